"""Structure generators (host logic): counts, geometry and seeded determinism."""
import numpy as np

from lmff_gb300 import structures as S


def test_c1_bilayer_geometry():
    s = S.ab_bilayer_graphene(30, 30)
    assert s.n == 7200
    assert np.allclose(s.box_hi[:2] - s.box_lo[:2], [73.79, 127.80], atol=0.01)
    assert set(np.unique(s.mol)) == {1, 2}
    z = np.unique(np.round(s.x[:, 2], 6))
    assert np.allclose(z, [0.0, 3.4])


def test_bond_lengths_and_coordination():
    s = S.ab_bilayer_graphene(6, 6)
    lay = s.x[s.mol == 1]
    L = s.box_hi - s.box_lo
    d = lay[:, None, :] - lay[None, :, :]
    d[..., :2] -= L[:2] * np.rint(d[..., :2] / L[:2])
    r = np.sqrt((d ** 2).sum(-1))
    nn = ((r > 0.1) & (r < 1.5)).sum(1)
    assert np.all(nn == 3)
    assert np.allclose(r[(r > 0.1) & (r < 1.5)], 1.42, atol=1e-9)


def test_graphite_slab_counts():
    s = S.graphite_slab(3, 8, 5, mol_mode="alternate")
    assert s.n == 3 * 160
    assert list(np.unique(s.mol)) == [1, 2]
    s2 = S.graphite_slab(3, 8, 5, mol_mode="unique")
    assert list(np.unique(s2.mol)) == [1, 2, 3]


def test_twisted_hbn_strain_reported_and_small():
    s = S.twisted_bilayer(40, 23, 0.6, top="hbn")
    assert s.meta["strain_max"] < 0.03
    assert set(np.unique(s.type)) == {1, 2, 3}


def test_replica_set_seeded():
    a = S.replica_set(count=6, seed=3)
    b = S.replica_set(count=6, seed=3)
    for s, t in zip(a, b):
        assert s.n == t.n and np.array_equal(s.x, t.x)
        assert np.all(s.box_hi[:2] - s.box_lo[:2] >= 20.0)
        assert 400 <= s.n <= 25000


def test_thermalize_exact_temperature():
    s = S.thermalize(S.ab_bilayer_graphene(8, 5), 300.0, seed=5)
    m = s.masses()
    ke = 0.5 * S.MVV2E_METAL * (m[:, None] * s.v ** 2).sum()
    t = 2 * ke / ((3 * s.n - 3) * S.BOLTZ_METAL)
    assert abs(t - 300.0) < 1e-9
    assert np.allclose((m[:, None] * s.v).sum(0), 0.0, atol=1e-9)
