"""The request server (lmff_server_*): batched single points equal the same systems
alone bit for bit, NVE requests in a mix match the same run alone, admission keeps the
admitted set within the device-memory budget, and a failing request fails alone.
The stream generator's properties are checked on the CPU."""
import numpy as np
import pytest
from conftest import ILP, TERSOFF, min_image, rel_max

from lmff_gb300 import build, capi, serve
from lmff_gb300 import structures as S


@pytest.fixture(scope="module")
def _built():
    build.build()


def _systems(count=5, seed=21):
    out = S.replica_set(count=count, nmin=600, nmax=4000, seed=seed)
    return [S.displace(s, 0.03, seed=k) for k, s in enumerate(out)]


def _bad_system():
    """An atom pushed onto a neighbour's bond: more than three intralayer neighbours."""
    s = S.ab_bilayer_graphene(8, 5)
    s.x[1] = s.x[0] + np.array([0.9, 0.0, 0.0])
    s.x[2] = s.x[0] + np.array([-0.9, 0.3, 0.0])
    s.x[3] = s.x[0] + np.array([0.0, -0.9, 0.0])
    s.x[4] = s.x[0] + np.array([0.2, 0.9, 0.0])
    return s


def _alone_md(s, nsteps, precision):
    eng = capi.Engine(TERSOFF, ILP, precision=precision)
    eng.upload(s)
    th = eng.run_nve(nsteps, 0.001, thermo_every=nsteps)
    x, v, f = eng.download()
    return x, v, f, th[-1]


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [capi.FP64, capi.MIXED])
def test_points_in_a_batch_are_bitwise_the_points_alone(_built, prec):
    systems = _systems()
    srv = serve.Server(capi.Engine(TERSOFF, ILP, precision=prec))
    tickets = srv.submit_many([(s, 0) for s in systems])
    res = [srv.wait(t) for t in tickets]
    st = srv.stats()
    srv.close()
    assert st["point_batches"] == 1 and st["point_systems"] == len(systems)
    for s, r in zip(systems, res):
        alone = capi.Engine(TERSOFF, ILP, precision=prec).compute_system(s)
        assert np.array_equal(r["f"], alone["f"])
        assert r["e_ilp"] == alone["e_ilp"] and r["e_tersoff"] == alone["e_tersoff"]
        assert np.array_equal(r["virial"], alone["virial"])


@pytest.mark.gpu
def test_nve_requests_in_a_mix_match_the_runs_alone(_built):
    """Three NVE requests of different lengths and two single points in one stream: the
    NVE batch re-forms when the shortest finishes.  FP64: the batch shares list rebuilds,
    so only the summation order differs from the run alone."""
    systems = [S.thermalize(s, 300.0, seed=5 + k) for k, s in enumerate(_systems(3, seed=33))]
    lengths = [15, 40, 27]
    points = _systems(2, seed=44)
    srv = serve.Server(capi.Engine(TERSOFF, ILP), md_chunk_steps=10)
    tickets = srv.submit_many([(s, n) for s, n in zip(systems, lengths)] + [(p, 0) for p in points])
    res = [srv.wait(t) for t in tickets]
    st = srv.stats()
    srv.close()
    assert st["md_reforms"] >= 3 and st["completed"] == 5
    for s, n, r in zip(systems, lengths, res):
        x, v, f, th = _alone_md(s, n, capi.FP64)
        assert np.abs(min_image(r["x"] - x, s.box_lo, s.box_hi, s.periodic)).max() < 1e-9
        assert rel_max(r["v"], v) < 1e-7 and rel_max(r["f"], f) < 1e-7
        assert abs(r["e_ilp"] + r["e_tersoff"] - th["pe"]) <= 1e-10 * abs(th["pe"])
    for p, r in zip(points, res[3:]):
        alone = capi.Engine(TERSOFF, ILP).compute_system(p)
        assert np.array_equal(r["f"], alone["f"])


@pytest.mark.gpu
def test_admission_keeps_the_admitted_set_within_the_budget(_built):
    systems = _systems(6, seed=55)
    bpa = 8192.0
    budget = 1.2 * bpa * max(s.n for s in systems)   # about one request at a time
    srv = serve.Server(capi.Engine(TERSOFF, ILP), hbm_budget_bytes=budget, bytes_per_atom=bpa)
    tickets = srv.submit_many([(s, 0) for s in systems])
    res = [srv.wait(t) for t in tickets]
    st = srv.stats()
    assert st["max_admitted_bytes"] <= budget
    # FIFO admission: each batch is the longest prefix of the queue that fits the budget
    expected, cur = 1, 0.0
    for s in systems:
        if cur > 0 and cur + bpa * s.n > budget:
            expected, cur = expected + 1, 0.0
        cur += bpa * s.n
    assert expected >= 2 and st["point_batches"] == expected
    for s, r in zip(systems, res):
        assert np.array_equal(r["f"], capi.Engine(TERSOFF, ILP).compute_system(s)["f"])
    big = S.ab_bilayer_graphene(60, 40)
    with pytest.raises(capi.LmffError) as ei:
        srv.submit(big)
    assert ei.value.code == -9 and "budget" in str(ei.value)
    srv.close()


@pytest.mark.gpu
def test_a_failing_request_fails_alone(_built):
    good = _systems(3, seed=66)
    bad = _bad_system()
    md_good = S.thermalize(good[0], 300.0, seed=3)
    srv = serve.Server(capi.Engine(TERSOFF, ILP), md_chunk_steps=5)
    tickets = srv.submit_many([(good[1], 0), (bad, 0), (good[2], 0), (md_good, 12), (bad, 12)])
    out = []
    for t in tickets:
        try:
            out.append(srv.wait(t))
        except capi.LmffError as e:
            out.append(e)
    srv.close()
    assert isinstance(out[1], capi.LmffError) and out[1].code == -4
    assert isinstance(out[4], capi.LmffError) and out[4].code == -4
    for s, r in ((good[1], out[0]), (good[2], out[2])):
        assert np.array_equal(r["f"], capi.Engine(TERSOFF, ILP).compute_system(s)["f"])
    x, v, f, th = _alone_md(md_good, 12, capi.FP64)
    assert np.abs(min_image(out[3]["x"] - x, md_good.box_lo, md_good.box_hi, md_good.periodic)).max() < 1e-9


def test_poisson_stream_is_seeded_and_shaped():
    a = serve.poisson_stream(count=60, rate=200.0, nmin=1000, nmax=20000, sizes=6, seed=3)
    b = serve.poisson_stream(count=60, rate=200.0, nmin=1000, nmax=20000, sizes=6, seed=3)
    assert [it.t_arrival for it in a] == [it.t_arrival for it in b]
    assert all(np.array_equal(p.system.x, q.system.x) for p, q in zip(a, b))
    t = np.array([it.t_arrival for it in a])
    assert np.all(np.diff(t) > 0) and 0.1 < t[-1] < 0.6          # 60 arrivals at 200/s
    n = np.array([it.system.n for it in a])
    assert n.min() >= 900 and n.max() <= 22000
    md = [it for it in a if it.nsteps > 0]
    assert 5 <= len(md) <= 35 and all(it.nsteps == 100 and it.system.v is not None for it in md)
    kinds = {int(it.system.type.max()) for it in a}
    assert kinds == {1, 3}                                        # graphene/graphene and graphene/hBN
