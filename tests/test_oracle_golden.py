"""The oracle restatement against the reference's own outputs (tests/golden/*.npz, made by
tests/golden/make_golden.py from the reference sources).  This pins the oracle: every GPU
parity test compares the engine with it."""
import numpy as np
import pytest
from conftest import GOLDEN_LISTS, GOLDEN_SINGLE, GOLDEN_VATOM, ILP, TERSOFF, load_golden, min_image, rel_max, rel_rms

from oracle import Oracle

TOL = 1e-12    # forces, virial: the two reference implementations agree to ~1e-12
E_TOL = 1e-10  # energies: the reference sums ~1e6 pair terms serially into one running
               # total, so its own rounding reaches ~1e-11 relative on the 7,200-atom case


def _oracle_for(g):
    o = Oracle(TERSOFF, ILP, cut_global=float(g["cut_global"]), tap_flag=int(g["tap_flag"]),
               skin=float(g["skin"]), nthreads=4)
    o.set_atoms(g["x"], g["type"], g["mol"], g["tag"], g["box_lo"], g["box_hi"], g["periodic"])
    return o


@pytest.mark.parametrize("name", GOLDEN_SINGLE)
def test_oracle_matches_reference(name):
    g = load_golden(name)
    o = _oracle_for(g)
    r = o.forces(eatom=True)
    assert rel_max(r["f"], g["f"]) < TOL
    assert rel_rms(r["f"], g["f"]) < TOL
    assert abs(r["e_tersoff"] - g["e_tersoff"]) <= E_TOL * abs(g["e_tersoff"])
    assert abs(r["e_ilp"] - g["e_ilp"]) <= E_TOL * abs(g["e_ilp"])
    assert rel_max(r["pvector"], g["pvector"]) < E_TOL
    assert rel_max(r["virial"], g["virial"]) < TOL
    assert rel_max(r["eatom"], g["eatom"]) < TOL


@pytest.mark.parametrize("name", GOLDEN_VATOM)
def test_oracle_per_atom_virial_matches_reference(name):
    """Each style's per-atom virial as the reference's ev_tally / ev_tally_xyz / v_tally3
    calls split it (pair_tersoff.cpp:173,223,253; pair_ilp_graphene_hbn.cpp:536,667,671),
    ghost shares folded into their owners."""
    g = load_golden(name)
    r = _oracle_for(g).forces(vatom=True)
    assert rel_max(r["vatom_tersoff"], g["vatom_tersoff"]) < TOL
    assert rel_max(r["vatom_ilp"], g["vatom_ilp"]) < TOL


def periodic_images(x, lo, hi, tilt, periodic, cut):
    """The atoms of a triclinic periodic cell wrapped into it by whole lattice vectors,
    then every image whose fractional coordinate lies within `cut` of the cell along each
    periodic edge (domain.cpp h / h_inv; the images a LAMMPS rank holds as ghosts).
    Returns the positions and each one's owner index (owners first)."""
    lx, ly, lz = np.asarray(hi) - np.asarray(lo)
    xy, xz, yz = tilt
    col = np.array([[lx, 0, 0], [xy, ly, 0], [xz, yz, lz]])
    rows = np.array([[1 / lx, -xy / (lx * ly), (xy * yz - ly * xz) / (lx * ly * lz)], [0, 1 / ly, -yz / (ly * lz)],
                     [0, 0, 1 / lz]])
    per = np.asarray(periodic, bool)
    lam = (x - lo) @ rows.T
    s = np.where(per, np.floor(lam), 0.0)
    xw, lam = x - s @ col, lam - s
    cl = cut * np.linalg.norm(rows, axis=1)
    K = [int(np.ceil(cl[d])) if per[d] else 0 for d in range(3)]
    xs, own = [xw], [np.arange(len(x))]
    for sh in np.stack(np.meshgrid(*[np.arange(-k, k + 1) for k in K], indexing="ij"), -1).reshape(-1, 3):
        if not sh.any():
            continue
        ok = np.all([(lam[:, d] + sh[d] >= -cl[d]) & (lam[:, d] + sh[d] < 1 + cl[d]) if per[d] else
                     np.ones(len(x), bool) for d in range(3)], axis=0)
        xs.append(xw[ok] + sh @ col)
        own.append(np.nonzero(ok)[0])
    return np.concatenate(xs), np.concatenate(own)


@pytest.mark.parametrize("name", ["tri_bilayer", "tri_tilted_bn", "tri_small"])
def test_triclinic_fixtures_match_the_oracle_on_explicit_images(name):
    """The reference's triclinic cells (tilt xy; xy, xz, yz with z periodic; a cell
    smaller than the cutoff) against the oracle on a non-periodic system of the cell's
    atoms and their images 40 A deep: the forces on the cell's atoms agree."""
    g = load_golden(name)
    xa, own = periodic_images(g["x"], g["box_lo"], g["box_hi"], g["tilt"], g["periodic"], 40.0)
    o = Oracle(TERSOFF, ILP, tap_flag=int(g["tap_flag"]), nthreads=4)
    o.set_atoms(xa, g["type"][own], g["mol"][own], g["tag"][own], xa.min(0) - 5.0, xa.max(0) + 5.0, [0, 0, 0])
    n = len(g["tag"])
    assert rel_max(o.forces()["f"][:n], g["f"]) < TOL


def _set(a):
    return set(map(tuple, np.asarray(a).reshape(-1, 3).tolist()))


@pytest.mark.parametrize("name", GOLDEN_LISTS)
def test_oracle_lists_match_reference(name):
    g = load_golden(name)
    o = _oracle_for(g)
    assert _set(o.full_list()) == _set(g["nlist"])
    assert _set(o.ilp_list()) == _set(g["ilplist"])


def test_oracle_nve_trajectory_matches_reference():
    """100 velocity-Verlet steps of the 7,200-atom bilayer from the reference's own start."""
    g = load_golden("c1_t100")
    o = Oracle(TERSOFF, ILP, nthreads=8)
    x = g["x0"].copy()
    v = g["v0"].copy()
    o.set_atoms(x, g["type"], g["mol"], g["tag"], g["box_lo"], g["box_hi"], g["periodic"])
    f = o.forces()["f"]
    o.nve(100, 0.001, [12.011, 10.811, 14.0067], x, v, f)
    dx = min_image(x - g["x"], g["box_lo"], g["box_hi"], g["periodic"])
    assert np.abs(dx).max() < 1e-9
    assert rel_max(v, g["v"]) < 1e-8
    assert rel_max(f, g["f"]) < 1e-8


def test_oracle_edges_cover_all_normal_cases():
    """The edge fixture has atoms with 0, 1, 2 and 3 intralayer neighbours."""
    g = load_golden("edges")
    il = g["ilplist"]
    counts = np.bincount(il[:, 0], minlength=int(g["tag"].max()) + 1)[g["tag"]]
    assert set(np.unique(counts)) >= {0, 1, 2, 3}
