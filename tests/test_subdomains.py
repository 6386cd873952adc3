"""Subdomain mode (lmff_compute_ghost): the system split over ranks as LAMMPS's brick
decomposition does, each rank's owned atoms plus the ghost atoms within the ghost
cutoff (cut_global + skin) of its subdomain, periodic images included.  Each subdomain
is evaluated on its own; folding the ghosts' forces and per-atom energies back onto
their owners (LAMMPS's reverse communication) and summing energies, pvector and virial
over the subdomains must give the reference's whole-system result (the golden
fixtures, made by the reference itself).

Bars as in tests/test_gpu_parity.py: FP64 1e-10 (max-norm relative), mixed 1e-5 eV/A.
"""
import itertools

import numpy as np
import pytest
from conftest import ILP, TERSOFF, load_golden, rel_max

from lmff_gb300 import build, capi

pytestmark = pytest.mark.gpu

F64_TOL = 1e-10
MIX_F_ABS = 1e-5
MIX_E_REL = 1e-6
MIX_W_REL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def decompose(x, lo, hi, periodic, splits, cutghost):
    """Brick decomposition of the atoms x (wrapped into the box on periodic dims):
    for each subdomain the caller indices of its owned atoms and of its ghosts with
    their positions (images shifted by whole box lengths).  Owned atoms come first."""
    lo, hi = np.asarray(lo, float), np.asarray(hi, float)
    L = hi - lo
    x = np.array(x, float)
    for d in range(3):
        if periodic[d]:
            x[:, d] = lo[d] + np.mod(x[:, d] - lo[d], L[d])
    edges = [np.linspace(lo[d], hi[d], splits[d] + 1) for d in range(3)]
    cell = np.stack([np.clip(np.searchsorted(edges[d], x[:, d], side="right") - 1, 0, splits[d] - 1)
                     for d in range(3)], axis=1)
    reach = [int(np.ceil(cutghost / L[d])) + 1 if periodic[d] else 0 for d in range(3)]
    shifts = list(itertools.product(*[range(-r, r + 1) for r in reach]))
    out = []
    for c in itertools.product(*[range(n) for n in splits]):
        slo = np.array([edges[d][c[d]] for d in range(3)])
        shi = np.array([edges[d][c[d] + 1] for d in range(3)])
        own = np.nonzero((cell == np.array(c)).all(axis=1))[0]
        gidx, gx = [], []
        for s in shifts:
            y = x + np.array(s) * L
            inside = np.ones(len(x), bool)
            for d in range(3):
                inside &= (y[:, d] >= slo[d] - cutghost) & (y[:, d] < shi[d] + cutghost)
            if s == (0, 0, 0):
                inside[own] = False
            sel = np.nonzero(inside)[0]
            gidx.append(sel)
            gx.append(y[sel])
        gidx = np.concatenate(gidx)
        gx = np.concatenate(gx)
        out.append((own, np.vstack([x[own], gx]), np.concatenate([own, gidx])))
    return out


def run_decomposed(g, splits, precision=capi.FP64, eatom=True, engine=None, x=None):
    eng = engine or capi.Engine(TERSOFF, ILP, cut_global=float(g["cut_global"]), tap_flag=int(g["tap_flag"]),
                                skin=float(g["skin"]), precision=precision)
    x = g["x"] if x is None else x
    n = len(g["tag"])
    f = np.zeros((n, 3))
    ea = np.zeros(n)
    tot = {"e_tersoff": 0.0, "e_ilp": 0.0, "pvector": np.zeros(2), "virial": np.zeros(6)}
    cutghost = float(g["cut_global"]) + float(g["skin"])
    for own, xs, idx in decompose(x, g["box_lo"], g["box_hi"], g["periodic"], splits, cutghost):
        r = eng.compute_ghost(len(own), xs, g["type"][idx], g["mol"][idx], g["tag"][idx], eatom=eatom)
        np.add.at(f, idx, r["f"])                 # reverse communication: fold ghost forces
        if eatom:
            np.add.at(ea, idx, r["eatom"])
        for k in ("e_tersoff", "e_ilp"):
            tot[k] += r[k]
        tot["pvector"] += r["pvector"]
        tot["virial"] += r["virial"]
    tot["f"], tot["eatom"] = f, ea
    return tot


CASES = [("bilayer_small", (2, 1, 1)), ("hetero_small", (2, 2, 1)), ("tiny_images", (2, 1, 1)),
         ("trilayer_alt", (1, 2, 1)), ("edges", (2, 1, 1)), ("c1_t0", (2, 2, 1))]


@pytest.mark.parametrize("name,splits", CASES)
def test_fp64_subdomains_sum_to_reference(name, splits):
    g = load_golden(name)
    r = run_decomposed(g, splits)
    assert rel_max(r["f"], g["f"]) <= F64_TOL
    assert abs(r["e_tersoff"] - g["e_tersoff"]) <= F64_TOL * abs(g["e_tersoff"])
    assert abs(r["e_ilp"] - g["e_ilp"]) <= F64_TOL * abs(g["e_ilp"])
    assert rel_max(r["pvector"], g["pvector"]) <= F64_TOL
    assert rel_max(r["virial"], g["virial"]) <= F64_TOL
    assert rel_max(r["eatom"], g["eatom"]) <= F64_TOL


@pytest.mark.parametrize("name,splits", [("hetero_small", (2, 2, 1)), ("c1_t0", (2, 2, 1)), ("edges", (2, 1, 1))])
def test_mixed_subdomains_sum_to_reference(name, splits):
    g = load_golden(name)
    r = run_decomposed(g, splits, precision=capi.MIXED)
    assert np.abs(r["f"] - g["f"]).max() <= MIX_F_ABS
    assert abs(r["e_tersoff"] - g["e_tersoff"]) <= MIX_E_REL * abs(g["e_tersoff"])
    assert abs(r["e_ilp"] - g["e_ilp"]) <= MIX_E_REL * abs(g["e_ilp"])
    assert rel_max(r["virial"], g["virial"]) <= MIX_W_REL


def test_one_subdomain_equals_periodic_mode():
    """One rank owning every atom, the periodic images as ghosts: the same forces,
    energies and virial as the periodic-system call."""
    g = load_golden("trilayer_alt")
    r = run_decomposed(g, (1, 1, 1))
    eng = capi.Engine(TERSOFF, ILP, cut_global=float(g["cut_global"]), tap_flag=int(g["tap_flag"]),
                      skin=float(g["skin"]))
    eng.set_box(g["box_lo"], g["box_hi"], g["periodic"])
    p = eng.compute(g["x"], g["type"], g["mol"], g["tag"], eatom=True)
    assert rel_max(r["f"], p["f"]) <= 1e-12
    assert abs(r["e_ilp"] - p["e_ilp"]) <= 1e-12 * abs(p["e_ilp"])
    assert rel_max(r["virial"], p["virial"]) <= 1e-12


def test_same_atoms_reuse_and_mode_switch():
    """Consecutive calls on the same subdomain atoms (LAMMPS between reneighbourings)
    reuse the engine's lists; a periodic-system call is refused until lmff_set_box."""
    g = load_golden("bilayer_small")
    eng = capi.Engine(TERSOFF, ILP, cut_global=float(g["cut_global"]), tap_flag=int(g["tap_flag"]),
                      skin=float(g["skin"]))
    (own, xs, idx), = decompose(g["x"], g["box_lo"], g["box_hi"], g["periodic"], (1, 1, 1), 18.0)
    r0 = eng.compute_ghost(len(own), xs, g["type"][idx], g["mol"][idx], g["tag"][idx])
    nb = eng.stats()["rebuilds"]
    xs2 = xs + np.random.default_rng(3).normal(0.0, 0.01, xs.shape)
    r1 = eng.compute_ghost(len(own), xs2, g["type"][idx], g["mol"][idx], g["tag"][idx], same_atoms=True)
    assert eng.stats()["rebuilds"] == nb
    fresh = capi.Engine(TERSOFF, ILP, cut_global=float(g["cut_global"]), tap_flag=int(g["tap_flag"]),
                        skin=float(g["skin"])).compute_ghost(len(own), xs2, g["type"][idx], g["mol"][idx],
                                                             g["tag"][idx])
    assert rel_max(r1["f"], fresh["f"]) <= 1e-12
    assert not np.array_equal(r0["f"], r1["f"])
    with pytest.raises(capi.LmffError):
        eng.compute(g["x"], g["type"], g["mol"], g["tag"])
    eng.set_box(g["box_lo"], g["box_hi"], g["periodic"])
    p = eng.compute(g["x"], g["type"], g["mol"], g["tag"])
    assert rel_max(p["f"], g["f"]) <= F64_TOL
