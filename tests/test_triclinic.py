"""Triclinic boxes (lmff_set_box with LAMMPS's tilt factors xy, xz, yz) against the
reference run on the same cells (tests/golden/tri_*.npz): an AB bilayer in a hexagonal
cell, four layers with B/N in a cell periodic in z with all three tilts, and a 24-atom
cell much smaller than the neighbour cutoff.  lmff_compute evaluates a triclinic cell
through the subdomain form on the cell's atoms and their periodic images; the images'
shares of forces, per-atom energies and per-atom virials are folded into their owners.

Bars as the orthogonal parity tests: FP64 1e-10 (max-norm relative), mixed max |dF| <=
1e-5 eV/A, energies 1e-6 and virial 1e-5 relative; per-atom virial 1e-10 in the FP64
mode, max |dW| <= 1e-4 eV in the mixed mode (its interlayer shares take the pair
kernel's FP32 form)."""
import numpy as np
import pytest
from conftest import ILP, TERSOFF, load_golden, rel_max, rel_rms

from lmff_gb300 import build, capi

pytestmark = pytest.mark.gpu

F64_TOL = 1e-10
MIX_F_ABS = 1e-5
MIX_E_REL = 1e-6
MIX_W_REL = 1e-5
NAMES = ["tri_bilayer", "tri_tilted_bn", "tri_small"]


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _engine(g, precision=capi.FP64):
    eng = capi.Engine(TERSOFF, ILP, tap_flag=int(g["tap_flag"]), precision=precision)
    eng.set_box(g["box_lo"], g["box_hi"], g["periodic"], g["tilt"])
    return eng


@pytest.mark.parametrize("name", NAMES)
def test_fp64_triclinic_matches_reference(name):
    g = load_golden(name)
    r = _engine(g).compute(g["x"], g["type"], g["mol"], g["tag"], eatom=True, vatom=True)
    assert rel_max(r["f"], g["f"]) <= F64_TOL and rel_rms(r["f"], g["f"]) <= F64_TOL
    assert abs(r["e_tersoff"] - g["e_tersoff"]) <= F64_TOL * abs(g["e_tersoff"])
    assert abs(r["e_ilp"] - g["e_ilp"]) <= F64_TOL * abs(g["e_ilp"])
    assert rel_max(r["pvector"], g["pvector"]) <= F64_TOL
    assert rel_max(r["virial"], g["virial"]) <= F64_TOL
    assert rel_max(r["eatom"], g["eatom"]) <= F64_TOL
    assert rel_max(r["vatom_tersoff"], g["vatom_tersoff"]) <= F64_TOL
    assert rel_max(r["vatom_ilp"], g["vatom_ilp"]) <= F64_TOL


@pytest.mark.parametrize("name", NAMES)
def test_mixed_triclinic_matches_reference(name):
    g = load_golden(name)
    r = _engine(g, capi.MIXED).compute(g["x"], g["type"], g["mol"], g["tag"], vatom=True)
    assert np.abs(r["f"] - g["f"]).max() <= MIX_F_ABS
    assert abs(r["e_tersoff"] - g["e_tersoff"]) <= MIX_E_REL * abs(g["e_tersoff"])
    assert abs(r["e_ilp"] - g["e_ilp"]) <= MIX_E_REL * abs(g["e_ilp"])
    assert rel_max(r["virial"], g["virial"]) <= MIX_W_REL
    assert np.abs(r["vatom"] - (g["vatom_tersoff"] + g["vatom_ilp"])).max() <= 1e-4


def test_triclinic_atoms_outside_the_cell_are_wrapped():
    """Atoms given one or two lattice vectors away from the cell: the same forces, in the
    caller's order, accumulated into f (OVERWRITE off)."""
    g = load_golden("tri_tilted_bn")
    lx, ly, lz = g["box_hi"] - g["box_lo"]
    xy, xz, yz = g["tilt"]
    col = np.array([[lx, 0, 0], [xy, ly, 0], [xz, yz, lz]])
    rng = np.random.default_rng(9)
    sh = rng.integers(-2, 3, size=(len(g["tag"]), 3))
    perm = rng.permutation(len(g["tag"]))
    x = (g["x"] + sh @ col)[perm]
    f0 = np.full((len(perm), 3), 0.25)
    r = _engine(g).compute(x, g["type"][perm], g["mol"][perm], g["tag"][perm], f=f0.copy())
    assert rel_max(r["f"] - 0.25, g["f"][perm]) <= F64_TOL


def test_triclinic_box_is_refused_by_the_other_calls_and_can_be_left():
    g = load_golden("tri_small")
    eng = _engine(g)
    eng.compute(g["x"], g["type"], g["mol"], g["tag"])
    with pytest.raises(capi.LmffError) as e:
        eng.compute_resident()
    assert e.value.code == -8    # LMFF_EUNSUPPORTED
    o = load_golden("bilayer_small")
    eng2 = capi.Engine(TERSOFF, ILP, tap_flag=int(o["tap_flag"]))
    eng2.set_box(g["box_lo"], g["box_hi"], g["periodic"], g["tilt"])
    eng2.compute(g["x"], g["type"], g["mol"], g["tag"])
    eng2.set_box(o["box_lo"], o["box_hi"], o["periodic"])    # back to an orthogonal box
    r = eng2.compute(o["x"], o["type"], o["mol"], o["tag"])
    assert rel_max(r["f"], o["f"]) <= F64_TOL
