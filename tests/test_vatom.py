"""Per-atom virial (lmff_compute_vatom, the LAMMPS styles' vflag_atom) against the
reference: each style's Pair::vatom as its ev_tally / ev_tally_xyz / v_tally3 calls split
it (pair_tersoff.cpp:173, :223, :253; pair_ilp_graphene_hbn.cpp:536, :667, :671;
pair_kolmogorov_crespi_full.cpp:536, :668, :675), from the reference harness's fixtures
(tests/golden/*.npz, vatom_tersoff / vatom_ilp, ghost rows folded into their owners).

Bars: Tersoff's shares come from an FP64 pass in either precision mode, max-norm relative
error <= 1e-10; the interlayer shares are FP64 in the FP64 mode (1e-10) and in the mixed
mode take the pair kernel's FP32 form with FP64 sums, max |dW| <= 1e-4 eV per component
(the per-atom counterpart of the 1e-5 eV/A force bar: pair forces times separations of a
few A)."""
import os

import numpy as np
import pytest
from conftest import GOLDEN_VATOM, ILP, POT, TERSOFF, load_golden, rel_max

from lmff_gb300 import build, capi

pytestmark = pytest.mark.gpu

TOL = 1e-10
MIX_VA_ABS = 1e-4
KC = os.path.join(POT, "CC.KC-full")
EINVAL = -1
BOTH = capi.TERSOFF | capi.ILP


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _engine(g, precision, kc=False, **opts):
    if kc:
        eng = capi.Engine(TERSOFF, None, elements=("C", "B", "N"), ilp_elements=("C", "NULL", "NULL"), kc_file=KC,
                          tap_flag=int(g["tap_flag"]), precision=precision)
    else:
        eng = capi.Engine(TERSOFF, ILP, cut_global=float(g["cut_global"]), tap_flag=int(g["tap_flag"]),
                          skin=float(g["skin"]), precision=precision)
    for k, v in opts.items():
        eng.set_option(k, v)
    eng.set_box(g["box_lo"], g["box_hi"], g["periodic"])
    return eng


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
@pytest.mark.parametrize("name", GOLDEN_VATOM + ["c1_t0"])
def test_vatom_matches_reference(name, precision):
    g = load_golden(name)
    r = _engine(g, precision).compute(g["x"], g["type"], g["mol"], g["tag"], vatom=True)
    assert rel_max(r["vatom_tersoff"], g["vatom_tersoff"]) <= TOL
    if precision == capi.FP64:
        assert rel_max(r["vatom_ilp"], g["vatom_ilp"]) <= TOL
    else:
        assert np.abs(r["vatom_ilp"] - g["vatom_ilp"]).max() <= MIX_VA_ABS


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
@pytest.mark.parametrize("name", ["kc_bilayer", "kc_bilayer_notaper"])
def test_vatom_kolmogorov_crespi_matches_reference(name, precision):
    g = load_golden(name)
    r = _engine(g, precision, kc=True).compute(g["x"], g["type"], g["mol"], g["tag"], vatom=True)
    assert rel_max(r["vatom_tersoff"], g["vatom_tersoff"]) <= TOL
    if precision == capi.FP64:
        assert rel_max(r["vatom_ilp"], g["vatom_ilp"]) <= TOL
    else:
        assert np.abs(r["vatom_ilp"] - g["vatom_ilp"]).max() <= MIX_VA_ABS


def test_vatom_force_only_evaluation_and_overwrite():
    """After the force-only fast path (no energy, no virial), with an atom order that is
    not the tag order, and LMFF_OVERWRITE against accumulation."""
    g = load_golden("hetero_small")
    perm = np.random.default_rng(5).permutation(len(g["tag"]))
    eng = _engine(g, capi.MIXED)
    eng.compute(g["x"][perm], g["type"][perm], g["mol"][perm], g["tag"][perm], eflag=False, vflag=False)
    v = np.ones((len(perm), 6))
    capi._lib.lmff_compute_vatom(eng._h, BOTH, len(perm), capi._p(v))
    want = (g["vatom_tersoff"] + g["vatom_ilp"])[perm]
    assert np.abs(v - 1.0 - want).max() <= MIX_VA_ABS
    eng.compute(g["x"][perm], g["type"][perm], g["mol"][perm], g["tag"][perm], same_atoms=True)
    rc = capi._lib.lmff_compute_vatom(eng._h, BOTH | capi.OVERWRITE, len(perm), capi._p(v))
    assert rc == 0 and np.abs(v - want).max() <= MIX_VA_ABS


def test_vatom_needs_a_directly_preceding_evaluation():
    g = load_golden("bilayer_small")
    eng = _engine(g, capi.FP64)
    v = np.zeros((len(g["tag"]), 6))
    assert capi._lib.lmff_compute_vatom(eng._h, BOTH, len(v), capi._p(v)) == EINVAL
    eng.compute(g["x"], g["type"], g["mol"], g["tag"])
    assert capi._lib.lmff_compute_vatom(eng._h, BOTH, len(v) - 1, capi._p(v)) == EINVAL
    eng.compute(g["x"], g["type"], g["mol"], g["tag"])
    assert capi._lib.lmff_compute_vatom(eng._h, capi.TERSOFF, len(v), capi._p(v)) == 0
    assert capi._lib.lmff_compute_vatom(eng._h, capi.ILP, len(v), capi._p(v)) == 0    # the other style may follow
    assert rel_max(v, g["vatom_tersoff"] + g["vatom_ilp"]) <= TOL
    eng.set_option("count_pairs", 1)     # another call that runs on the device
    assert capi._lib.lmff_compute_vatom(eng._h, BOTH, len(v), capi._p(v)) == EINVAL
