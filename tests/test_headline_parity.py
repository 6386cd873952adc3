"""The benchmarked workloads themselves against the oracle (the CPU restatement of the
reference, pinned to the reference binary by tests/test_oracle_golden.py).

- The 10-layer AB graphite slab with alternating molecule ids and 3.35 A spacing (the
  2.7M-atom benchmark's environment: ~937 list entries per atom, odd layer separations
  interacting), as the 36,800-atom periodic patch that the benchmark's CPU baseline
  times (bench.cpu_sample), with an N(0, 0.03 A) displacement on top of its 300 K
  state.
- A commensurate graphene/hBN bilayer with the twisted-heterostructure workload's
  parameters (0.6 degree twist, hBN B-N 1.45 A, 3.4 A spacing, N(0, 0.02 A) per-atom
  displacement), small enough for the oracle.

Bars: FP64 1e-10 (max-norm relative forces, RMS forces, per-style energies, pvector,
virial, per-atom energy); mixed max |dF| <= 1e-5 eV/A, energies <= 1e-6 relative,
virial <= 1e-5 relative.  Both the energy/virial kernels and the force-only kernels of
an MD step are checked.
"""
import os

import numpy as np
import pytest
from conftest import ILP, TERSOFF, rel_max, rel_rms

from lmff_gb300 import build, capi
from lmff_gb300 import structures as S

pytestmark = pytest.mark.gpu

F64_TOL = 1e-10
MIX_F_ABS = 1e-5
MIX_E_REL = 1e-6
MIX_W_REL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _graphite_patch():
    import bench
    return S.displace(bench.cpu_sample(), 0.03, seed=21)


def _twisted_hetero():
    s = S.twisted_bilayer(60, 35, 0.6, top="hbn", spacing=3.4)
    assert s.meta["strain_max"] < 0.02
    return S.displace(s, 0.02, seed=22)


# workload -> (builder, type -> element map as the benchmark gives it: pure carbon maps
# its one type to C, which selects the single-element pair loops)
_CASES = {"graphite_10layer_alt_36800": (_graphite_patch, ("C",)),
          "twisted_graphene_hbn_0p6deg": (_twisted_hetero, ("C", "B", "N"))}
_REF = {}


def _oracle(name):
    if name not in _REF:
        from oracle import Oracle
        build_fn, elements = _CASES[name]
        s = build_fn()
        o = Oracle(TERSOFF, ILP, elements=elements, nthreads=os.cpu_count() or 1)
        o.set_system(s)
        _REF[name] = (s, o.forces(eatom=True, vatom=True))
    return _REF[name]


def _engine(name, **kw):
    return capi.Engine(TERSOFF, ILP, elements=_CASES[name][1], **kw)


@pytest.mark.parametrize("name", sorted(_CASES))
def test_fp64_matches_oracle_on_benchmark_workloads(name):
    s, ref = _oracle(name)
    got = _engine(name).compute_system(s, eatom=True)
    assert rel_max(got["f"], ref["f"]) <= F64_TOL
    assert rel_rms(got["f"], ref["f"]) <= F64_TOL
    assert abs(got["e_tersoff"] - ref["e_tersoff"]) <= F64_TOL * abs(ref["e_tersoff"])
    assert abs(got["e_ilp"] - ref["e_ilp"]) <= F64_TOL * abs(ref["e_ilp"])
    assert rel_max(got["pvector"], ref["pvector"]) <= F64_TOL
    assert rel_max(got["virial"], ref["virial"]) <= F64_TOL
    assert rel_max(got["eatom"], ref["eatom"]) <= F64_TOL


@pytest.mark.parametrize("name", sorted(_CASES))
def test_mixed_matches_oracle_on_benchmark_workloads(name):
    s, ref = _oracle(name)
    got = _engine(name, precision=capi.MIXED).compute_system(s, eatom=True)
    assert np.abs(got["f"] - ref["f"]).max() <= MIX_F_ABS
    assert abs(got["e_tersoff"] - ref["e_tersoff"]) <= MIX_E_REL * abs(ref["e_tersoff"])
    assert abs(got["e_ilp"] - ref["e_ilp"]) <= MIX_E_REL * abs(ref["e_ilp"])
    assert rel_max(got["pvector"], ref["pvector"]) <= MIX_E_REL
    assert rel_max(got["virial"], ref["virial"]) <= MIX_W_REL


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
@pytest.mark.parametrize("name", sorted(_CASES))
def test_vatom_matches_oracle_on_benchmark_workloads(name, precision):
    """Per-atom virial at 1e-10 per style (Tersoff an FP64 pass in either mode; the
    interlayer shares in the mixed mode at max |dW| <= 1e-4 eV); with three intralayer
    neighbours for every atom each style's per-atom virials sum to its fdotr virial (the
    reference leaves out only the dn_i/dx_i term of atoms with two): 1e-9, the mixed
    interlayer sum at the mixed virial bar."""
    s, ref = _oracle(name)
    got = _engine(name, precision=precision).compute_system(s, vatom=True)
    assert rel_max(got["vatom_tersoff"], ref["vatom_tersoff"]) <= F64_TOL
    assert rel_max(got["vatom_tersoff"].sum(0), ref["virial_tersoff"]) <= 1e-9
    if precision == capi.FP64:
        assert rel_max(got["vatom_ilp"], ref["vatom_ilp"]) <= F64_TOL
        assert rel_max(got["vatom_ilp"].sum(0), ref["virial_ilp"]) <= 1e-9
    else:
        assert np.abs(got["vatom_ilp"] - ref["vatom_ilp"]).max() <= 1e-4
        assert rel_max(got["vatom_ilp"].sum(0), ref["virial_ilp"]) <= MIX_W_REL


@pytest.mark.parametrize("name", sorted(_CASES))
@pytest.mark.parametrize("tpa", [8, 16])
def test_mixed_force_only_matches_oracle_on_benchmark_workloads(name, tpa):
    """The kernels an MD step runs (no energy, no virial) at the benchmark's launch shapes."""
    s, ref = _oracle(name)
    eng = _engine(name, precision=capi.MIXED)
    eng.set_option("tpa", tpa)
    got = eng.compute_system(s, eflag=False, vflag=False)
    assert np.abs(got["f"] - ref["f"]).max() <= MIX_F_ABS
