"""The allocation-free entry point, lmff_compute_device_noalloc, called through the C ABI.

It serves callers that must not allocate device memory while they run (an application
that gives all GPU memory to its own pool at start-up, or a code path where cudaMalloc
is not allowed).  Its results must equal those of the regular device entry point,
lmff_compute_device, and the reference's own outputs (the golden fixtures), within the
parity tolerances used everywhere else in the tests, and must stay equal when it is
called twice in a row: the second call reuses the same static scratch array that the
first call left behind.  The call must also leave the device's free memory unchanged.
"""
import numpy as np
import pytest
from conftest import ILP, TERSOFF, load_golden, rel_max

from lmff_gb300 import build, capi

pytestmark = pytest.mark.gpu

F64_TOL = 1e-10   # the FP64 parity bar of tests/test_gpu_parity.py
MIX_F_ABS = 1e-5  # the mixed-precision force bar of tests/test_gpu_parity.py
MIX_E_REL = 1e-6
MIX_W_REL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _inputs(g):
    import torch
    x = torch.tensor(g["x"], dtype=torch.float64, device="cuda")
    t = torch.tensor(g["type"], dtype=torch.int32, device="cuda")
    m = torch.tensor(g["mol"], dtype=torch.int64, device="cuda")
    return x, t, m


def _check(got_f, got, ref_f, ref, precision, what):
    """Forces, per-style energies, pvector and virial against a reference result."""
    if precision == capi.FP64:
        assert rel_max(got_f, ref_f) <= F64_TOL, what
        e_tol, w_tol = F64_TOL, F64_TOL
    else:
        assert np.abs(got_f - ref_f).max() <= MIX_F_ABS, what
        e_tol, w_tol = MIX_E_REL, MIX_W_REL
    assert abs(got["e_tersoff"] - ref["e_tersoff"]) <= e_tol * abs(ref["e_tersoff"]), what
    assert abs(got["e_ilp"] - ref["e_ilp"]) <= e_tol * abs(ref["e_ilp"]), what
    assert rel_max(got["pvector"], ref["pvector"]) <= max(e_tol, 1e-10), what
    assert rel_max(got["virial"], ref["virial"]) <= w_tol, what


@pytest.mark.parametrize("name", ["bilayer_small", "hetero_small", "tiny_images"])
@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
def test_noalloc_matches_compute_device_on_two_calls(name, precision):
    import torch
    g = load_golden(name)
    eng = capi.Engine(TERSOFF, ILP, tap_flag=int(g["tap_flag"]), precision=precision)
    eng.set_box(g["box_lo"], g["box_hi"], g["periodic"])
    x, t, m = _inputs(g)
    n = x.shape[0]
    f_ref = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    ref = eng.compute_device(x, t, m, None, f_ref, overwrite=True)
    fr = f_ref.cpu().numpy()
    for call in range(2):
        f = torch.full((n, 3), float("nan"), dtype=torch.float64, device="cuda")
        got = eng.compute_device_noalloc(x, t, m, f)
        fg = f.cpu().numpy()
        assert np.isfinite(fg).all(), call
        # against the regular device entry point ...
        _check(fg, got, fr, ref, precision, ("compute_device", call))
        # ... and against the reference's own outputs for the same atoms
        _check(fg, got, g["f"], {k: g[k] for k in ("e_tersoff", "e_ilp", "pvector", "virial")}, precision,
               ("golden", call))


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
def test_noalloc_leaves_free_device_memory_unchanged(precision):
    """After a first call (which looks the static array up and loads the kernels), further
    calls change neither cudaMemGetInfo's free-memory figure nor torch's allocator."""
    import torch
    g = load_golden("hetero_small")
    eng = capi.Engine(TERSOFF, ILP, tap_flag=int(g["tap_flag"]), precision=precision)
    eng.set_box(g["box_lo"], g["box_hi"], g["periodic"])
    x, t, m = _inputs(g)
    f = torch.zeros((x.shape[0], 3), dtype=torch.float64, device="cuda")
    eng.compute_device_noalloc(x, t, m, f)
    torch.cuda.synchronize()
    for call in range(2):
        free0 = torch.cuda.mem_get_info()[0]
        alloc0 = torch.cuda.memory_allocated()
        eng.compute_device_noalloc(x, t, m, f)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0, call
        assert torch.cuda.memory_allocated() == alloc0, call


def test_noalloc_empty_subdomain_returns_zero():
    """natoms = 0 (a rank whose subdomain holds no atoms) succeeds with zero energies."""
    import torch
    eng = capi.Engine(TERSOFF, ILP)
    eng.set_box([0, 0, -15], [100, 100, 18], [1, 1, 0])
    x = torch.zeros((0, 3), dtype=torch.float64, device="cuda")
    t = torch.zeros(0, dtype=torch.int32, device="cuda")
    m = torch.zeros(0, dtype=torch.int64, device="cuda")
    f = torch.zeros((0, 3), dtype=torch.float64, device="cuda")
    got = eng.compute_device_noalloc(x, t, m, f)
    assert got["e_tersoff"] == 0.0 and got["e_ilp"] == 0.0
    assert not np.any(got["virial"])


def test_noalloc_rejects_systems_above_its_limit():
    import torch
    eng = capi.Engine(TERSOFF, ILP)
    eng.set_box([0, 0, -15], [100, 100, 18], [1, 1, 0])
    n = 2049
    x = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    t = torch.ones(n, dtype=torch.int32, device="cuda")
    m = torch.ones(n, dtype=torch.int64, device="cuda")
    f = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    with pytest.raises(capi.LmffError) as ei:
        eng.compute_device_noalloc(x, t, m, f)
    assert ei.value.code == -1 and "2048" in str(ei.value)
