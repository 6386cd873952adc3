"""The allocation-free entry point, lmff_compute_device_noalloc, called through the C ABI.

It serves callers that must not allocate device memory while they run (an application
that gives all GPU memory to its own pool at start-up, or a code path where cudaMalloc
is not allowed).  Its results must equal those of the regular device entry point,
lmff_compute_device, within the parity tolerances used everywhere else in the tests,
and must stay equal when it is called twice in a row: the second call reuses the same
static scratch array that the first call left behind.
"""
import numpy as np
import pytest
from conftest import ILP, TERSOFF, load_golden, rel_max

from lmff_gb300 import build, capi

pytestmark = pytest.mark.gpu

F64_TOL = 1e-10   # the FP64 parity bar of tests/test_gpu_parity.py
MIX_F_ABS = 1e-5  # the mixed-precision force bar of tests/test_gpu_parity.py


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _inputs(g):
    import torch
    x = torch.tensor(g["x"], dtype=torch.float64, device="cuda")
    t = torch.tensor(g["type"], dtype=torch.int32, device="cuda")
    m = torch.tensor(g["mol"], dtype=torch.int64, device="cuda")
    return x, t, m


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
    for call in range(2):
        f = torch.full((n, 3), float("nan"), dtype=torch.float64, device="cuda")
        got = eng.compute_device_noalloc(x, t, m, f)
        fr, fg = f_ref.cpu().numpy(), f.cpu().numpy()
        assert np.isfinite(fg).all(), call
        if precision == capi.FP64:
            assert rel_max(fg, fr) <= F64_TOL, call
            tol = F64_TOL
        else:
            assert np.abs(fg - fr).max() <= MIX_F_ABS, call
            tol = 1e-6
        assert abs(got["e_tersoff"] - ref["e_tersoff"]) <= tol * abs(ref["e_tersoff"]), call
        assert abs(got["e_ilp"] - ref["e_ilp"]) <= tol * abs(ref["e_ilp"]), call
        assert rel_max(got["virial"], ref["virial"]) <= max(tol, 1e-10) * 10, call


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
