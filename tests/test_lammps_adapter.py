"""The LAMMPS-side host code (lammps-lmff_gb300/lammps/lmff_lammps_adapter.cpp) on a GPU,
driven as the tersoff/gb300 and ilp/graphene/hbn/gb300 pair styles drive it inside
LAMMPS (tests/lammps_adapter_driver.cpp), against the reference's golden outputs:
- one engine per style or one engine the two styles share (hybrid/overlay: the first
  style's call evaluates both, the second takes its energies from that call);
- the periodic form (one MPI rank) and the subdomain form (the system split over ranks
  with ghost shells built as LAMMPS's brick decomposition does; the ghost forces and
  per-atom energies and virials folded onto their owners as LAMMPS's reverse
  communication does)."""
import os
import subprocess

import numpy as np
import pytest
from conftest import POT, ROOT, load_golden, rel_max
from test_subdomains import decompose

from lmff_gb300 import build

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    lib = build.build()
    out = str(tmp_path_factory.mktemp("drv") / "lammps_adapter_driver")
    src = [os.path.join(ROOT, "tests", "lammps_adapter_driver.cpp"),
           os.path.join(ROOT, "lammps-lmff_gb300", "lammps", "lmff_lammps_adapter.cpp"),
           os.path.join(ROOT, "lammps-lmff_gb300", "csrc", "potentials.cpp")]
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "lammps-lmff_gb300", "lammps"),
           "-I" + os.path.join(ROOT, "lammps-lmff_gb300", "csrc")]
    libdir = os.path.dirname(lib)
    subprocess.check_call(["g++", "-O2", "-std=c++17", *inc, *src, "-o", out, "-L" + libdir, "-llmff_gb300",
                           "-Wl,-rpath," + libdir])
    return out


def run_driver(driver, tmp_path, g, shared, splits=None):
    """Returns, per call (two), the folded whole-system f, eatom, vatom, energies,
    pvector, virial."""
    n = len(g["tag"])
    if splits is None:
        systems = [(np.arange(n), np.asarray(g["x"], float), np.arange(n), n)]
    else:
        cg = float(g["cut_global"]) + float(g["skin"])
        systems = [(own, xs, idx, len(own))
                   for own, xs, idx in decompose(g["x"], g["box_lo"], g["box_hi"], g["periodic"], splits, cg)]
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as fh:
        np.array([int(shared), 0 if splits is None else len(systems)], np.int32).tofile(fh)
        np.concatenate([g["box_lo"], g["box_hi"]]).astype(np.float64).tofile(fh)
        np.asarray(g["periodic"], np.int32).tofile(fh)
        np.array([int(g["tap_flag"])], np.int32).tofile(fh)
        for own, xs, idx, nlocal in systems:
            np.array([nlocal, len(idx)], np.int32).tofile(fh)
            np.asarray(xs, np.float64).tofile(fh)
            for a in (g["type"], g["mol"], g["tag"]):
                np.asarray(a[idx], np.int32).tofile(fh)
    out = tmp_path / "out.bin"
    subprocess.check_call([driver, POT, str(inp), str(out)])
    raw = np.fromfile(out, np.float64)
    pos = 0
    calls = []
    for call in range(2):
        f = np.zeros((n, 3))
        ea = np.zeros(n)
        va = np.zeros((n, 6))
        tot = np.zeros(10)   # e_tersoff, e_ilp, pvector[2], virial[6]
        for own, xs, idx, nlocal in systems:
            m = len(idx) if splits is not None else n
            np.add.at(f, idx, raw[pos:pos + 3 * m].reshape(m, 3))
            pos += 3 * m
            np.add.at(ea, idx, raw[pos:pos + m])
            pos += m
            np.add.at(va, idx, raw[pos:pos + 6 * m].reshape(m, 6))
            pos += 6 * m
            tot += raw[pos:pos + 10]
            pos += 10
        calls.append((f, ea, va, tot))
    assert pos == raw.size
    return calls


def check(calls, g):
    for call, (f, ea, va, tot) in enumerate(calls):
        assert rel_max(f, g["f"]) <= TOL, call
        assert rel_max(ea, g["eatom"]) <= TOL, call
        if "vatom_ilp" in g:   # per-atom virial (vflag_atom) of both styles together
            assert rel_max(va, g["vatom_tersoff"] + g["vatom_ilp"]) <= TOL, call
        assert abs(tot[0] - g["e_tersoff"]) <= TOL * abs(g["e_tersoff"]), call
        assert abs(tot[1] - g["e_ilp"]) <= TOL * abs(g["e_ilp"]), call
        assert rel_max(tot[2:4], g["pvector"]) <= TOL, call
        assert rel_max(tot[4:10], g["virial"]) <= TOL, call


@pytest.mark.parametrize("shared", [0, 1])
@pytest.mark.parametrize("name", ["bilayer_small", "hetero_small", "tiny_images"])
def test_adapter_matches_reference(driver, tmp_path, name, shared):
    g = load_golden(name)
    check(run_driver(driver, tmp_path, g, shared), g)


@pytest.mark.parametrize("shared", [0, 1])
@pytest.mark.parametrize("name,splits", [("bilayer_small", (2, 1, 1)), ("hetero_small", (2, 2, 1)),
                                         ("c1_t0", (2, 2, 1))])
def test_adapter_subdomains_match_reference(driver, tmp_path, name, splits, shared):
    g = load_golden(name)
    check(run_driver(driver, tmp_path, g, shared, splits), g)
