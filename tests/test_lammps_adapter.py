"""The LAMMPS-side host code (lammps-lmff_gb300/lammps/lmff_lammps_adapter.cpp) on a GPU,
driven as the tersoff/gb300 and ilp/graphene/hbn/gb300 pair styles drive it inside
LAMMPS (tests/lammps_adapter_driver.cpp), against the reference's golden outputs."""
import os
import subprocess

import numpy as np
import pytest
from conftest import POT, ROOT, load_golden, rel_max

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


@pytest.mark.parametrize("name", ["bilayer_small", "hetero_small", "tiny_images"])
def test_adapter_matches_reference(driver, tmp_path, name):
    g = load_golden(name)
    n = len(g["tag"])
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as fh:
        np.array([n], np.int32).tofile(fh)
        np.concatenate([g["box_lo"], g["box_hi"]]).astype(np.float64).tofile(fh)
        np.asarray(g["periodic"], np.int32).tofile(fh)
        np.array([int(g["tap_flag"])], np.int32).tofile(fh)
        np.asarray(g["x"], np.float64).tofile(fh)
        for a in (g["type"], g["mol"], g["tag"]):
            np.asarray(a, np.int32).tofile(fh)
    out = tmp_path / "out.bin"
    subprocess.check_call([driver, POT, str(inp), str(out)])
    raw = np.fromfile(out, np.float64)
    per = 3 * n + n + 2 + 2 + 6
    assert raw.size == 2 * per
    for call in range(2):
        r = raw[call * per:(call + 1) * per]
        f = r[:3 * n].reshape(n, 3)
        eatom = r[3 * n:4 * n]
        et, ei = r[4 * n], r[4 * n + 1]
        pv = r[4 * n + 2:4 * n + 4]
        vir = r[4 * n + 4:4 * n + 10]
        assert rel_max(f, g["f"]) <= TOL, call
        assert rel_max(eatom, g["eatom"]) <= TOL, call
        assert abs(et - g["e_tersoff"]) <= TOL * abs(g["e_tersoff"]), call
        assert abs(ei - g["e_ilp"]) <= TOL * abs(g["e_ilp"]), call
        assert rel_max(pv, g["pvector"]) <= TOL, call
        assert rel_max(vir, g["virial"]) <= TOL, call
