"""Kolmogorov-Crespi full (pair_style kolmogorov/crespi/full) as the interlayer style,
with Tersoff, on the same normals machinery as ILP.  The oracle restatement is pinned
against the reference run on the same inputs (tests/golden/kc_*.npz, made by
tests/golden/make_golden.py with CC.KC-full: the Kolmogorov-Crespi 2005 graphene
parameters); the engine is checked against both on the GPU."""
import os

import numpy as np
import pytest
from conftest import POT, TERSOFF, load_golden, min_image, rel_max, rel_rms

from lmff_gb300 import build, capi
from lmff_gb300 import structures as S
from oracle import Oracle

KC = os.path.join(POT, "CC.KC-full")
KC_ELEMS = ("C", "NULL", "NULL")
TOL = 1e-12
E_TOL = 1e-10
F64_TOL = 1e-10
MIX_F_ABS = 1e-5


def _oracle(g):
    o = Oracle(TERSOFF, None, kc_file=KC, interlayer_elements=KC_ELEMS, tap_flag=int(g["tap_flag"]), nthreads=4)
    o.set_atoms(g["x"], g["type"], g["mol"], g["tag"], g["box_lo"], g["box_hi"], g["periodic"])
    return o


def _engine(g, precision=capi.FP64):
    eng = capi.Engine(TERSOFF, None, elements=("C", "B", "N"), ilp_elements=KC_ELEMS, kc_file=KC,
                      tap_flag=int(g["tap_flag"]), precision=precision)
    eng.set_box(g["box_lo"], g["box_hi"], g["periodic"])
    return eng


@pytest.mark.parametrize("name", ["kc_bilayer", "kc_bilayer_notaper"])
def test_kc_oracle_matches_reference(name):
    g = load_golden(name)
    r = _oracle(g).forces(eatom=True, vatom=True)
    assert rel_max(r["f"], g["f"]) < TOL and rel_rms(r["f"], g["f"]) < TOL
    assert rel_max(r["vatom_tersoff"], g["vatom_tersoff"]) < TOL
    assert rel_max(r["vatom_ilp"], g["vatom_ilp"]) < TOL
    assert abs(r["e_tersoff"] - g["e_tersoff"]) <= E_TOL * abs(g["e_tersoff"])
    assert abs(r["e_ilp"] - g["e_ilp"]) <= E_TOL * abs(g["e_ilp"])
    assert rel_max(r["pvector"], g["pvector"]) < E_TOL
    assert rel_max(r["virial"], g["virial"]) < TOL
    assert rel_max(r["eatom"], g["eatom"]) < TOL


def test_kc_oracle_trajectory_start_matches_reference():
    g = load_golden("kc_trilayer_t30")
    o = Oracle(TERSOFF, None, kc_file=KC, interlayer_elements=KC_ELEMS, tap_flag=1, nthreads=4)
    o.set_atoms(g["x0"], g["type"], g["mol"], g["tag"], g["box_lo"], g["box_hi"], g["periodic"])
    r = o.forces()
    assert rel_max(r["f"], g["f0"]) < TOL
    assert abs(r["e_ilp"] - g["e0"]) <= E_TOL * abs(g["e0"])


def test_kc_parser_errors(tmp_path):
    """The reference's read_file errors for this format (12 words per entry)."""
    good = open(KC).read()
    bad = {"missing": good.replace("C C 3.34", "C B 3.34"),
           "duplicate": good + "C C 3.34 15.71 12.29 4.933 3.030 0.578 3.629 10.238 1.0 2.0\n",
           "short": good.replace(" 2.0\n", "\n")}
    lib = capi.load_library() if os.path.exists(capi.LIB_PATH) else None
    if lib is None:
        build.build()
        lib = capi.load_library()
    import ctypes as C
    for kind, txt in bad.items():
        p = str(tmp_path / f"{kind}.KC")
        open(p, "w").write(txt)
        h = C.c_void_p()
        t = (C.c_char_p * 3)(b"C", b"B", b"N")
        k = (C.c_char_p * 3)(b"C", b"B", b"NULL") if kind == "missing" else (C.c_char_p * 3)(b"C", b"NULL", b"NULL")
        rc = lib.lmff_create_kc_from_files(C.byref(h), TERSOFF.encode(), t, p.encode(), k, 3, 16.0, 1, 2.0, 0)
        msg = lib.lmff_last_error(None).decode()
        assert rc == -6, (kind, rc, msg)
        want = {"missing": "missing an entry", "duplicate": "duplicate entry", "short": "KC"}[kind]
        assert want in msg, (kind, msg)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["kc_bilayer", "kc_bilayer_notaper"])
def test_kc_engine_matches_reference(name):
    build.build()
    g = load_golden(name)
    r = _engine(g).compute(g["x"], g["type"], g["mol"], g["tag"], eatom=True)
    assert rel_max(r["f"], g["f"]) <= F64_TOL and rel_rms(r["f"], g["f"]) <= F64_TOL
    assert abs(r["e_ilp"] - g["e_ilp"]) <= F64_TOL * abs(g["e_ilp"])
    assert rel_max(r["pvector"], g["pvector"]) <= F64_TOL
    assert rel_max(r["virial"], g["virial"]) <= F64_TOL
    assert rel_max(r["eatom"], g["eatom"]) <= F64_TOL
    m = _engine(g, capi.MIXED).compute(g["x"], g["type"], g["mol"], g["tag"])
    assert np.abs(m["f"] - g["f"]).max() <= MIX_F_ABS
    assert abs(m["e_ilp"] - g["e_ilp"]) <= 1e-6 * abs(g["e_ilp"])


@pytest.mark.gpu
def test_kc_nve_trajectory_matches_reference():
    """30 velocity-Verlet steps of a displaced, thermal 3-layer slab (unique molecule
    ids), device resident, against the reference's own trajectory."""
    build.build()
    g = load_golden("kc_trilayer_t30")
    eng = _engine(g)
    s = S.System(g["x0"], g["type"], g["mol"], g["tag"], g["box_lo"], g["box_hi"], g["periodic"].astype(bool),
                 g["v0"])
    eng.upload(s)
    eng.run_nve(30, 0.001)
    x, v, f = eng.download()
    dx = min_image(x - g["x"], g["box_lo"], g["box_hi"], g["periodic"])
    assert np.abs(dx).max() < 1e-9
    assert rel_max(v, g["v"]) < 1e-8 and rel_max(f, g["f"]) < 1e-8


@pytest.mark.gpu
def test_kc_engine_vs_oracle_larger():
    """A 10k-atom twisted bilayer graphene (0.9 deg, strained commensurate) against the
    oracle, FP64 and mixed."""
    build.build()
    s = S.displace(S.twisted_bilayer(24, 14, 0.9, top="graphene"), 0.03, seed=5)
    o = Oracle(TERSOFF, None, kc_file=KC, interlayer_elements=KC_ELEMS, tap_flag=1, nthreads=8)
    o.set_system(s)
    ro = o.forces()
    eng = capi.Engine(TERSOFF, None, elements=("C", "B", "N"), ilp_elements=KC_ELEMS, kc_file=KC)
    r = eng.compute_system(s)
    assert rel_max(r["f"], ro["f"]) <= F64_TOL
    assert abs(r["e_ilp"] - ro["e_ilp"]) <= F64_TOL * abs(ro["e_ilp"])
    m = capi.Engine(TERSOFF, None, elements=("C", "B", "N"), ilp_elements=KC_ELEMS, kc_file=KC,
                    precision=capi.MIXED).compute_system(s)
    assert np.abs(m["f"] - ro["f"]).max() <= MIX_F_ABS
