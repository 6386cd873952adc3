"""The reference's own case through the engine: its data file (Cases/case_5016/inf0.data,
6 graphene layers, 5016 atoms) read with ``structures.read_lammps_data``, ``replicate``
with LAMMPS semantics, the case's pair setup (Tersoff C.opt.tersoff with type 1 NULL,
ILP BNCH.ILP, taper off), and its minimisation (layer 1 held by setforce, CG with the
quadratic line search) -- each against the reference run on the same input
(tests/golden/case5016*.npz, made by tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest
from conftest import REFERENCE, ROOT, load_golden, min_image, rel_max, rel_rms

from lmff_gb300 import build, capi
from lmff_gb300 import structures as S

POT = os.path.join(ROOT, "lammps-lmff_gb300", "potentials")
TERSOFF_ELEMS = ("NULL", "C(O)", "C(O)", "C(O)", "C(O)", "C(O)")
ILP_ELEMS = ("C",) * 6
CASE_DATA = os.path.join(REFERENCE, "Cases", "case_5016", "inf0.data")
F64_TOL = 1e-10
MIX_F_ABS = 1e-5


def case_system(g, x=None):
    s = S.System(np.array(g["x"] if x is None else x), g["type"].astype(np.int32), g["mol"].astype(np.int64),
                 g["tag"].astype(np.int64), g["box_lo"], g["box_hi"], g["periodic"].astype(bool))
    s.meta["type_masses"] = np.full(6, 12.0107)
    return s


def case_engine(precision=capi.FP64):
    return capi.Engine(os.path.join(POT, "C.opt.tersoff"), os.path.join(POT, "BNCH.ILP"), elements=TERSOFF_ELEMS,
                       ilp_elements=ILP_ELEMS, tap_flag=0, precision=precision)


# ------------------------------------------------------------------ CPU: the format

@pytest.mark.skipif(not os.path.exists(CASE_DATA), reason="reference checkout not present")
def test_reader_matches_read_data_on_the_reference_case():
    g = load_golden("case5016")
    s = S.read_lammps_data(CASE_DATA)
    order = np.argsort(s.tag)
    assert s.n == 5016 and np.array_equal(s.tag[order], g["tag"])
    assert np.array_equal(s.type[order], g["type"]) and np.array_equal(s.mol[order], g["mol"])
    assert np.array_equal(s.box_lo, g["box_lo"]) and np.array_equal(s.box_hi, g["box_hi"])
    # read_data wraps coordinates on the box edge into the box; compare modulo the box
    d = min_image(s.x[order] - g["x"], g["box_lo"], g["box_hi"], g["periodic"])
    assert np.abs(d).max() < 1e-12
    assert np.allclose(s.type_masses(), 12.0107)


def test_reader_round_trip_and_errors(tmp_path):
    s = S.thermalize(S.twisted_bilayer(5, 3, 2.0, top="hbn"), 300.0, seed=4)
    p = str(tmp_path / "a.data")
    S.write_lammps_data(s, p)
    r = S.read_lammps_data(p)
    for k in ("x", "v", "type", "mol", "tag", "box_lo", "box_hi"):
        assert np.array_equal(getattr(r, k), getattr(s, k)), k
    txt = open(p).read()
    # a tilted box: its xy xz yz line round-trips through tilt
    t = S.hex_layers(5, 3, nlayers=2, periodic_z=True, xz=0.3, yz=-0.2)
    q = str(tmp_path / "t.data")
    S.write_lammps_data(t, q)
    rt = S.read_lammps_data(q)
    assert np.array_equal(rt.tilt, t.tilt) and np.array_equal(rt.x, t.x)
    assert r.tilt is None
    bad = {"section": txt.replace("Atoms # full", "Ellipse"),
           "columns": txt.replace("Atoms # full\n\n1 ", "Atoms # full\n\n1 1 ", 1),
           "short": txt[:txt.index("Velocities")].rsplit("\n", 5)[0]}
    for name, t in bad.items():
        q = str(tmp_path / f"{name}.data")
        open(q, "w").write(t)
        with pytest.raises(ValueError):
            S.read_lammps_data(q)


def test_replicate_matches_lammps():
    g = load_golden("case5016")
    r = load_golden("case5016_rep2")
    rep = S.replicate(case_system(g), 2, 1, 1)
    order = np.argsort(rep.tag)
    assert np.array_equal(rep.tag[order], r["tag"])
    assert np.array_equal(rep.type[order], r["type"]) and np.array_equal(rep.mol[order], r["mol"])
    assert np.allclose(rep.box_hi, r["box_hi"], rtol=0, atol=1e-12)
    d = min_image(rep.x[order] - r["x"], r["box_lo"], r["box_hi"], r["periodic"])
    assert np.abs(d).max() < 1e-11


# ------------------------------------------------------------------ GPU: forces, minimise

@pytest.mark.gpu
@pytest.mark.parametrize("name", ["case5016", "case5016_rep2"])
def test_case_forces_match_reference(name):
    build.build()
    g = load_golden(name)
    s = case_system(g)
    r = case_engine().compute_system(s)
    assert rel_max(r["f"], g["f"]) <= F64_TOL and rel_rms(r["f"], g["f"]) <= F64_TOL
    assert abs(r["e_tersoff"] - g["e_tersoff"]) <= F64_TOL * abs(g["e_tersoff"])
    assert abs(r["e_ilp"] - g["e_ilp"]) <= F64_TOL * abs(g["e_ilp"])
    assert rel_max(r["virial"], g["virial"]) <= F64_TOL
    m = case_engine(capi.MIXED).compute_system(s)
    assert np.abs(m["f"] - g["f"]).max() <= MIX_F_ABS


def _minimize(g, etol, ftol, maxiter, maxeval):
    s = case_system(g, g["x0"])
    eng = case_engine()
    eng.upload(s)
    out = eng.minimize(etol, ftol, maxiter, maxeval, 0.1, frozen=(s.type == 1).astype(np.int32))
    x, _, f = eng.download()
    return out, x, f


@pytest.mark.gpu
def test_case_minimisation_matches_reference():
    """The case's own `minimize 1.0e-5 1.0e-5 1000 10000`: one CG iteration, two
    evaluations, energy-tolerance stop -- counts, energies, positions and forces."""
    build.build()
    g = load_golden("case5016_min")
    out, x, f = _minimize(g, 1e-5, 1e-5, 1000, 10000)
    niter, neval, stop = (int(v) for v in g["min_counts"])
    einit, efin, fn2, fninf, alpha = g["min_values"]
    assert (out["niter"], out["neval"], out["stop_condition"]) == (niter, neval, stop)
    assert abs(out["einitial"] - einit) <= F64_TOL * abs(einit)
    assert abs(out["efinal"] - efin) <= F64_TOL * abs(efin)
    assert abs(out["fnorm2_final"] - fn2) <= 1e-8 * fn2 and abs(out["fnorminf_final"] - fninf) <= 1e-8 * fninf
    assert out["alpha_final"] == alpha
    d = min_image(x - g["x"], g["box_lo"], g["box_hi"], g["periodic"])
    assert np.abs(d).max() < 1e-10
    assert rel_max(f, g["f"]) <= 1e-8
    assert np.all(f[g["type"] == 1] == 0.0)              # setforce on layer 1


@pytest.mark.gpu
def test_case_long_minimisation_matches_reference():
    """`minimize 1.0e-10 1.0e-3 300 3000`: 135 CG iterations in the reference.  The
    line search branches on energy differences near 1e-8 eV, so summation-order noise
    can move the path slightly: same stop condition, iteration count within 10 %, final
    energy within 1e-9 relative."""
    build.build()
    g = load_golden("case5016_min_long")
    out, x, f = _minimize(g, 1e-10, 1e-3, 300, 3000)
    niter, neval, stop = (int(v) for v in g["min_counts"])
    einit, efin = g["min_values"][:2]
    assert out["stop_condition"] == stop
    assert abs(out["niter"] - niter) <= 0.1 * niter
    assert abs(out["einitial"] - einit) <= F64_TOL * abs(einit)
    assert abs(out["efinal"] - efin) <= 1e-9 * abs(efin)
    assert np.all(f[g["type"] == 1] == 0.0)
