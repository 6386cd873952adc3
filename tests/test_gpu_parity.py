"""Parity of the CUDA engine (through the C ABI) with the reference and the oracle.

Bars (max-norm relative unless stated):
  FP64 drop-in   forces max and RMS <= 1e-10, per-style energies and pvector <= 1e-10,
                 fdotr virial <= 1e-10, per-atom energy <= 1e-10 (of max |eatom|)
  mixed          forces: max |dF| <= 1e-5 eV/A absolute; energies <= 1e-6 relative;
                 virial <= 1e-5 relative
  lists          bit-exact as sets (tag_i, tag_j, periodic image)
"""
import numpy as np
import pytest
from conftest import (GOLDEN_LISTS, GOLDEN_SINGLE, ILP, TERSOFF, load_golden, min_image, rel_max,
                      rel_rms)

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


def engine_for(g, precision=capi.FP64, **kw):
    eng = capi.Engine(TERSOFF, ILP, cut_global=float(g["cut_global"]), tap_flag=int(g["tap_flag"]),
                      skin=float(g["skin"]), precision=precision)
    for k, v in kw.items():
        eng.set_option(k, v)
    eng.set_box(g["box_lo"], g["box_hi"], g["periodic"])
    return eng


def compute_golden(eng, g, **kw):
    return eng.compute(g["x"], g["type"], g["mol"], g["tag"], eatom=True, **kw)


@pytest.mark.parametrize("name", GOLDEN_SINGLE)
def test_fp64_matches_reference(name):
    g = load_golden(name)
    r = compute_golden(engine_for(g), g)
    assert rel_max(r["f"], g["f"]) <= F64_TOL
    assert rel_rms(r["f"], g["f"]) <= F64_TOL
    assert abs(r["e_tersoff"] - g["e_tersoff"]) <= F64_TOL * abs(g["e_tersoff"])
    assert abs(r["e_ilp"] - g["e_ilp"]) <= F64_TOL * abs(g["e_ilp"])
    assert rel_max(r["pvector"], g["pvector"]) <= F64_TOL
    assert rel_max(r["virial"], g["virial"]) <= F64_TOL
    assert rel_max(r["eatom"], g["eatom"]) <= F64_TOL


@pytest.mark.parametrize("tpa", [4, 8, 32])
def test_fp64_threads_per_atom_variants(tpa):
    g = load_golden("hetero_small")
    r = compute_golden(engine_for(g, tpa=tpa), g)
    assert rel_max(r["f"], g["f"]) <= F64_TOL
    assert rel_max(r["virial"], g["virial"]) <= F64_TOL


def _set(a):
    return set(map(tuple, np.asarray(a).reshape(-1, 3).tolist()))


@pytest.mark.parametrize("name", GOLDEN_LISTS)
def test_lists_match_reference(name):
    g = load_golden(name)
    eng = engine_for(g, list_full=1)
    compute_golden(eng, g)
    assert _set(eng.export_list(0)) == _set(g["nlist"])
    assert _set(eng.export_list(1)) == _set(g["ilplist"])
    # default (interlayer) pair list = the reference list restricted to mol_i != mol_j
    eng2 = engine_for(g)
    compute_golden(eng2, g)
    mol = dict(zip(g["tag"].tolist(), g["mol"].tolist()))
    ref = {t for t in _set(g["nlist"]) if mol[t[0]] != mol[t[1]]}
    assert _set(eng2.export_list(0)) == ref


@pytest.mark.parametrize("name", ["c1_t0", "hetero_small", "trilayer_alt", "edges", "tiny_images"])
def test_mixed_precision_accuracy(name):
    g = load_golden(name)
    r = compute_golden(engine_for(g, precision=capi.MIXED), g)
    assert np.abs(r["f"] - g["f"]).max() <= MIX_F_ABS
    assert abs(r["e_tersoff"] - g["e_tersoff"]) <= MIX_E_REL * abs(g["e_tersoff"])
    assert abs(r["e_ilp"] - g["e_ilp"]) <= MIX_E_REL * abs(g["e_ilp"])
    assert rel_max(r["virial"], g["virial"]) <= MIX_W_REL


@pytest.mark.parametrize("name", ["c1_t0", "hetero_small", "trilayer_alt", "edges", "tiny_images"])
@pytest.mark.parametrize("tpa", [8, 16, 32])
def test_mixed_forces_without_energy_match_reference(name, tpa):
    """The production force-only pair kernels (no energy/virial: the single-element loop
    with two list entries per iteration and compact j records, and the multi-element
    loop), against the reference."""
    g = load_golden(name)
    eng = engine_for(g, precision=capi.MIXED, tpa=tpa)
    r = eng.compute(g["x"], g["type"], g["mol"], g["tag"], eflag=False, vflag=False)
    assert np.abs(r["f"] - g["f"]).max() <= MIX_F_ABS


def test_mixed_forces_without_energy_large():
    """Force-only mixed evaluation of a 97k-atom displaced graphite slab against the FP64
    engine, and against the mixed evaluation with energies (another kernel instance)."""
    s = S.displace(S.graphite_slab(6, 60, 34, mol_mode="alternate"), 0.03, seed=5)
    r64 = capi.Engine(TERSOFF, ILP).compute_system(s)
    eng = capi.Engine(TERSOFF, ILP, precision=capi.MIXED)
    rf = eng.compute_system(s, eflag=False, vflag=False)
    re = capi.Engine(TERSOFF, ILP, precision=capi.MIXED).compute_system(s)
    assert np.abs(rf["f"] - r64["f"]).max() <= MIX_F_ABS
    assert np.abs(rf["f"] - re["f"]).max() <= MIX_F_ABS


def test_mixed_forces_without_energy_hetero_large():
    """Force-only mixed evaluation of a displaced graphene/hBN twisted bilayer (the
    multi-element loop with two list entries per iteration) against the FP64 engine."""
    # a 2,640-atom cell (most atoms near a periodic face: the image-decoding loop) and the
    # 489,632-atom 0.6 degree cell (mostly the loop without image decode)
    for s in (S.displace(S.twisted_bilayer(24, 14, 0.9, top="hbn"), 0.03, seed=6),
              S.displace(S.twisted_graphene_hbn_500k(seed=2), 0.03, seed=7)):
        r64 = capi.Engine(TERSOFF, ILP).compute_system(s, eflag=False, vflag=False)
        for tpa in (8, 16):
            eng = capi.Engine(TERSOFF, ILP, precision=capi.MIXED)
            eng.set_option("tpa", tpa)
            rf = eng.compute_system(s, eflag=False, vflag=False)
            assert np.abs(rf["f"] - r64["f"]).max() <= MIX_F_ABS, (s.n, tpa)


def test_nve_trajectory_matches_reference():
    """100 velocity-Verlet steps of the 7,200-atom bilayer, device resident, vs the
    reference's own trajectory from the same start."""
    g = load_golden("c1_t100")
    eng = engine_for(g)
    s = S.System(g["x0"], g["type"], g["mol"], g["tag"], g["box_lo"], g["box_hi"], g["periodic"].astype(bool),
                 g["v0"])
    eng.upload(s)
    eng.run_nve(100, 0.001)
    x, v, f = eng.download()
    dx = min_image(x - g["x"], g["box_lo"], g["box_hi"], g["periodic"])
    assert np.abs(dx).max() < 1e-9
    assert rel_max(v, g["v"]) < 1e-8
    assert rel_max(f, g["f"]) < 1e-8


def test_nve_hetero_matches_reference():
    g = load_golden("hetero_t20")
    eng = engine_for(g)
    s = S.System(g["x0"], g["type"], g["mol"], g["tag"], g["box_lo"], g["box_hi"], g["periodic"].astype(bool),
                 g["v0"])
    eng.upload(s)
    eng.run_nve(20, 0.001)
    x, v, f = eng.download()
    dx = min_image(x - g["x"], g["box_lo"], g["box_hi"], g["periodic"])
    assert np.abs(dx).max() < 1e-9
    assert rel_max(f, g["f"]) < 1e-8


def test_deterministic_bitwise():
    g = load_golden("hetero_small")
    e1 = compute_golden(engine_for(g), g)
    e2 = compute_golden(engine_for(g), g)
    assert np.array_equal(e1["f"], e2["f"])
    assert e1["e_ilp"] == e2["e_ilp"] and np.array_equal(e1["virial"], e2["virial"])


def test_same_atoms_fast_path_and_identity_change():
    g = load_golden("bilayer_small")
    eng = engine_for(g)
    r0 = compute_golden(eng, g)
    r1 = eng.compute(g["x"], g["type"], g["mol"], g["tag"], same_atoms=True, eatom=True)
    assert np.array_equal(r0["f"], r1["f"])
    # permuted atom order: identity check notices and reloads
    p = np.random.default_rng(0).permutation(len(g["tag"]))
    r2 = eng.compute(g["x"][p], g["type"][p], g["mol"][p], g["tag"][p])
    assert rel_max(r2["f"], g["f"][p]) <= F64_TOL


def test_force_accumulates():
    g = load_golden("bilayer_small")
    eng = engine_for(g)
    f = np.ones((len(g["tag"]), 3))
    r = eng.compute(g["x"], g["type"], g["mol"], g["tag"], f=f)
    assert rel_max(r["f"] - 1.0, g["f"]) <= F64_TOL


def test_batch_equals_single():
    systems = S.replica_set(count=4, nmin=500, nmax=3000, seed=9)
    systems = [S.displace(s, 0.03, seed=k) for k, s in enumerate(systems)]
    eng = capi.Engine(TERSOFF, ILP)
    eng.batch_set(systems)
    out = eng.batch_compute()
    for s, b in zip(systems, out):
        single = capi.Engine(TERSOFF, ILP).compute_system(s)
        assert np.array_equal(b["f"], single["f"])
        assert b["e_ilp"] == single["e_ilp"] and b["e_tersoff"] == single["e_tersoff"]


def _oracle_vs_engine(s, precision=capi.FP64, tap=1):
    from oracle import Oracle
    o = Oracle(TERSOFF, ILP, tap_flag=tap, nthreads=8)
    o.set_system(s)
    ref = o.forces(eatom=True)
    eng = capi.Engine(TERSOFF, ILP, tap_flag=tap, precision=precision)
    got = eng.compute_system(s, eatom=True)
    return ref, got


@pytest.mark.parametrize("seed", [101, 102, 103])
def test_fp64_vs_oracle_random_heterostructures(seed):
    rng = np.random.default_rng(seed)
    top = ["hbn", "graphene"][seed % 2]
    s = S.twisted_bilayer(int(rng.integers(8, 14)), int(rng.integers(5, 9)), float(rng.uniform(0, 5)), top=top,
                          spacing=float(rng.uniform(3.2, 3.6)), shift=tuple(rng.uniform(0, 2, 2)))
    s = S.displace(s, 0.05, seed=seed)
    ref, got = _oracle_vs_engine(s)
    assert rel_max(got["f"], ref["f"]) <= F64_TOL
    assert abs(got["e_ilp"] - ref["e_ilp"]) <= F64_TOL * abs(ref["e_ilp"])
    assert abs(got["e_tersoff"] - ref["e_tersoff"]) <= F64_TOL * abs(ref["e_tersoff"])
    assert rel_max(got["virial"], ref["virial"]) <= F64_TOL
    assert rel_max(got["eatom"], ref["eatom"]) <= F64_TOL


def test_fp64_vs_oracle_graphite_unique_mols():
    s = S.displace(S.graphite_slab(5, 10, 6, mol_mode="unique"), 0.04, seed=7)
    ref, got = _oracle_vs_engine(s)
    assert rel_max(got["f"], ref["f"]) <= F64_TOL
    assert rel_max(got["virial"], ref["virial"]) <= F64_TOL


def test_too_many_ilp_neighbours_is_reported():
    s = S.ab_bilayer_graphene(8, 5)
    # a fourth intralayer neighbour within 2 A of atom 0
    x = np.vstack([s.x, s.x[0] + np.array([0.0, -1.3, 0.0])])
    s2 = S.System(x, np.append(s.type, 1), np.append(s.mol, 1), np.arange(1, len(x) + 1), s.box_lo, s.box_hi,
                  s.periodic)
    eng = capi.Engine(TERSOFF, ILP)
    with pytest.raises(capi.LmffError) as ei:
        eng.compute_system(s2)
    assert ei.value.code == -4 and "too many neighbors" in str(ei.value)


def test_newton_third_law_and_translation_invariance_large():
    """Size-independent properties on a 97k-atom graphite slab (FP64 and mixed)."""
    s = S.displace(S.graphite_slab(6, 60, 34, mol_mode="alternate"), 0.03, seed=3)
    for prec in (capi.FP64, capi.MIXED):
        eng = capi.Engine(TERSOFF, ILP, precision=prec)
        r = eng.compute_system(s)
        ftot = r["f"].sum(0)
        if prec == capi.FP64:
            assert np.abs(ftot).max() <= 1e-9 * np.abs(r["f"]).sum(0).max()
        else:   # per-atom FP32 rounding does not cancel between the two ends of a pair
            assert np.abs(ftot).max() <= MIX_F_ABS * np.sqrt(s.n)
        s2 = s.copy()
        s2.x = s2.x + np.array([0.37, -1.1, 0.25])
        s2.box_lo = s2.box_lo + np.array([0.37, -1.1, 0.25])
        s2.box_hi = s2.box_hi + np.array([0.37, -1.1, 0.25])
        r2 = capi.Engine(TERSOFF, ILP, precision=prec).compute_system(s2)
        tol = 1e-10 if prec == capi.FP64 else 1e-5
        assert np.abs(r2["f"] - r["f"]).max() <= tol * max(1.0, np.abs(r["f"]).max())


def test_mixed_vs_fp64_large():
    s = S.displace(S.graphite_slab(4, 60, 34, mol_mode="unique"), 0.03, seed=4)
    r64 = capi.Engine(TERSOFF, ILP).compute_system(s)
    r32 = capi.Engine(TERSOFF, ILP, precision=capi.MIXED).compute_system(s)
    assert np.abs(r32["f"] - r64["f"]).max() <= MIX_F_ABS
    assert abs(r32["e_ilp"] - r64["e_ilp"]) <= MIX_E_REL * abs(r64["e_ilp"])


def test_benchmark_slab_full_size():
    """The 2,694,960-atom 10-layer AB graphite slab at 300 K, at full size, through
    size-independent properties: 150 mixed NVE steps through the step graph (the first
    build runs count + fill, the rebuilds inside the graph the single pass with
    compaction) conserve the total energy; the forces the engine holds at the end, on
    its rebuilt list, equal a fresh FP64 evaluation at the same positions; the FP64
    forces sum to zero."""
    s0 = S.thermalize(S.graphite_slab(10, 342, 197, spacing=3.35, mol_mode="alternate"), 300.0, seed=3)
    assert s0.n == 2_694_960
    eng = capi.Engine(TERSOFF, ILP, precision=capi.MIXED, skin=1.0)
    eng.set_option("tpa", 8)
    eng.set_option("block", 128)
    eng.upload(s0)
    th = eng.run_nve(150, 0.001, thermo_every=150)
    assert eng.stats()["rebuilds"] >= 2
    assert abs(th[-1]["etotal"] - th[0]["etotal"]) <= 5e-4 * s0.n
    x, _, f = eng.download()
    eng.close()
    s1 = s0.copy()
    s1.x = x
    r64 = capi.Engine(TERSOFF, ILP).compute_system(s1, eflag=False, vflag=False)
    assert np.abs(f - r64["f"]).max() <= MIX_F_ABS
    assert np.abs(r64["f"].sum(0)).max() <= 1e-9 * np.abs(r64["f"]).sum(0).max()


def test_two_engines_interleaved_share_constant_memory_safely():
    """Two engines with different parameter sets (Tersoff-only, ILP-only, as the two
    LAMMPS sub-styles hold them) alternate on one device; each call must use its own
    engine's tables."""
    g = load_golden("bilayer_small")
    et = capi.Engine(TERSOFF, None)
    ei = capi.Engine(None, ILP)
    for eng in (et, ei):
        eng.set_box(g["box_lo"], g["box_hi"], g["periodic"])
    for call in range(3):
        rt = et.compute(g["x"], g["type"], g["mol"], g["tag"], which=capi.TERSOFF, same_atoms=call > 0)
        ri = ei.compute(g["x"], g["type"], g["mol"], g["tag"], which=capi.ILP, same_atoms=call > 0)
        assert abs(rt["e_tersoff"] - g["e_tersoff"]) <= F64_TOL * abs(g["e_tersoff"]), call
        assert abs(ri["e_ilp"] - g["e_ilp"]) <= F64_TOL * abs(g["e_ilp"]), call
        assert rel_max(rt["f"] + ri["f"], g["f"]) <= F64_TOL, call


def _graph_vs_host_loop(prec, graph_list_cap=0, steps=60, thermo_every=20, check_every=0, temp=1500.0):
    """The same NVE run through the step graph and through the host-driven loop."""
    s = S.thermalize(S.twisted_bilayer(8, 8, 3.0, top="hbn"), temp, seed=11)
    out = []
    for graphs in (1, 0):
        eng = capi.Engine(TERSOFF, ILP, precision=prec, skin=0.4)
        eng.set_option("graphs", graphs)
        if check_every:
            eng.set_option("check_every", check_every)
        if graph_list_cap:
            eng.set_option("graph_list_cap", graph_list_cap)
        eng.upload(s)
        th = eng.run_nve(steps, 0.001, thermo_every=thermo_every)
        x, v, f = eng.download()
        out.append((x, v, f, th, eng.stats()))
    out.append(s)
    return out


@pytest.mark.parametrize("prec", [capi.FP64, capi.MIXED])
def test_step_graph_bitwise_equals_host_loop(prec):
    """Steps replayed as CUDA graphs (conditional rebuild node) give the bitwise-same
    trajectory, thermo output and rebuild count as the host-driven loop."""
    (xg, vg, fg, thg, sg), (xe, ve, fe, the, se), _ = _graph_vs_host_loop(prec)
    assert sg["graph_steps"] > 0 and se["graph_steps"] == 0
    assert se["rebuilds"] > 2                        # the small skin forces rebuilds inside graph chunks
    assert sg["rebuilds"] == se["rebuilds"]
    assert np.array_equal(xg, xe) and np.array_equal(vg, ve) and np.array_equal(fg, fe)
    assert [t["etotal"] for t in thg] == [t["etotal"] for t in the]
    assert len(thg) == 60 // 20 + 1


@pytest.mark.parametrize("check_every", [1, 4])
def test_step_graph_with_check_interval_bitwise_equals_host_loop(check_every):
    """A fixed rebuild-check interval (every step; every 4th with the look-ahead, one
    conditional node per 4-step graph) gives the same trajectory and rebuild count
    through the graphs as through the host-driven loop; forces equal a fresh FP64
    evaluation of the final positions (no pair was missed)."""
    (xg, vg, fg, thg, sg), (xe, ve, fe, the, se), s = _graph_vs_host_loop(capi.FP64, check_every=check_every,
                                                                          temp=300.0, steps=80)
    assert sg["graph_steps"] > 0 and sg["graph_redos"] == 0
    assert se["rebuilds"] >= 2 and sg["rebuilds"] == se["rebuilds"]
    assert np.array_equal(xg, xe) and np.array_equal(vg, ve) and np.array_equal(fg, fe)
    assert [t["etotal"] for t in thg] == [t["etotal"] for t in the]
    s1 = s.copy()
    s1.x = xg
    r = capi.Engine(TERSOFF, ILP).compute_system(s1, eflag=False, vflag=False)
    assert rel_max(fg, r["f"]) < 1e-10


@pytest.mark.parametrize("prec", [capi.FP64, capi.MIXED])
def test_programmatic_dependent_launch_changes_nothing(prec):
    """The chain kernels launched with programmatic dependent launch (option pdl = 31:
    every chain kernel early, dependents scheduled as each kernel starts, each waiting on
    the device for the kernel before it) and with ordinary launches: the same trajectory, thermo output and rebuild count through
    the step graphs (every 4th step a rebuild check), and the same single-point forces,
    energies and per-atom energies, to the bit."""
    s = S.thermalize(S.twisted_bilayer(8, 8, 3.0, top="hbn"), 1500.0, seed=11)
    out = []
    for pdl in (31, 0):
        eng = capi.Engine(TERSOFF, ILP, precision=prec, skin=0.4)
        eng.set_option("pdl", pdl)
        eng.set_option("check_every", 4)
        r = eng.compute_system(s, eatom=True)
        eng.upload(s)
        th = eng.run_nve(80, 0.001, thermo_every=20)
        out.append((r, eng.download(), th, eng.stats()))
        eng.close()
    (r1, (x1, v1, f1), th1, s1), (r0, (x0, v0, f0), th0, s0) = out
    assert np.array_equal(r1["f"], r0["f"]) and np.array_equal(r1["eatom"], r0["eatom"])
    assert r1["e_tersoff"] == r0["e_tersoff"] and r1["e_ilp"] == r0["e_ilp"]
    assert np.array_equal(r1["virial"], r0["virial"])
    assert s1["graph_steps"] > 0 and s1["rebuilds"] == s0["rebuilds"] >= 2
    assert np.array_equal(x1, x0) and np.array_equal(v1, v0) and np.array_equal(f1, f0)
    assert [t["etotal"] for t in th1] == [t["etotal"] for t in th0]


def test_step_graph_skin_trip_redo():
    """A check interval far too long for the motion (16 steps at 1500 K, skin 0.4 A):
    atoms move more than skin/2 between checks, the graph raises the trip and the chunk
    is redone on the host-driven loop, which rebuilds at such steps.  The result agrees
    with the host-driven run to FP64 rounding and its forces with a fresh evaluation."""
    (xg, vg, fg, thg, sg), (xe, ve, fe, the, se), s = _graph_vs_host_loop(capi.FP64, check_every=16)
    assert sg["graph_redos"] > 0
    assert sg["steps"] == se["steps"]
    assert np.abs(min_image(xg - xe, s.box_lo, s.box_hi, s.periodic)).max() < 1e-9
    assert rel_max(vg, ve) < 1e-7 and rel_max(fg, fe) < 1e-7
    for a, b in zip(thg, the):
        assert abs(a["etotal"] - b["etotal"]) <= 1e-10 * abs(b["etotal"])
    s1 = s.copy()
    s1.x = xg
    r = capi.Engine(TERSOFF, ILP).compute_system(s1, eflag=False, vflag=False)
    assert rel_max(fg, r["f"]) < 1e-10


def test_step_graph_overflow_redo():
    """A graph whose rebuild overflows its captured list capacity redoes the chunk on
    the host-driven path from a checkpoint of the chunk's first step.  The redo builds
    the list at that step, so sums run in another order: FP64 agreement, not bitwise."""
    (xg, vg, fg, thg, sg), (xe, ve, fe, the, se), s = _graph_vs_host_loop(capi.FP64, graph_list_cap=1000)
    assert sg["graph_redos"] > 0
    assert sg["steps"] == se["steps"]
    # positions are wrapped at rebuilds, which the redo moves: compare modulo the box
    assert np.abs(min_image(xg - xe, s.box_lo, s.box_hi, s.periodic)).max() < 1e-9
    assert rel_max(vg, ve) < 1e-7 and rel_max(fg, fe) < 1e-7
    for a, b in zip(thg, the):
        assert abs(a["etotal"] - b["etotal"]) <= 1e-10 * abs(b["etotal"])


@pytest.mark.parametrize("ev", [True, False])
@pytest.mark.parametrize("prec", [capi.FP64, capi.MIXED])
def test_moved_atoms_rebuild_the_list(prec, ev):
    """lmff_compute on already loaded atoms (LMFF_SAME_ATOMS) rebuilds the list when an
    atom moved past skin/2 since the last build and only then (force-only calls test the
    displacement after the evaluation and redo it on a rebuilt list).  Either way the
    accumulated forces (input f + forces) equal a fresh engine's, energies too."""
    g = load_golden("bilayer_small")
    eng = engine_for(g, precision=prec)
    compute_golden(eng, g)
    rb = eng.stats()["rebuilds"]
    skin = float(g["skin"])
    x1 = np.array(g["x"])
    x1[5, 2] += 0.25 * skin                            # out of plane, |d| = skin / 4: no rebuild
    f_in = np.random.default_rng(3).normal(0.0, 1.0, x1.shape)
    r1 = eng.compute(x1, g["type"], g["mol"], g["tag"], f=f_in.copy(), same_atoms=True, eflag=ev, vflag=ev)
    assert eng.stats()["rebuilds"] == rb
    x2 = x1 + [0.6 * skin, 0.25 * skin, 0.0]           # rigid shift, |d| > skin / 2: rebuild
    r2 = eng.compute(x2, g["type"], g["mol"], g["tag"], f=f_in.copy(), same_atoms=True, eflag=ev, vflag=ev)
    assert eng.stats()["rebuilds"] == rb + 1
    f_tol = F64_TOL * 10.0 if prec == capi.FP64 else MIX_F_ABS   # eV/A; the sums run in another order
    e_tol = 1e-12 if prec == capi.FP64 else MIX_E_REL
    for x, r in ((x1, r1), (x2, r2)):
        fresh = engine_for(g, precision=prec).compute(x, g["type"], g["mol"], g["tag"])
        assert np.abs(r["f"] - f_in - fresh["f"]).max() <= f_tol
        if ev:
            assert abs(r["e_ilp"] - fresh["e_ilp"]) <= e_tol * abs(fresh["e_ilp"])
            assert abs(r["e_tersoff"] - fresh["e_tersoff"]) <= e_tol * abs(fresh["e_tersoff"])
        else:
            assert r["e_ilp"] == 0.0 and r["e_tersoff"] == 0.0


@pytest.mark.parametrize("prec", [capi.FP64, capi.MIXED])
@pytest.mark.parametrize("name", ["bilayer_small", "hetero_small", "edges"])
def test_force_only_tersoff_lanes_equal_one_thread_routine(name, prec):
    """Small systems evaluate force-only Tersoff with one lane per bond (k_tersoff_lanes)
    and energy/virial evaluations with one thread per atom (k_tersoff): the lanes add the
    per-partner sums in the one-thread routine's order, so the forces agree to rounding."""
    g = load_golden(name)
    eng = engine_for(g, precision=prec)
    r_ev = eng.compute(g["x"], g["type"], g["mol"], g["tag"], which=capi.TERSOFF)
    r_f = eng.compute(g["x"], g["type"], g["mol"], g["tag"], which=capi.TERSOFF, eflag=False, vflag=False,
                      same_atoms=True)
    d = np.abs(r_f["f"] - r_ev["f"]).max()
    assert d <= 1e-13 * np.abs(r_ev["f"]).max(), d


@pytest.mark.parametrize("prec", [capi.FP64, capi.MIXED])
@pytest.mark.parametrize("name", ["bilayer_small", "hetero_small", "edges", "tiny_images"])
def test_small_system_variants_equal_large_system_kernels(name, prec):
    """The kernel variants small systems run (one warp per atom in the list build, 16
    lanes per atom in the intralayer lists, 8 in the gather, one lane per bond in
    Tersoff alone) against the large-system kernels (option small_variants 0): the same
    lists entry for entry and the same forces, energies and per-atom energies to the bit;
    Tersoff alone with one lane per bond agrees with the one-thread kernel to rounding: the
    one-thread force-only kernel adds each three-body product into its partner's sum in
    one FMA, the lanes (like the one-thread energy/virial kernel, which uses the product
    twice) round it first (FP64 ~1e-15, the FP32 sums of the mixed mode ~1e-8 relative)."""
    g = load_golden(name)
    out = {}
    for sv in (1, 0):
        eng = engine_for(g, precision=prec, small_variants=sv)
        args = (g["x"], g["type"], g["mol"], g["tag"])
        rf = eng.compute(*args, eflag=False, vflag=False)
        lists = (eng.export_list(0), eng.export_list(1))
        rt = eng.compute(*args, which=capi.TERSOFF, eflag=False, vflag=False, same_atoms=True)
        re = eng.compute(*args, eatom=True, same_atoms=True)
        out[sv] = (rf, lists, rt, re)
        eng.close()
    (rf1, l1, rt1, re1), (rf0, l0, rt0, re0) = out[1], out[0]
    assert np.array_equal(l1[0], l0[0]) and np.array_equal(l1[1], l0[1])
    assert np.array_equal(rf1["f"], rf0["f"])
    rel = 1e-13 if prec == capi.FP64 else 1e-6
    assert np.abs(rt1["f"] - rt0["f"]).max() <= rel * np.abs(rt0["f"]).max()
    assert np.array_equal(re1["f"], re0["f"]) and np.array_equal(re1["eatom"], re0["eatom"])
    for k in ("e_tersoff", "e_ilp"):
        assert re1[k] == re0[k]
    assert np.array_equal(re1["virial"], re0["virial"])


def test_host_positions_in_another_periodic_image_need_no_rebuild():
    """A caller may pass unwrapped coordinates, or wrap some atoms between calls (LAMMPS
    does at reneighbouring): the engine takes each position in the image its list was
    built with, so the forces are unchanged and no rebuild is triggered."""
    g = load_golden("bilayer_small")
    eng = engine_for(g)
    r0 = compute_golden(eng, g)
    rb = eng.stats()["rebuilds"]
    L = g["box_hi"] - g["box_lo"]
    x = np.array(g["x"])
    x[::3, 0] += L[0]
    x[1::5, 1] -= 2 * L[1]
    r1 = eng.compute(x, g["type"], g["mol"], g["tag"], same_atoms=True)
    assert eng.stats()["rebuilds"] == rb
    assert rel_max(r1["f"], r0["f"]) < 1e-12
    assert abs(r1["e_ilp"] - r0["e_ilp"]) <= 1e-12 * abs(r0["e_ilp"])
