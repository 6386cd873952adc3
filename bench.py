"""Benchmark: atom-steps/s of the Tersoff + ILP path on the 2.7M-atom graphite slab.

Workload (default): 10-layer AB graphite, 342 x 197 rectangular cells per layer
(269,496 atoms/layer, 2,694,960 atoms, 841 x 839 A, 3.35 A spacing, periodic x/y),
alternating molecule ids, 300 K Gaussian velocities from a seed; velocity-Verlet NVE
with dt = 1 fs, device resident, mixed precision (FP32 pair arithmetic, FP64
integration and accumulation).  One step = integrate + [neighbour check/rebuild] +
Tersoff + ILP forces.  Synthetic inputs generated here (the reference's own large data
files are not available).

Timing: W untimed warm-up steps, then exactly K steps timed on the device with CUDA
events on the engine's stream (lmff_stats.ms_last_run), bracketed by
torch.cuda.synchronize() (and a barrier with N > 1).  On the 2.7M-atom slab the
inputs are far larger than L2 (the pair list alone is 10 GB), so no L2 flush is needed;
config.l2 states the list size of each workload.  A second, host-driven run of
max(K, --kernel-steps) steps times every kernel launch with CUDA events: the roofline
averages, the launches per step, and the neighbour rebuilds (time per rebuild, steps
between rebuilds, the amortised cost per step); rebuilds_in_timed_region counts the
rebuilds inside the K timed steps.  Algorithmic flops come from bench/flops.h (the
oracle's arithmetic, op-counted by oracle/opcount.py).

With one GPU the line also carries the chosen forms' targets, measured in the same run:
plain_fp64 (the all-FP64 drop-in on the same slab), batched (256 bilayer replicas,
batched mixed vs one-at-a-time FP64), served (the Poisson stream, the server's
closed-loop capacity vs one-at-a-time FP64 over the whole stream, and open-loop
p50/p99), and form_ratios (the ratios and their targets).  --no-forms skips them.

Multi-GPU: the path is run as independent replicas (one system per GPU, no data-path
collective): value = total atom-steps of all ranks / max rank time, scaling "weak".

--impl reference: the CPU arm (the oracle restatement of the reference's CPU algorithm,
OpenMP over all host cores) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "lammps-lmff_gb300"))

import numpy as np  # noqa: E402

METRIC = "atom-steps/s at 2.7M-atom graphite"
UNIT = "atom-steps/s"
TERSOFF_FILE = os.path.join(ROOT, "lammps-lmff_gb300", "potentials", "BNC.tersoff")
ILP_FILE = os.path.join(ROOT, "lammps-lmff_gb300", "potentials", "BNCH.ILP")

# DRAM bytes per pair-list entry of the mixed pair kernel, from one ncu capture of the
# 331,200-atom graphite slab (k_ilp<16,0,0,1,0,0,1>: 1.297 GB read + 20.1 MB written for
# 310,301,280 entries; the list is larger than L2, so traffic grows with the entries)
K_ILP_DRAM_BYTES_PER_ENTRY = (1.297430e9 + 20.068096e6) / 310301280
# FP64-pipe activity of the two FP64-bound per-atom kernels of the mixed step (ncu
# sm__pipe_fp64_cycles_active on the 331,200-atom slab, profiles/)
FP64_PIPE_ACTIVE_NCU = {"k_tersoff": 0.624, "k_nderiv": 0.824}
L2_BYTES = 129e6   # GB300 L2
FLOPS_H = os.path.join(ROOT, "bench", "flops.h")


def read_flops(path: str = FLOPS_H) -> dict:
    """The algorithmic operation counts frozen in bench/flops.h (oracle/opcount.py: the
    oracle compiled with an operation-counting double on the benchmark's CPU sample)."""
    out = {}
    for line in open(path):
        p = line.split()
        if len(p) == 3 and p[0] == "#define" and p[1].startswith("LMFF_"):
            out[p[1][5:]] = float(p[2])
    return out


FLOPS = read_flops()


def alg_flops_pair_kernel(pairs: int, entries: int) -> float:
    """The reference's arithmetic for one pair-kernel launch: every list candidate's
    displacement and r^2, and per directed pair in the cutoff the repulsion term with
    the normal of i and its share of the vdW term (calc_FRep / calc_FvdW).  calc_FRep's
    normal-derivative terms (dn_i/dx_i and the intralayer neighbours k) are counted with
    the normal-derivative kernel, which applies them once per atom."""
    per_pair = FLOPS["FLOPS_ILP_PAIR"] + FLOPS["VDW_PER_PAIR"] * FLOPS["FLOPS_ILP_VDW"]
    return entries * FLOPS["FLOPS_ILP_CAND"] + pairs * per_pair


def alg_flops_nderiv(n_ilp_atoms: int) -> float:
    """calc_normal's Jacobians and their application to dE/dn_i: the dn_i/dx_i term and
    one term per intralayer neighbour, once per atom (reverse-accumulated, as LMFF's
    dprodni)."""
    return n_ilp_atoms * (FLOPS["FLOPS_NORMAL"] + (1.0 + FLOPS["KTERMS_PER_PAIR"]) * FLOPS["FLOPS_ILP_KTERM"])


def alg_flops_tersoff(natoms: int) -> float:
    """Tersoff arithmetic of sp2 carbon (3 bonds, 6 triplets per atom), per atom as
    counted on the graphite sample."""
    return natoms * FLOPS["FLOPS_TERSOFF_ATOM"]


def workload(name: str):
    from lmff_gb300 import structures as S
    if name == "graphite_2p7m":
        s = S.graphite_slab(10, 342, 197, spacing=3.35, mol_mode="alternate")
    elif name == "bilayer_7200":
        s = S.ab_bilayer_graphene(30, 30)
    elif name == "graphite_small":
        s = S.graphite_slab(10, 40, 23, spacing=3.35, mol_mode="alternate")
    elif name == "graphite_330k":
        s = S.graphite_slab(10, 120, 69, spacing=3.35, mol_mode="alternate")
    elif name == "twisted_500k":
        s = S.twisted_graphene_hbn_500k(seed=2)
    else:
        raise SystemExit(f"unknown workload {name}")
    return S.thermalize(s, 300.0, seed=3)


def cpu_sample():
    """Bounded CPU sample of the same workload: a 98 x 98 A periodic patch of the same
    10-layer graphite slab (36,800 atoms), same density and per-atom neighbour counts."""
    from lmff_gb300 import structures as S
    return S.thermalize(S.graphite_slab(10, 40, 23, spacing=3.35, mol_mode="alternate"), 300.0, seed=3)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        load = [v for v in sm if v > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        try:
            return json.load(open(path))
        except ValueError:
            return {}
    return {}


def fp_peak_tflops(dtype_name: str) -> float:
    """SIMT peak measured here: cuBLAS GEMM at 8192^3 in FP32 (TF32 off) or FP64, best of 5
    after warm-up (MEASURED_PEAKS.json carries HBM and bf16 tensor peaks only)."""
    import torch
    torch.backends.cuda.matmul.allow_tf32 = False
    dt = torch.float32 if dtype_name == "fp32" else torch.float64
    n = 8192 if dt == torch.float32 else 4096
    a = torch.randn(n, n, device="cuda", dtype=dt)
    b = torch.randn(n, n, device="cuda", dtype=dt)
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    torch.cuda.empty_cache()
    return 2.0 * n ** 3 / best / 1e12


def time_cpu_baseline(nsteps: int, warm: int, nthreads: int):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    s = cpu_sample()
    o = Oracle(TERSOFF_FILE, ILP_FILE, nthreads=nthreads)
    x = s.x.copy()
    v = s.v.copy()
    o.set_atoms(x, s.type, s.mol, s.tag, s.box_lo, s.box_hi, s.periodic)
    f = o.forces()["f"]
    masses = [12.011, 10.811, 14.0067]
    if warm:
        o.nve(warm, 0.001, masses, x, v, f)
    t0 = time.perf_counter()
    o.nve(nsteps, 0.001, masses, x, v, f)
    dt = time.perf_counter() - t0
    return s.n * nsteps / dt, s.n, dt


def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    nthreads = os.cpu_count() or 1
    steps = max(1, args.steps)
    value, natoms, dt = time_cpu_baseline(steps, args.warmup, nthreads)
    sample = (f"{natoms}-atom 98x98 A periodic patch of the same 10-layer graphite, {steps} NVE steps "
              f"(+{args.warmup} warm-up), oracle restatement of the reference CPU algorithm")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": steps, "warmup": args.warmup, "ms_per_step": dt / steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "10-layer AB graphite, 2.7M atoms (CPU runs a 36.8k-atom patch of it)",
                       "precision": "fp64", "sample_atoms": natoms},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def max_over_ranks(x: float, dist=None) -> float:
    """The largest x over the ranks of the default process group (x itself without one):
    the job's time is its slowest rank's.  CPU tensor under gloo, device tensor under
    NCCL."""
    if dist is None or not dist.is_initialized():
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world: int, natoms: int, steps: int, tmax: float) -> float:
    """Whole-job atom-steps/s of `world` independent replicas of `natoms` atoms, each
    running `steps` steps, the slowest taking `tmax` seconds (weak scaling)."""
    return world * natoms * steps / tmax


def _sync_wall(fn, reps: int) -> float:
    """Wall seconds per call of fn (every call returns with its GPU work finished)."""
    t0 = time.perf_counter()
    for _ in range(reps):
        fn()
    return (time.perf_counter() - t0) / reps


def bench_replicas(args, local: int) -> dict:
    """256 independent bilayer replicas, 50/50 graphene/graphene and graphene/hBN, atom
    counts log-uniform in [500, 20000], twist U[0, 5] deg, spacing U[3.2, 3.6] A (seeded),
    each displaced by N(0, 0.02 A): energies, forces and virial of every replica.
    Batched = one launch per kernel over all replicas (lmff_batch_set +
    lmff_batch_compute: host arrays in, forces and per-replica energies/virials out).
    Baseline = the same evaluations one replica at a time through lmff_compute.  Single
    points reuse no list, so both build theirs without a skin (skin 0)."""
    from lmff_gb300 import capi
    from lmff_gb300 import structures as S
    systems = [S.displace(s, 0.02, seed=k) for k, s in enumerate(S.replica_set(256, 500, 20000, seed=4))]
    ntot = sum(s.n for s in systems)
    out = {}
    for name, prec in (("mixed", capi.MIXED), ("fp64", capi.FP64)):
        eng = capi.Engine(TERSOFF_FILE, ILP_FILE, device=local, precision=prec, skin=0.0)
        eng.batch_set(systems)
        eng.batch_compute()

        def batched():
            eng.batch_set(systems)
            eng.batch_compute()
        reps = max(3, args.steps // 4)
        t_b = _sync_wall(batched, reps)
        t_set = _sync_wall(lambda: eng.batch_set(systems), reps)
        t_cmp = _sync_wall(eng.batch_compute, reps)
        st = eng.stats()
        # device-resident re-evaluation of the loaded batch (no host copies, no rebuild)
        t_r = _sync_wall(lambda: eng.compute_resident(eflag=True, vflag=True), max(3, args.steps // 4))
        seq = capi.Engine(TERSOFF_FILE, ILP_FILE, device=local, precision=prec, skin=0.0)
        for s_ in systems[:8]:
            seq.compute_system(s_)
        t0 = time.perf_counter()
        for s_ in systems:
            seq.compute_system(s_)
        t_s = time.perf_counter() - t0
        out[name] = {"batched_s": t_b, "batch_set_s": t_set, "batch_compute_s": t_cmp,
                     "build_ms": st["ms_last_build"], "forces_ms": st["ms_last_forces"],
                     "resident_s": t_r, "one_at_a_time_s": t_s,
                     "batched_replicas_per_s": len(systems) / t_b, "one_at_a_time_replicas_per_s": len(systems) / t_s}
        del eng, seq
    value = out["mixed"]["batched_replicas_per_s"]
    return {"metric": "replica evaluations/s (E+F+W), 256 bilayer replicas", "value": value,
            "unit": "replicas/s", "n_gpus": 1, "higher_is_better": True, "data": "synthetic",
            "dtype": "f32", "config": {"workload": "256 bilayer replicas, 500-20000 atoms log-uniform",
                                       "atoms_total": ntot, "precision": "mixed", "skin": 0.0},
            "batched_mixed_vs_one_at_a_time_fp64": value / out["fp64"]["one_at_a_time_replicas_per_s"],
            "atom_evals_per_s_batched_mixed": ntot / out["mixed"]["batched_s"],
            "atom_evals_per_s_resident_mixed": ntot / out["mixed"]["resident_s"],
            "detail": out}


def bench_serving(args, local: int) -> dict:
    """Poisson request stream: 200 requests/s, 70 % single points and 30 % 100-step NVE
    runs at 300 K, bilayers of 1k-200k atoms (log-uniform on a 24-value grid), seeded.
    The server (mixed precision, 150 GB admission budget) replays the stream in real time
    (open loop: latency p50/p99, solves/s) and all at once (closed loop: capacity); the
    baseline serves the same whole stream one request at a time in plain FP64 (and in
    mixed precision, for reference)."""
    from lmff_gb300 import capi, serve
    stream = serve.poisson_stream(count=args.serve_requests, rate=200.0, seed=7)
    proto = capi.Engine(TERSOFF_FILE, ILP_FILE, device=local, precision=capi.MIXED)
    srv = serve.Server(proto, hbm_budget_bytes=150e9, md_chunk_steps=args.serve_chunk)
    serve.replay(srv, stream[:8], realtime=False)          # warm-up: allocations, graphs
    openl = serve.replay(srv, stream, realtime=True)
    closed = serve.replay(srv, stream, realtime=False)
    st = srv.stats()
    srv.close()
    seq64 = serve.replay_sequential(capi.Engine(TERSOFF_FILE, ILP_FILE, device=local, precision=capi.FP64),
                                    stream, realtime=False)
    seqmx = serve.replay_sequential(capi.Engine(TERSOFF_FILE, ILP_FILE, device=local, precision=capi.MIXED),
                                    stream, realtime=False)
    return {"metric": "solves/s, Poisson 200 req/s stream", "value": openl["solves_per_s"], "unit": "solves/s",
            "n_gpus": 1, "higher_is_better": True, "data": "synthetic", "dtype": "f32",
            "config": {"workload": f"{len(stream)} requests, 200 req/s, 30% 100-step NVE, 1k-200k atom bilayers",
                       "precision": "mixed", "md_chunk_steps": args.serve_chunk, "budget_gb": 150},
            "open_loop": openl, "closed_loop": closed,
            "one_at_a_time_fp64": seq64, "one_at_a_time_mixed": seqmx,
            "capacity_vs_one_at_a_time_fp64": closed["solves_per_s"] / seq64["solves_per_s"],
            "server_stats": st}


def bench_drift(args, local: int) -> dict:
    """NVE energy drift of the 7,200-atom AB bilayer at 300 K, dt 1 fs: slope of a
    least-squares line through the total energy sampled every 1000 steps."""
    from lmff_gb300 import capi
    from lmff_gb300 import structures as S
    s = S.thermalize(S.ab_bilayer_graphene(30, 30), 300.0, seed=3)
    out = {}
    for name, prec, nsteps in (("mixed", capi.MIXED, args.drift_steps_mixed),
                               ("fp64", capi.FP64, args.drift_steps_fp64)):
        eng = capi.Engine(TERSOFF_FILE, ILP_FILE, device=local, precision=prec)
        eng.upload(s)
        t0 = time.perf_counter()
        th = eng.run_nve(nsteps, 0.001, thermo_every=1000)
        wall = time.perf_counter() - t0
        t_ps = np.array([t["step"] for t in th]) * 0.001
        e = np.array([t["etotal"] for t in th])
        slope = np.polyfit(t_ps, e, 1)[0]                  # eV / ps
        out[name] = {"steps": nsteps, "ns": nsteps * 1e-6, "drift_mev_per_atom_per_ns": slope * 1e3 * 1e3 / s.n,
                     "etotal_first": float(e[0]), "etotal_last": float(e[-1]),
                     "max_abs_dev_mev_per_atom": float(np.abs(e - e[0]).max() * 1e3 / s.n),
                     "temp_last": th[-1]["temp"], "wall_s": wall, "atom_steps_per_s": s.n * nsteps / wall,
                     "graph_steps": eng.stats()["graph_steps"]}
    return {"metric": "NVE energy drift, 7200-atom bilayer, 300 K, dt 1 fs", "value":
            out["mixed"]["drift_mev_per_atom_per_ns"], "unit": "meV/atom/ns", "n_gpus": 1,
            "higher_is_better": False, "data": "synthetic", "dtype": "f32", "detail": out}


SPECIAL = {"replicas_256": bench_replicas, "serve_poisson": bench_serving, "drift_c1": bench_drift}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="graphite_2p7m")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--tpa", type=int, default=0, help="threads per atom (0: autotune)")
    ap.add_argument("--block", type=int, default=0, help="threads per block (0: autotune)")
    ap.add_argument("--skin", type=float, default=0.0, help="neighbour skin in A (0: autotune)")
    ap.add_argument("--tile", type=int, default=0, help="pair-loop tile, list entries per lane and iteration "
                                                         "(1 or 2; 0: autotune)")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-peak", action="store_true", help="skip the cuBLAS peak measurement")
    ap.add_argument("--kernel-steps", type=int, default=200,
                    help="steps of the per-kernel timing run (also gives the rebuild interval)")
    ap.add_argument("--fp64-steps", type=int, default=3, help="timed steps of the plain FP64 sub-record")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the plain-FP64, batched and served sub-records")
    ap.add_argument("--serve-requests", type=int, default=200)
    ap.add_argument("--serve-chunk", type=int, default=20)
    ap.add_argument("--drift-steps-mixed", type=int, default=1000000)
    ap.add_argument("--drift-steps-fp64", type=int, default=100000)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo" if args.impl == "reference" else "nccl")
    if args.impl == "reference":
        run_reference(args, rank, world)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    import torch
    torch.cuda.set_device(local)
    from lmff_gb300 import build, capi
    if rank == 0:
        build.build()
    if dist:
        dist.barrier()
    if rank != 0:
        build.build()

    if args.workload in SPECIAL:
        line = SPECIAL[args.workload](args, local)
        if rank == 0:
            print(json.dumps(line), flush=True)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    s = workload(args.workload)
    prec = capi.MIXED if args.precision == "mixed" else capi.FP64
    # pure carbon: one atom type mapped to C (pair_coeff * * <style> <file> C)
    elements = ("C",) if set(np.unique(s.type)) == {1} else ("C", "B", "N")
    tuned = None
    if not (args.tpa and args.block and args.skin and args.tile):
        from lmff_gb300 import tune
        # tuned on the workload itself: a smaller patch of the same slab ranks the launch
        # shapes differently (measured: 16 threads per atom best at 331k, 8 at 2.7M)
        # small systems also try 32 threads per atom: the pair kernel's time there is one
        # thread's walk over its share of the list
        tuned = tune.tune(s, TERSOFF_FILE, ILP_FILE, elements=elements, precision=prec, device=local,
                          tpas=(8, 16, 32) if s.n < 100_000 else (8, 16), blocks=(128, 256),
                          skins=(1.0, 1.5, 2.0) if s.n < 100_000 else (1.0, 2.0),
                          use_cache=False, n_full=s.n, tiles=(2, 1))
        args.tpa = args.tpa or tuned["tpa"]
        args.block = args.block or tuned["block"]
        args.skin = args.skin or tuned["skin"]
        args.tile = args.tile or tuned.get("tile", 2)
    m = run_md(s, prec, elements, local, args.tpa, args.block, args.skin, args.warmup, args.steps,
               args.kernel_steps, dist, clocks=True, tile=args.tile)
    value = replica_throughput(world, s.n, args.steps, m["tmax"])
    ms_per_step = m["tmax"] / args.steps * 1e3
    launches_total = sum(m["launches_per_step"].values()) * args.steps

    # e2e through the drop-in call (lmff_compute) with pinned host buffers
    e2e = None
    if args.e2e_steps > 0:
        e2e = bench_e2e(s, prec, elements, local, args, world)

    peaks = measured_peaks()
    pk = {"fp32": 0.0, "fp64": 0.0}
    if rank == 0 and not args.no_peak:
        pk = {"fp32": fp_peak_tflops("fp32"), "fp64": fp_peak_tflops("fp64")}
    rl = rooflines(m, s, prec, pk, peaks)

    cpu = None
    if rank == 0 and not args.no_cpu:
        nthreads = os.cpu_count() or 1
        cv, cn, cdt = time_cpu_baseline(args.cpu_steps, 1, nthreads)
        cpu = {"value": cv, "unit": UNIT, "cores": nthreads, "kind": "port",
               "sample": f"{cn}-atom 98x98 A patch of the same slab, {args.cpu_steps} NVE steps, "
                         f"oracle restatement, {cdt:.1f} s"}

    # the chosen forms' targets, on one GPU: plain FP64 on the same system, batched
    # replicas and the served Poisson stream against one-at-a-time FP64
    forms = None
    if rank == 0 and world == 1 and not args.no_forms and args.workload == "graphite_2p7m":
        forms = form_records(args, s, elements, local, value, pk)

    if rank == 0:
        # the pair list is what every step streams from HBM; say whether it fits in the
        # 129 MB L2 (no flush between steps either way: the steps of an MD run re-read it)
        st = m["stats"]
        list_bytes = 4.0 * st["list_per_atom"] * s.n
        l2_note = (f"inputs larger than L2 (pair list {list_bytes / 1e9:.1f} GB), no flush"
                   if list_bytes > L2_BYTES else
                   f"pair list {list_bytes / 1e6:.1f} MB fits in L2; no flush (MD steps re-read it)")
        metric = METRIC if args.workload == "graphite_2p7m" else f"atom-steps/s, workload {args.workload}"
        line = {"metric": metric, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32" if prec == capi.MIXED else "f64", "data": "synthetic",
                "config": {"workload": "10-layer AB graphite slab, 2,694,960 atoms, 300 K NVE dt 1 fs"
                           if args.workload == "graphite_2p7m" else args.workload,
                           "natoms": s.n, "precision": args.precision, "tpa": args.tpa, "block": args.block,
                           "skin": args.skin, "pair_tile": args.tile, "elements": list(elements),
                           "autotune": None if tuned is None else {
                               "probe_atoms": tuned["probe_atoms"],
                               "picked": [tuned["tpa"], tuned["block"], tuned["skin"], tuned.get("tile", 2)],
                               "score_ms_probe": tuned["score_ms"]},
                           "l2": l2_note,
                           "parallelism": f"replicas x{world}", "wall_s": m["wall"]},
                "clocks": m["clocks"], "roofline": rl["k_ilp"],
                "rooflines_other": {k: v for k, v in rl.items() if k != "k_ilp"},
                "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": launches_total, "graph_steps_timed": m["graph_steps"],
                "rebuilds_in_timed_region": m["rebuilds_timed"], "rebuild": m["rebuild"],
                "kernel_ms_avg": m["kernel_ms_avg"], "list_per_atom": st["list_per_atom"]}
        if forms is not None:
            line.update(forms)
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def run_md(s, prec, elements, local, tpa, block, skin, warmup, steps, kernel_steps, dist=None, clocks=False,
           tile=2):
    """Device-resident NVE of system s: `warmup` untimed steps, `steps` timed steps (the
    production loop: steps replayed as CUDA graphs, device time from CUDA events on the
    engine's stream), then a host-driven run of max(steps, kernel_steps) steps with CUDA
    events around every kernel launch: per-kernel averages, launches per step and the
    neighbour-rebuild statistics."""
    import torch
    from lmff_gb300 import capi
    eng = capi.Engine(TERSOFF_FILE, ILP_FILE, elements=elements, device=local, precision=prec)
    eng.set_option("tpa", tpa)
    eng.set_option("block", block)
    eng.set_option("skin", skin)
    eng.set_option("pair_tile", tile)
    eng.upload(s)
    eng.run_nve(warmup, 0.001)
    eng.set_option("count_pairs", 1)
    sampler = ClockSampler(local) if clocks else None
    if sampler:
        sampler.start()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    r0 = eng.stats()["rebuilds"]
    t0 = time.perf_counter()
    eng.run_nve(steps, 0.001)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    clk = sampler.stop() if sampler else None
    st = eng.stats()
    out = {"wall": wall, "clocks": clk, "graph_steps": st["graph_steps"], "rebuilds_timed": st["rebuilds"] - r0,
           "tmax": max_over_ranks(st["ms_last_run"] / 1e3, dist)}
    nk = max(steps, kernel_steps)
    r1 = st["rebuilds"]
    eng.set_option("kernel_timing", 1)
    eng.set_option("reset_timing", 1)
    eng.run_nve(nk, 0.001)
    eng.set_option("kernel_timing", 0)
    st = eng.stats()
    kms, kn = st["kernel_ms"], st["kernel_launches"]
    out["stats"] = st
    out["kernel_ms_avg"] = {k: (kms[k] / kn[k] if kn[k] else None) for k in kms}
    out["launches_per_step"] = {k: kn[k] / nk for k in kn}
    rb = st["rebuilds"] - r1
    rb_ms = kms["neighbor_build"] / kn["neighbor_build"] if kn["neighbor_build"] else None
    out["rebuild"] = {"steps_observed": nk, "rebuilds_observed": rb, "ms_per_rebuild": rb_ms,
                      "steps_per_rebuild": nk / rb if rb else None,
                      "amortised_ms_per_step": rb_ms * rb / nk if rb else 0.0}
    eng.close()
    return out


def rooflines(m, s, prec, pk, peaks) -> dict:
    """Roofline entries of the pair kernel (the dominant one) and of the two FP64-bound
    per-atom kernels; algorithmic flops from bench/flops.h over the CUDA-event average."""
    from lmff_gb300 import capi
    st = m["stats"]
    ka = m["kernel_ms_avg"]
    pairs, cands = st["pairs_in_cutoff"], st["list_entries"]
    name = "fp32" if prec == capi.MIXED else "fp64"
    k_s = ka["pair_ilp"] / 1e3
    achieved = alg_flops_pair_kernel(pairs, cands) / k_s / 1e12
    out = {"k_ilp": {
        "bound": name, "achieved": achieved, "peak": pk[name], "unit": "TFLOP/s",
        "frac": achieved / pk[name] if pk[name] else None,
        "traffic": K_ILP_DRAM_BYTES_PER_ENTRY * cands if prec == capi.MIXED else None,
        "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_ilp launch on the "
                          "331,200-atom slab (1.317 GB for 310.3 M list entries), scaled by list entries",
        "kernel": "k_ilp (pair kernel)", "kernel_ms_avg": ka["pair_ilp"],
        "peak_source": f"cuBLAS {name.upper()} GEMM measured in this run (SIMT; MEASURED_PEAKS.json has HBM "
                       f"{peaks.get('hbm_gbs')} GB/s and bf16 tensor only)",
        "pairs_in_cutoff": pairs, "list_entries": cands,
        "alg_flops_source": "bench/flops.h (op count of the oracle)",
        "alg_flops_per_pair": FLOPS["FLOPS_ILP_CAND"] + FLOPS["FLOPS_ILP_PAIR"]
        + FLOPS["VDW_PER_PAIR"] * FLOPS["FLOPS_ILP_VDW"],
        "alg_flops_per_rejected": FLOPS["FLOPS_ILP_CAND"],
        "hbm_gbs_of_list_stream": cands * 4 / k_s / 1e9, "hbm_peak_gbs": peaks.get("hbm_gbs")}}
    for kern, key, flops in (("k_tersoff", "tersoff", alg_flops_tersoff(s.n)),
                             ("k_nderiv", "normal_deriv", alg_flops_nderiv(s.n))):
        t = ka.get(key)
        if not t:
            continue
        a = flops / (t / 1e3) / 1e12
        e = {"bound": "fp64", "kernel_ms_avg": t, "alg_flops": flops, "achieved_alg": a, "unit": "TFLOP/s",
             "peak_fp64": pk["fp64"], "peak_fp32": pk["fp32"]}
        if prec == capi.FP64:
            e["frac"] = a / pk["fp64"] if pk["fp64"] else None
            e["frac_source"] = "algorithmic flops over the measured DGEMM peak"
        else:
            # the mixed kernels do the reference's FP64 arithmetic partly in FP32 and in
            # fewer FP64 operations, so their position on the FP64 roofline is the
            # measured FP64-pipe activity
            e["frac"] = FP64_PIPE_ACTIVE_NCU[kern]
            e["frac_source"] = "ncu sm__pipe_fp64_cycles_active, 331,200-atom slab (profiles/)"
            e["alg_frac_of_fp32_peak"] = a / pk["fp32"] if pk["fp32"] else None
        out[kern] = e
    return out


def bench_e2e(s, prec, elements, local, args, world) -> dict:
    """The same force evaluation through lmff_compute with pinned host x in and host f
    out per step (host<->device copies inside the timed region)."""
    import torch
    from lmff_gb300 import capi
    xa = torch.empty((s.n, 3), dtype=torch.float64, pin_memory=True).numpy()
    xb = torch.empty((s.n, 3), dtype=torch.float64, pin_memory=True).numpy()
    fb = torch.empty((s.n, 3), dtype=torch.float64, pin_memory=True).numpy()
    xa[:] = s.x
    xb[:] = s.x + np.random.default_rng(1).normal(0.0, 0.01, s.x.shape)
    eng2 = capi.Engine(TERSOFF_FILE, ILP_FILE, elements=elements, device=local, precision=prec)
    eng2.set_option("tpa", args.tpa)
    eng2.set_option("block", args.block)
    eng2.set_option("skin", args.skin)
    eng2.set_option("pair_tile", args.tile)
    eng2.set_box(s.box_lo, s.box_hi, s.periodic)
    eng2.compute(xa, s.type, s.mol, s.tag, eflag=False, vflag=False, f=fb, overwrite=True)
    eng2.compute(xb, s.type, s.mol, s.tag, eflag=False, vflag=False, f=fb, overwrite=True, same_atoms=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.e2e_steps):
        eng2.compute(xa if k % 2 == 0 else xb, s.type, s.mol, s.tag, eflag=False, vflag=False, f=fb,
                     overwrite=True, same_atoms=True)
    torch.cuda.synchronize()
    te = time.perf_counter() - t0
    eng2.close()
    return {"value": world * s.n * args.e2e_steps / te, "unit": UNIT, "h2d_bytes_per_step": int(xa.nbytes),
            "d2h_bytes_per_step": int(fb.nbytes),
            "path": "lmff_compute: pinned host x in, host f out, per force evaluation"}


def form_records(args, s, elements, local, mixed_value, pk) -> dict:
    """Sub-records for the chosen forms' targets, measured in the same run:
    plain_fp64 -- the all-FP64 drop-in on the same slab (tpa 16, block 128, skin 1 A);
    batched -- 256 bilayer replicas, E+F+W, batched mixed vs one-at-a-time FP64;
    served -- the Poisson stream, server (mixed) vs one-at-a-time FP64, whole stream."""
    from lmff_gb300 import capi
    out = {}
    m = run_md(s, capi.FP64, elements, local, 16, 128, 1.0, 1, args.fp64_steps, 0)
    v64 = s.n * args.fp64_steps / m["tmax"]
    rl = rooflines(m, s, capi.FP64, pk, measured_peaks())
    out["plain_fp64"] = {"value": v64, "unit": UNIT, "steps": args.fp64_steps,
                         "ms_per_step": m["tmax"] / args.fp64_steps * 1e3, "tpa": 16, "block": 128, "skin": 1.0,
                         "roofline": rl["k_ilp"], "roofline_tersoff": rl.get("k_tersoff"),
                         "roofline_nderiv": rl.get("k_nderiv"), "kernel_ms_avg": m["kernel_ms_avg"],
                         "rebuilds_in_timed_region": m["rebuilds_timed"]}
    rep = bench_replicas(args, local)
    out["batched"] = {"value": rep["value"], "unit": rep["unit"], "config": rep["config"],
                      "one_at_a_time_fp64_replicas_per_s": rep["detail"]["fp64"]["one_at_a_time_replicas_per_s"],
                      "batched_fp64_replicas_per_s": rep["detail"]["fp64"]["batched_replicas_per_s"],
                      "resident_mixed_replicas_per_s": 256 / rep["detail"]["mixed"]["resident_s"],
                      "ratio_vs_one_at_a_time_fp64": rep["batched_mixed_vs_one_at_a_time_fp64"]}
    srv = bench_serving(args, local)
    out["served"] = {"open_loop": srv["open_loop"], "closed_loop": srv["closed_loop"],
                     "one_at_a_time_fp64": srv["one_at_a_time_fp64"], "config": srv["config"],
                     "capacity_vs_one_at_a_time_fp64": srv["capacity_vs_one_at_a_time_fp64"]}
    out["form_ratios"] = {"mixed_vs_plain_fp64": mixed_value / v64, "target_mixed_vs_plain": 1.8,
                         "batched_vs_one_at_a_time_fp64": rep["batched_mixed_vs_one_at_a_time_fp64"],
                         "served_capacity_vs_one_at_a_time_fp64": srv["capacity_vs_one_at_a_time_fp64"],
                         "target_batched_served": 5.0}
    return out


if __name__ == "__main__":
    main()
