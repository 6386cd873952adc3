"""Serving many independent requests on one GPU (the lmff_server_* C ABI).

A request is one bilayer system: a single point (forces, energies, virial) or an NVE
run.  ``Server`` wraps the native server (submission queue, admission by a device
memory budget, continuous batching; csrc/server.cpp).  ``poisson_stream`` builds a
seeded request stream, ``replay`` plays it against a server in real time (open loop)
or all at once (closed loop, capacity), and ``replay_sequential`` plays it one request
at a time on a plain engine: the one-at-a-time baseline.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import capi
from . import structures as S


class Request(C.Structure):
    _fields_ = [("natoms", C.c_int), ("x", C.c_void_p), ("v", C.c_void_p), ("type", C.c_void_p),
                ("mol", C.c_void_p), ("lo", C.c_double * 3), ("hi", C.c_double * 3), ("periodic", C.c_int * 3),
                ("nsteps", C.c_int), ("dt", C.c_double), ("f_out", C.c_void_p), ("x_out", C.c_void_p),
                ("v_out", C.c_void_p), ("res", C.c_void_p)]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_double), ("bytes_per_atom", C.c_double), ("max_batch_atoms", C.c_int64),
                ("md_chunk_steps", C.c_int)]


class ServerStats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ("submitted", "completed", "failed", "queued", "active", "point_batches",
                                         "point_systems", "md_chunks", "md_reforms", "md_steps")] + \
               [(k, C.c_double) for k in ("admitted_bytes", "bytes_per_atom", "busy_s", "max_admitted_bytes")]


PENDING = 1


class Server:
    """Native request server.  The engine parameters (potential files, elements,
    precision, tunables) come from a prototype ``capi.Engine``; masses are set on it."""

    def __init__(self, proto: capi.Engine, hbm_budget_bytes: float = 150e9, max_batch_atoms: int = 8 << 20,
                 md_chunk_steps: int = 20, bytes_per_atom: float = 0.0,
                 masses: Sequence[float] = (12.011, 10.811, 14.0067)):
        self._lib = capi.load_library()
        proto.set_masses(masses)
        cfg = ServerConfig(hbm_budget_bytes, bytes_per_atom, max_batch_atoms, md_chunk_steps)
        self._h = C.c_void_p()
        rc = self._lib.lmff_server_create(C.byref(self._h), proto._h, C.cast(C.pointer(cfg), C.c_void_p))
        if rc != 0:
            raise capi.LmffError(rc, capi.load_library().lmff_last_error(None).decode())
        self._out: Dict[int, Dict] = {}

    def submit(self, s: S.System, nsteps: int = 0, dt: float = 0.001) -> int:
        return self.submit_many([(s, nsteps)], dt)[0]

    def submit_many(self, items, dt: float = 0.001) -> List[int]:
        """Queue [(system, nsteps), ...] together (one worker iteration sees all)."""
        reqs = (Request * len(items))()
        outs = []
        keep = []
        for k, (s, nsteps) in enumerate(items):
            out, arrs = self._fill(reqs[k], s, nsteps, dt)
            outs.append(out)
            keep.append(arrs)
        tickets = (C.c_int64 * len(items))()
        rc = self._lib.lmff_server_submit_many(self._h, len(items), C.cast(reqs, C.c_void_p),
                                               C.cast(tickets, C.c_void_p))
        if rc != 0:
            raise capi.LmffError(rc, self._lib.lmff_server_last_error().decode())
        for t, out in zip(tickets, outs):
            self._out[t] = out
        return list(tickets)

    def _fill(self, r: Request, s: S.System, nsteps: int, dt: float):
        n = s.n
        x = capi._f64(s.x)
        t = np.ascontiguousarray(s.type, dtype=np.int32)
        m = np.ascontiguousarray(s.mol, dtype=np.int64)
        v = capi._f64(s.v) if (nsteps > 0 and s.v is not None) else None
        out = {"f": np.zeros((n, 3)), "res": capi.Result()}
        if nsteps > 0:
            out["x"] = np.zeros((n, 3))
            out["v"] = np.zeros((n, 3))
        r.natoms = n
        r.x = x.ctypes.data
        r.v = None if v is None else v.ctypes.data
        r.type = t.ctypes.data
        r.mol = m.ctypes.data
        for c in range(3):
            r.lo[c] = float(s.box_lo[c])
            r.hi[c] = float(s.box_hi[c])
            r.periodic[c] = int(bool(s.periodic[c]))
        r.nsteps = nsteps
        r.dt = dt
        r.f_out = out["f"].ctypes.data
        r.x_out = out["x"].ctypes.data if nsteps > 0 else None
        r.v_out = out["v"].ctypes.data if nsteps > 0 else None
        r.res = C.cast(C.pointer(out["res"]), C.c_void_p)
        return out, (x, t, m, v)   # inputs are copied at submission; keep them alive until then

    def wait(self, ticket: int, timeout: float = -1.0) -> Optional[Dict]:
        """The request's result dict (f, energies, virial, latency_s; x and v for NVE),
        None if still running after ``timeout`` seconds; raises LmffError if it failed."""
        lat = C.c_double()
        rc = self._lib.lmff_server_wait(self._h, ticket, timeout, C.byref(lat))
        if rc == PENDING:
            return None
        out = self._out.pop(ticket)
        if rc != 0:
            raise capi.LmffError(rc, self._lib.lmff_server_last_error().decode())
        d = out["res"].to_dict()
        d["f"] = out["f"]
        if "x" in out:
            d["x"], d["v"] = out["x"], out["v"]
        d["latency_s"] = lat.value
        return d

    def stats(self) -> Dict:
        st = ServerStats()
        self._lib.lmff_server_get_stats(self._h, C.cast(C.pointer(st), C.c_void_p))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def close(self) -> None:
        if self._h:
            self._lib.lmff_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass


# ------------------------------------------------------------------ request streams

@dataclass
class StreamItem:
    t_arrival: float
    system: S.System
    nsteps: int


def _bilayer(ntot: int, top: str, theta: float, spacing: float) -> S.System:
    a = math.sqrt(3.0) * S.A_CC_GRAPHENE
    nx, ny = S._rect_for_count(int(ntot / 2))
    nx = max(nx, math.ceil(20.0 / a))
    ny = max(ny, math.ceil(20.0 / (3 * S.A_CC_GRAPHENE)))
    if top == "graphene" and theta == 0.0:
        return S.ab_bilayer_graphene(nx, ny, spacing=spacing)
    return S.twisted_bilayer(nx, ny, theta, top=top, spacing=spacing)


def poisson_stream(count: int = 400, rate: float = 200.0, frac_md: float = 0.3, md_steps: int = 100,
                   nmin: int = 1000, nmax: int = 200000, sizes: int = 24, temp: float = 300.0,
                   seed: int = 7) -> List[StreamItem]:
    """Poisson arrivals at ``rate`` per second; a fraction ``frac_md`` are NVE runs of
    ``md_steps`` at ``temp``, the rest single points.  Systems are bilayers (half AB
    graphene, half graphene/hBN twisted 0.5-3 degrees) with atom counts log-uniform over a
    geometric grid of ``sizes`` values in [nmin, nmax]; each request gets its own
    displacement (single point, 0.02 A) or velocities (NVE) from the seeded generator."""
    rng = np.random.default_rng(seed)
    grid = np.unique(np.round(np.exp(np.linspace(math.log(nmin), math.log(nmax), sizes))).astype(int))
    bases: Dict = {}
    out = []
    t = 0.0
    for k in range(count):
        t += float(rng.exponential(1.0 / rate))
        ntot = int(grid[rng.integers(len(grid))])
        top = "graphene" if rng.random() < 0.5 else "hbn"
        key = (ntot, top)
        if key not in bases:
            theta = 0.0 if top == "graphene" else float(rng.uniform(0.5, 3.0))
            bases[key] = _bilayer(ntot, top, theta, 3.4)
        md = rng.random() < frac_md
        sub_seed = int(rng.integers(1 << 31))
        if md:
            s = S.thermalize(bases[key], temp, seed=sub_seed)
        else:
            s = S.displace(bases[key], 0.02, seed=sub_seed)
        out.append(StreamItem(t, s, md_steps if md else 0))
    return out


def _summary(lat: List[float], t_first: float, t_last_done: float, atom_steps: float) -> Dict:
    lat = np.asarray(lat)
    span = max(t_last_done - t_first, 1e-9)
    return {"requests": int(len(lat)), "solves_per_s": len(lat) / span, "makespan_s": span,
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3), "atom_steps_per_s": atom_steps / span}


def _atom_steps(stream: Sequence[StreamItem]) -> float:
    return float(sum(it.system.n * max(1, it.nsteps) for it in stream))


def replay(server: Server, stream: Sequence[StreamItem], realtime: bool = True, dt: float = 0.001) -> Dict:
    """Submit every request at its arrival time (realtime) or all at once, wait for
    all; latency = completion - submission, measured by the server."""
    t0 = time.perf_counter()
    sub = []
    for it in stream:
        if realtime:
            d = t0 + it.t_arrival - time.perf_counter()
            if d > 0:
                time.sleep(d)
        sub.append((server.submit(it.system, it.nsteps, dt), time.perf_counter()))
    lat, done = [], []
    for ticket, ts in sub:
        r = server.wait(ticket)
        lat.append(r["latency_s"])
        done.append(ts + r["latency_s"])
    return _summary(lat, t0, max(done), _atom_steps(stream))


def replay_sequential(engine: capi.Engine, stream: Sequence[StreamItem], realtime: bool = True,
                      dt: float = 0.001) -> Dict:
    """The one-request-at-a-time baseline on a plain engine: each request waits for the
    previous one; latency = completion - arrival."""
    t0 = time.perf_counter()
    lat, done = [], []
    for it in stream:
        if realtime:
            d = t0 + it.t_arrival - time.perf_counter()
            if d > 0:
                time.sleep(d)
        arrival = t0 + it.t_arrival if realtime else t0
        if it.nsteps > 0:
            engine.upload(it.system)
            engine.run_nve(it.nsteps, dt)
            engine.download()
        else:
            engine.compute_system(it.system)
        t = time.perf_counter()
        lat.append(t - arrival)
        done.append(t)
    return _summary(lat, t0, max(done), _atom_steps(stream))
