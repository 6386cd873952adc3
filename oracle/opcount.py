"""Freeze the benchmark's algorithmic operation counts (TEST INFRASTRUCTURE).

Compiles oracle/opcount.cpp (the oracle's own C source with an operation-counting
double, g++), runs one Tersoff + ILP force evaluation of the benchmark's CPU sample --
the 36,800-atom periodic patch of the 10-layer alternating-molecule graphite slab with
an N(0, 0.03 A) displacement -- and writes the per-unit counts to bench/flops.h, which
bench.py reads for its rooflines.  Run: python oracle/opcount.py [--check]
(--check recounts and compares with the committed header instead of writing it).
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "opcount.cpp")
LIB = os.path.join(HERE, "_build", "libopcount.so")
HEADER = os.path.join(ROOT, "bench", "flops.h")
POT = os.path.join(ROOT, "lammps-lmff_gb300", "potentials")

CATS = ["OTHER", "ILP_CAND", "ILP_PAIR", "ILP_VDW", "ILP_KTERM", "NORMAL", "TERS_CAND", "TERS_REP", "TERS_BOND",
        "TERS_ZETA", "TERS_ATTR", "ILP_DSELF"]

DOC = {
    "FLOPS_ILP_CAND": "an interlayer list candidate: displacement and r^2 (every candidate)",
    "FLOPS_ILP_PAIR": "a directed pair in the cutoff, beyond the candidate's: r, taper, the repulsion term with "
                      "the normal of i, forces on i and j, energy",
    "FLOPS_ILP_VDW": "one vdW evaluation (calc_FvdW, tag-parity half of the pairs)",
    "FLOPS_ILP_DSELF": "calc_FRep's term of dn_i/dx_i (per pair; with the reverse-accumulated normal derivative "
                       "it is applied once per atom)",
    "FLOPS_ILP_KTERM": "calc_FRep's force on one intralayer neighbour k of i (per pair and k; applied once per "
                       "atom and k with the reverse-accumulated normal derivative)",
    "FLOPS_NORMAL": "calc_normal of one atom: its normal and the Jacobians",
    "FLOPS_TERS_REP": "Tersoff repulsive term of a bond (tag-parity half)",
    "FLOPS_TERS_BOND": "force_zeta and the bond force of a directed bond",
    "FLOPS_TERS_ZETA": "zeta term of a triplet",
    "FLOPS_TERS_ATTR": "three-body (attractive) force of a triplet",
    "VDW_PER_PAIR": "vdW evaluations per directed pair in the cutoff",
    "KTERMS_PER_PAIR": "intralayer neighbours k of i per directed pair (k-terms of calc_FRep)",
    "FLOPS_TERSOFF_ATOM": "Tersoff arithmetic per atom (repulsive + bond + zeta + attractive)",
    "TERS_BONDS_PER_ATOM": "directed Tersoff bonds per atom",
    "TERS_TRIPLETS_PER_ATOM": "Tersoff triplets per atom",
    "ILP_PAIRS_PER_ATOM": "directed interlayer pairs in the cutoff per atom",
    "ILP_CANDIDATES_PER_ATOM": "interlayer list candidates per atom (the oracle's list: cutoff + 2 A skin)",
}


def build() -> str:
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    deps = [SRC, os.path.join(HERE, "lmff_oracle.c"), os.path.join(HERE, "lmff_oracle.h")]
    if not os.path.exists(LIB) or any(os.path.getmtime(d) > os.path.getmtime(LIB) for d in deps):
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-o", tmp, SRC])
        os.replace(tmp, LIB)
    return LIB


def sample():
    for p in (os.path.join(ROOT, "lammps-lmff_gb300"), ROOT):
        if p not in sys.path:
            sys.path.insert(0, p)
    import bench
    from lmff_gb300 import structures as S
    return S.displace(bench.cpu_sample(), 0.03, seed=21)


def count(s, elements=("C",)) -> dict:
    """{category: (operations, library calls, units)} of one evaluation of system s."""
    lib = C.CDLL(build())
    P = C.c_void_p
    lib.opc_count.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.POINTER(C.c_char_p), C.c_double, C.c_int, C.c_int,
                              P, P, P, P, P, P, P, C.c_int, P, P, P, C.c_char_p, C.c_int]
    arr = (C.c_char_p * len(elements))(*[e.encode() for e in elements])
    x = np.ascontiguousarray(s.x, dtype=np.float64)
    t = np.ascontiguousarray(s.type, dtype=np.int32)
    m = np.ascontiguousarray(s.mol, dtype=np.int64)
    g = np.ascontiguousarray(s.tag, dtype=np.int64)
    lo = np.ascontiguousarray(s.box_lo, dtype=np.float64)
    hi = np.ascontiguousarray(s.box_hi, dtype=np.float64)
    per = np.ascontiguousarray(np.asarray(s.periodic).astype(np.int32))
    ops = np.zeros(16, dtype=np.uint64)
    calls = np.zeros(16, dtype=np.uint64)
    units = np.zeros(16, dtype=np.uint64)
    err = C.create_string_buffer(512)

    def ptr(a):
        return a.ctypes.data_as(P)
    rc = lib.opc_count(os.path.join(POT, "BNC.tersoff").encode(), os.path.join(POT, "BNCH.ILP").encode(),
                       len(elements), arr, 16.0, 1, s.n, ptr(x), ptr(t), ptr(m), ptr(g), ptr(lo), ptr(hi), ptr(per),
                       3, ptr(ops), ptr(calls), ptr(units), err, 512)
    if rc:
        raise RuntimeError(f"opc_count: {rc} {err.value.decode()}")
    return {c: (int(ops[k]), int(calls[k]), int(units[k])) for k, c in enumerate(CATS)}


def constants(cnt: dict, natoms: int) -> dict:
    """Per-unit operation counts (and per-unit library calls) from the category totals."""
    def per(cat):
        o, c, u = cnt[cat]
        return (o / u, c / u) if u else (0.0, 0.0)
    out = {}
    for cat in ("ILP_CAND", "ILP_PAIR", "ILP_VDW", "ILP_DSELF", "ILP_KTERM", "NORMAL", "TERS_REP", "TERS_BOND",
                "TERS_ZETA", "TERS_ATTR"):
        out[f"FLOPS_{cat}"], out[f"CALLS_{cat}"] = per(cat)
    u = {c: cnt[c][2] for c in cnt}
    out["VDW_PER_PAIR"] = u["ILP_VDW"] / u["ILP_PAIR"]
    out["KTERMS_PER_PAIR"] = u["ILP_KTERM"] / u["ILP_PAIR"]
    ters = sum(cnt[c][0] for c in ("TERS_REP", "TERS_BOND", "TERS_ZETA", "TERS_ATTR"))
    out["FLOPS_TERSOFF_ATOM"] = ters / natoms
    out["TERS_BONDS_PER_ATOM"] = u["TERS_BOND"] / natoms
    out["TERS_TRIPLETS_PER_ATOM"] = u["TERS_ATTR"] / natoms
    out["ILP_PAIRS_PER_ATOM"] = u["ILP_PAIR"] / natoms
    out["ILP_CANDIDATES_PER_ATOM"] = u["ILP_CAND"] / natoms
    return out


def header(consts: dict, n: int) -> str:
    lines = ["/* Algorithmic operation counts of the Tersoff + ILP force evaluation, frozen by",
             " * oracle/opcount.py: the oracle (oracle/lmff_oracle.c, pinned to the reference) compiled",
             " * with an operation-counting double (oracle/opcount.cpp), one evaluation of the",
             f" * {n}-atom periodic patch of the 10-layer alternating-molecule graphite slab",
             " * (3.35 A, 300 K lattice, N(0, 0.03 A) displacement), BNC.tersoff + BNCH.ILP, 16 A, taper.",
             " * Convention: add, subtract, multiply, divide, sqrt = 1; a*b + c = 2; each exp, pow,",
             " * sin, cos call = 1 (CALLS_* counts them per unit, already inside FLOPS_*).",
             " * Generated file: regenerate with python oracle/opcount.py. */",
             "#pragma once", ""]
    for k, v in consts.items():
        if k.startswith("CALLS_"):
            continue
        lines.append(f"/* {DOC[k]} */")
        lines.append(f"#define LMFF_{k} {v:.4f}")
        ck = k.replace("FLOPS_", "CALLS_")
        if ck != k and ck in consts:
            lines.append(f"#define LMFF_{ck} {consts[ck]:.4f}")
    return "\n".join(lines) + "\n"


def read_header(path: str = HEADER) -> dict:
    out = {}
    for line in open(path):
        p = line.split()
        if len(p) == 3 and p[0] == "#define" and p[1].startswith("LMFF_"):
            out[p[1][5:]] = float(p[2])
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--check", action="store_true")
    args = ap.parse_args()
    s = sample()
    consts = constants(count(s), s.n)
    if args.check:
        old = read_header()
        bad = {k: (old.get(k), v) for k, v in consts.items() if abs(old.get(k, -1.0) - round(v, 4)) > 1e-3}
        print("ok" if not bad else f"differs: {bad}")
        sys.exit(1 if bad else 0)
    os.makedirs(os.path.dirname(HEADER), exist_ok=True)
    with open(HEADER, "w") as fh:
        fh.write(header(consts, s.n))
    print(open(HEADER).read())


if __name__ == "__main__":
    main()
