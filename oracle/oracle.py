"""ctypes wrapper of the C oracle (oracle/lmff_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the benchmark's
CPU-baseline leg, never by the engine.  ``build()`` compiles the oracle library into
oracle/_build/ (gcc, OpenMP, -ffp-contract=off so x86 and Arm hosts agree).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Dict, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liblmff_oracle.so")
SRC = os.path.join(HERE, "lmff_oracle.c")
HDR = os.path.join(HERE, "lmff_oracle.h")
_lib = None


def build(force: bool = False) -> str:
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    stale = force or not os.path.exists(LIB) or any(
        os.path.getmtime(s) > os.path.getmtime(LIB) for s in (SRC, HDR))
    if stale:
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                               "-o", tmp, SRC, "-lm"])
        os.replace(tmp, LIB)
    return LIB


class _Result(C.Structure):
    _fields_ = [("e_tersoff", C.c_double), ("e_ilp", C.c_double), ("pvector", C.c_double * 2),
                ("virial", C.c_double * 6), ("virial_tersoff", C.c_double * 6),
                ("virial_ilp", C.c_double * 6), ("nghost", C.c_int64), ("nlist", C.c_int64)]


def _load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(LIB)
        P = C.c_void_p
        lib.orc_pot_init.argtypes = [P, C.c_int, C.c_double, C.c_int, C.c_double]
        lib.orc_read_tersoff.argtypes = [P, C.c_char_p, C.POINTER(C.c_char_p)]
        lib.orc_read_ilp.argtypes = [P, C.c_char_p, C.POINTER(C.c_char_p)]
        lib.orc_read_kc.argtypes = [P, C.c_char_p, C.POINTER(C.c_char_p)]
        lib.orc_pot_error.argtypes = [P]
        lib.orc_pot_error.restype = C.c_char_p
        lib.orc_new.argtypes = [P, C.c_int]
        lib.orc_new.restype = P
        lib.orc_free.argtypes = [P]
        lib.orc_error.argtypes = [P]
        lib.orc_error.restype = C.c_char_p
        lib.orc_set_atoms.argtypes = [P, C.c_int, P, P, P, P, P, P, P]
        lib.orc_update_x.argtypes = [P, P]
        lib.orc_forces.argtypes = [P, C.c_int, P, P, C.POINTER(_Result)]
        lib.orc_forces_va.argtypes = [P, C.c_int, P, P, P, P, C.POINTER(_Result)]
        lib.orc_nve.argtypes = [P, C.c_int, C.c_double, P, P, P, P, C.POINTER(_Result)]
        lib.orc_nrebuilds.argtypes = [P]
        lib.orc_nrebuilds.restype = C.c_int64
        lib.orc_full_list.argtypes = [P, P, C.c_int64]
        lib.orc_full_list.restype = C.c_int64
        lib.orc_ilp_list.argtypes = [P, P, C.c_int64]
        lib.orc_ilp_list.restype = C.c_int64
        _lib = lib
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class OracleError(RuntimeError):
    pass


class Oracle:
    """CPU oracle for one system.  Potential files and element names follow
    ``pair_coeff * * <style> <file> <elem per type>``."""

    def __init__(self, tersoff_file: Optional[str], ilp_file: Optional[str],
                 elements: Sequence[str] = ("C", "B", "N"), cut_global: float = 16.0,
                 tap_flag: int = 1, skin: float = 2.0, nthreads: int = 0, kc_file: Optional[str] = None,
                 interlayer_elements: Optional[Sequence[str]] = None):
        """kc_file: a kolmogorov/crespi/full parameter file used as the interlayer style
        instead of ilp_file; interlayer_elements: its own element list (default
        `elements`)."""
        lib = _load()
        self._pot = C.create_string_buffer(1 << 20)
        ntypes = len(elements)
        if lib.orc_pot_init(self._pot, ntypes, cut_global, tap_flag, skin):
            raise OracleError(lib.orc_pot_error(self._pot).decode())
        arr = (C.c_char_p * ntypes)(*[e.encode() for e in elements])
        if tersoff_file and lib.orc_read_tersoff(self._pot, tersoff_file.encode(), arr):
            raise OracleError(lib.orc_pot_error(self._pot).decode())
        arr2 = arr if interlayer_elements is None else (C.c_char_p * ntypes)(*[e.encode() for e in interlayer_elements])
        if ilp_file and lib.orc_read_ilp(self._pot, ilp_file.encode(), arr2):
            raise OracleError(lib.orc_pot_error(self._pot).decode())
        if kc_file and lib.orc_read_kc(self._pot, kc_file.encode(), arr2):
            raise OracleError(lib.orc_pot_error(self._pot).decode())
        self.nthreads = nthreads or (os.cpu_count() or 1)
        self._ctx = lib.orc_new(self._pot, self.nthreads)
        self.n = 0

    def __del__(self):
        if getattr(self, "_ctx", None) and _lib is not None:
            _lib.orc_free(self._ctx)
            self._ctx = None

    def _check(self, rc: int):
        if rc != 0:
            raise OracleError(f"{rc}: {_lib.orc_error(self._ctx).decode()}")

    def set_system(self, s) -> None:
        self.set_atoms(s.x, s.type, s.mol, s.tag, s.box_lo, s.box_hi, s.periodic)

    def set_atoms(self, x, type_, mol, tag, lo, hi, periodic) -> None:
        x = np.ascontiguousarray(x, dtype=np.float64)
        self._type = np.ascontiguousarray(type_, dtype=np.int32)
        self._mol = np.ascontiguousarray(mol, dtype=np.int64)
        self._tag = np.ascontiguousarray(tag, dtype=np.int64)
        lo = np.ascontiguousarray(lo, dtype=np.float64)
        hi = np.ascontiguousarray(hi, dtype=np.float64)
        per = np.ascontiguousarray(np.asarray(periodic, dtype=bool).astype(np.int32))
        self.n = x.shape[0]
        self._check(_lib.orc_set_atoms(self._ctx, self.n, _ptr(x), _ptr(self._type), _ptr(self._mol),
                                       _ptr(self._tag), _ptr(lo), _ptr(hi), _ptr(per)))

    def update_x(self, x) -> None:
        x = np.ascontiguousarray(x, dtype=np.float64)
        self._check(_lib.orc_update_x(self._ctx, _ptr(x)))

    def forces(self, which: int = 3, eatom: bool = False, vatom: bool = False) -> Dict:
        """vatom: also each style's per-atom virial (n x 6, xx yy zz xy xz yz) as
        "vatom_tersoff" / "vatom_ilp" and their sum "vatom"."""
        f = np.zeros((self.n, 3))
        ea = np.zeros(self.n) if eatom else None
        r = _Result()
        if vatom:
            vt, vi = np.zeros((self.n, 6)), np.zeros((self.n, 6))
            self._check(_lib.orc_forces_va(self._ctx, which, _ptr(f), _ptr(ea) if eatom else None, _ptr(vt),
                                           _ptr(vi), C.byref(r)))
        else:
            self._check(_lib.orc_forces(self._ctx, which, _ptr(f), _ptr(ea) if eatom else None, C.byref(r)))
        out = {"f": f, "e_tersoff": r.e_tersoff, "e_ilp": r.e_ilp, "pvector": np.array(r.pvector[:]),
               "virial": np.array(r.virial[:]), "virial_tersoff": np.array(r.virial_tersoff[:]),
               "virial_ilp": np.array(r.virial_ilp[:]), "nghost": r.nghost, "nlist": r.nlist}
        out["e_pair"] = out["e_tersoff"] + out["e_ilp"]
        if eatom:
            out["eatom"] = ea
        if vatom:
            out["vatom_tersoff"], out["vatom_ilp"], out["vatom"] = vt, vi, vt + vi
        return out

    def nve(self, nsteps: int, dt: float, mass_of_type, x, v, f) -> Dict:
        """Velocity-Verlet in place on x, v, f (f must be the forces of x)."""
        m = np.ascontiguousarray(mass_of_type, dtype=np.float64)
        r = _Result()
        self._check(_lib.orc_nve(self._ctx, nsteps, dt, _ptr(m), _ptr(x), _ptr(v), _ptr(f), C.byref(r)))
        return {"e_tersoff": r.e_tersoff, "e_ilp": r.e_ilp, "virial": np.array(r.virial[:])}

    def nrebuilds(self) -> int:
        return int(_lib.orc_nrebuilds(self._ctx))

    def full_list(self) -> np.ndarray:
        n = _lib.orc_full_list(self._ctx, None, 0)
        out = np.zeros((n, 3), dtype=np.int64)
        _lib.orc_full_list(self._ctx, _ptr(out), n)
        return out

    def ilp_list(self) -> np.ndarray:
        n = _lib.orc_ilp_list(self._ctx, None, 0)
        if n < 0:
            raise OracleError(_lib.orc_error(self._ctx).decode())
        out = np.zeros((n, 3), dtype=np.int64)
        _lib.orc_ilp_list(self._ctx, _ptr(out), n)
        return out
