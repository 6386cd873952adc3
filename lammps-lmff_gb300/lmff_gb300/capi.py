"""ctypes binding of the engine's C ABI (include/lmff_gb300.h).

This is plumbing for the tests, the benchmark and the serving loop; the compute path is
the CUDA library itself.  There is no CPU fallback: loading fails loudly when
liblmff_gb300.so is missing or cannot be loaded, and every non-zero status code raises
``LmffError`` with the engine's message.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Dict, List, Optional, Sequence

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "liblmff_gb300.so")
POTENTIALS = os.path.join(os.path.dirname(PKG), "potentials")

LMFF_OK = 0
CODES = {-1: "LMFF_EINVAL", -2: "LMFF_ECUDA", -3: "LMFF_EOVERFLOW", -4: "LMFF_ETOO_MANY_ILP_NEIGH",
         -5: "LMFF_EZERO_NORMAL", -6: "LMFF_EBADPARAM", -7: "LMFF_ETIMEDOUT", -8: "LMFF_EUNSUPPORTED",
         -9: "LMFF_ENOMEM", -10: "LMFF_ENODEV"}
FP64 = 0
MIXED = 1
TERSOFF = 1
ILP = 2
SAME_ATOMS = 4
OVERWRITE = 8


class LmffError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{CODES.get(code, code)}: {msg}")
        self.code = code


class Result(C.Structure):
    _fields_ = [("e_tersoff", C.c_double), ("e_ilp", C.c_double), ("pvector", C.c_double * 2),
                ("virial_tersoff", C.c_double * 6), ("virial_ilp", C.c_double * 6)]

    def to_dict(self) -> Dict:
        vt = np.array(self.virial_tersoff[:])
        vi = np.array(self.virial_ilp[:])
        return {"e_tersoff": self.e_tersoff, "e_ilp": self.e_ilp, "pvector": np.array(self.pvector[:]),
                "virial_tersoff": vt, "virial_ilp": vi, "virial": vt + vi,
                "e_pair": self.e_tersoff + self.e_ilp}


def _results(res, n: int) -> List[Dict]:
    """Result.to_dict of each of the n entries of a Result array, by columns (a batch has
    hundreds of systems)."""
    a = np.frombuffer(res, dtype=np.float64, count=16 * n).reshape(n, 16).copy()
    et, ei, pv, vt, vi = a[:, 0], a[:, 1], a[:, 2:4], a[:, 4:10], a[:, 10:16]
    vs, ep = vt + vi, et + ei
    return [{"e_tersoff": float(et[k]), "e_ilp": float(ei[k]), "pvector": pv[k], "virial_tersoff": vt[k],
             "virial_ilp": vi[k], "virial": vs[k], "e_pair": float(ep[k])} for k in range(n)]


class Thermo(C.Structure):
    _fields_ = [("step", C.c_int64), ("pe", C.c_double), ("ke", C.c_double), ("etotal", C.c_double),
                ("temp", C.c_double), ("virial", C.c_double * 6)]


class Stats(C.Structure):
    _fields_ = [("natoms", C.c_int64), ("list_entries", C.c_int64), ("short_entries", C.c_int64),
                ("list_capacity", C.c_int64), ("rebuilds", C.c_int64), ("steps", C.c_int64),
                ("list_per_atom", C.c_double), ("bytes_device", C.c_double), ("ms_last_build", C.c_double),
                ("ms_last_forces", C.c_double), ("precision", C.c_int), ("tpa", C.c_int), ("block", C.c_int),
                ("ms_last_run", C.c_double), ("kernel_ms", C.c_double * 7), ("kernel_launches", C.c_int64 * 7),
                ("pairs_in_cutoff", C.c_int64), ("graph_steps", C.c_int64), ("graph_redos", C.c_int64),
                ("bytes_per_atom_need", C.c_double)]
class MinResult(C.Structure):
    _fields_ = [("niter", C.c_int), ("neval", C.c_int), ("stop_condition", C.c_int), ("einitial", C.c_double),
                ("efinal", C.c_double), ("fnorm2_init", C.c_double), ("fnorminf_init", C.c_double),
                ("fnorm2_final", C.c_double), ("fnorminf_final", C.c_double), ("alpha_final", C.c_double)]


KERNELS = ["pair_ilp", "tersoff", "intralayer_normals", "gather", "integrate", "neighbor_build", "normal_deriv"]


class SystemDesc(C.Structure):
    _fields_ = [("natoms", C.c_int), ("x", C.c_void_p), ("type", C.c_void_p), ("mol", C.c_void_p),
                ("lo", C.c_double * 3), ("hi", C.c_double * 3), ("periodic", C.c_int * 3), ("v", C.c_void_p)]


# a numpy view of a SystemDesc array, so a large batch's descriptors are filled by column
_DESC_DTYPE = np.dtype({"names": ["natoms", "x", "type", "mol", "lo", "hi", "periodic", "v"],
                        "formats": ["<i4", "<u8", "<u8", "<u8", ("<f8", 3), ("<f8", 3), ("<i4", 3), "<u8"],
                        "offsets": [SystemDesc.natoms.offset, SystemDesc.x.offset, SystemDesc.type.offset,
                                    SystemDesc.mol.offset, SystemDesc.lo.offset, SystemDesc.hi.offset,
                                    SystemDesc.periodic.offset, SystemDesc.v.offset],
                        "itemsize": C.sizeof(SystemDesc)})


def _addr(a: np.ndarray) -> int:
    return a.__array_interface__["data"][0]


_lib = None


def load_library(path: str = LIB_PATH):
    """Load liblmff_gb300.so (built by lmff_gb300.build); raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"{path} not found: build it with lmff_gb300.build.build()")
    lib = C.CDLL(path)
    P = C.c_void_p
    I = C.c_int
    D = C.c_double
    sig = {
        "lmff_device_count": ([], I),
        "lmff_create": ([C.POINTER(P), P, I], I),
        "lmff_create_from_files": ([C.POINTER(P), C.c_char_p, C.c_char_p, I, C.POINTER(C.c_char_p), D, I, D, I], I),
        "lmff_create_from_files2": ([C.POINTER(P), C.c_char_p, C.POINTER(C.c_char_p), C.c_char_p,
                                     C.POINTER(C.c_char_p), I, D, I, D, I], I),
        "lmff_minimize": ([P, D, D, I, I, D, P, P], I),
        "lmff_create_kc_from_files": ([C.POINTER(P), C.c_char_p, C.POINTER(C.c_char_p), C.c_char_p,
                                       C.POINTER(C.c_char_p), I, D, I, D, I], I),
        "lmff_destroy": ([P], None),
        "lmff_set_precision": ([P, I], I),
        "lmff_set_box": ([P, P, P, D, D, D, P], I),
        "lmff_set_option": ([P, C.c_char_p, D], I),
        "lmff_compute": ([P, I, P, P, P, P, I, I, I, P, P, C.POINTER(Result)], I),
        "lmff_compute_device": ([P, I, P, P, P, P, I, I, I, P, C.POINTER(Result)], I),
        "lmff_compute_ghost": ([P, I, I, P, P, P, P, I, I, I, P, P, C.POINTER(Result)], I),
        "lmff_compute_vatom": ([P, I, I, P], I),
        "lmff_compute_device_noalloc": ([P, I, P, P, P, I, I, I, P, C.POINTER(Result)], I),
        "lmff_upload": ([P, I, P, P, P, P, P, P], I),
        "lmff_compute_resident": ([P, I, I, I, C.POINTER(Result)], I),
        "lmff_run_nve": ([P, I, D, I, P], I),
        "lmff_download": ([P, P, P, P], I),
        "lmff_batch_set": ([P, I, P], I),
        "lmff_batch_compute": ([P, P, P], I),
        "lmff_batch_results": ([P, I, P], I),
        "lmff_set_masses": ([P, I, P], I),
        "lmff_clone": ([P, C.POINTER(P)], I),
        "lmff_server_create": ([C.POINTER(P), P, P], I),
        "lmff_server_submit": ([P, P, C.POINTER(C.c_int64)], I),
        "lmff_server_submit_many": ([P, I, P, P], I),
        "lmff_server_wait": ([P, C.c_int64, D, C.POINTER(D)], I),
        "lmff_server_get_stats": ([P, P], I),
        "lmff_server_last_error": ([], C.c_char_p),
        "lmff_server_destroy": ([P], None),
        "lmff_get_stats": ([P, C.POINTER(Stats)], I),
        "lmff_export_list": ([P, I, P, C.c_int64], C.c_int64),
        "lmff_last_error": ([P], C.c_char_p),
        "lmff_strerror": ([I], C.c_char_p),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


class Engine:
    """One engine handle: one GPU, one stream, one resident system or batch."""

    def __init__(self, tersoff_file: Optional[str] = None, ilp_file: Optional[str] = None,
                 elements: Sequence[str] = ("C", "B", "N"), cut_global: float = 16.0, tap_flag: int = 1,
                 skin: float = 2.0, device: int = 0, precision: int = FP64,
                 ilp_elements: Optional[Sequence[str]] = None, kc_file: Optional[str] = None):
        """elements: type -> element name for both files (pair_coeff * * ... C B N);
        ilp_elements, if given, a separate list for the interlayer file (the Tersoff file
        then uses `elements`), e.g. elements = NULL C(O) ... with ilp_elements = C C ...
        kc_file: a kolmogorov/crespi/full parameter file as the interlayer style instead
        of ilp_file."""
        lib = load_library()
        if tersoff_file is None and ilp_file is None and kc_file is None:
            tersoff_file = os.path.join(POTENTIALS, "BNC.tersoff")
            ilp_file = os.path.join(POTENTIALS, "BNCH.ILP")
        self._h = C.c_void_p()
        arr = (C.c_char_p * len(elements))(*[e.encode() for e in elements])
        if kc_file is not None:
            ie = elements if ilp_elements is None else ilp_elements
            arr2 = (C.c_char_p * len(ie))(*[e.encode() for e in ie])
            rc = lib.lmff_create_kc_from_files(C.byref(self._h), tersoff_file.encode() if tersoff_file else None, arr,
                                               kc_file.encode(), arr2, len(elements), cut_global, tap_flag, skin,
                                               device)
        elif ilp_elements is None:
            rc = lib.lmff_create_from_files(C.byref(self._h), tersoff_file.encode() if tersoff_file else None,
                                            ilp_file.encode() if ilp_file else None, len(elements), arr, cut_global,
                                            tap_flag, skin, device)
        else:
            if len(ilp_elements) != len(elements):
                raise ValueError("elements and ilp_elements must name the same number of types")
            arr2 = (C.c_char_p * len(ilp_elements))(*[e.encode() for e in ilp_elements])
            rc = lib.lmff_create_from_files2(C.byref(self._h), tersoff_file.encode() if tersoff_file else None, arr,
                                             ilp_file.encode() if ilp_file else None, arr2, len(elements),
                                             cut_global, tap_flag, skin, device)
        if rc != 0:
            raise LmffError(rc, lib.lmff_last_error(None).decode())
        self.ntypes = len(elements)
        self.set_precision(precision)

    def close(self):
        if getattr(self, "_h", None) and self._h.value and _lib is not None:
            _lib.lmff_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        self.close()

    def _ck(self, rc: int):
        if rc != 0:
            raise LmffError(rc, _lib.lmff_last_error(self._h).decode())

    # -------------------------------------------------------------- configuration
    def set_precision(self, mode: int):
        self._ck(_lib.lmff_set_precision(self._h, mode))

    def set_box(self, lo, hi, periodic, tilt=None):
        """tilt: LAMMPS's (xy, xz, yz) of a triclinic box (lmff_compute evaluates it)."""
        lo = _f64(lo)
        hi = _f64(hi)
        per = np.ascontiguousarray(np.asarray(periodic, dtype=bool).astype(np.int32))
        xy, xz, yz = (0.0, 0.0, 0.0) if tilt is None else (float(t) for t in tilt)
        self._ck(_lib.lmff_set_box(self._h, _p(lo), _p(hi), xy, xz, yz, _p(per)))

    def set_option(self, key: str, value: float):
        self._ck(_lib.lmff_set_option(self._h, key.encode(), float(value)))

    # -------------------------------------------------------------- one-shot compute
    def compute(self, x, type_, mol=None, tag=None, which: int = TERSOFF | ILP, eflag: bool = True,
                vflag: bool = True, eatom: bool = False, same_atoms: bool = False, f=None,
                overwrite: bool = False, vatom: bool = False) -> Dict:
        """vatom: also each style's per-atom virial ("vatom_tersoff", "vatom_ilp" [n, 6]
        and their sum "vatom"), from lmff_compute_vatom right after the evaluation."""
        x = _f64(x)
        n = x.shape[0]
        t = np.ascontiguousarray(type_, dtype=np.int32)
        m = None if mol is None else np.ascontiguousarray(mol, dtype=np.int64)
        g = None if tag is None else np.ascontiguousarray(tag, dtype=np.int64)
        out_f = np.zeros((n, 3)) if f is None else f
        ea = np.zeros(n) if eatom else None
        r = Result()
        flags = which | (SAME_ATOMS if same_atoms else 0) | (OVERWRITE if overwrite else 0)
        self._ck(_lib.lmff_compute(self._h, n, _p(x), _p(t), _p(m), _p(g), flags, int(eflag), int(vflag),
                                   _p(out_f), _p(ea), C.byref(r)))
        self._last_n = n
        out = r.to_dict()
        out["f"] = out_f
        if eatom:
            out["eatom"] = ea
        if vatom:
            self._add_vatom(out, which)
        return out

    def vatom(self, which: int = TERSOFF | ILP, natoms: Optional[int] = None) -> np.ndarray:
        """Per-atom virial (lmff_compute_vatom) of the evaluation the previous call on this
        engine made: [n, 6], rows xx yy zz xy xz yz in that call's atom order (nall rows
        after compute_ghost), the styles selected by `which`."""
        n = getattr(self, "_last_n", 0) if natoms is None else int(natoms)
        v = np.zeros((n, 6))
        self._ck(_lib.lmff_compute_vatom(self._h, which, n, _p(v)))
        return v

    def _add_vatom(self, out: Dict, which: int):
        vt = self.vatom(TERSOFF) if which & TERSOFF else np.zeros((self._last_n, 6))
        vi = self.vatom(ILP) if which & ILP else np.zeros((self._last_n, 6))
        out["vatom_tersoff"], out["vatom_ilp"], out["vatom"] = vt, vi, vt + vi

    def compute_system(self, s, **kw) -> Dict:
        self.set_box(s.box_lo, s.box_hi, s.periodic, getattr(s, "tilt", None))
        return self.compute(s.x, s.type, s.mol, s.tag, **kw)

    def compute_ghost(self, nlocal: int, x, type_, mol, tag, which: int = TERSOFF | ILP, eflag=True, vflag=True,
                      eatom=False, same_atoms=False, vatom=False) -> Dict:
        """Subdomain evaluation (lmff_compute_ghost): x[nall,3] holds the owned atoms
        [0, nlocal) then the ghost atoms; returns f[nall,3] (ghost shares included),
        eatom[nall] and the per-atom virials [nall, 6] if asked, and the energies/virials
        of the owned interactions."""
        x = _f64(x).reshape(-1, 3)
        nall = x.shape[0]
        t = np.ascontiguousarray(type_, dtype=np.int32)
        m = np.ascontiguousarray(mol, dtype=np.int64)
        g = np.ascontiguousarray(tag, dtype=np.int64)
        f = np.zeros((nall, 3))
        ea = np.zeros(nall) if eatom else None
        r = Result()
        flags = which | (SAME_ATOMS if same_atoms else 0)
        self._ck(_lib.lmff_compute_ghost(self._h, int(nlocal), nall, _p(x), _p(t), _p(m), _p(g), flags, int(eflag),
                                         int(vflag), _p(f), _p(ea), C.byref(r)))
        self._last_n = nall
        out = r.to_dict()
        out["f"] = f
        if eatom:
            out["eatom"] = ea
        if vatom:
            self._add_vatom(out, which)
        return out

    def compute_device(self, x, type_, mol, tag, f, which: int = TERSOFF | ILP, eflag=True, vflag=True,
                       same_atoms=False, overwrite=True) -> Dict:
        """Device-pointer variant: x, type, mol, tag, f are torch CUDA tensors
        (float64 [n,3], int32 [n], int64 [n], int64 [n] or None, float64 [n,3])."""
        r = Result()
        flags = which | (SAME_ATOMS if same_atoms else 0) | (OVERWRITE if overwrite else 0)
        self._ck(_lib.lmff_compute_device(self._h, int(x.shape[0]), x.data_ptr(), type_.data_ptr(),
                                          mol.data_ptr() if mol is not None else None,
                                          tag.data_ptr() if tag is not None else None, flags, int(eflag),
                                          int(vflag), f.data_ptr(), C.byref(r)))
        self._last_n = int(x.shape[0])
        return r.to_dict()

    def compute_device_noalloc(self, x, type_, mol, f, which: int = TERSOFF | ILP, eflag=True, vflag=True) -> Dict:
        """Allocation-free evaluation (lmff_compute_device_noalloc) on torch CUDA tensors:
        x float64 [n,3], type int32 [n], mol int64 [n], f float64 [n,3] (overwritten)."""
        r = Result()
        self._ck(_lib.lmff_compute_device_noalloc(self._h, int(x.shape[0]), x.data_ptr(), type_.data_ptr(),
                                                  mol.data_ptr(), which, int(eflag), int(vflag), f.data_ptr(),
                                                  C.byref(r)))
        return r.to_dict()

    # -------------------------------------------------------------- resident MD
    def upload(self, s, masses=None):
        """Make `s` the resident system.  masses (per type) default to the system's
        (a data file's Masses section), else C, B, N."""
        if masses is None:
            masses = s.type_masses() if hasattr(s, "type_masses") else (12.011, 10.811, 14.0067)
        self.set_box(s.box_lo, s.box_hi, s.periodic)
        x = _f64(s.x)
        v = None if s.v is None else _f64(s.v)
        t = np.ascontiguousarray(s.type, dtype=np.int32)
        m = np.ascontiguousarray(s.mol, dtype=np.int64)
        g = np.ascontiguousarray(s.tag, dtype=np.int64)
        ms = _f64(list(masses) + [1.0] * (self.ntypes - len(masses)))
        self._n = x.shape[0]
        self._ck(_lib.lmff_upload(self._h, self._n, _p(x), _p(v), _p(t), _p(m), _p(g), _p(ms)))

    def compute_resident(self, which: int = TERSOFF | ILP, eflag=True, vflag=True) -> Dict:
        r = Result()
        self._ck(_lib.lmff_compute_resident(self._h, which, int(eflag), int(vflag), C.byref(r)))
        self._last_n = self._n
        return r.to_dict()

    def run_nve(self, nsteps: int, dt: float = 0.001, thermo_every: int = 0) -> List[Dict]:
        nth = (nsteps // thermo_every + 1) if thermo_every > 0 else 0
        th = (Thermo * max(nth, 1))()
        self._ck(_lib.lmff_run_nve(self._h, nsteps, dt, thermo_every, C.cast(th, C.c_void_p) if nth else None))
        return [{"step": t.step, "pe": t.pe, "ke": t.ke, "etotal": t.etotal, "temp": t.temp,
                 "virial": np.array(t.virial[:])} for t in th[:nth]]

    def minimize(self, etol: float, ftol: float, maxiter: int, maxeval: int, dmax: float = 0.1,
                 frozen: Optional[np.ndarray] = None) -> Dict:
        """LAMMPS `minimize etol ftol maxiter maxeval` (min_style cg, line quadratic) on
        the resident system; frozen atoms (nonzero, upload order) keep zero force."""
        r = MinResult()
        fz = None if frozen is None else np.ascontiguousarray(frozen, dtype=np.int32)
        self._ck(_lib.lmff_minimize(self._h, etol, ftol, maxiter, maxeval, dmax, _p(fz),
                                    C.cast(C.pointer(r), C.c_void_p)))
        return {k: getattr(r, k) for k, _ in MinResult._fields_}

    def download(self):
        x = np.zeros((self._n, 3))
        v = np.zeros((self._n, 3))
        f = np.zeros((self._n, 3))
        self._ck(_lib.lmff_download(self._h, _p(x), _p(v), _p(f)))
        return x, v, f

    # -------------------------------------------------------------- batch
    def set_masses(self, masses=(12.011, 10.811, 14.0067)) -> None:
        m = _f64(masses)
        self._ck(_lib.lmff_set_masses(self._h, len(m), _p(m)))

    def batch_set(self, systems, velocities: bool = False) -> None:
        """Load many systems as one resident batch; with velocities=True each system's
        v (or zeros) is loaded too, for run_nve on the whole batch."""
        xs = [_f64(s.x) for s in systems]
        ts = [np.ascontiguousarray(s.type, dtype=np.int32) for s in systems]
        ms = [np.ascontiguousarray(s.mol, dtype=np.int64) for s in systems]
        vs = [_f64(s.v) if velocities and s.v is not None else None for s in systems]
        self._batch_keep = [xs, ts, ms, vs]
        descs = (SystemDesc * len(systems))()
        d = np.frombuffer(descs, dtype=_DESC_DTYPE)
        d["natoms"] = [s.n for s in systems]
        d["x"] = [_addr(x) for x in xs]
        d["type"] = [_addr(t) for t in ts]
        d["mol"] = [_addr(m) for m in ms]
        d["v"] = [0 if v is None else _addr(v) for v in vs]
        d["lo"] = [s.box_lo for s in systems]
        d["hi"] = [s.box_hi for s in systems]
        d["periodic"] = [[int(bool(p)) for p in s.periodic] for s in systems]
        self._batch_n = [s.n for s in systems]
        self._n = sum(self._batch_n)
        self._ck(_lib.lmff_batch_set(self._h, len(systems), C.cast(descs, C.c_void_p)))

    def batch_results(self) -> List[Dict]:
        """Per-system energies and virials of the last evaluation that computed them."""
        res = (Result * len(self._batch_n))()
        self._ck(_lib.lmff_batch_results(self._h, len(self._batch_n), C.cast(res, C.c_void_p)))
        return _results(res, len(self._batch_n))

    def split(self, a: np.ndarray) -> List[np.ndarray]:
        """Split a batch-ordered per-atom array into the systems of the batch."""
        return np.split(a, np.cumsum(self._batch_n)[:-1])

    def batch_compute(self):
        ntot = sum(self._batch_n)
        f = np.empty((ntot, 3))   # lmff_batch_compute writes every element
        res = (Result * len(self._batch_n))()
        self._ck(_lib.lmff_batch_compute(self._h, _p(f), C.cast(res, C.c_void_p)))
        out = _results(res, len(self._batch_n))
        o = 0
        for d, n in zip(out, self._batch_n):
            d["f"] = f[o:o + n]
            o += n
        return out

    # -------------------------------------------------------------- diagnostics
    def stats(self) -> Dict:
        s = Stats()
        self._ck(_lib.lmff_get_stats(self._h, C.byref(s)))
        out = {k: getattr(s, k) for k, _ in Stats._fields_}
        out["kernel_ms"] = dict(zip(KERNELS, s.kernel_ms[:]))
        out["kernel_launches"] = dict(zip(KERNELS, s.kernel_launches[:]))
        return out

    def export_list(self, which: int = 0) -> np.ndarray:
        n = _lib.lmff_export_list(self._h, which, None, 0)
        if n < 0:
            self._ck(int(n))
        out = np.zeros((n, 3), dtype=np.int64)
        _lib.lmff_export_list(self._h, which, _p(out), n)
        return out


def device_count() -> int:
    return int(load_library().lmff_device_count())
