"""latttmat_gb300 -- GB300 transfer-matrix operators and eigensolver.

Python mirror of the reference's operator interface over the C ABI in
``include/latttmat.h`` (liblatttmat_gb300.so, sm_103a).  ``TMatOp`` plays the
part of one reference MatVecProd class (TMat/tmat.hpp:82-144):
``rows()/cols()/perform_op(x, y)/getnormfactor()/getLayerSize()/moments()/
phys_extend()/get_t_instance()``.  ``pfunc`` and ``read_input`` mirror
TMat/pfunc.hpp / TMat/read_input.cpp (see ``latttmat_gb300.driver``).

The CUDA library is required: there is no CPU fallback.  Importing works on a
machine without a GPU (tests check the exported symbols there), but every
compute call needs a CUDA device.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liblatttmat_gb300.so")

TM_OK = 0
TM_ERR_ARG = 1
TM_ERR_UNSUPPORTED = 2
TM_ERR_CUDA = 3
TM_ERR_NOMEM = 4
TM_ERR_NOCONV = 5
TM_ERR_NONFINITE = 6
TM_ERR_NOTRANSPOSE = 7
TM_ERR_LIMIT = 8

TM_F64 = 0
TM_F32 = 1
TM_F64_DF = 2
TM_EIGS_F64 = 0
TM_EIGS_MIXED = 1

# every symbol include/latttmat.h declares
EXPORTED_SYMBOLS = (
    "tm_create", "tm_transpose", "tm_destroy", "tm_rows", "tm_cols", "tm_normfactor", "tm_layer_size",
    "tm_is_symmetric", "tm_suggested_ncv", "tm_matvec_count", "tm_perform_op", "tm_perform_op_dev",
    "tm_orbit_table", "tm_eigs", "tm_moments", "tm_phys_extend", "tm_grad", "tm_last_error", "tm_version",
    "tm_profile_matvec", "tm_launch_count", "tm_alloc_count", "tm_perform_op_dev_noalloc", "tm_eigs_batch",
    "tm_debug_set_eo_tile_bits", "tm_sweep_create", "tm_sweep_destroy", "tm_sweep_count", "tm_sweep_rows",
    "tm_sweep_normfactor", "tm_sweep_set_wave_bytes", "tm_sweep_stats", "tm_sweep_eigs_vec",
    "tm_sweep_set_transpose", "tm_sweep_grad", "tm_sweep_perform_op_dev", "tm_sweep_eigs",
    "tm_chain_autotune", "tm_chain_set_tuning", "tm_dump_configs", "tm_dump_configs_lr",
)


class TMError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class tm_params(ctypes.Structure):
    _fields_ = [("betaJ", ctypes.c_double), ("kappa", ctypes.c_double), ("kappa2", ctypes.c_double),
                ("h", ctypes.c_double), ("size", ctypes.c_int)]


class tm_eigs_info(ctypes.Structure):
    _fields_ = [("nconv", ctypes.c_int), ("matvecs", ctypes.c_int), ("matvecs_f64", ctypes.c_int),
                ("restarts", ctypes.c_int), ("ncv", ctypes.c_int), ("max_resid", ctypes.c_double),
                ("seconds", ctypes.c_double), ("refine_rounds", ctypes.c_int), ("refine_checks", ctypes.c_int),
                ("refine_outcome", ctypes.c_int), ("refine_est", ctypes.c_double),
                ("refine_true", ctypes.c_double), ("matvecs_phase1", ctypes.c_int),
                ("seconds_phase1", ctypes.c_double), ("seconds_refine", ctypes.c_double)]


_lib = None


def load_library(path: Optional[str] = None) -> ctypes.CDLL:
    """Load liblatttmat_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError(f"{p} not found; build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(p)
    P = ctypes.c_void_p
    lib.tm_create.argtypes = [ctypes.POINTER(tm_params), ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                              ctypes.POINTER(P)]
    lib.tm_transpose.argtypes = [P, ctypes.POINTER(P)]
    lib.tm_destroy.argtypes = [P]
    for f in ("tm_rows", "tm_cols", "tm_matvec_count"):
        getattr(lib, f).argtypes = [P]
        getattr(lib, f).restype = ctypes.c_int64
    lib.tm_normfactor.argtypes = [P]
    lib.tm_normfactor.restype = ctypes.c_double
    lib.tm_layer_size.argtypes = [P]
    lib.tm_is_symmetric.argtypes = [P]
    lib.tm_suggested_ncv.argtypes = [P, ctypes.c_int]
    lib.tm_perform_op.argtypes = [P, P, P]
    lib.tm_perform_op_dev.argtypes = [P, P, P, ctypes.c_int, P]
    lib.tm_orbit_table.argtypes = [P, P, P, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]
    lib.tm_eigs.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_uint64, ctypes.c_int, P, P, P,
                            P, ctypes.POINTER(tm_eigs_info)]
    lib.tm_moments.argtypes = [P, P, P, P, ctypes.POINTER(ctypes.c_int)]
    lib.tm_phys_extend.argtypes = [P, P, P, P, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                   ctypes.POINTER(ctypes.c_int)]
    lib.tm_grad.argtypes = [P, P, P, ctypes.c_double, P]
    lib.tm_profile_matvec.argtypes = [P, ctypes.c_int, ctypes.c_int, P, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    lib.tm_eigs_batch.argtypes = [P, ctypes.c_int, ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, P, P, P, P]
    lib.tm_eigs_batch.restype = ctypes.c_int
    lib.tm_launch_count.restype = ctypes.c_int64
    lib.tm_alloc_count.restype = ctypes.c_int64
    lib.tm_debug_set_eo_tile_bits.argtypes = [ctypes.c_int]
    lib.tm_debug_set_eo_tile_bits.restype = None
    lib.tm_sweep_create.argtypes = [P, ctypes.c_int, ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.POINTER(P)]
    lib.tm_sweep_destroy.argtypes = [P]
    lib.tm_sweep_count.argtypes = [P]
    lib.tm_sweep_rows.argtypes = [P, ctypes.c_int]
    lib.tm_sweep_rows.restype = ctypes.c_int64
    lib.tm_sweep_normfactor.argtypes = [P, ctypes.c_int]
    lib.tm_sweep_normfactor.restype = ctypes.c_double
    lib.tm_sweep_set_wave_bytes.argtypes = [P, ctypes.c_size_t]
    lib.tm_sweep_stats.argtypes = [P, P, ctypes.c_int]
    lib.tm_sweep_eigs_vec.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, P, P, P, P, P]
    lib.tm_sweep_set_transpose.argtypes = [P, ctypes.c_int]
    lib.tm_sweep_grad.argtypes = [P, P, P, P, P]
    for f in ("tm_sweep_eigs_vec", "tm_sweep_set_transpose", "tm_sweep_grad"):
        getattr(lib, f).restype = ctypes.c_int
    lib.tm_sweep_perform_op_dev.argtypes = [P, P, P, ctypes.c_int]
    lib.tm_sweep_eigs.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, P, P, P, P]
    lib.tm_chain_autotune.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_double)]
    lib.tm_chain_set_tuning.argtypes = [ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    for f in ("tm_sweep_create", "tm_sweep_destroy", "tm_sweep_set_wave_bytes", "tm_sweep_perform_op_dev",
              "tm_sweep_eigs", "tm_chain_autotune", "tm_chain_set_tuning"):
        getattr(lib, f).restype = ctypes.c_int
    lib.tm_dump_configs.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_uint32, P]
    lib.tm_dump_configs.restype = ctypes.c_int
    lib.tm_dump_configs_lr.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_uint32, P]
    lib.tm_dump_configs_lr.restype = ctypes.c_int
    lib.tm_last_error.restype = ctypes.c_char_p
    lib.tm_version.restype = ctypes.c_char_p
    for f in ("tm_create", "tm_transpose", "tm_destroy", "tm_perform_op", "tm_perform_op_dev", "tm_orbit_table",
              "tm_eigs", "tm_moments", "tm_phys_extend", "tm_grad", "tm_profile_matvec"):
        getattr(lib, f).restype = ctypes.c_int
    if path is None:
        _lib = lib
    return lib


def eigs_batch(model: str, dim: int, axialdir: int, points, nev: int = 2, tol: float = 1e-10,
               mode: int = TM_EIGS_MIXED, extend_cond: int = 0, nthreads: int = 0):
    """Solve many parameter points concurrently (tm_eigs_batch).

    points: sequence of (betaJ, kappa, kappa2, h, size) tuples.  Returns
    (vals complex [count, nev] already divided by normfactor, info dicts,
    per-instance status codes)."""
    lib = load_library()
    count = len(points)
    arr = (tm_params * max(count, 1))()
    for i, (bj, k, k2, h, size) in enumerate(points):
        arr[i] = tm_params(float(bj), float(k), float(k2), float(h), int(size))
    vr = np.zeros(count * nev)
    vi = np.zeros(count * nev)
    infos = (tm_eigs_info * max(count, 1))()
    st = np.zeros(max(count, 1), dtype=np.int32)
    code = lib.tm_eigs_batch(ctypes.byref(arr), count, model.encode()[:1], int(dim), int(axialdir),
                             int(extend_cond), int(nev), float(tol), int(mode), int(nthreads), _ptr(vr), _ptr(vi),
                             ctypes.byref(infos), _ptr(st))
    if code != TM_OK and not np.any(st[:count] == TM_OK):
        _check(code)
    vals = (vr + 1j * vi).reshape(count, nev)
    info = [{k: getattr(infos[i], k) for k, _ in tm_eigs_info._fields_} for i in range(count)]
    return vals, info, st[:count].copy()


class Sweep:
    """A parameter sweep of aux-bit operators (models B and D) solved as one
    device batch (tm_sweep_*): points are (betaJ, kappa, kappa2, h, size)
    tuples, widths may differ."""

    def __init__(self, model: str, dim: int, axialdir: int, points, extend_cond: int = 0):
        lib = load_library()
        self._lib = lib
        count = len(points)
        arr = (tm_params * max(count, 1))()
        for i, (bj, k, k2, h, size) in enumerate(points):
            arr[i] = tm_params(float(bj), float(k), float(k2), float(h), int(size))
        h_ = ctypes.c_void_p()
        _check(lib.tm_sweep_create(ctypes.byref(arr), count, model.encode()[:1], int(dim), int(axialdir),
                                   int(extend_cond), ctypes.byref(h_)))
        self._h = h_
        self.points = list(points)

    def count(self) -> int:
        return int(self._lib.tm_sweep_count(self._h))

    def rows(self, i: int) -> int:
        return int(self._lib.tm_sweep_rows(self._h, int(i)))

    def normfactor(self, i: int) -> float:
        return float(self._lib.tm_sweep_normfactor(self._h, int(i)))

    def stats(self) -> dict:
        """Diagnostics of the last eigs(): waves, steps, seconds per phase."""
        out = np.zeros(5)
        n = self._lib.tm_sweep_stats(self._h, _ptr(out), 5)
        keys = ("waves", "steps", "wave_build_s", "step_s", "restart_s")
        return {k: float(out[i]) for i, k in enumerate(keys[:n])}

    def set_wave_bytes(self, nbytes: int) -> None:
        _check(self._lib.tm_sweep_set_wave_bytes(self._h, int(nbytes)))

    def perform_op_dev(self, x_ptrs, y_ptrs, dtype: int = TM_F64) -> None:
        """y_i = T_i x_i for every member; x_ptrs / y_ptrs: device pointers to FP64 vectors."""
        n = self.count()
        xa = (ctypes.c_void_p * n)(*[ctypes.c_void_p(int(p)) for p in x_ptrs])
        ya = (ctypes.c_void_p * n)(*[ctypes.c_void_p(int(p)) for p in y_ptrs])
        _check(self._lib.tm_sweep_perform_op_dev(self._h, ctypes.cast(xa, ctypes.c_void_p),
                                                 ctypes.cast(ya, ctypes.c_void_p), int(dtype)))

    def eigs(self, nev: int = 2, tol: float = 1e-10, mode: int = TM_EIGS_MIXED, ncv: int = 0,
             vectors: bool = False):
        """(vals complex [count, nev] / normfactor, info dicts, status codes),
        and with vectors=True a fourth item: each member's leading eigenvector."""
        n = self.count()
        vr = np.zeros(n * nev)
        vi = np.zeros(n * nev)
        infos = (tm_eigs_info * n)()
        st = np.zeros(n, dtype=np.int32)
        if vectors:
            vecs = [np.zeros(self.rows(i)) for i in range(n)]
            ptrs = (ctypes.c_void_p * n)(*[ctypes.c_void_p(v.ctypes.data) for v in vecs])
            code = self._lib.tm_sweep_eigs_vec(self._h, int(nev), int(ncv), float(tol), int(mode), _ptr(vr),
                                               _ptr(vi), ctypes.cast(ptrs, ctypes.c_void_p), ctypes.byref(infos),
                                               _ptr(st))
        else:
            code = self._lib.tm_sweep_eigs(self._h, int(nev), int(ncv), float(tol), int(mode), _ptr(vr), _ptr(vi),
                                           ctypes.byref(infos), _ptr(st))
        if code != TM_OK and not np.any(st == TM_OK):
            _check(code)
        vals = (vr + 1j * vi).reshape(n, nev)
        info = [{k: getattr(infos[i], k) for k, _ in tm_eigs_info._fields_} for i in range(n)]
        if vectors:
            return vals, info, st.copy(), vecs
        return vals, info, st.copy()

    def set_transpose(self, transpose: bool = True) -> None:
        """Solve the members' transposes (left eigenvectors)."""
        _check(self._lib.tm_sweep_set_transpose(self._h, int(bool(transpose))))

    def grad(self, qr, ql, lambda_internal) -> np.ndarray:
        """Batched adjoint: d ln(lambda_i)/d(betaJ, kappa, kappa2, h), shape (count, 4)."""
        n = self.count()
        qr = [np.ascontiguousarray(v, dtype=np.float64) for v in qr]
        pr = (ctypes.c_void_p * n)(*[ctypes.c_void_p(v.ctypes.data) for v in qr])
        pl = None
        if ql is not None:
            ql = [np.ascontiguousarray(v, dtype=np.float64) for v in ql]
            pl = (ctypes.c_void_p * n)(*[ctypes.c_void_p(v.ctypes.data) for v in ql])
        lam = np.ascontiguousarray(lambda_internal, dtype=np.float64)
        g = np.zeros(n * 4)
        _check(self._lib.tm_sweep_grad(self._h, ctypes.cast(pr, ctypes.c_void_p),
                                       ctypes.cast(pl, ctypes.c_void_p) if pl is not None else None, _ptr(lam),
                                       _ptr(g)))
        return g.reshape(n, 4)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.tm_sweep_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def chain_autotune(op: "TMatOp", dtype: int = TM_F32):
    """Time the aux-bit operator's product over the chain kernels' tile and
    block sizes; the fastest goes into the library's tuning table.
    Returns (tile_bits, threads, ms per product)."""
    tb = ctypes.c_int()
    th = ctypes.c_int()
    ms = ctypes.c_double()
    _check(load_library().tm_chain_autotune(op._h, int(dtype), ctypes.byref(tb), ctypes.byref(th), ctypes.byref(ms)))
    return tb.value, th.value, ms.value


def write_configs(states: np.ndarray, L: int, prefix: str) -> None:
    """Write planted configurations as the reference does: <prefix>_config_<k>.dat,
    one line per layer, L digits, site 0 first (DumpConfig/dumpconfig.hpp:32-40)."""
    for k, row in enumerate(np.asarray(states)):
        with open(f"{prefix}_config_{k}.dat", "w") as fh:
            for st in row:
                st = int(st)
                fh.write("".join("1" if (st >> i) & 1 else "0" for i in range(L)) + "\n")


def chain_set_tuning(model: str, L: int, dtype: int, tile_bits: int, threads: int) -> None:
    """Set one entry of the chain tuning table (0, 0: the default)."""
    _check(load_library().tm_chain_set_tuning(model.encode()[:1], int(L), int(dtype), int(tile_bits), int(threads)))


def launch_count() -> int:
    """Kernels launched by the library since load."""
    return int(load_library().tm_launch_count())


def alloc_count() -> int:
    """Device allocations requested by the library since load."""
    return int(load_library().tm_alloc_count())


def debug_set_eo_tile_bits(bits: int) -> None:
    """Cap the even/odd passes' tiles at 2^bits elements for operators created
    afterwards (0: no cap), so small operators take the clustered code paths."""
    load_library().tm_debug_set_eo_tile_bits(int(bits))


def _check(code: int):
    if code != TM_OK:
        msg = load_library().tm_last_error().decode(errors="replace")
        raise TMError(code, msg)


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class TMatOp:
    """One transfer-matrix operator on the GPU (a reference MatVecProd).

    model: 'A' (ANNNI), 'B' (BNNNI+3NN), 'D' (DNNI); dim 2 or 3; axialdir as
    in the reference input file; extend_cond as the reference constructors take
    it (bit 0 open boundary, bit 1 no spin-flip reduction).  For dim=3 pass
    size=(size1, size2).
    """

    def __init__(self, model: str, dim: int, axialdir: int, betaJ: float, kappa: float, h: float = 0.0,
                 size=12, kappa2: float = 0.0, extend_cond: int = 0, _handle=None, _parent=None):
        lib = load_library()
        self._lib = lib
        self._parent = _parent
        if _handle is not None:
            self._h = _handle
        else:
            if dim == 3:
                s1, s2 = size
                packed = (int(s1) << 16) | int(s2)
            else:
                packed = int(size)
            p = tm_params(float(betaJ), float(kappa), float(kappa2), float(h), packed)
            h_ = ctypes.c_void_p()
            _check(lib.tm_create(ctypes.byref(p), model.encode()[:1], int(dim), int(axialdir), int(extend_cond),
                                 ctypes.byref(h_)))
            self._h = h_
        self.model, self.dim, self.axialdir = model, dim, axialdir

    # --- Spectra operator concept -------------------------------------
    def rows(self) -> int:
        return int(self._lib.tm_rows(self._h))

    def cols(self) -> int:
        return int(self._lib.tm_cols(self._h))

    def getnormfactor(self) -> float:
        return float(self._lib.tm_normfactor(self._h))

    def getLayerSize(self) -> int:
        return int(self._lib.tm_layer_size(self._h))

    def is_symmetric(self) -> bool:
        return bool(self._lib.tm_is_symmetric(self._h))

    def suggested_nev(self, neig: int) -> int:
        return int(self._lib.tm_suggested_ncv(self._h, int(neig)))

    def matvec_count(self) -> int:
        return int(self._lib.tm_matvec_count(self._h))

    def perform_op(self, x_in: np.ndarray, y_out: Optional[np.ndarray] = None) -> np.ndarray:
        x = np.ascontiguousarray(x_in, dtype=np.float64)
        if x.shape != (self.cols(),):
            raise ValueError(f"x has shape {x.shape}, expected ({self.cols()},)")
        y = y_out if y_out is not None else np.empty_like(x)
        _check(self._lib.tm_perform_op(self._h, _ptr(x), _ptr(y)))
        return y

    def perform_op_dev(self, x_ptr: int, y_ptr: int, dtype: int = TM_F64, stream: int = 0):
        """y = T x on device buffers (raw pointers, e.g. torch tensor.data_ptr())."""
        _check(self._lib.tm_perform_op_dev(self._h, ctypes.c_void_p(x_ptr), ctypes.c_void_p(y_ptr), int(dtype),
                                           ctypes.c_void_p(stream)))

    def get_t_instance(self) -> "TMatOp":
        h_ = ctypes.c_void_p()
        _check(self._lib.tm_transpose(self._h, ctypes.byref(h_)))
        return TMatOp(self.model, self.dim, self.axialdir, 0, 0, _handle=h_, _parent=self)

    # --- reduced basis ------------------------------------------------
    def orbit_table(self):
        """(idxlist uint64, duplist uint16) of a reduced operator."""
        n = ctypes.c_int64()
        _check(self._lib.tm_orbit_table(self._h, None, None, 0, ctypes.byref(n)))
        idx = np.empty(n.value, np.uint64)
        dup = np.empty(n.value, np.uint16)
        _check(self._lib.tm_orbit_table(self._h, _ptr(idx), _ptr(dup), n.value, ctypes.byref(n)))
        return idx, dup

    # --- eigensolver --------------------------------------------------
    def eigs(self, nev: int, ncv: int = 0, tol: float = 1e-10, seed: int = 0, mode: int = TM_EIGS_F64,
             vectors: bool = False, left: bool = False, vecs_out: Optional[np.ndarray] = None):
        """Largest-magnitude eigenvalues (already divided by normfactor).

        Returns (vals, vecs or None, vecl or None, info dict)."""
        vr = np.zeros(nev)
        vi = np.zeros(nev)
        n = self.rows()
        sym = self.is_symmetric()
        vecs = None
        if vectors:
            shape = (nev, n) if sym else (nev, n, 2)
            if vecs_out is not None:  # caller-provided (e.g. pinned) host buffer
                if vecs_out.shape != shape or vecs_out.dtype != np.float64 or not vecs_out.flags.c_contiguous:
                    raise ValueError(f"vecs_out must be a C-contiguous float64 array of shape {shape}")
                vecs = vecs_out
            else:
                vecs = np.zeros(shape)
        vecl = np.zeros(n) if (left and not sym) else None
        info = tm_eigs_info()
        _check(self._lib.tm_eigs(self._h, int(nev), int(ncv), float(tol), int(seed), int(mode), _ptr(vr), _ptr(vi),
                                 _ptr(vecs) if vecs is not None else None,
                                 _ptr(vecl) if vecl is not None else None, ctypes.byref(info)))
        vals = vr if sym else vr + 1j * vi
        if vecs is not None and not sym:
            vecs = vecs[..., 0] + 1j * vecs[..., 1]
        d = {k: getattr(info, k) for k, _ in tm_eigs_info._fields_}
        return vals, vecs, vecl, d

    # --- observables --------------------------------------------------
    def moments(self, ql: np.ndarray, qr: Optional[np.ndarray] = None):
        ql = np.ascontiguousarray(ql, dtype=np.float64)
        qr = ql if qr is None else np.ascontiguousarray(qr, dtype=np.float64)
        out = np.zeros(4)
        st = ctypes.c_int()
        _check(self._lib.tm_moments(self._h, _ptr(ql), _ptr(qr), _ptr(out), ctypes.byref(st)))
        return out, st.value

    def phys_extend(self, ql: np.ndarray, qr: Optional[np.ndarray] = None):
        ql = np.ascontiguousarray(ql, dtype=np.float64)
        qr = ql if qr is None else np.ascontiguousarray(qr, dtype=np.float64)
        out = np.zeros(8)
        nout = ctypes.c_int()
        st = ctypes.c_int()
        _check(self._lib.tm_phys_extend(self._h, _ptr(ql), _ptr(qr), _ptr(out), 8, ctypes.byref(nout),
                                        ctypes.byref(st)))
        return out[: nout.value].copy(), st.value

    def grad(self, qr: np.ndarray, lambda_internal: float, ql: Optional[np.ndarray] = None) -> np.ndarray:
        """d ln(lambda)/d(betaJ, kappa, kappa2, h) of the eigenvalue of qr (ql for general operators)."""
        qr = np.ascontiguousarray(qr, dtype=np.float64)
        qlp = None
        if ql is not None:
            ql = np.ascontiguousarray(ql, dtype=np.float64)
            qlp = _ptr(ql)
        g = np.zeros(4)
        _check(self._lib.tm_grad(self._h, _ptr(qr), qlp, float(lambda_internal), _ptr(g)))
        return g

    def dump_configs(self, vec: np.ndarray, nconfig: int, length: int, seed: int,
                     vecl: Optional[np.ndarray] = None) -> np.ndarray:
        """Plant configurations from the leading eigenvector (the reference's
        DumpConfig, operators A/1, A/5 and D/5): uint64 layer states, shape
        (nconfig, length).  The two-layer parallel TMs (A/2, A/6, B/6) plant
        from their right and left eigenvectors (vecl); the full one (A/2)
        gives length + 1 layers per chain, as the reference writes them."""
        v = np.ascontiguousarray(vec, dtype=np.float64)
        if v.shape != (self.rows(),):
            raise ValueError(f"vec has shape {v.shape}, expected ({self.rows()},)")
        if vecl is None:
            out = np.zeros((int(nconfig), int(length)), dtype=np.uint64)
            _check(self._lib.tm_dump_configs(self._h, _ptr(v), int(nconfig), int(length), int(seed), _ptr(out)))
            return out
        vl = np.ascontiguousarray(vecl, dtype=np.float64)
        if vl.shape != (self.rows(),):
            raise ValueError(f"vecl has shape {vl.shape}, expected ({self.rows()},)")
        layers = int(length) + 1 if (self.model, self.axialdir) == ("A", 2) else int(length)
        out = np.zeros((int(nconfig), layers), dtype=np.uint64)
        _check(self._lib.tm_dump_configs_lr(self._h, _ptr(v), _ptr(vl), int(nconfig), int(length), int(seed),
                                            _ptr(out)))
        return out

    def profile_matvec(self, dtype: int = TM_F32, iters: int = 10):
        """Per-stage average ms of the internal-order product (CUDA events)."""
        out = np.zeros(8)
        ns = ctypes.c_int()
        _check(self._lib.tm_profile_matvec(self._h, int(dtype), int(iters), _ptr(out), 8, ctypes.byref(ns)))
        return out[: ns.value].copy()

    def close(self):
        if getattr(self, "_h", None):
            self._lib.tm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
