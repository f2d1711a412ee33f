"""ctypes binding to oracle/_ref/libtmat_ref.so -- the reference's own operator
sources compiled by oracle/build_ref.sh.  Test infrastructure only (golden
fixture generation and CPU-side pinning of the oracle); never used by the
product path.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(HERE, "_ref", "libtmat_ref.so")


def available() -> bool:
    return os.path.exists(REF_LIB)


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(REF_LIB)
        P = ctypes.c_void_p
        L.ref_create.restype = P
        L.ref_create.argtypes = [ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int]
        L.ref_destroy.argtypes = [P]
        L.ref_rows.restype = ctypes.c_int64
        L.ref_rows.argtypes = [P]
        L.ref_normfactor.restype = ctypes.c_double
        L.ref_normfactor.argtypes = [P]
        L.ref_perform_op.argtypes = [P, P, P]
        L.ref_has_transpose.argtypes = [P]
        L.ref_perform_op_t.argtypes = [P, P, P]
        L.ref_orbit.restype = ctypes.c_int64
        L.ref_orbit.argtypes = [P, P, P, ctypes.c_int64]
        L.ref_moments.argtypes = [P, P, P, P]
        L.ref_phys_extend.argtypes = [P, P, P, P, ctypes.c_int]
        L.ref_dump.argtypes = [ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                               ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p,
                               ctypes.c_int, ctypes.c_int, ctypes.c_uint, ctypes.c_char_p]
        _lib = L
    return _lib


def ref_dump(model, axialdir, extend_cond, betaJ, kappa, kappa2, h, size, vecfile, veclfile, nconfig, length,
             seed, prefix):
    """Run the reference's DumpConfig dump() (fixed seed); returns its status."""
    return lib().ref_dump(model.encode(), int(axialdir), int(extend_cond), float(betaJ), float(kappa),
                          float(kappa2), float(h), int(size), vecfile.encode(), (veclfile or "").encode(),
                          int(nconfig), int(length), int(seed), prefix.encode())


def read_configs(prefix, nconfig, L):
    """Layer states of <prefix>_config_<k>.dat files (L digits per line, site 0 first)."""
    out = []
    for k in range(nconfig):
        rows = []
        for line in open(f"{prefix}_config_{k}.dat").read().split():
            rows.append(sum(1 << i for i, ch in enumerate(line[:L]) if ch == "1"))
        out.append(rows)
    return np.array(out, dtype=np.uint64)


class RefOp:
    """One reference operator (constructed exactly as TMat/pfunc.cpp does)."""

    def __init__(self, model, dim, axialdir, betaJ, kappa, h=0.0, size=12, kappa2=0.0, extend_cond=0):
        packed = (size[0] << 16) | size[1] if dim == 3 else int(size)
        self.h = lib().ref_create(model.encode(), dim, axialdir, extend_cond, betaJ, kappa, kappa2, h, packed)
        if not self.h:
            raise ValueError("reference does not provide this operator")
        self.n = lib().ref_rows(self.h)
        self.normfactor = lib().ref_normfactor(self.h)

    def perform_op(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        lib().ref_perform_op(self.h, x.ctypes.data, y.ctypes.data)
        return y

    def has_transpose(self):
        return bool(lib().ref_has_transpose(self.h))

    def perform_op_t(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        lib().ref_perform_op_t(self.h, x.ctypes.data, y.ctypes.data)
        return y

    def orbit(self):
        idx = np.zeros(self.n, np.uint64)
        dup = np.zeros(self.n, np.uint32)
        n = lib().ref_orbit(self.h, idx.ctypes.data, dup.ctypes.data, self.n)
        if n < 0:
            return None, None
        return idx, dup

    def moments(self, ql, qr=None):
        ql = np.ascontiguousarray(ql, dtype=np.float64)
        qr = ql if qr is None else np.ascontiguousarray(qr, dtype=np.float64)
        out = np.zeros(4)
        st = lib().ref_moments(self.h, ql.ctypes.data, qr.ctypes.data, out.ctypes.data)
        return out, st

    def phys_extend(self, ql, qr=None):
        ql = np.ascontiguousarray(ql, dtype=np.float64)
        qr = ql if qr is None else np.ascontiguousarray(qr, dtype=np.float64)
        out = np.zeros(8)
        n = lib().ref_phys_extend(self.h, ql.ctypes.data, qr.ctypes.data, out.ctypes.data, 8)
        st = 0
        if n < 0:
            n = -1 - n
            st = -1
        return out[:n].copy(), st

    def __del__(self):
        try:
            lib().ref_destroy(self.h)
        except Exception:
            pass
