"""ctypes front end of the oracle (oracle/tm_oracle.c) plus a CPU eigensolver.

OracleOp mirrors a reference MatVecProd (rows/perform_op/normfactor/orbit
table/moments/phys_extend).  eigs() drives its perform_op with ARPACK (scipy),
the same implicitly-restarted Lanczos/Arnoldi family as the reference's
Spectra solver, at tol 1e-13.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build_oracle

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.LIB
        if not os.path.exists(path):
            path = build_oracle.build()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        L.orc_create.restype = P
        L.orc_create.argtypes = [ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int]
        L.orc_destroy.argtypes = [P]
        L.orc_rows.restype = ctypes.c_int64
        L.orc_rows.argtypes = [P]
        L.orc_normfactor.restype = ctypes.c_double
        L.orc_normfactor.argtypes = [P]
        L.orc_symmetric.argtypes = [P]
        L.orc_perform_op.argtypes = [P, P, P]
        L.orc_perform_op_t.argtypes = [P, P, P]
        L.orc_orbit.restype = ctypes.c_int64
        L.orc_orbit.argtypes = [P, P, P]
        L.orc_moments.argtypes = [P, P, P, P]
        L.orc_phys_extend.argtypes = [P, P, P, P, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.orc_xam_slices.restype = ctypes.c_int64
        L.orc_xam_slices.argtypes = [P, P, P, ctypes.c_int64, ctypes.c_int64]
        L.orc_xam_nslices.restype = ctypes.c_int64
        L.orc_xam_nslices.argtypes = [P]
        _lib = L
    return _lib


class OracleOp:
    def __init__(self, model, dim, axialdir, betaJ, kappa, h=0.0, size=12, kappa2=0.0, extend_cond=0):
        packed = (size[0] << 16) | size[1] if dim == 3 else int(size)
        self.h = lib().orc_create(model.encode(), dim, axialdir, extend_cond, betaJ, kappa, kappa2, h, packed)
        if not self.h:
            raise ValueError("operator not provided by the reference dispatch")
        self.n = int(lib().orc_rows(self.h))
        self.normfactor = float(lib().orc_normfactor(self.h))
        self.symmetric = bool(lib().orc_symmetric(self.h))

    def rows(self):
        return self.n

    def perform_op(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        lib().orc_perform_op(self.h, x.ctypes.data, y.ctypes.data)
        return y

    def perform_op_t(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        lib().orc_perform_op_t(self.h, x.ctypes.data, y.ctypes.data)
        return y

    def orbit(self):
        n = lib().orc_orbit(self.h, None, None)
        if n < 0:
            return None, None
        idx = np.empty(n, np.uint64)
        dup = np.empty(n, np.uint16)
        lib().orc_orbit(self.h, idx.ctypes.data, dup.ctypes.data)
        return idx, dup

    def moments(self, ql, qr=None):
        ql = np.ascontiguousarray(ql, dtype=np.float64)
        qr = ql if qr is None else np.ascontiguousarray(qr, dtype=np.float64)
        out = np.zeros(4)
        st = lib().orc_moments(self.h, ql.ctypes.data, qr.ctypes.data, out.ctypes.data)
        return out, st

    def phys_extend(self, ql, qr=None):
        ql = np.ascontiguousarray(ql, dtype=np.float64)
        qr = ql if qr is None else np.ascontiguousarray(qr, dtype=np.float64)
        out = np.zeros(8)
        nout = ctypes.c_int()
        st = lib().orc_phys_extend(self.h, ql.ctypes.data, qr.ctypes.data, out.ctypes.data, 8, ctypes.byref(nout))
        return out[: nout.value].copy(), st

    def xam_slices(self, x, first, count):
        """Run `count` leading-bit slices of the reduced x-ANNNI product (timing samples)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        done = lib().orc_xam_slices(self.h, x.ctypes.data, y.ctypes.data, int(first), int(count))
        return y, int(done)

    def xam_nslices(self):
        return int(lib().orc_xam_nslices(self.h))

    def eigs(self, nev, tol=1e-13, seed=0, return_vectors=False):
        import scipy.sparse.linalg as sla

        n = self.n
        lin = sla.LinearOperator((n, n), matvec=lambda v: self.perform_op(np.ravel(v)), dtype=np.float64)
        v0 = np.random.default_rng(seed).uniform(0, 1, n)
        ncv = min(n - 1, max(2 * nev + 8, 20))
        if self.symmetric:
            w, v = sla.eigsh(lin, k=nev, which="LM", tol=tol, v0=v0, ncv=ncv)
        else:
            w, v = sla.eigs(lin, k=nev, which="LM", tol=tol, v0=v0, ncv=ncv)
        o = np.argsort(-np.abs(w), kind="stable")
        w = w[o] / self.normfactor
        if return_vectors:
            return w, v[:, o]
        return w

    def __del__(self):
        try:
            lib().orc_destroy(self.h)
        except Exception:
            pass
