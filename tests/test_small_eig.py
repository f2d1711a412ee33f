"""CPU: the small dense eigen-solvers used on the device (tm_hqr.cuh: Hessenberg
reduction + Francis double-shift QR, complex inverse iteration) compiled with
the host compiler and checked against numpy.linalg.eig on random and
structured matrices."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = r"""
#include <vector>
#include "tm_hqr.cuh"
extern "C" int hqr_values(double* H, int m, double* wr, double* wi) { return ltm::geneig_values(H, m, wr, wi); }
extern "C" void hqr_vector(const double* A, int m, double lr, double li, double* yr, double* yi) {
  std::vector<double> Br(m * m), Bi(m * m);
  ltm::geneig_vector(A, m, m, lr, li, Br.data(), Bi.data(), yr, yi);
}
"""


@pytest.fixture(scope="module")
def lib():
    d = tempfile.mkdtemp()
    src = os.path.join(d, "shim.cpp")
    out = os.path.join(d, "libhqr.so")
    open(src, "w").write(SHIM)
    subprocess.run(["g++", "-O2", "-shared", "-fPIC", "-I", os.path.join(ROOT, "latttmat_gb300", "csrc"), src, "-o",
                    out], check=True)
    L = ctypes.CDLL(out)
    L.hqr_values.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    L.hqr_vector.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
                             ctypes.c_void_p]
    return L


def eig(lib, A):
    m = A.shape[0]
    H = np.asfortranarray(A.copy())
    wr = np.zeros(m)
    wi = np.zeros(m)
    st = lib.hqr_values(H.ctypes.data, m, wr.ctypes.data, wi.ctypes.data)
    return st, wr + 1j * wi


def matrices():
    rng = np.random.default_rng(5)
    for m in (3, 4, 5, 7, 11, 16, 23, 32, 46):
        yield rng.standard_normal((m, m))
        # Krylov-Schur-like: upper Hessenberg with a dense leading block and a coupling row
        H = np.triu(rng.standard_normal((m, m)), -1)
        k = m // 2
        H[k, :k] = rng.standard_normal(k)
        yield H
        # positive matrix with a dominant real eigenvalue and a negative second one
        P = np.abs(rng.standard_normal((m, m)))
        yield P - 0.6 * np.diag(rng.uniform(size=m))


@pytest.mark.parametrize("A", list(matrices()))
def test_eigenvalues_match_numpy(lib, A):
    st, w = eig(lib, A)
    assert st == 0
    ref = np.linalg.eigvals(A)
    scale = max(1.0, np.max(np.abs(ref)))
    for z in ref:
        assert np.min(np.abs(w - z)) < 1e-9 * scale


@pytest.mark.parametrize("A", list(matrices())[:12])
def test_eigenvectors(lib, A):
    m = A.shape[0]
    Af = np.asfortranarray(A)
    for z in np.linalg.eigvals(A):
        yr = np.zeros(m)
        yi = np.zeros(m)
        lib.hqr_vector(Af.ctypes.data, m, z.real, z.imag, yr.ctypes.data, yi.ctypes.data)
        y = yr + 1j * yi
        assert abs(np.linalg.norm(y) - 1) < 1e-12
        assert np.linalg.norm(A @ y - z * y) < 1e-8 * max(1.0, np.linalg.norm(A))
