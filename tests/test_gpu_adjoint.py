"""GPU: adjoint d ln(lambda)/d(betaJ, kappa, kappa2, h) against central finite
differences (step 1e-5) of the GPU FP64 eigenvalues, and against the reference
magnetisation moment: d ln(lambda0)/dh = -betaJ * L * <M>/L
(TMat/tmatphys.cpp:13-38 with the field term of genTvec, TMat/tmat.hpp:213).
Tolerances: 2e-6 relative to max(|grad|, 1) for the FD check (the FD error of
1e-12-accurate eigenvalues at step 1e-5 is about 1e-7)."""
import numpy as np
import pytest

import latttmat_gb300 as lt

pytestmark = pytest.mark.gpu

STEP = 1e-5
# (model, dim, axialdir, extend_cond, betaJ, kappa, h, size, nev)
POINTS = [
    ("A", 2, 1, 0, 0.5, 0.3, 0.1, 10, 2),
    ("A", 2, 5, 2, 0.4, 0.6, 0.0, 14, 2),
    ("A", 2, 5, 0, 0.35, 0.55, 0.05, 16, 2),
    ("A", 3, 1, 0, 0.25, 0.4, 0.0, (3, 4), 2),
    ("A", 3, 1, 0, 0.3, 0.2, 0.05, (3, 3), 2),
]


def lam(model, dim, ax, ec, bj, k, h, size, nev, which=0):
    op = lt.TMatOp(model, dim, ax, bj, k, h, size, 0.0, ec)
    vals, vecs, _, _ = op.eigs(nev, tol=1e-13, mode=lt.TM_EIGS_F64, vectors=True)
    return op, vals, vecs


@pytest.mark.parametrize("pt", POINTS)
def test_grad_vs_finite_differences(pt):
    model, dim, ax, ec, bj, k, h, size, nev = pt
    op, vals, vecs = lam(model, dim, ax, ec, bj, k, h, size, nev)
    g = op.grad(vecs[0], vals[0] * op.getnormfactor())
    params = [bj, k, 0.0, h]
    for t in (0, 1, 3):
        if t == 3 and h == 0.0 and ec == 0 and ax in (5, 13):
            continue  # the flip-reduced sector is only defined at h = 0
        if dim == 3 and t == 3 and h == 0.0:
            continue
        if t == 1 and k == 0.5:
            continue
        pp, pm = list(params), list(params)
        pp[t] += STEP
        pm[t] -= STEP
        _, vp, _ = lam(model, dim, ax, ec, pp[0], pp[1], pp[3], size, nev)
        _, vm, _ = lam(model, dim, ax, ec, pm[0], pm[1], pm[3], size, nev)
        fd = (np.log(vp[0]) - np.log(vm[0])) / (2 * STEP)
        assert abs(g[t] - fd) < 2e-6 * max(1.0, abs(fd)), (t, g[t], fd)


@pytest.mark.parametrize("pt", [p for p in POINTS if p[0] == "A"])
def test_field_derivative_equals_magnetisation(pt):
    model, dim, ax, ec, bj, k, h, size, nev = pt
    op, vals, vecs = lam(model, dim, ax, ec, bj, k, h, size, nev)
    g = op.grad(vecs[0], vals[0] * op.getnormfactor())
    q = vecs[0] / np.linalg.norm(vecs[0])
    m, _ = op.moments(q)
    L = op.getLayerSize()
    assert g[3] == pytest.approx(-bj * L * m[0], rel=1e-9, abs=1e-10)


# The two adjoint points of the gradient workload: A/5 reduced perpendicular
# TM at L=24 (betaJ=0.35, kappa=0.55, h=0.05; h != 0 keeps the flip reduction
# off) and the 3D ANNNI perpendicular TM on a 5x5 periodic layer (betaJ=0.2,
# kappa=0.4, h=0; R = 170,440).
CFG5 = [
    ("A", 2, 5, 0, 0.35, 0.55, 0.05, 24, 2),
    ("A", 3, 1, 0, 0.2, 0.4, 0.0, (5, 5), 2),
]


@pytest.mark.parametrize("pt", CFG5)
def test_grad_at_the_workload_points(pt):
    """Adjoint gradient of ln(lambda0) and of xi at the workload's two points
    against central finite differences (step 1e-5) of FP64 eigenvalues, and
    d ln(lambda0)/dh against the magnetisation moment."""
    model, dim, ax, ec, bj, k, h, size, nev = pt
    op, vals, vecs = lam(model, dim, ax, ec, bj, k, h, size, nev)
    nf = op.getnormfactor()
    g0 = op.grad(vecs[0], vals[0] * nf)
    g1 = op.grad(vecs[1], vals[1] * nf)
    xi = 1.0 / np.log(vals[0] / abs(vals[1]))
    dxi = -xi * xi * (g0 - g1)
    params = [bj, k, 0.0, h]
    for t in (0, 1, 3):
        if t == 3 and h == 0.0:
            continue  # the flip-reduced sector is only defined at h = 0
        pp, pm = list(params), list(params)
        pp[t] += STEP
        pm[t] -= STEP
        _, vp, _ = lam(model, dim, ax, ec, pp[0], pp[1], pp[3], size, nev)
        _, vm, _ = lam(model, dim, ax, ec, pm[0], pm[1], pm[3], size, nev)
        fd = (np.log(vp[0]) - np.log(vm[0])) / (2 * STEP)
        assert abs(g0[t] - fd) < 2e-6 * max(1.0, abs(fd)), (t, g0[t], fd)
        xp = 1.0 / np.log(vp[0] / abs(vp[1]))
        xm = 1.0 / np.log(vm[0] / abs(vm[1]))
        fdx = (xp - xm) / (2 * STEP)
        assert abs(dxi[t] - fdx) < 1e-5 * max(1.0, abs(fdx)), (t, dxi[t], fdx)
    if dim == 2 or h != 0.0:
        q = vecs[0] / np.linalg.norm(vecs[0])
        m, _ = op.moments(q)
        L = op.getLayerSize()
        assert g0[3] == pytest.approx(-bj * L * m[0], rel=1e-9, abs=1e-10)


def test_grad_xi_from_lambda1():
    """d xi from lambda1's eigenpair: xi = 1/ln(lambda0/|lambda1|)."""
    args = ("A", 2, 5, 2, 0.4, 0.6, 0.0, 14, 3)
    op, vals, vecs = lam(*args)
    nf = op.getnormfactor()
    g0 = op.grad(vecs[0], vals[0] * nf)
    g1 = op.grad(vecs[1], vals[1] * nf)
    xi = 1.0 / np.log(vals[0] / abs(vals[1]))
    dxi = -xi * xi * (g0[0] - g1[0])
    _, vp, _ = lam("A", 2, 5, 2, 0.4 + STEP, 0.6, 0.0, 14, 3)
    _, vm, _ = lam("A", 2, 5, 2, 0.4 - STEP, 0.6, 0.0, 14, 3)
    xp = 1.0 / np.log(vp[0] / abs(vp[1]))
    xm = 1.0 / np.log(vm[0] / abs(vm[1]))
    assert dxi == pytest.approx((xp - xm) / (2 * STEP), rel=1e-5)


@pytest.mark.parametrize("args", [("A", 2, 5, 0, 0.35, 0.55, 0.05, 16), ("A", 2, 1, 0, 0.5, 0.3, 0.1, 10)])
def test_cpp_eigen_function_forward_backward(tmp_path, args):
    """The C++ forward/backward pair of include/latttmat.hpp (EigenFunction),
    compiled here against the library, one forward and one backward on the GPU
    checked against central differences of its own forward pass."""
    import os
    import subprocess

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    pkg = os.path.join(root, "latttmat_gb300")
    exe = tmp_path / "eigen_function_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(root, "include"),
                    os.path.join(root, "tests", "cpp", "eigen_function_check.cpp"), "-o", str(exe), "-L", pkg,
                    "-llatttmat_gb300", "-Wl,-rpath," + pkg], check=True)
    r = subprocess.run([str(exe)] + [str(a) for a in args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "MISMATCH" not in r.stdout


# aux-bit operators: (model, axialdir, extend_cond, betaJ, kappa, kappa2, h, L)
AUX_POINTS = [
    ("B", 7, 2, 0.45, 0.6, 0.2, 0.0, 12),
    ("B", 7, 0, 0.5, 0.35, 0.1, 0.05, 10),
    ("B", 3, 0, 0.4, 0.7, 0.15, 0.1, 8),
    ("D", 5, 2, 0.5, 0.4, 0.0, 0.1, 10),
    ("D", 1, 0, 0.45, 0.6, 0.0, 0.05, 8),
]


def _lam_vecs(model, ax, ec, bj, k, k2, h, L):
    op = lt.TMatOp(model, 2, ax, bj, k, h, L, k2, ec)
    vals, vecs, vecl, _ = op.eigs(2, tol=1e-13, mode=lt.TM_EIGS_F64, vectors=True, left=True)
    return op, vals, vecs, vecl


@pytest.mark.parametrize("pt", AUX_POINTS)
def test_aux_grad_vs_finite_differences(pt):
    """Adjoint of the DNNI and diagonal BNNNI operators (Boltzmann-weight
    term plus the chain's tangent product) against central differences
    (step 1e-5) of FP64 eigenvalues, for every parameter."""
    model, ax, ec, bj, k, k2, h, L = pt
    op, vals, vecs, vecl = _lam_vecs(model, ax, ec, bj, k, k2, h, L)
    lam0 = float(np.real(vals[0]))
    qr = np.real(vecs[0])
    ql = None if op.is_symmetric() else np.asarray(vecl)
    g = op.grad(qr, lam0 * op.getnormfactor(), ql)
    params = [bj, k, k2, h]
    for t in range(4):
        if t == 3 and h == 0.0:
            continue  # the flip-reduced sector is only defined at h = 0
        if model == "D" and t == 2:
            assert g[2] == 0.0
            continue
        pp, pm = list(params), list(params)
        pp[t] += STEP
        pm[t] -= STEP
        vp = float(np.real(_lam_vecs(model, ax, ec, pp[0], pp[1], pp[2], pp[3], L)[1][0]))
        vm = float(np.real(_lam_vecs(model, ax, ec, pm[0], pm[1], pm[2], pm[3], L)[1][0]))
        fd = (np.log(vp) - np.log(vm)) / (2 * STEP)
        assert abs(g[t] - fd) < 2e-6 * max(1.0, abs(fd)), (t, g[t], fd)
