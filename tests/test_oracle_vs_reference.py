"""CPU: oracle restatement vs the reference compiled from its own sources
(oracle/_ref), on randomised parameter points.  Runs only where the reference
library was built (the reference sources exist on the build machine only)."""
import numpy as np
import pytest

refbind = pytest.importorskip("oracle.refbind")
oracle = pytest.importorskip("oracle.oracle")

if not refbind.available():
    pytest.skip("oracle/_ref not built on this machine", allow_module_level=True)

OPS = [("A", 2, 1), ("A", 2, 5), ("A", 2, 9), ("A", 2, 13), ("A", 2, 17), ("A", 2, 18), ("A", 2, 19),
       ("A", 2, 20), ("D", 2, 1), ("D", 2, 5), ("D", 2, 17), ("D", 2, 18), ("B", 2, 3), ("B", 2, 7)]


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("model,dim,ax", OPS)
def test_random_points(model, dim, ax, seed):
    rng = np.random.default_rng(1000 + seed)
    L = int(rng.choice([6, 8, 9, 10, 11, 12]))
    if model == "B":
        L = int(rng.choice([6, 8, 10, 12]))
    bj = float(rng.uniform(0.05, 1.2))
    k = float(rng.choice([0.0, rng.uniform(0, 1.2), 0.5]))
    k2 = float(rng.uniform(0, 0.8)) if model == "B" else 0.0
    h = float(rng.choice([0.0, rng.uniform(-0.3, 0.3)]))
    ec = int(rng.choice([0, 2]))
    r = refbind.RefOp(model, dim, ax, bj, k, h, L, k2, ec)
    o = oracle.OracleOp(model, dim, ax, bj, k, h, L, k2, ec)
    assert r.n == o.n and r.normfactor == o.normfactor
    x = rng.uniform(-1, 1, r.n)
    yr, yo = r.perform_op(x), o.perform_op(x)
    np.testing.assert_allclose(yo, yr, rtol=1e-13, atol=1e-13 * np.max(np.abs(yr)))
    if r.has_transpose():
        np.testing.assert_allclose(o.perform_op_t(x), r.perform_op_t(x), rtol=1e-13,
                                   atol=1e-13 * np.max(np.abs(yr)))
    ir, dr = r.orbit()
    if ir is not None:
        io, do = o.orbit()
        np.testing.assert_array_equal(io, ir)
        np.testing.assert_array_equal(do, dr.astype(np.uint16))


@pytest.mark.parametrize("shape,k,h", [((3, 3), 0.3, 0.0), ((3, 4), 0.0, 0.0), ((4, 4), 0.0, 0.0),
                                       ((2, 5), 0.6, 0.1), ((4, 3), 0.2, 0.05)])
def test_3d_points(shape, k, h):
    r = refbind.RefOp("A", 3, 1, 0.25, k, h, shape)
    o = oracle.OracleOp("A", 3, 1, 0.25, k, h, shape)
    assert r.n == o.n
    x = np.random.default_rng(7).uniform(-1, 1, r.n)
    np.testing.assert_allclose(o.perform_op(x), r.perform_op(x), rtol=1e-13, atol=1e-13)
    ir, dr = r.orbit()
    io, do = o.orbit()
    np.testing.assert_array_equal(io, ir)
    np.testing.assert_array_equal(do, dr.astype(np.uint16))


TWO_LAYER = [("A", 2, 2), ("A", 2, 0), ("A", 2, 6), ("B", 2, 6)]


@pytest.mark.parametrize("seed", range(5))
@pytest.mark.parametrize("model,dim,ax", TWO_LAYER)
def test_two_layer_points(model, dim, ax, seed):
    rng = np.random.default_rng(2000 + seed)
    L = int(rng.choice([3, 4, 5, 6, 7]))
    if ax == 2 and L % 2:
        L += 1  # odd L: see test_yat_odd_width
    bj = float(rng.uniform(0.05, 1.0))
    k = float(rng.choice([0.0, rng.uniform(0, 1.2), 0.5]))
    k2 = float(rng.uniform(0, 0.8)) if model == "B" else 0.0
    h = float(rng.choice([0.0, rng.uniform(-0.3, 0.3)]))
    ec = int(rng.choice([0, 2]))
    r = refbind.RefOp(model, dim, ax, bj, k, h, L, k2, ec)
    o = oracle.OracleOp(model, dim, ax, bj, k, h, L, k2, ec)
    assert r.n == o.n
    np.testing.assert_allclose(o.normfactor, r.normfactor, rtol=1e-15)
    x = rng.uniform(-1, 1, r.n)
    yr = r.perform_op(x)
    np.testing.assert_allclose(o.perform_op(x), yr, rtol=1e-13, atol=1e-13 * np.max(np.abs(yr)))
    if r.has_transpose():
        np.testing.assert_allclose(o.perform_op_t(x), r.perform_op_t(x), rtol=1e-13,
                                   atol=1e-13 * np.max(np.abs(yr)))
    ir, dr = r.orbit()
    if ir is not None:
        io, do = o.orbit()
        np.testing.assert_array_equal(io, ir)
        np.testing.assert_array_equal(do, dr.astype(np.uint16))


@pytest.mark.parametrize("L", [3, 5])
def test_yat_odd_width(L):
    """At odd L the reference YATMatVecProd2D ends its L ping-pong steps on the
    output buffer and then permutes that buffer in place (TMat/tmat.cpp:213-240),
    so its output is not T x.  The oracle computes T x; its spectrum equals the
    reference's own reduced operator YAMMatVecProd2D at the same point, and the
    two agree with the reference full operator at even L."""
    bj, k, h = 0.4, 0.3, 0.1

    def top(op, n):
        A = np.array([op.perform_op(np.eye(n)[i]) for i in range(n)]).T
        ev = np.linalg.eigvals(A) / op.normfactor
        return ev[np.argsort(-np.abs(ev))][:3]

    o = oracle.OracleOp("A", 2, 2, bj, k, h, L, 0.0, 0)
    ry = refbind.RefOp("A", 2, 6, bj, k, h, L, 0.0, 2)
    np.testing.assert_allclose(top(o, o.n), top(ry, ry.n), rtol=1e-11)
