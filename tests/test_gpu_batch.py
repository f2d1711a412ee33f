"""GPU: the parameter sweep entry point (tm_eigs_batch) on instances of the
256-point B/7 sweep (reduced diagonal BNNNI, widths 16..24 mixed in one call)
against the reference's eigenvalues (ARPACK on the reference product, tol
1e-13) and against one tm_eigs solve per point.  Bars: 1e-10 relative, both
precision modes."""
import numpy as np
import pytest

import latttmat_gb300 as lt
from cases import CASES, case_dict
from gpu_util import checksum_weights, fixture, rel_err, seeded_input

pytestmark = pytest.mark.gpu

SWEEP = [case_dict(c) for c in CASES if c[0].startswith("zbm_sw")]


def _points():
    return [(d["betaJ"], d["kappa"], d["kappa2"], d["h"], d["size"]) for d in SWEEP]


def _match(vals, ref, rtol):
    """Multisets up to complex conjugation (the operators are real)."""
    both = np.concatenate([vals, np.conj(vals)])
    for z in ref:
        assert np.min(np.abs(both - z)) / abs(z) < rtol, (z, vals)


@pytest.mark.parametrize("mode", [lt.TM_EIGS_F64, lt.TM_EIGS_MIXED])
def test_batch_against_reference(mode):
    vals, info, st = lt.eigs_batch("B", 2, 7, _points(), nev=2, tol=1e-12, mode=mode, extend_cond=2)
    assert list(st) == [lt.TM_OK] * len(SWEEP)
    for i, d in enumerate(SWEEP):
        f = fixture(d["name"])
        _match(vals[i], f["evals_re"] + 1j * f["evals_im"], 1e-10)
        assert info[i]["nconv"] == 2


def test_batch_against_single_solves():
    pts = _points()
    vals, _, st = lt.eigs_batch("B", 2, 7, pts, nev=2, tol=1e-12, mode=lt.TM_EIGS_MIXED, extend_cond=2)
    assert list(st) == [lt.TM_OK] * len(pts)
    for i, (bj, k, k2, h, L) in enumerate(pts):
        op = lt.TMatOp("B", 2, 7, bj, k, h, L, k2, 2)
        v1, _, _, _ = op.eigs(2, tol=1e-12, mode=lt.TM_EIGS_F64)
        _match(vals[i], v1, 1e-10)
        op.close()


# ---------------------------------------------------------------- device sweep
def _dev_product(torch, op_or_none, x, dt):
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    op_or_none.perform_op_dev(xd.data_ptr(), yd.data_ptr(), dt)
    torch.cuda.synchronize()
    return yd.cpu().numpy()


MIXED_B7 = [(0.45, 0.3, 0.0, 0.0, 12), (0.3, 0.8, 0.1, 0.0, 16), (0.6, 0.45, 0.0, 0.0, 14),
            (0.2, 0.5118216247002567, 0.0, 0.0, 24), (0.8, 0.2, 0.0, 0.0, 18), (0.5, 0.6, 0.2, 0.0, 20)]


@pytest.mark.parametrize("model,ax,ec,points", [
    ("B", 7, 2, MIXED_B7),
    ("B", 3, 0, [(0.5, 0.6, 0.2, 0.1, 8), (0.4, 0.3, 0.0, 0.0, 12), (0.6, 0.5, 0.1, 0.0, 10)]),
    ("D", 5, 2, [(0.4, 0.3, 0.0, 0.1, 13), (0.5, 0.7, 0.0, 0.0, 16), (0.4, 0.3, 0.0, 0.0, 10)]),
    ("D", 1, 0, [(0.4, 0.3, 0.0, 0.1, 8), (0.6, 0.7, 0.0, 0.0, 10), (0.4, 0.3, 0.0, 0.1, 13)]),
])
@pytest.mark.parametrize("waves", ["one", "each"])
def test_sweep_product_matches_single_operators(model, ax, ec, points, waves):
    """One batched product over members of several widths (one launch per
    chain pass over all members) equals each member's own product: FP64 and
    double-float within 1e-12, FP32 within 2e-5 of the single FP64 product;
    with every member in one wave, and with one member per wave."""
    torch = pytest.importorskip("torch")
    sw = lt.Sweep(model, 2, ax, points, extend_cond=ec)
    if waves == "each":
        sw.set_wave_bytes(1)
    xs, refs, ops = [], [], []
    for i, (bj, k, k2, h, L) in enumerate(points):
        op = lt.TMatOp(model, 2, ax, bj, k, h, L, k2, ec)
        assert op.rows() == sw.rows(i)
        assert op.getnormfactor() == sw.normfactor(i)
        x = seeded_input(op.rows(), 11 + i)
        xs.append(torch.from_numpy(x).cuda())
        refs.append(_dev_product(torch, op, x, lt.TM_F64))
        ops.append(op)
    for dt, bar in ((lt.TM_F64, 1e-12), (lt.TM_F64_DF, 1e-12), (lt.TM_F32, 2e-5)):
        ys = [torch.full_like(x, float("nan")) for x in xs]
        sw.perform_op_dev([x.data_ptr() for x in xs], [y.data_ptr() for y in ys], dt)
        torch.cuda.synchronize()
        for y, ref in zip(ys, refs):
            assert rel_err(y.cpu().numpy(), ref) < bar, (dt, rel_err(y.cpu().numpy(), ref))
    sw.close()


def test_sweep_fixture_products():
    """Batched FP64 products of the sweep instances against the reference's
    own products (weighted checksums and stored values)."""
    torch = pytest.importorskip("torch")
    pts = _points()
    sw = lt.Sweep("B", 2, 7, pts, extend_cond=2)
    xs = [torch.from_numpy(seeded_input(sw.rows(i), 1)).cuda() for i in range(len(pts))]
    ys = [torch.empty_like(x) for x in xs]
    sw.perform_op_dev([x.data_ptr() for x in xs], [y.data_ptr() for y in ys], lt.TM_F64)
    torch.cuda.synchronize()
    for i, d in enumerate(SWEEP):
        f = fixture(d["name"])
        y = ys[i].cpu().numpy()
        w = checksum_weights(len(y))
        np.testing.assert_allclose([np.dot(w, y), np.linalg.norm(y)], f["y_chk"], rtol=1e-12)
        if "y" in f:
            assert rel_err(y, f["y"]) < 1e-12
        else:
            assert rel_err(y[f["samp_idx"]], f["y_samp"]) < 1e-12
    sw.close()


@pytest.mark.parametrize("mode", [lt.TM_EIGS_F64, lt.TM_EIGS_MIXED])
def test_sweep_waves_do_not_change_results(mode):
    """Members are independent: solving them in one wave or one per wave
    gives the same eigenvalues bit for bit."""
    a = lt.Sweep("B", 2, 7, MIXED_B7, extend_cond=2)
    va, ia, sa = a.eigs(2, tol=1e-12, mode=mode)
    b = lt.Sweep("B", 2, 7, MIXED_B7, extend_cond=2)
    b.set_wave_bytes(1)
    vb, ib, sb = b.eigs(2, tol=1e-12, mode=mode)
    assert list(sa) == list(sb) == [lt.TM_OK] * len(MIXED_B7)
    np.testing.assert_array_equal(va, vb)
    assert [x["matvecs"] for x in ia] == [x["matvecs"] for x in ib]
    for i, (bj, k, k2, h, L) in enumerate(MIXED_B7):
        op = lt.TMatOp("B", 2, 7, bj, k, h, L, k2, 2)
        v1, _, _, _ = op.eigs(2, tol=1e-12, mode=lt.TM_EIGS_F64)
        _match(va[i], v1, 1e-10)
    a.close()
    b.close()


def test_sweep_dnni_eigenvalues():
    """A reduced DNNI sweep (model D axialdir 5) against single solves."""
    pts = [(0.4, 0.3, 0.0, 0.1, 13), (0.5, 0.7, 0.0, 0.0, 16), (0.4, 0.3, 0.0, 0.0, 10), (0.7, 0.2, 0.0, 0.0, 14)]
    sw = lt.Sweep("D", 2, 5, pts, extend_cond=2)
    vals, info, st = sw.eigs(2, tol=1e-12, mode=lt.TM_EIGS_MIXED)
    assert list(st) == [lt.TM_OK] * len(pts)
    for i, (bj, k, k2, h, L) in enumerate(pts):
        op = lt.TMatOp("D", 2, 5, bj, k, h, L, k2, 2)
        v1, _, _, _ = op.eigs(2, tol=1e-12, mode=lt.TM_EIGS_F64)
        _match(vals[i], v1, 1e-10)


@pytest.mark.parametrize("model,ax,L", [("B", 7, 16), ("D", 1, 12)])
def test_chain_autotune_choices_give_the_same_product(model, ax, L):
    """The autotuner returns a valid tile / block size, and the product is the
    same (to rounding) under every tuning it can choose."""
    torch = pytest.importorskip("torch")
    oracle = pytest.importorskip("oracle.oracle")
    op = lt.TMatOp(model, 2, ax, 0.45, 0.35, 0.0, L, 0.1, 2)
    ref = oracle.OracleOp(model, 2, ax, 0.45, 0.35, 0.0, L, 0.1, 2)
    x = seeded_input(op.rows(), 3)
    yr = ref.perform_op(x)
    try:
        for dt in (lt.TM_F32, lt.TM_F64_DF):
            tb, th, ms = lt.chain_autotune(op, dt)
            assert 11 <= tb <= 14 and th in (128, 256) and ms > 0
            for tb2 in ((11, 12, 13, 14) if dt == lt.TM_F32 else (11, 12, 13)):
                for th2 in (128, 256):
                    lt.chain_set_tuning(model, L, dt, tb2, th2)
                    xd = torch.tensor(x, dtype=torch.float32 if dt == lt.TM_F32 else torch.float64, device="cuda")
                    yd = torch.empty_like(xd)
                    op.perform_op_dev(xd.data_ptr(), yd.data_ptr(), dt)
                    torch.cuda.synchronize()
                    bar = 2e-5 if dt == lt.TM_F32 else 1e-12
                    assert rel_err(yd.double().cpu().numpy(), yr) < bar, (dt, tb2, th2)
    finally:
        for dt in (lt.TM_F32, lt.TM_F64_DF):
            lt.chain_set_tuning(model, L, dt, 0, 0)


@pytest.mark.parametrize("model,ax,ec,points", [
    ("B", 7, 2, MIXED_B7[:4] + [(0.55, 0.35, 0.1, 0.0, 14)]),
    ("B", 7, 0, [(0.5, 0.35, 0.1, 0.05, 10), (0.4, 0.6, 0.2, 0.02, 12)]),
    ("D", 5, 2, [(0.4, 0.3, 0.0, 0.1, 13), (0.5, 0.7, 0.0, 0.0, 16), (0.45, 0.5, 0.0, 0.05, 12)]),
])
def test_sweep_adjoint_matches_single_operators(model, ax, ec, points):
    """Batched adjoint: leading right eigenvectors from the sweep, left ones
    from the sweep of the transposes, gradients from one batched reduction
    and batched tangent products -- against tm_grad on each operator with its
    own tm_eigs eigenvectors (1e-8 relative to max(|grad|, 1))."""
    right = lt.Sweep(model, 2, ax, points, extend_cond=ec)
    vals, _, st, vr = right.eigs(2, tol=1e-12, mode=lt.TM_EIGS_MIXED, vectors=True)
    assert list(st) == [lt.TM_OK] * len(points)
    sym = model == "D"
    vl = None
    if not sym:
        left = lt.Sweep(model, 2, ax, points, extend_cond=ec)
        left.set_transpose(True)
        vals_l, _, st_l, vl = left.eigs(2, tol=1e-12, mode=lt.TM_EIGS_MIXED, vectors=True)
        assert list(st_l) == [lt.TM_OK] * len(points)
        np.testing.assert_allclose(np.abs(vals_l[:, 0]), np.abs(vals[:, 0]), rtol=1e-10)
        left.close()
    lam = np.array([np.real(vals[i, 0]) * right.normfactor(i) for i in range(len(points))])
    g = right.grad(vr, vl, lam)
    for i, (bj, k, k2, h, L) in enumerate(points):
        op = lt.TMatOp(model, 2, ax, bj, k, h, L, k2, ec)
        v1, vecs, vecl, _ = op.eigs(2, tol=1e-13, mode=lt.TM_EIGS_F64, vectors=True, left=not sym)
        qr = np.real(vecs[0])
        g1 = op.grad(qr, float(np.real(v1[0])) * op.getnormfactor(), None if sym else np.asarray(vecl))
        assert np.max(np.abs(g[i] - g1)) < 1e-8 * max(1.0, np.max(np.abs(g1))), (i, g[i], g1)
        # the sweep's eigenvector is the operator's (up to sign)
        q = vr[i] * np.sign(vr[i].sum())
        qq = qr / np.linalg.norm(qr)
        qq = qq * np.sign(qq.sum())
        assert rel_err(q, qq) < 1e-7
        op.close()
    right.close()
