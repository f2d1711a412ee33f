"""GPU parity: operators through the C ABI against the reference's own outputs.

Bars: orbit tables bit-exact; FP64 matvec (native or double-float) within
1e-12 of the reference (relative to max|y|); FP32 device matvec within 2e-5; eigenvalues within
1e-10 relative of the reference (ARPACK on the reference perform_op).
"""
import numpy as np
import pytest

import latttmat_gb300 as lt
from gpu_util import case_names, checksum_weights, fixture, make_op, rel_err, seeded_input

pytestmark = pytest.mark.gpu

IMPLEMENTED = ["xat", "xam", "x3d", "xdt", "xdm", "zbt", "zbm", "yat", "y2at", "yam", "ybm"]
SYM = ["xat", "xam", "x3d", "xdt", "xdm"]


def _skip_if_unavailable(fn):
    try:
        return fn()
    except lt.TMError as e:
        if e.code == lt.TM_ERR_UNSUPPORTED:
            pytest.skip(str(e))
        raise


@pytest.mark.parametrize("name", case_names(IMPLEMENTED))
def test_matvec_fp64(name):
    f = fixture(name)
    op = _skip_if_unavailable(lambda: make_op(name))
    n = op.rows()
    assert n == int(f["n"])
    assert op.getnormfactor() == pytest.approx(float(f["normfactor"]), rel=1e-14)
    x = seeded_input(n, 1)
    y = op.perform_op(x)
    w = checksum_weights(n)
    if "y" in f:
        assert rel_err(y, f["y"]) < 1e-12
    chk = np.array([np.dot(w, y), np.linalg.norm(y)])
    np.testing.assert_allclose(chk, f["y_chk"], rtol=1e-12)


@pytest.mark.parametrize("name", case_names(["xam", "x3d", "xdm", "zbm", "yam", "ybm"]))
def test_orbit_table_bit_exact(name):
    f = fixture(name)
    op = _skip_if_unavailable(lambda: make_op(name))
    idx, dup = op.orbit_table()
    import hashlib

    assert len(idx) == int(f["orbit_n"])
    assert hashlib.sha256(idx.astype(np.uint64).tobytes()).hexdigest() == str(f["idx_sha"])
    assert hashlib.sha256(dup.astype(np.uint16).tobytes()).hexdigest() == str(f["dup_sha"])
    if "idx" in f:
        np.testing.assert_array_equal(idx, f["idx"])
        np.testing.assert_array_equal(dup, f["dup"])


@pytest.mark.parametrize("name", case_names(["xat", "xam", "x3d", "xdt", "xdm"]))
def test_matvec_fp32_device(name):
    torch = pytest.importorskip("torch")
    f = fixture(name)
    op = _skip_if_unavailable(lambda: make_op(name))
    n = op.rows()
    x = seeded_input(n, 1)
    xd = torch.tensor(x, dtype=torch.float32, device="cuda")
    yd = torch.empty_like(xd)
    op.perform_op_dev(xd.data_ptr(), yd.data_ptr(), lt.TM_F32, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    y = yd.double().cpu().numpy()
    ref = f["y"] if "y" in f else op.perform_op(x)
    assert rel_err(y, ref) < 2e-5
    xd64 = torch.tensor(x, dtype=torch.float64, device="cuda")
    yd64 = torch.empty_like(xd64)
    op.perform_op_dev(xd64.data_ptr(), yd64.data_ptr(), lt.TM_F64, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rel_err(yd64.cpu().numpy(), ref) < 1e-12


@pytest.mark.parametrize("name", case_names(["xat", "xam", "x3d", "xdt", "xdm", "zbt", "zbm"]))
def test_matvec_double_float_device(name):
    """TM_F64_DF device product (double-float engines for the even/odd and
    aux-bit operators, native FP64 for the rest) within the FP64 bar, for
    the operator and, where it has one, its transpose."""
    torch = pytest.importorskip("torch")
    f = fixture(name)
    op = _skip_if_unavailable(lambda: make_op(name))
    n = op.rows()
    x = seeded_input(n, 1)

    def dev_df(o):
        xd = torch.tensor(x, dtype=torch.float64, device="cuda")
        yd = torch.empty_like(xd)
        o.perform_op_dev(xd.data_ptr(), yd.data_ptr(), lt.TM_F64_DF, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        return yd.cpu().numpy()

    y = dev_df(op)
    if "y" in f:
        assert rel_err(y, f["y"]) < 1e-12
    w = checksum_weights(n)
    np.testing.assert_allclose([np.dot(w, y), np.linalg.norm(y)], f["y_chk"], rtol=1e-12)
    try:
        t = op.get_t_instance()
    except lt.TMError as e:
        if e.code == lt.TM_ERR_NOTRANSPOSE:
            return
        raise
    assert rel_err(dev_df(t), t.perform_op(x)) < 1e-12


@pytest.mark.parametrize("name", case_names(["yat", "y2at", "yam", "ybm"]))
def test_two_layer_fp64_only(name):
    """The two-layer operators run in FP64 only: an FP32 device product is
    refused with TM_ERR_UNSUPPORTED, the FP64 one matches the reference."""
    torch = pytest.importorskip("torch")
    f = fixture(name)
    op = make_op(name)
    x = seeded_input(op.rows(), 1)
    x32 = torch.tensor(x, dtype=torch.float32, device="cuda")
    y32 = torch.empty_like(x32)
    with pytest.raises(lt.TMError) as e:
        op.perform_op_dev(x32.data_ptr(), y32.data_ptr(), lt.TM_F32)
    assert e.value.code == lt.TM_ERR_UNSUPPORTED
    x64 = torch.tensor(x, dtype=torch.float64, device="cuda")
    y64 = torch.empty_like(x64)
    op.perform_op_dev(x64.data_ptr(), y64.data_ptr(), lt.TM_F64)
    torch.cuda.synchronize()
    assert rel_err(y64.cpu().numpy(), f["y"]) < 1e-12


@pytest.mark.parametrize("L", [5, 7])
def test_yat_odd_width_against_oracle(L):
    """Odd widths: the reference's YATMatVecProd2D output is not T x there (its
    final permutation reads its own output buffer); the oracle computes T x,
    and its spectrum matches the reference's reduced YAMMatVecProd2D."""
    oracle = pytest.importorskip("oracle.oracle")
    op = lt.TMatOp("A", 2, 2, 0.4, 0.3, 0.1, L)
    ref = oracle.OracleOp("A", 2, 2, 0.4, 0.3, 0.1, L)
    x = seeded_input(op.rows(), 3)
    assert rel_err(op.perform_op(x), ref.perform_op(x)) < 1e-12
    assert rel_err(op.get_t_instance().perform_op(x), ref.perform_op_t(x)) < 1e-12


@pytest.mark.parametrize("mode", [lt.TM_EIGS_F64, lt.TM_EIGS_MIXED])
@pytest.mark.parametrize("name", case_names(SYM))
def test_eigenvalues(name, mode):
    f = fixture(name)
    op = _skip_if_unavailable(lambda: make_op(name))
    nev = len(f["evals_re"])
    if op.rows() <= nev + 2:
        pytest.skip("operator too small for the Krylov solver")
    vals, vecs, _, info = op.eigs(nev, tol=1e-12, mode=mode, vectors=True)
    ref = f["evals_re"]
    np.testing.assert_allclose(vals, ref, rtol=1e-10, atol=0)
    # leading eigenvector (up to sign) against the reference's
    if "q0" in f:
        q = vecs[0] / np.linalg.norm(vecs[0])
        q = q * np.sign(q.sum())
        assert rel_err(q, f["q0"]) < 1e-6
    assert info["nconv"] == nev


@pytest.mark.parametrize("name", case_names(SYM))
def test_moments_phys(name):
    f = fixture(name)
    op = _skip_if_unavailable(lambda: make_op(name))
    if "q0" not in f:
        pytest.skip("no stored eigenvector")
    m, st = op.moments(f["q0"])
    np.testing.assert_allclose(m, f["moments"], rtol=1e-12, atol=1e-12)
    assert st == int(f["moments_status"])
    p, pst = op.phys_extend(f["q0"])
    if len(f["phys"]):
        np.testing.assert_allclose(p, f["phys"], rtol=1e-12, atol=1e-12)
    assert pst == int(f["phys_status"])


@pytest.mark.parametrize("L,ec", [(16, 2), (20, 0), (24, 2)])
def test_double_float_refinement_product(L, ec):
    """The solver's refinement product (double-float on FP32 pipes) against the
    native FP64 product: relative error below 1e-12 of max|y|."""
    torch = pytest.importorskip("torch")
    op = lt.TMatOp("A", 2, 5, 0.45, 0.35, 0.0, L, 0.0, ec)
    n = op.rows()
    ms64 = op.profile_matvec(lt.TM_F64, iters=1)  # exercises the FP64 path
    assert len(ms64) >= 1
    vals64, _, _, info64 = op.eigs(3, tol=1e-12, mode=lt.TM_EIGS_F64)
    valsm, _, _, infom = op.eigs(3, tol=1e-12, mode=lt.TM_EIGS_MIXED)
    np.testing.assert_allclose(valsm, vals64, rtol=1e-10)
    assert infom["matvecs_f64"] < info64["matvecs_f64"]


@pytest.mark.parametrize("mode", [lt.TM_EIGS_F64, lt.TM_EIGS_MIXED])
@pytest.mark.parametrize("L,ec", [(20, 2), (16, 0), (18, 2)])
def test_eigenvectors_into_pinned_host_memory(mode, L, ec):
    """Eigenvectors written into pinned (device-mapped) host memory come
    straight from a gather kernel (16-byte stores for even row lengths); they
    equal those copied into pageable memory bit for bit."""
    torch = pytest.importorskip("torch")
    op = lt.TMatOp("A", 2, 5, 0.3, 0.5, 0.0, L, 0.0, ec)
    nev = 3
    vals_a, vecs_a, _, _ = op.eigs(nev, tol=1e-12, mode=mode, vectors=True)
    pinned = torch.empty((nev, op.rows()), dtype=torch.float64, pin_memory=True).numpy()
    pinned[:] = np.nan
    vals_b, vecs_b, _, _ = op.eigs(nev, tol=1e-12, mode=mode, vectors=True, vecs_out=pinned)
    np.testing.assert_array_equal(vals_a, vals_b)
    np.testing.assert_array_equal(vecs_a, vecs_b)
    # eigenvector check in the reference's order against the oracle
    oracle = pytest.importorskip("oracle.oracle")
    ref = oracle.OracleOp("A", 2, 5, 0.3, 0.5, 0.0, L, 0.0, ec)
    for c in range(nev):
        y = ref.perform_op(vecs_b[c]) / op.getnormfactor()
        assert rel_err(y, vals_b[c] * vecs_b[c]) < 1e-9


@pytest.mark.parametrize("L,bits,bj", [(20, 9, 0.3), (20, 8, -0.4), (24, 11, 0.45), (24, 10, -0.3)])
def test_even_odd_cluster_split(L, bits, bj):
    """Tiles split over 2- and 4-CTA clusters (the layout L >= 30 uses),
    forced at small L by capping the tile bits: the FP32 and double-float
    passes combine through the L2 exchange slots, native FP64 through DSMEM.
    All products against the oracle, and the mixed solve against FP64."""
    torch = pytest.importorskip("torch")
    oracle = pytest.importorskip("oracle.oracle")
    lt.debug_set_eo_tile_bits(bits)
    try:
        op = lt.TMatOp("A", 2, 5, bj, 0.5, 0.0, L, 0.0, 2)
    finally:
        lt.debug_set_eo_tile_bits(0)
    ref = oracle.OracleOp("A", 2, 5, bj, 0.5, 0.0, L, 0.0, 2)
    x = seeded_input(op.rows(), 7)
    yr = ref.perform_op(x)
    assert rel_err(op.perform_op(x), yr) < 1e-12
    stream = torch.cuda.current_stream().cuda_stream
    for dt, tdt, bar in ((lt.TM_F32, torch.float32, 2e-5), (lt.TM_F64_DF, torch.float64, 1e-12),
                         (lt.TM_F64, torch.float64, 1e-12)):
        xd = torch.tensor(x, dtype=tdt, device="cuda")
        yd = torch.empty_like(xd)
        op.perform_op_dev(xd.data_ptr(), yd.data_ptr(), dt, stream)
        torch.cuda.synchronize()
        assert rel_err(yd.double().cpu().numpy(), yr) < bar, dt
    vals64, _, _, _ = op.eigs(3, tol=1e-12, mode=lt.TM_EIGS_F64)
    valsm, _, _, infom = op.eigs(3, tol=1e-12, mode=lt.TM_EIGS_MIXED)
    np.testing.assert_allclose(valsm, vals64, rtol=1e-10)
    assert infom["nconv"] == 3


@pytest.mark.parametrize("L,ec,bj", [(12, 2, -0.4), (14, 0, -0.35), (16, 2, -0.6), (20, 2, -0.3)])
def test_even_odd_negative_coupling(L, ec, bj):
    """betaJ < 0 swaps the roles of the butterfly coefficients in the even/odd
    engines (x0' = x1 + r x0): the FP64 and FP32 products against the oracle,
    and the mixed solve (FP32 and double-float engines) against the FP64 one."""
    torch = pytest.importorskip("torch")
    oracle = pytest.importorskip("oracle.oracle")
    op = lt.TMatOp("A", 2, 5, bj, 0.5, 0.0, L, 0.0, ec)
    ref = oracle.OracleOp("A", 2, 5, bj, 0.5, 0.0, L, 0.0, ec)
    x = seeded_input(op.rows(), 5)
    yr = ref.perform_op(x)
    assert rel_err(op.perform_op(x), yr) < 1e-12
    xd = torch.tensor(x, dtype=torch.float32, device="cuda")
    yd = torch.empty_like(xd)
    op.perform_op_dev(xd.data_ptr(), yd.data_ptr(), lt.TM_F32, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rel_err(yd.double().cpu().numpy(), yr) < 2e-5
    xd64 = torch.tensor(x, dtype=torch.float64, device="cuda")
    yd64 = torch.empty_like(xd64)
    op.perform_op_dev(xd64.data_ptr(), yd64.data_ptr(), lt.TM_F64_DF, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rel_err(yd64.cpu().numpy(), yr) < 1e-12
    nev = 3
    vals64, _, _, _ = op.eigs(nev, tol=1e-12, mode=lt.TM_EIGS_F64)
    valsm, _, _, infom = op.eigs(nev, tol=1e-12, mode=lt.TM_EIGS_MIXED)
    np.testing.assert_allclose(valsm, vals64, rtol=1e-10)
    assert infom["nconv"] == nev
