"""GPU: general (non-symmetric) operators -- diagonal BNNNI full (ZBT) and
reduced (ZBM), the two-layer y-ANNNI / y2-ANNNI / BNNNI operators (YAT, Y2AT,
YAM, YBM) -- transpose products, complex-capable eigenvalues and the left
eigenvector from the transpose solve, against the reference's own outputs."""
import numpy as np
import pytest

import latttmat_gb300 as lt
from gpu_util import case_names, checksum_weights, fixture, make_op, rel_err, seeded_input

pytestmark = pytest.mark.gpu


def assert_eigs_match(vals, ref, rtol):
    """Match as multisets up to complex conjugation: the operators are real, so
    z and conj(z) are both eigenvalues; which member of a conjugate pair (equal
    modulus) is reported is a convention, not part of the result."""
    both = np.concatenate([vals, np.conj(vals)])
    for z in ref:
        err = np.min(np.abs(both - z)) / abs(z)
        assert err < rtol, (z, vals)


@pytest.mark.parametrize("name", case_names(["zbt", "zbm", "yat", "yam", "ybm"]))
def test_transpose_product(name):
    f = fixture(name)
    op = make_op(name)
    t = op.get_t_instance()
    x = seeded_input(op.rows(), 1)
    yt = t.perform_op(x)
    if "yt" in f:
        assert rel_err(yt, f["yt"]) < 1e-12
    else:
        assert rel_err(yt[f["samp_idx"]], f["yt_samp"]) < 1e-12
        w = checksum_weights(op.rows())
        np.testing.assert_allclose([np.dot(w, yt), np.linalg.norm(yt)], f["yt_chk"], rtol=1e-12)
    # <y, T x> == <T^T y, x>
    z = seeded_input(op.rows(), 2)
    assert np.dot(z, op.perform_op(x)) == pytest.approx(np.dot(t.perform_op(z), x), rel=1e-11)


@pytest.mark.parametrize("mode", [lt.TM_EIGS_F64, lt.TM_EIGS_MIXED])
@pytest.mark.parametrize("name", case_names(["zbt", "zbm", "yat", "y2at", "yam", "ybm"]))
def test_general_eigenvalues_and_left_vector(name, mode):
    f = fixture(name)
    op = make_op(name)
    nev = len(f["evals_re"])
    vals, vecs, vecl, info = op.eigs(nev, tol=1e-12, mode=mode, vectors=True, left=True)
    ref = f["evals_re"] + 1j * f["evals_im"]
    assert_eigs_match(vals, ref, 1e-10)
    q = np.real(vecs[0])
    q = q / np.linalg.norm(q) * np.sign(q.sum())
    ql = vecl / np.linalg.norm(vecl) * np.sign(vecl.sum())
    if "q0" in f:
        assert rel_err(q, f["q0"]) < 1e-6
        assert rel_err(ql, f["ql"]) < 1e-6
    else:  # long vectors: the values at the sampled positions
        assert rel_err(q[f["samp_idx"]], f["q0_samp"]) < 1e-6
        assert rel_err(ql[f["samp_idx"]], f["ql_samp"]) < 1e-6
    m, st = op.moments(ql, q)
    np.testing.assert_allclose(m, f["moments"], rtol=1e-6, atol=1e-9)
    assert st == int(f["moments_status"])


def test_y2at_transpose_is_the_operator():
    """Y2ATMatVecProd2D's get_t_instance returns the operator itself
    (TMat/tmat.hpp:382-384); the transposed view here does the same."""
    op = make_op("y2at_L5_h")
    x = seeded_input(op.rows(), 4)
    assert rel_err(op.get_t_instance().perform_op(x), op.perform_op(x)) == 0.0
