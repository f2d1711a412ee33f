"""GPU: the Krylov sweeps staged through shared memory by bulk copies
(update-and-dot over 9-16 basis columns, the refinement's block dots) at the
edges of their chunking: bases shorter than one 1024-element chunk, a
partial last chunk, and lengths with 1, 2 or 3 elements past the last full
float4.  The mixed-precision solve runs those sweeps on every step from the
ninth basis column on; its eigenvalues must equal the plain FP64 solve's
(which uses none of them) to the solver tolerance, and its eigenvectors must
be unit eigenvectors of the oracle's operator."""
import numpy as np
import pytest

import latttmat_gb300 as lt

oracle = pytest.importorskip("oracle.oracle")

# reduced x-ANNNI, betaJ 0.4, kappa 0.5, flip off: rows 13 (n % 4 = 1, below
# one chunk), 18 (2), 687 (3), 1224 (one full chunk and a partial one), 2250,
# 7685 (1, several chunks)
WIDTHS = [6, 7, 14, 15, 16, 18]


def test_widths_cover_the_chunk_edges():
    ns = [oracle.OracleOp("A", 2, 5, 0.4, 0.5, 0.0, L, 0.0, 2).n for L in WIDTHS]
    assert {n % 4 for n in ns} >= {1, 2, 3}
    assert min(ns) < 1024 < max(ns)
    assert any(n % 1024 and n > 1024 for n in ns)


@pytest.mark.gpu
@pytest.mark.parametrize("L", WIDTHS)
def test_mixed_solve_through_staged_sweeps(L):
    nev = 4
    op = lt.TMatOp("A", 2, 5, 0.4, 0.5, 0.0, L, 0.0, 2)
    n = op.rows()
    ref = oracle.OracleOp("A", 2, 5, 0.4, 0.5, 0.0, L, 0.0, 2)
    assert n == ref.n
    vm, vecs, _, info = op.eigs(nev, tol=1e-10, mode=lt.TM_EIGS_MIXED, vectors=True)
    vf, _, _, _ = op.eigs(nev, tol=1e-10, mode=lt.TM_EIGS_F64)
    np.testing.assert_allclose(np.real(vm), np.real(vf), rtol=1e-10)
    vecs = np.asarray(vecs).reshape(nev, n)
    lam0 = None
    for c in range(nev):
        q = vecs[c]
        assert abs(np.linalg.norm(q) - 1.0) < 1e-9
        tq = ref.perform_op(q)
        lam = float(q @ tq)
        lam0 = lam0 or abs(lam)
        assert np.linalg.norm(tq - lam * q) <= 1e-8 * lam0
