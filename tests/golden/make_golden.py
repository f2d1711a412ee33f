"""Generate the golden fixtures in tests/golden/*.npz from the reference itself.

Runs the reference's own operator sources (TMat/utility, tmat, tmatreduce,
tmat3d, tmatphys), compiled here by oracle/build_ref.sh into
oracle/_ref/libtmat_ref.so, on the seeded inputs of cases.py:
  * y = perform_op(x), and y = T^T x where the reference has a transpose;
  * orbit tables (idxlist, duplist) of reduced operators;
  * eigenvalues from ARPACK (scipy) driving the reference perform_op, tol 1e-13
    (Spectra, the reference's solver, is not vendored);
  * moments / phys_extend of the leading eigenvector through the reference's own
    functions.
Long outputs are stored as checksums (sum w*y with fixed weights, ||y||).

Usage: python tests/golden/make_golden.py   (needs oracle/_ref built)
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np
import scipy.sparse.linalg as sla

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from cases import CASES, FULL_VECTOR_MAX, case_dict, checksum_weights, general, seeded_input  # noqa: E402
from oracle.refbind import RefOp, available  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def gen(c):
    d = case_dict(c)
    op = RefOp(d["model"], d["dim"], d["axialdir"], d["betaJ"], d["kappa"], d["h"], d["size"], d["kappa2"],
               d["extend_cond"])
    n = op.n
    out = dict(n=np.int64(n), normfactor=np.float64(op.normfactor))
    x = seeded_input(n, 1)
    y = op.perform_op(x)
    w = checksum_weights(n)
    out["y_chk"] = np.array([np.dot(w, y), np.linalg.norm(y)])
    if n <= FULL_VECTOR_MAX:
        out["y"] = y
    if op.has_transpose():
        yt = op.perform_op_t(x)
        out["yt_chk"] = np.array([np.dot(w, yt), np.linalg.norm(yt)])
        if n <= FULL_VECTOR_MAX:
            out["yt"] = yt
    idx, dup = op.orbit()
    if idx is not None:
        out["orbit_n"] = np.int64(len(idx))
        out["idx_sha"] = np.array(sha(idx.astype(np.uint64)))
        out["dup_sha"] = np.array(sha(dup.astype(np.uint16)))
        out["dup_sum"] = np.int64(dup.astype(np.int64).sum())
        if n <= FULL_VECTOR_MAX:
            out["idx"] = idx.astype(np.uint64)
            out["dup"] = dup.astype(np.uint16)
    # eigenvalues through ARPACK on the reference matvec
    nev = d["nev"]
    lin = sla.LinearOperator((n, n), matvec=lambda v: op.perform_op(np.ravel(v)), dtype=np.float64)
    sym = not op.has_transpose() and not general(d)
    v0 = np.random.default_rng(0).uniform(0, 1, n)
    if sym:
        vals, vecs = sla.eigsh(lin, k=nev, which="LM", tol=1e-13, v0=v0, ncv=min(n - 1, max(2 * nev + 8, 20)))
    else:
        vals, vecs = sla.eigs(lin, k=nev, which="LM", tol=1e-13, v0=v0, ncv=min(n - 1, max(2 * nev + 8, 20)))
    order = np.argsort(-np.abs(vals), kind="stable")
    vals = vals[order]
    vecs = vecs[:, order]
    out["evals_re"] = np.real(vals) / op.normfactor
    out["evals_im"] = np.imag(vals) / op.normfactor
    q = np.real(vecs[:, 0])
    q = q / np.linalg.norm(q)
    if q.sum() < 0:
        q = -q
    if sym:
        ql = q
    else:
        lt = sla.LinearOperator((n, n), matvec=lambda v: op.perform_op_t(np.ravel(v)), dtype=np.float64)
        lv, lvec = sla.eigs(lt, k=1, which="LM", tol=1e-13, v0=v0, ncv=min(n - 1, 20))
        ql = np.real(lvec[:, 0])
        ql = ql / np.linalg.norm(ql)
        if ql.sum() < 0:
            ql = -ql
        out["left_eval"] = np.real(lv[0]) / op.normfactor
        if n <= FULL_VECTOR_MAX:
            out["ql"] = ql
    if n <= FULL_VECTOR_MAX:
        out["q0"] = q
    mom, mst = op.moments(ql, q)
    phys, pst = op.phys_extend(ql, q)
    out["moments"] = mom
    out["moments_status"] = np.int64(mst)
    out["phys"] = phys
    out["phys_status"] = np.int64(pst)
    return d["name"], out


def main(names=None):
    if not available():
        raise SystemExit("oracle/_ref/libtmat_ref.so missing: run oracle/build_ref.sh first")
    for c in CASES:
        if names and c[0] not in names:
            continue
        name, out = gen(c)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(f"{name}: n={int(out['n'])} evals={out['evals_re'][:2]}")


if __name__ == "__main__":
    main(sys.argv[1:] or None)
