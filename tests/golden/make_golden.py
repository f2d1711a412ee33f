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
Long outputs are stored as checksums (sum w*y with fixed weights, ||y||) and
as values at seeded sample positions (cases.sample_indices).

The LARGE_CASES of cases.py (x-ANNNI reduced at L = 26..32) run only when named
or with --large; their eigenvalues use the reference solver's Krylov size
(ncv = 2*nev+3, TMat/tmat.hpp:88) at tol 1e-12, and the number of reference
products each ARPACK solve took is stored beside them.  At L = 32 a product
takes about two minutes on 8 cores and the eigenvalues about an hour and a half.

The DUMP_CASES (configuration planting) run when named or with --dump.

Usage: python tests/golden/make_golden.py [--large] [--dump] [names...]   (needs oracle/_ref built)
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

import time  # noqa: E402

from cases import (CASES, DUMP_CASES, FULL_VECTOR_MAX, LARGE_CASES, case_dict, checksum_weights,  # noqa: E402
                   general, sample_indices, seeded_input)
from oracle.refbind import RefOp, available, read_configs, ref_dump  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def log(msg):
    print(f"[{time.strftime('%H:%M:%S')}] {msg}", flush=True)


def gen(c, large=False):
    d = case_dict(c)
    t0 = time.perf_counter()
    op = RefOp(d["model"], d["dim"], d["axialdir"], d["betaJ"], d["kappa"], d["h"], d["size"], d["kappa2"],
               d["extend_cond"])
    n = op.n
    log(f"{d['name']}: n={n}, constructed in {time.perf_counter() - t0:.1f} s")
    out = dict(n=np.int64(n), normfactor=np.float64(op.normfactor))
    samp = sample_indices(n) if n > FULL_VECTOR_MAX else None
    if samp is not None:
        out["samp_idx"] = samp
    x = seeded_input(n, 1)
    t0 = time.perf_counter()
    y = op.perform_op(x)
    log(f"{d['name']}: one product in {time.perf_counter() - t0:.1f} s")
    w = checksum_weights(n)
    out["y_chk"] = np.array([np.dot(w, y), np.linalg.norm(y)])
    if n <= FULL_VECTOR_MAX:
        out["y"] = y
    else:
        out["y_samp"] = y[samp]
    del y
    if op.has_transpose():
        yt = op.perform_op_t(x)
        out["yt_chk"] = np.array([np.dot(w, yt), np.linalg.norm(yt)])
        if n <= FULL_VECTOR_MAX:
            out["yt"] = yt
        else:
            out["yt_samp"] = yt[samp]
        del yt
    del x, w
    idx, dup = op.orbit()
    if idx is not None:
        out["orbit_n"] = np.int64(len(idx))
        out["idx_sha"] = np.array(sha(idx.astype(np.uint64)))
        out["dup_sha"] = np.array(sha(dup.astype(np.uint16)))
        out["dup_sum"] = np.int64(dup.astype(np.int64).sum())
        if n <= FULL_VECTOR_MAX:
            out["idx"] = idx.astype(np.uint64)
            out["dup"] = dup.astype(np.uint16)
        else:
            out["idx_samp"] = idx[samp].astype(np.uint64)
            out["dup_samp"] = dup[samp].astype(np.uint16)
    del idx, dup
    # eigenvalues through ARPACK on the reference matvec
    nev = d["nev"]
    if nev == 0:
        return d["name"], out
    count = [0]

    def mv(v):
        count[0] += 1
        return op.perform_op(np.ravel(v))

    lin = sla.LinearOperator((n, n), matvec=mv, dtype=np.float64)
    sym = not op.has_transpose() and not general(d)
    v0 = np.random.default_rng(0).uniform(0, 1, n)
    if large:
        # the reference solver's Krylov size (suggested_nev, TMat/tmat.hpp:88)
        ncv, tol = 2 * nev + 3, 1e-12
        if n <= (1 << 28):
            # product count of the reference's settings (Spectra's default tol 1e-10)
            sla.eigsh(lin, k=nev, which="LM", tol=1e-10, v0=v0, ncv=ncv)
            out["arpack_matvecs_tol1e10"] = np.int64(count[0])
            log(f"{d['name']}: ARPACK ncv={ncv} tol=1e-10 took {count[0]} products")
            count[0] = 0
    else:
        ncv, tol = min(n - 1, max(2 * nev + 8, 20)), 1e-13
    t0 = time.perf_counter()
    if sym:
        vals, vecs = sla.eigsh(lin, k=nev, which="LM", tol=tol, v0=v0, ncv=ncv)
    else:
        vals, vecs = sla.eigs(lin, k=nev, which="LM", tol=tol, v0=v0, ncv=ncv)
    if large:
        out["arpack_matvecs"] = np.int64(count[0])
        out["arpack_ncv_tol"] = np.array([ncv, tol])
        log(f"{d['name']}: ARPACK ncv={ncv} tol={tol} took {count[0]} products, {time.perf_counter() - t0:.0f} s")
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
    else:
        out["q0_samp"] = q[samp]
        if not sym:
            out["ql_samp"] = ql[samp]
    mom, mst = op.moments(ql, q)
    phys, pst = op.phys_extend(ql, q)
    out["moments"] = mom
    out["moments_status"] = np.int64(mst)
    out["phys"] = phys
    out["phys_status"] = np.int64(pst)
    return d["name"], out


def gen_dump(c):
    """Leading eigenvector of the reference operator (ARPACK on its product),
    written as the reference's X_vec.dat, and the configurations the
    reference's dump() plants from it with the case's seed."""
    import tempfile

    name, model, ax, ec, bj, k, k2, h, size, nconf, length, seed = c
    op = RefOp(model, 2, ax, bj, k, h, size, k2, ec)
    n = op.n
    v0 = np.random.default_rng(0).uniform(0, 1, n)

    def leading(matvec, symmetric):
        lin = sla.LinearOperator((n, n), matvec=lambda v: matvec(np.ravel(v)), dtype=np.float64)
        if symmetric:
            vals, vecs = sla.eigsh(lin, k=2, which="LM", tol=1e-13, v0=v0, ncv=min(n - 1, 20))
        else:
            vals, vecs = sla.eigs(lin, k=2, which="LM", tol=1e-13, v0=v0, ncv=min(n - 1, 20))
        q = np.real(vecs[:, int(np.argmax(np.abs(vals)))])
        q = q / np.linalg.norm(q)
        return q * np.sign(q.sum())

    two_layer = (model, ax) in (("A", 2), ("A", 6), ("B", 6))  # GenDumpConfig: right and left vectors
    q = leading(op.perform_op, not two_layer)
    ql = leading(op.perform_op_t, False) if two_layer else None
    with tempfile.TemporaryDirectory() as td:
        vf = os.path.join(td, "RUN_vec.dat")
        q.astype(np.float64).tofile(vf)
        vlf = None
        if ql is not None:
            vlf = os.path.join(td, "RUN_vecl.dat")
            ql.astype(np.float64).tofile(vlf)
        st = ref_dump(model, ax, ec, bj, k, k2, h, size, vf, vlf, nconf, length, seed, os.path.join(td, "RUN"))
        if st != 0:
            raise RuntimeError(f"reference dump failed ({st})")
        configs = read_configs(os.path.join(td, "RUN"), nconf, size)
    out = dict(vec=q, configs=configs, n=np.int64(n))
    if ql is not None:
        out["vecl"] = ql
    log(f"{name}: n={n} configs {configs.shape}")
    return name, out


def main(args):
    if not available():
        raise SystemExit("oracle/_ref/libtmat_ref.so missing: run oracle/build_ref.sh first")
    large = "--large" in args
    names = [a for a in args if not a.startswith("--")]
    for c in DUMP_CASES:
        if (names and c[0] in names) or (not names and "--dump" in args):
            name, out = gen_dump(c)
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    if "--dump" in args and not names:
        return
    for c in CASES + LARGE_CASES:
        is_large = c in LARGE_CASES
        if names and c[0] not in names:
            continue
        if not names and is_large and not large:
            continue
        name, out = gen(c, large=is_large)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        log(f"{name}: n={int(out['n'])} evals={out.get('evals_re', [])[:2]}")


if __name__ == "__main__":
    main(sys.argv[1:])
