"""CPU: the oracle restatement (oracle/tm_oracle.c) pinned against the golden
fixtures made by the reference itself (tests/golden/make_golden.py).

Bit-exact for orbit tables; FP64 outputs equal to rounding (the restatement
keeps the reference's arithmetic order, so differences are expected to be 0).
"""
import hashlib

import numpy as np
import pytest

from cases import CASES, case_dict, checksum_weights, seeded_input
from gpu_util import fixture

oracle = pytest.importorskip("oracle.oracle")


def _op(d):
    return oracle.OracleOp(d["model"], d["dim"], d["axialdir"], d["betaJ"], d["kappa"], d["h"], d["size"],
                           d["kappa2"], d["extend_cond"])


@pytest.mark.parametrize("name", [c[0] for c in CASES])
def test_oracle_matches_reference_fixture(name):
    d = case_dict([c for c in CASES if c[0] == name][0])
    f = fixture(name)
    o = _op(d)
    assert o.n == int(f["n"])
    assert o.normfactor == float(f["normfactor"])
    x = seeded_input(o.n, 1)
    y = o.perform_op(x)
    w = checksum_weights(o.n)
    np.testing.assert_allclose([np.dot(w, y), np.linalg.norm(y)], f["y_chk"], rtol=1e-13)
    if "y" in f:
        np.testing.assert_allclose(y, f["y"], rtol=1e-13, atol=1e-13 * np.max(np.abs(f["y"])))
    if "yt" in f:
        yt = o.perform_op_t(x)
        np.testing.assert_allclose(yt, f["yt"], rtol=1e-13, atol=1e-13 * np.max(np.abs(f["yt"])))
    if "idx_sha" in f:
        idx, dup = o.orbit()
        assert hashlib.sha256(idx.astype(np.uint64).tobytes()).hexdigest() == str(f["idx_sha"])
        assert hashlib.sha256(dup.astype(np.uint16).tobytes()).hexdigest() == str(f["dup_sha"])
    if "q0" in f:
        ql = f["ql"] if "ql" in f else f["q0"]
        m, st = o.moments(ql, f["q0"])
        np.testing.assert_allclose(m, f["moments"], rtol=1e-12, atol=1e-13)
        assert st == int(f["moments_status"])
        p, pst = o.phys_extend(ql, f["q0"])
        if len(f["phys"]):
            np.testing.assert_allclose(p, f["phys"], rtol=1e-12, atol=1e-13)
        assert pst == int(f["phys_status"])


@pytest.mark.parametrize("name", ["xat_L12_cfg1", "xam_L12_noflip", "xam_L12_flip", "xdt_L13_cfg3",
                                  "zbm_L12_noflip", "x3d_3x4_h"])
def test_oracle_eigenvalues(name):
    d = case_dict([c for c in CASES if c[0] == name][0])
    f = fixture(name)
    o = _op(d)
    w = o.eigs(len(f["evals_re"]))
    np.testing.assert_allclose(np.real(w), f["evals_re"], rtol=1e-10)
    np.testing.assert_allclose(np.imag(w), f["evals_im"], atol=1e-8 * np.abs(f["evals_re"][0]))


def test_published_probe_values():
    """Leading eigenvalues of the reference run for A/1 and A/5 (flip on and
    off) at L=12, betaJ=kappa=0.5, as the reference's own probe printed them."""
    full = oracle.OracleOp("A", 2, 1, 0.5, 0.5, 0.0, 12).eigs(2)
    np.testing.assert_allclose(full, [84970.93472621, 59989.6215884], rtol=1e-11)
    nf = oracle.OracleOp("A", 2, 5, 0.5, 0.5, 0.0, 12, 0.0, 2).eigs(2)
    np.testing.assert_allclose(nf, [84970.93472621, 45042.94793585], rtol=1e-11)
    fl = oracle.OracleOp("A", 2, 5, 0.5, 0.5, 0.0, 12, 0.0, 0).eigs(2)
    np.testing.assert_allclose(fl, [84970.93472621, 36870.69770993], rtol=1e-11)


def test_dump_fixtures_are_well_formed():
    """The planted-configuration fixtures (made by the reference's own dump())
    hold one unit eigenvector of the operator's size (two, right and left,
    for the two-layer parallel TMs) and nconfig x length layer states of L
    bits each (length + 1 for the full two-layer TM, whose dumper writes the
    first layer, the partner layer of every step and the last layer).  The
    eigenvectors are checked against the oracle's operator: T q = lambda q."""
    from cases import DUMP_CASES, TWO_LAYER_DUMP

    for name, model, ax, ec, bj, k, k2, h, size, nconf, length, seed in DUMP_CASES:
        f = fixture(name)
        o = _op(dict(model=model, dim=2, axialdir=ax, betaJ=bj, kappa=k, h=h, size=size, kappa2=k2,
                     extend_cond=ec))
        q = f["vec"]
        assert q.shape == (o.n,) and abs(np.linalg.norm(q) - 1.0) < 1e-12
        tq = o.perform_op(q)
        lam = float(q @ tq)
        assert np.linalg.norm(tq - lam * q) < 1e-8 * abs(lam)
        two_layer = (model, ax) in TWO_LAYER_DUMP
        if two_layer:
            ql = f["vecl"]
            assert ql.shape == (o.n,) and abs(np.linalg.norm(ql) - 1.0) < 1e-12
            tl = o.perform_op_t(ql)
            assert np.linalg.norm(tl - float(ql @ tl) * ql) < 1e-8 * abs(lam)
        assert f["configs"].shape == (nconf, length + 1 if (model, ax) == ("A", 2) else length)
        assert int(f["configs"].max()) < (1 << size)
