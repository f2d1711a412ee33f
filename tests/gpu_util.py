"""Helpers for the GPU parity tests (fixture loading, op construction)."""
from __future__ import annotations

import os

import numpy as np

import latttmat_gb300 as lt
from cases import by_name, case_dict, CASES, seeded_input, checksum_weights

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def fixture(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))


def make_op(name) -> lt.TMatOp:
    d = by_name(name)
    return lt.TMatOp(d["model"], d["dim"], d["axialdir"], d["betaJ"], d["kappa"], d["h"], d["size"], d["kappa2"],
                     d["extend_cond"])


def case_names(prefixes):
    return [c[0] for c in CASES if c[0].split("_")[0] in prefixes]


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
