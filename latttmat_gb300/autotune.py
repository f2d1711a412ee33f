"""Autotuner of the aux-bit chain kernels (tile size and threads per block).

For each width it builds one operator of the family, times its FP32 and
double-float products over the candidate tile sizes (2^11..2^14 elements)
and block sizes (128, 256 threads) with tm_chain_autotune, and prints the
fastest per width and element size -- the table the library carries as its
built-in choices (kTunedBNNNI in csrc/tm_aux.cu) -- optionally as JSON.

  python -m latttmat_gb300.autotune [--model B] [--axialdir 7] [--widths 16 18 20 22 24] [--json out.json]
"""
from __future__ import annotations

import argparse
import json

import latttmat_gb300 as lt


def tune(model: str, axialdir: int, widths, betaJ: float = 0.6, kappa: float = 0.4):
    rows = []
    for L in widths:
        op = lt.TMatOp(model, 2, axialdir, betaJ, kappa, 0.0, L, 0.0, 2)
        row = {"L": L}
        for dt, tag in ((lt.TM_F32, "4"), (lt.TM_F64_DF, "8")):
            lt.chain_set_tuning(model, L, dt, 0, 0)
            tb, th, ms = lt.chain_autotune(op, dt)
            row.update({f"tb{tag}": tb, f"th{tag}": th, f"ms{tag}": ms})
        op.close()
        rows.append(row)
    return rows


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--model", default="B")
    ap.add_argument("--axialdir", type=int, default=7)
    ap.add_argument("--widths", type=int, nargs="+", default=[16, 18, 20, 22, 24])
    ap.add_argument("--json", default=None)
    a = ap.parse_args()
    rows = tune(a.model, a.axialdir, a.widths)
    for r in rows:
        print(f"    {{{r['L']}, {r['tb4']}, {r['th4']}, {r['tb8']}, {r['th8']}}},  "
              f"// {r['ms4']:.3f} ms FP32, {r['ms8']:.3f} ms double-float")
    if a.json:
        with open(a.json, "w") as fh:
            json.dump(rows, fh, indent=1)


if __name__ == "__main__":
    main()
