"""Parity cases shared by the golden-fixture generator and the tests.

Each case names one reference operator (model, dim, axialdir, extend_cond as
TMat/pfunc.cpp constructs it) and a parameter point.  Inputs are seeded:
x = default_rng(seed).uniform(-1, 1, n).  Fixtures hold the reference's own
outputs on those inputs (generated by make_golden.py from the reference
sources compiled here).
"""
from __future__ import annotations

import numpy as np

# (name, model, dim, axialdir, extend_cond, betaJ, kappa, kappa2, h, size, nev)
CASES = [
    # x-ANNNI full perpendicular TM (XATMatVecProd2D), incl. every boundary case
    ("xat_L4", "A", 2, 1, 0, 0.5, 0.5, 0.0, 0.0, 4, 2),
    ("xat_L8_h", "A", 2, 1, 0, 0.3, 0.7, 0.0, 0.1, 8, 2),
    ("xat_L12_cfg1", "A", 2, 1, 0, 0.5, 0.5, 0.0, 0.0, 12, 2),
    ("xat_L13", "A", 2, 1, 0, 0.45, 0.3, 0.0, 0.0, 13, 2),
    ("xat_L14_h", "A", 2, 1, 0, 0.9, 0.2, 0.0, 0.05, 14, 2),
    ("xat_open_L10", "A", 2, 9, 0, 0.4, 0.6, 0.0, 0.0, 10, 2),
    ("xat_b5_L10", "A", 2, 17, 0, 0.4, 0.6, 0.0, 0.1, 10, 2),
    ("xat_b9_L10", "A", 2, 18, 0, 0.4, 0.6, 0.0, 0.0, 10, 2),
    ("xat_b13_L10", "A", 2, 19, 0, 0.35, 0.8, 0.0, 0.0, 10, 2),
    ("xat_b17_L11", "A", 2, 20, 0, 0.35, 0.8, 0.0, 0.2, 11, 2),
    # x-ANNNI reduced (XAMMatVecProd2D): flip on (ec 0, h 0) / off (ec 2 or h != 0)
    ("xam_L8_flip", "A", 2, 5, 0, 0.5, 0.5, 0.0, 0.0, 8, 2),
    ("xam_L8_noflip", "A", 2, 5, 2, 0.5, 0.5, 0.0, 0.0, 8, 2),
    ("xam_L12_flip", "A", 2, 5, 0, 0.5, 0.5, 0.0, 0.0, 12, 2),
    ("xam_L12_noflip", "A", 2, 5, 2, 0.5, 0.5, 0.0, 0.0, 12, 2),
    ("xam_L13_noflip", "A", 2, 5, 2, 0.3, 0.6, 0.0, 0.0, 13, 2),
    ("xam_L14_h", "A", 2, 5, 0, 0.35, 0.55, 0.0, 0.05, 14, 2),
    ("xam_L16_flip", "A", 2, 5, 0, 0.3, 0.6, 0.0, 0.0, 16, 4),
    ("xam_L16_noflip", "A", 2, 5, 2, 0.3, 0.6, 0.0, 0.0, 16, 4),
    ("xam_L18_noflip", "A", 2, 5, 2, 0.7, 0.3, 0.0, 0.0, 18, 2),
    ("xam_L20_noflip", "A", 2, 5, 2, 0.3, 0.6, 0.0, 0.0, 20, 4),
    ("xam_L24_noflip", "A", 2, 5, 2, 0.3, 0.6, 0.0, 0.0, 24, 4),
    ("xam_L24_h_cfg5", "A", 2, 5, 0, 0.35, 0.55, 0.0, 0.05, 24, 4),
    ("xam_open_L12", "A", 2, 13, 2, 0.4, 0.6, 0.0, 0.0, 12, 2),
    ("xam_open_L13_flip", "A", 2, 13, 0, 0.4, 0.6, 0.0, 0.0, 13, 2),
    # DNNI full (XDTMatVecProd2D) and reduced (XDMMatVecProd2D)
    ("xdt_L8", "D", 2, 1, 0, 0.4, 0.3, 0.0, 0.1, 8, 2),
    ("xdt_L13_cfg3", "D", 2, 2, 0, 0.4, 0.3, 0.0, 0.1, 13, 2),
    ("xdt_L10_k", "D", 2, 1, 0, 0.6, 0.7, 0.0, 0.0, 10, 2),
    ("xdt_b5_L10", "D", 2, 17, 0, 0.4, 0.3, 0.0, 0.1, 10, 2),
    ("xdt_b9_L10", "D", 2, 18, 0, 0.4, 0.3, 0.0, 0.0, 10, 2),
    ("xdm_L10_flip", "D", 2, 5, 0, 0.4, 0.3, 0.0, 0.0, 10, 2),
    ("xdm_L13_noflip", "D", 2, 5, 2, 0.4, 0.3, 0.0, 0.1, 13, 2),
    ("xdm_L16_noflip", "D", 2, 6, 2, 0.5, 0.7, 0.0, 0.0, 16, 2),
    # diagonal BNNNI+3NN full (ZBTMatVecProd2D) and reduced (ZBMMatVecProd2D)
    ("zbt_L8", "B", 2, 3, 0, 0.5, 0.6, 0.2, 0.1, 8, 2),
    ("zbt_L12", "B", 2, 3, 0, 0.4, 0.3, 0.0, 0.0, 12, 2),
    ("zbm_L12_flip", "B", 2, 7, 0, 0.4, 0.3, 0.0, 0.0, 12, 2),
    ("zbm_L12_noflip", "B", 2, 7, 2, 0.5, 0.6, 0.2, 0.0, 12, 2),
    ("zbm_L16_noflip", "B", 2, 7, 2, 0.6, 0.8, 0.0, 0.0, 16, 2),
    ("zbm_L14_h", "B", 2, 7, 0, 0.5, 0.45, 0.1, 0.05, 14, 2),
    # instances of the 256-point B/7 parameter sweep (widths 16..24, betaJ grid
    # on [0.2, 1.0], kappa1 uniform; bench.batch_points), numbered by position
    ("zbm_sw000_L24", "B", 2, 7, 2, 0.2, 0.5118216247002567, 0.0, 0.0, 24, 2),
    ("zbm_sw001_L22", "B", 2, 7, 2, 0.2031372549019608, 0.9504636963259353, 0.0, 0.0, 22, 2),
    ("zbm_sw002_L20", "B", 2, 7, 2, 0.2062745098039216, 0.14415961271963373, 0.0, 0.0, 20, 2),
    ("zbm_sw003_L18", "B", 2, 7, 2, 0.20941176470588235, 0.9486494471372439, 0.0, 0.0, 18, 2),
    ("zbm_sw005_L16", "B", 2, 7, 2, 0.21568627450980393, 0.42332644897257565, 0.0, 0.0, 16, 2),
    ("zbm_sw128_L24", "B", 2, 7, 2, 0.6015686274509804, 0.2838064889441311, 0.0, 0.0, 24, 2),
    ("zbm_sw192_L18", "B", 2, 7, 2, 0.8023529411764707, 0.3626968570578484, 0.0, 0.0, 18, 2),
    ("zbm_sw255_L18", "B", 2, 7, 2, 1.0, 0.3856578446575508, 0.0, 0.0, 18, 2),
    # two-layer parallel TMs: y-ANNNI full (YATMatVecProd2D and its _T, even L:
    # at odd L the reference's final permutation reads its own output buffer),
    # y2-ANNNI full (Y2ATMatVecProd2D), y-ANNNI and BNNNI reduced
    # (YAMMatVecProd2D, YBMMatVecProd2D)
    ("yat_L4", "A", 2, 2, 0, 0.5, 0.3, 0.0, 0.0, 4, 2),
    ("yat_L6_h", "A", 2, 2, 0, 0.4, 0.7, 0.0, 0.1, 6, 2),
    ("yat_L8", "A", 2, 2, 0, 0.3, 0.6, 0.0, 0.0, 8, 2),
    ("y2at_L4", "A", 2, 0, 0, 0.5, 0.3, 0.0, 0.0, 4, 2),
    ("y2at_L5_h", "A", 2, 0, 0, 0.4, 0.6, 0.0, 0.1, 5, 2),
    ("y2at_L7", "A", 2, 0, 0, 0.3, 0.6, 0.0, 0.0, 7, 2),
    ("yam_L6_flip", "A", 2, 6, 0, 0.5, 0.3, 0.0, 0.0, 6, 2),
    ("yam_L7_noflip", "A", 2, 6, 2, 0.4, 0.7, 0.0, 0.0, 7, 2),
    ("yam_L8_h", "A", 2, 6, 0, 0.4, 0.6, 0.0, 0.1, 8, 2),
    ("yam_L10_noflip", "A", 2, 6, 2, 0.3, 0.6, 0.0, 0.0, 10, 2),
    ("ybm_L6_flip", "B", 2, 6, 0, 0.5, 0.6, 0.4, 0.0, 6, 2),
    ("ybm_L8_noflip", "B", 2, 6, 2, 0.5, 0.3, 0.2, 0.0, 8, 2),
    ("ybm_L7_h", "B", 2, 6, 0, 0.4, 0.6, 0.4, 0.05, 7, 2),
    # 3D ANNNI reduced (XAMMatVecProd3D)
    ("x3d_3x3", "A", 3, 1, 0, 0.3, 0.4, 0.0, 0.0, (3, 3), 2),
    ("x3d_3x4_h", "A", 3, 1, 0, 0.25, 0.5, 0.0, 0.1, (3, 4), 2),
    ("x3d_4x4_ising", "A", 3, 1, 0, 0.2, 0.0, 0.0, 0.0, (4, 4), 2),
    ("x3d_5x5_cfg5", "A", 3, 1, 0, 0.2, 0.4, 0.0, 0.0, (5, 5), 2),
]

# The headline x-ANNNI reduced operator (A/5, betaJ=0.3, kappa=0.6, h=0) at the
# widths where the even/odd product splits its tiles over CTA clusters (30, 32)
# and below; flip off as the reference driver runs neigs > 1 (extend_cond 2),
# and flip on at L=32.  nev = 0: tables and product only, no eigenvalues.
# Outputs are stored as checksums plus values at SAMPLE_COUNT seeded indices.
LARGE_CASES = [
    ("xam_L26_noflip", "A", 2, 5, 2, 0.3, 0.6, 0.0, 0.0, 26, 4),
    ("xam_L28_noflip", "A", 2, 5, 2, 0.3, 0.6, 0.0, 0.0, 28, 4),
    ("xam_L30_noflip", "A", 2, 5, 2, 0.3, 0.6, 0.0, 0.0, 30, 4),
    ("xam_L32_flip", "A", 2, 5, 0, 0.3, 0.6, 0.0, 0.0, 32, 0),
    ("xam_L32_cfg2", "A", 2, 5, 2, 0.3, 0.6, 0.0, 0.0, 32, 4),
]

# Configuration planting (the reference's DumpConfig) from the leading
# eigenvector: (name, model, axialdir, extend_cond, betaJ, kappa, kappa2, h,
# size, nconfig, length, seed).  Fixtures hold the eigenvector used and the
# layer states the reference's own dump() planted with that seed.
DUMP_CASES = [
    ("dump_xat_L10", "A", 1, 0, 0.4, 0.3, 0.0, 0.05, 10, 4, 64, 12345),
    ("dump_xat_L12", "A", 1, 0, 0.6, 0.5, 0.0, 0.0, 12, 3, 40, 7),
    ("dump_xam_L12", "A", 5, 2, 0.35, 0.5, 0.0, 0.0, 12, 4, 64, 777),
    ("dump_xam_L14_flip", "A", 5, 0, 0.45, 0.4, 0.0, 0.0, 14, 3, 48, 99),
    ("dump_xam_L16_h", "A", 5, 0, 0.3, 0.6, 0.0, 0.05, 16, 2, 40, 2024),
    ("dump_xdm_L12", "D", 5, 2, 0.4, 0.3, 0.0, 0.0, 12, 4, 48, 4242),
    ("dump_xdm_L13_h", "D", 5, 0, 0.5, 0.4, 0.0, 0.05, 13, 3, 40, 31),
    ("dump_xdm_L14_flip", "D", 5, 0, 0.35, 0.6, 0.0, 0.0, 14, 3, 36, 8),
    ("dump_yat_L6", "A", 2, 0, 0.4, 0.3, 0.0, 0.0, 6, 4, 40, 17),
    ("dump_yat_L8_h", "A", 2, 0, 0.6, 0.5, 0.0, 0.05, 8, 3, 32, 321),
    ("dump_yam_L8", "A", 6, 2, 0.5, 0.4, 0.0, 0.0, 8, 4, 40, 55),
    ("dump_yam_L9_flip", "A", 6, 0, 0.4, 0.6, 0.0, 0.0, 9, 3, 32, 6),
    ("dump_ybm_L8_flip", "B", 6, 0, 0.45, 0.3, 0.2, 0.0, 8, 3, 32, 1234),
]
TWO_LAYER_DUMP = (("A", 2), ("A", 6), ("B", 6))   # planted from right and left eigenvectors

FULL_VECTOR_MAX = 70000   # store full matvec outputs up to this length, else checksums and samples
SAMPLE_COUNT = 4096


def case_dict(c):
    name, model, dim, ax, ec, bj, k, k2, h, size, nev = c
    return dict(name=name, model=model, dim=dim, axialdir=ax, extend_cond=ec, betaJ=bj, kappa=k, kappa2=k2,
                h=h, size=size, nev=nev)


def general(d) -> bool:
    """Operators the reference solves with GenEigsSolver (complex Ritz pairs):
    the diagonal BNNNI and the two-layer families (TMat/tmat.hpp:158-176)."""
    return d["model"] == "B" or (d["model"] == "A" and d["dim"] == 2 and d["axialdir"] in (0, 2, 6))


def seeded_input(n: int, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).uniform(-1.0, 1.0, n)


def checksum_weights(n: int) -> np.ndarray:
    """Fixed weights for size-independent checksums of long outputs."""
    return np.random.default_rng(12345).uniform(0.5, 1.5, n)


def sample_indices(n: int) -> np.ndarray:
    """Sorted distinct seeded positions at which long outputs are stored."""
    idx = np.unique(np.random.default_rng(777).integers(0, n, SAMPLE_COUNT))
    return idx.astype(np.int64)


def by_name(name):
    for c in CASES + LARGE_CASES:
        if c[0] == name:
            return case_dict(c)
    raise KeyError(name)
