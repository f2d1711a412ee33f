"""GPU: the tmat CLI end to end on reference-format input files; output files
checked against the reference's own eigenvalues and formats."""
import os
import subprocess

import numpy as np
import pytest

from gpu_util import fixture

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TMAT = os.path.join(ROOT, "latttmat_gb300", "tmat")

INPUT = """modeltype = {model} # model type. A: ANNNI; B: BNNNI and 3NN; D: DNNI
dim = {dim}       # dimensionality. 2 or 3
axialdir = {ax}  # type of transfer matrix
neigs = {neigs}     # number of eigenvalues
savevec = 1 1 # save vectors, compute layer magnetisation
outfile = {out}  # prefix for output files
size = {size}        # system width L
J = {bj}          # inverse temperature beta * J
kappa = {k} {k2}    # kappa1 and kappa2 values
h = {h}            # external field
"""


def run(tmp_path, **kw):
    p = tmp_path / "in.dat"
    p.write_text(INPUT.format(**kw))
    r = subprocess.run([TMAT, str(p)], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def read_vals(path):
    out = []
    for line in open(path).read().split("\n"):
        s = line.strip()
        if s.startswith("("):
            re_, im = s[1:-1].split(",")
            out.append(complex(float(re_), float(im)))
        elif s:
            out.append(float(s))
    return np.array(out)


@pytest.mark.parametrize("name,kw", [
    ("xat_L12_cfg1", dict(model="A", dim=2, ax=1, neigs=2, size=12, bj=0.5, k=0.5, k2=0, h=0)),
    ("xam_L12_noflip", dict(model="A", dim=2, ax=5, neigs=2, size=12, bj=0.5, k=0.5, k2=0, h=0)),
    ("xdt_L13_cfg3", dict(model="D", dim=2, ax=2, neigs=2, size=13, bj=0.4, k=0.3, k2=0, h=0.1)),
    ("zbm_L12_noflip", dict(model="B", dim=2, ax=7, neigs=2, size=12, bj=0.5, k=0.6, k2=0.2, h=0)),
])
def test_cli_outputs(tmp_path, name, kw):
    f = fixture(name)
    out = run(tmp_path, out="RUN", **kw)
    assert "MODEL : 2D_" in out and "Number of iteration" in out
    vals = read_vals(tmp_path / "RUN_val.dat")
    ref = f["evals_re"] + 1j * f["evals_im"]
    both = np.concatenate([vals, np.conj(vals)])
    for z in ref:
        assert np.min(np.abs(both - z)) / abs(z) < 1e-9, (z, vals)
    n = int(f["n"])
    sym = kw["model"] != "B"
    vec = np.fromfile(tmp_path / "RUN_vec.dat", dtype=np.float64)
    assert vec.size == (2 * n if sym else 2 * 2 * n)
    phys = open(tmp_path / "RUN_phys.dat").read().split("\n")
    mom = np.array([float(t) for t in phys[0].split("\t")])
    ql = f["ql"] if "ql" in f else f["q0"]
    np.testing.assert_allclose(mom, f["moments"], rtol=1e-6, atol=1e-8)
    if not sym:
        assert os.path.exists(tmp_path / "RUN_vecl.dat")
        assert "Eigensolver check" in out
