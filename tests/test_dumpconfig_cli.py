"""The dumpconfig CLI (the reference's DumpConfig driver, DumpConfig/main.cpp)
end to end: input file + <out>_vec.dat (+ <out>_vecl.dat) in, planted
<out>_config_<k>.dat files out, compared line by line with the configurations
the reference's own dump() planted from the same vectors and seed
(tests/golden/dump_*.npz).  The dispatch errors that stop before any device
work run on the CPU."""
import os
import subprocess

import numpy as np
import pytest

from cases import DUMP_CASES
from gpu_util import fixture

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DUMP = os.path.join(ROOT, "latttmat_gb300", "dumpconfig")

INPUT = """modeltype = {model} # model type. A: ANNNI; B: BNNNI and 3NN; D: DNNI
dim = {dim}       # dimensionality. 2 or 3
axialdir = {ax}  # type of transfer matrix
neigs = {neigs}     # number of eigenvalues
savevec = 1 1 # save vectors, compute layer magnetisation
outfile = RUN  # prefix for output files
size = {size}        # system width L
J = {bj}          # inverse temperature beta * J
kappa = {k} {k2}    # kappa1 and kappa2 values
h = {h}            # external field
"""


def _run(tmp_path, args, **kw):
    p = tmp_path / "in.dat"
    p.write_text(INPUT.format(**kw))
    return subprocess.run([DUMP, str(p)] + [str(a) for a in args], cwd=tmp_path, capture_output=True, text=True,
                          timeout=600)


def _need_binary():
    if not os.path.exists(DUMP):
        pytest.skip("dumpconfig not built")


def test_unsupported_dimension_is_reported_like_the_reference(tmp_path):
    _need_binary()
    r = _run(tmp_path, [2, 10], model="A", dim=3, ax=1, neigs=1, size="3 4", bj=0.5, k=0.5, k2=0, h=0)
    assert r.returncode == 0
    assert "Error: dimension not supported yet" in r.stderr
    assert not list(tmp_path.glob("RUN_config_*.dat"))


def test_unsupported_axial_direction_is_reported_like_the_reference(tmp_path):
    _need_binary()
    r = _run(tmp_path, [1, 10], model="D", dim=2, ax=2, neigs=1, size=8, bj=0.5, k=0.5, k2=0, h=0)
    assert r.returncode == 0
    assert "Error: axial direction not supported yet" in r.stderr


# the reference driver builds XAM / XDM with extend_cond = (neigs > 1 ? 2 : 0)
# and the two-layer dumpers with extend_cond 0: the cases below are the
# fixtures whose extend_cond a driver run reproduces
CLI_CASES = ["dump_xat_L10", "dump_xam_L12", "dump_xam_L14_flip", "dump_xdm_L13_h", "dump_yat_L6",
             "dump_yam_L9_flip", "dump_ybm_L8_flip"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", CLI_CASES)
def test_cli_plants_the_reference_configurations(tmp_path, name):
    _need_binary()
    case = [c for c in DUMP_CASES if c[0] == name][0]
    _, model, ax, ec, bj, k, k2, h, size, nconf, length, seed = case
    f = fixture(name)
    vec = f["vec"]
    two_layer = "vecl" in f
    if two_layer:
        # a tmat run with several eigenvalues writes complex (re, im) pairs;
        # the reader keeps the real parts
        pairs = np.zeros(2 * vec.size)
        pairs[0::2] = vec
        pairs[1::2] = 1e3
        (pairs if name == "dump_yam_L9_flip" else vec).tofile(tmp_path / "RUN_vec.dat")
        f["vecl"].tofile(tmp_path / "RUN_vecl.dat")
    else:
        # several saved vectors: the first column is the one planted from
        np.concatenate([vec, np.full(vec.size, 7.0)]).tofile(tmp_path / "RUN_vec.dat")
    r = _run(tmp_path, [nconf, length, "--seed", seed], model=model, dim=2, ax=ax, neigs=2 if ec == 2 else 1,
             size=size, bj=bj, k=k, k2=k2, h=h)
    assert r.returncode == 0, r.stdout + r.stderr
    for c in range(nconf):
        lines = (tmp_path / f"RUN_config_{c}.dat").read_text().split("\n")
        assert lines[-1] == ""
        want = ["".join("1" if (int(s) >> i) & 1 else "0" for i in range(size)) for s in f["configs"][c]]
        assert lines[:-1] == want
    assert not (tmp_path / f"RUN_config_{nconf}.dat").exists()


@pytest.mark.gpu
def test_cli_reports_a_missing_vector_file(tmp_path):
    _need_binary()
    r = _run(tmp_path, [1, 10], model="A", dim=2, ax=5, neigs=1, size=10, bj=0.5, k=0.5, k2=0, h=0)
    assert r.returncode == 1
    assert 'Open "RUN_vec.dat" failed' in r.stderr


@pytest.mark.gpu
def test_cli_reports_a_short_vector_file(tmp_path):
    _need_binary()
    np.ones(10).tofile(tmp_path / "RUN_vec.dat")
    r = _run(tmp_path, [1, 10], model="A", dim=2, ax=1, neigs=1, size=10, bj=0.5, k=0.5, k2=0, h=0)
    assert r.returncode == 1
    assert "size incorrect" in r.stderr
