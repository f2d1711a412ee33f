"""GPU: configuration planting (tm_dump_configs, the reference's DumpConfig)
against the configurations the reference's own dump() planted with the same
eigenvector and seed (tests/golden/dump_*.npz).  Bar: every layer state of
every chain equal."""
import numpy as np
import pytest

import latttmat_gb300 as lt
from cases import DUMP_CASES
from gpu_util import fixture

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", DUMP_CASES, ids=[c[0] for c in DUMP_CASES])
def test_planted_configurations_match_the_reference(case):
    name, model, ax, ec, bj, k, k2, h, size, nconf, length, seed = case
    f = fixture(name)
    op = lt.TMatOp(model, 2, ax, bj, k, h, size, k2, ec)
    assert op.rows() == int(f["n"])
    vecl = f["vecl"] if "vecl" in f else None  # the two-layer TM plants from both vectors
    states = op.dump_configs(f["vec"], nconf, length, seed, vecl=vecl)
    np.testing.assert_array_equal(states, f["configs"])
    # a second call with the same seed plants the same configurations
    np.testing.assert_array_equal(op.dump_configs(f["vec"], nconf, length, seed, vecl=vecl), states)


def test_planting_writes_the_reference_file_format(tmp_path):
    name, model, ax, ec, bj, k, k2, h, size, nconf, length, seed = DUMP_CASES[0]
    f = fixture(name)
    op = lt.TMatOp(model, 2, ax, bj, k, h, size, k2, ec)
    states = op.dump_configs(f["vec"], nconf, length, seed)
    prefix = str(tmp_path / "RUN")
    lt.write_configs(states, size, prefix)
    lines = open(prefix + "_config_0.dat").read().split("\n")
    assert len([ln for ln in lines if ln]) == length
    assert all(len(ln) == size and set(ln) <= {"0", "1"} for ln in lines if ln)
    first = int(states[0, 0])
    assert lines[0] == "".join("1" if (first >> i) & 1 else "0" for i in range(size))


def test_planting_refuses_other_operators():
    op = lt.TMatOp("B", 2, 7, 0.5, 0.5, 0.0, 12, 0.0, 2)
    with pytest.raises(lt.TMError) as e:
        op.dump_configs(np.ones(op.rows()), 1, 4, 0)
    assert e.value.code == lt.TM_ERR_UNSUPPORTED
    # left/right planting is the two-layer TM's; the two-layer TM needs both vectors
    sym = lt.TMatOp("A", 2, 5, 0.4, 0.3, 0.0, 10, 0.0, 2)
    with pytest.raises(lt.TMError) as e:
        sym.dump_configs(np.ones(sym.rows()), 1, 4, 0, vecl=np.ones(sym.rows()))
    assert e.value.code == lt.TM_ERR_UNSUPPORTED
    yat = lt.TMatOp("A", 2, 2, 0.4, 0.3, 0.0, 6, 0.0, 0)
    with pytest.raises(lt.TMError) as e:
        yat.dump_configs(np.ones(yat.rows()), 1, 4, 0)
    assert e.value.code == lt.TM_ERR_ARG
