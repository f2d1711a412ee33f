"""CPU: the C ABI library loads and exports every symbol include/latttmat.h
declares (no compute calls: there may be no GPU here)."""
import ctypes
import os
import re

import pytest

import latttmat_gb300 as lt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "latttmat.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(tm_[a-z_0-9]+)\s*\(", txt)))


def test_header_declares_expected_api():
    syms = header_symbols()
    for s in ("tm_create", "tm_perform_op", "tm_perform_op_dev", "tm_eigs", "tm_orbit_table", "tm_transpose",
              "tm_destroy", "tm_grad", "tm_moments", "tm_phys_extend"):
        assert s in syms
    assert set(syms) <= set(lt.EXPORTED_SYMBOLS) | {"tm_version", "tm_last_error"}


def test_library_exports_every_declared_symbol():
    if not os.path.exists(lt.LIB_PATH):
        pytest.skip("library not built")
    lib = ctypes.CDLL(lt.LIB_PATH)
    missing = [s for s in header_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_version_string_without_gpu():
    if not os.path.exists(lt.LIB_PATH):
        pytest.skip("library not built")
    assert b"sm_103a" in lt.load_library().tm_version()


def test_no_cpu_fallback_in_product_package():
    """The product package never imports the oracle."""
    pkg = os.path.join(ROOT, "latttmat_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp", ".hpp")):
                src = open(os.path.join(dirpath, f), errors="replace").read()
                assert "oracle" not in src.replace("oracle/_ref", ""), f
