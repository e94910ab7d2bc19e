"""The C-ABI library builds, loads without a GPU and exports every entry
point declared in include/qmc.h (no compute calls here)."""
import ctypes
import os
import re

import pytest

from jaqmc_gb300 import _native, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "qmc.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qmc_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib_path():
    return build.build()


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("qmc_forward", "qmc_local_energy", "qmc_mh_steps", "qmc_model_set_params",
                 "qmc_workspace_size", "qmc_reduce_mean_var"):
        assert must in names


def test_library_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(str(lib_path))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(lib_path):
    assert set(declared_functions()) == set(_native.exported_symbols())
    lib = _native.load(lib_path)
    assert lib.qmc_last_error() == b""
