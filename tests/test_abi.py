"""The C-ABI library builds, loads on a machine without a GPU, and exports exactly what
include/bqa_gb300.h declares (no compute calls here)."""
import ctypes
import re
from pathlib import Path

import pytest

from bqa_gb300 import _lib
from bqa_gb300.build import build_library

HEADER = Path(__file__).resolve().parents[1] / "include" / "bqa_gb300.h"


def declared_functions() -> set:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(bqa_[a-z0-9_]+)\s*\(", text))


@pytest.fixture(scope="module")
def lib():
    build_library()
    return _lib.Library()


def test_header_and_binding_agree():
    assert declared_functions() == set(_lib.SIGNATURES)


def test_every_declared_symbol_is_exported(lib):
    for name in declared_functions():
        assert hasattr(lib.dll, name), name


def test_abi_version_and_limits(lib):
    assert lib.dll.bqa_abi_version() == _lib.ABI_VERSION
    assert lib.max_bond_dim(3) == 16
    assert lib.max_bond_dim(4) == 8
    assert lib.max_bond_dim(-1) == 0
    assert lib.max_bond_dim(3, _lib.BQA_C128) == 13
    assert lib.max_bond_dim(3, 7) == 0


def test_bad_arguments_are_reported_not_crashing(lib):
    rc = lib.dll.bqa_env_factor(None, 4, 8, 0, 1e-6, None, None, None, None)
    assert rc == 1
    assert b"bqa_env_factor" in lib.dll.bqa_last_error()
    with pytest.raises(_lib.BqaError):
        lib.call("bqa_edge_zz", None, 4, 2, 0, None, None)
