"""The C-ABI library builds, loads on a machine without a GPU, and exports exactly what
include/bqa_gb300.h declares (no compute calls here)."""
import ctypes
import re
from pathlib import Path

import pytest

from bqa_gb300 import _lib
from bqa_gb300.build import build_library

HEADER = Path(__file__).resolve().parents[1] / "include" / "bqa_gb300.h"
PROBE_HEADER = Path(__file__).resolve().parents[1] / "include" / "bqa_gb300_probes.h"


def declared_functions(header=HEADER) -> set:
    text = header.read_text()
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


def test_probes_live_in_their_own_library(lib):
    """The measurement probes are declared and exported by the probe library only."""
    probes = declared_functions(PROBE_HEADER)
    assert probes == set(_lib.PROBE_SIGNATURES) == {"bqa_fp32_fma_probe", "bqa_mma_probe"}
    dll = _lib.load_probes()
    for name in probes:
        assert hasattr(dll, name), name
        assert not hasattr(lib.dll, name), name


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


def _c_offsets(tmp_path, struct: str, fields: list) -> dict:
    """offsetof each field and sizeof the struct, from the header, by a C compiler."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / f"{struct}.c"
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void) {",
             f'  printf("sizeof %zu\\n", sizeof({struct}));']
    lines += [f'  printf("{f} %zu\\n", offsetof({struct}, {f}));' for f in fields]
    lines += ["  return 0;", "}"]
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / struct
    subprocess.run([cc, "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {k: int(v) for k, v in (line.split() for line in out.strip().splitlines())}


@pytest.mark.parametrize("cls,struct", [(_lib.BqaClass, "bqa_class"), (_lib.BqaJob, "bqa_job"),
                                        (_lib.BqaLayerInfo, "bqa_layer_info")])
def test_struct_layout_matches_header(tmp_path, cls, struct):
    """The ctypes mirrors have the C structs' field offsets and sizes (a mismatch would pass
    garbage pointers to the library silently)."""
    names = [f[0] for f in cls._fields_]
    c = _c_offsets(tmp_path, struct, names)
    assert c["sizeof"] == ctypes.sizeof(cls)
    for n in names:
        assert c[n] == getattr(cls, n).offset, n
