"""Build ``libbqa_gb300.so`` from ``csrc/*.cu`` with nvcc for sm_103a (GB300).

Each translation unit compiles in its own nvcc process (in parallel), then one link
step makes the shared library next to this file.  ``python -m bqa_gb300.build`` runs it.
The library links the CUDA runtime dynamically, so a process that already loaded it
(e.g. through PyTorch) shares one runtime instance with it.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libbqa_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GB300 backend must be compiled with the CUDA toolkit")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + [PKG.parent / "include" / "bqa_gb300.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build_library(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-cudart", "shared",
                    "-I", str(PKG.parent / "include")] + (extra_flags or [])
    procs = []
    for src in sources():
        obj = BUILD / (src.stem + ".o")
        cmd = [cc, "-c", str(src), "-o", str(obj)] + flags
        procs.append((src, obj, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    objs = []
    for src, obj, cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{out.decode(errors='replace')}")
        if verbose and out:
            print(out.decode(errors="replace"))
        objs.append(str(obj))
    tmp = LIB.with_suffix(".so.tmp")
    link = [cc, "-shared", "-o", str(tmp)] + objs + ARCH + ["-cudart", "shared",
                                                           "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout.decode(errors='replace')}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    v = "-v" in sys.argv
    extra = ["-Xptxas", "-v"] if "--ptxas" in sys.argv else None
    print(build_library(force=True, verbose=v or bool(extra), extra_flags=extra))
