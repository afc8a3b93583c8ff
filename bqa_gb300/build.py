"""Build ``libbqa_gb300.so`` from ``csrc/*.cu`` with nvcc for sm_103a (GB300), and the
measurement probes' ``libbqa_gb300_probes.so`` from ``probes/*.cu``.

Each translation unit compiles in its own nvcc process (in parallel), then one link
step per library makes it next to this file.  ``python -m bqa_gb300.build`` runs it.
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
PROBES = PKG / "probes"
BUILD = PKG / "_build"
LIB = PKG / "libbqa_gb300.so"
PROBE_LIB = PKG / "libbqa_gb300_probes.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GB300 backend must be compiled with the CUDA toolkit")


def _stale(lib: Path, srcdir: Path) -> bool:
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    deps = list(srcdir.glob("*")) + list(CSRC.glob("*.cuh")) + list((PKG.parent / "include").glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build_library(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Build the backend library and the probes' library (each only if stale unless ``force``);
    returns the backend library's path."""
    jobs = [(lib, srcdir) for lib, srcdir in ((LIB, CSRC), (PROBE_LIB, PROBES)) if force or _stale(lib, srcdir)]
    if not jobs:
        return LIB
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-cudart", "shared",
                    "-I", str(PKG.parent / "include")] + (extra_flags or [])
    procs = []
    for lib, srcdir in jobs:
        for src in sorted(srcdir.glob("*.cu")):
            obj = BUILD / (srcdir.name + "_" + src.stem + ".o")
            cmd = [cc, "-c", str(src), "-o", str(obj)] + flags
            procs.append((lib, src, obj, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    objs: dict = {lib: [] for lib, _ in jobs}
    for lib, src, obj, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{out.decode(errors='replace')}")
        if verbose and out:
            print(out.decode(errors="replace"))
        objs[lib].append(str(obj))
    for lib, files in objs.items():
        tmp = lib.with_suffix(".so.tmp")
        link = [cc, "-shared", "-o", str(tmp)] + files + ARCH + ["-cudart", "shared",
                                                                "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
        r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc link of {lib.name} failed:\n{r.stdout.decode(errors='replace')}")
        os.replace(tmp, lib)
    return LIB


if __name__ == "__main__":
    v = "-v" in sys.argv
    extra = ["-Xptxas", "-v"] if "--ptxas" in sys.argv else None
    print(build_library(force=True, verbose=v or bool(extra), extra_flags=extra))
