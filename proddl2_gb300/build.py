"""Build libfftdock.so in-tree for sm_103a with nvcc.

Each translation unit under ``csrc/`` is compiled in parallel to an object in
``_build/`` and linked into ``proddl2_gb300/libfftdock.so``.  A unit is only
recompiled when it or a header it includes is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libfftdock.so"
CLI = PKG / "fftdock-scan"
CLI_MAIN = CSRC / "fftdock_scan_main.cpp"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-I", str(ROOT / "include"), "-I", str(CSRC),
]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = Path("/usr/local/cuda/bin/nvcc")
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfftdock.so")


def _headers():
    return [p for p in CSRC.glob("*.cuh")] + [p for p in CSRC.glob("*.h")] + [ROOT / "include" / "fftdock.h"]


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src] + _headers())


def _compile(src: Path, extra):
    obj = BUILD / (src.stem + ".o")
    if not _stale(obj, src):
        return obj, None
    cmd = [nvcc()] + NVCC_FLAGS + list(extra) + ["-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, "%s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr)
    return obj, None


def build(verbose=False, extra_flags=(), jobs=None):
    """Compile and link; returns the library path."""
    BUILD.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu")) + sorted(p for p in CSRC.glob("*.cpp") if p != CLI_MAIN)
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    errors = []
    objs = []
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for obj, err in ex.map(lambda s: _compile(s, extra_flags), srcs):
            objs.append(obj)
            if err:
                errors.append(err)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    if not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs] + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    # command-line front end, linked against the library beside it
    if not CLI.exists() or CLI.stat().st_mtime < max(LIB.stat().st_mtime, CLI_MAIN.stat().st_mtime):
        cmd = [nvcc(), "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off", "-I", str(ROOT / "include"),
               str(CLI_MAIN), "-o", str(CLI),
               "-L", str(PKG), "-lfftdock", "-Xlinker", "-rpath=$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("fftdock-scan link failed:\n%s\n%s" % (r.stdout, r.stderr))
    if verbose:
        print("built", LIB, "and", CLI)
    return LIB


if __name__ == "__main__":
    extra = sys.argv[1:]
    build(verbose=True, extra_flags=extra)
