"""Build the reference's own code that compiles from its sources alone into
oracle/_ref (test infrastructure; never part of the product).

* libgdiam_ref.so: the gdiam bounding-box / diameter library vendored in the
  reference (src/PRODDL/External/Gdiam/gdiam.cpp) with its PRODDL wrapper
  (src/PRODDL/Geom/gdiam_simple.cpp) and oracle/gdiam_shim.cpp for C entry
  points.  The rest of the reference needs FFTW3, Blitz++, Boost and HDF5 and
  is not built.

The reference tree is taken from the FFTDOCK_REFERENCE_DIR environment
variable or the ``reference`` argument of build(), else from the checkout
beside this repository (../reference).  Runs only where that tree exists;
elsewhere it does nothing.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"


def reference_dir(reference=None):
    if reference:
        return Path(reference)
    env = os.environ.get("FFTDOCK_REFERENCE_DIR")
    if env:
        return Path(env)
    return HERE.parent.parent / "reference"


def build(verbose=False, reference=None):
    REFERENCE = reference_dir(reference)
    srcs = [REFERENCE / "src/PRODDL/External/Gdiam/gdiam.cpp", REFERENCE / "src/PRODDL/Geom/gdiam_simple.cpp"]
    if not all(p.exists() for p in srcs):
        return None
    gxx = shutil.which("g++")
    if not gxx:
        return None
    OUT.mkdir(exist_ok=True)
    lib = OUT / "libgdiam_ref.so"
    inputs = srcs + [HERE / "gdiam_shim.cpp"]
    if lib.exists() and all(p.stat().st_mtime <= lib.stat().st_mtime for p in inputs):
        return lib
    cmd = [gxx, "-O2", "-fPIC", "-shared", "-w", "-I", str(REFERENCE / "include")] + [str(p) for p in inputs] + \
          ["-o", str(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        if verbose:
            print(r.stderr)
        return None
    return lib


if __name__ == "__main__":
    print(build(verbose=True, reference=sys.argv[1] if len(sys.argv) > 1 else None))
