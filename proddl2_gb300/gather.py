"""Gather of scan records into the ranked pose list, and the pose file.

Host side of the reference's ``gather`` task (``Foreman``,
``include/PRODDL/docking_app.hpp:117-313``): per-rotation records from any
number of ``rot-scan`` outputs (this library's or the reference's) are merged
into the ``maxNRigidMatches`` lowest-energy poses, which are written in the
reference's IORigid format for its export step.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import FFTDockError


def gather_records(paths, max_matches=20000):
    """Poses (structured ``value, rot[9], t[3]``) ascending by value."""
    lib = _lib.lib()
    paths = [str(p).encode() for p in paths]
    arr = (C.c_char_p * len(paths))(*paths)
    out = np.zeros(max_matches, dtype=_lib.pose_dtype())
    n = C.c_int32()
    rc = lib.fftdock_gather_records(arr, len(paths), int(max_matches), C.c_void_p(out.ctypes.data), C.byref(n))
    if rc:
        raise FFTDockError(rc, "gathering scan records")
    return out[: n.value]


def gather_list(list_path, max_matches=20000):
    lib = _lib.lib()
    out = np.zeros(max_matches, dtype=_lib.pose_dtype())
    n = C.c_int32()
    rc = lib.fftdock_gather_list(str(list_path).encode(), int(max_matches), C.c_void_p(out.ctypes.data),
                                 C.byref(n))
    if rc:
        raise FFTDockError(rc, "gathering scan records from %s" % list_path)
    return out[: n.value]


def _frame(f):
    if f is None:
        return None
    r, v = f
    a = np.ascontiguousarray(np.concatenate([np.asarray(r, dtype=np.float64).reshape(9),
                                             np.asarray(v, dtype=np.float64).reshape(3)]))
    return a


def write_rigid(path, poses, rec_frame=None, lig_frame=None, text=False):
    """IORigid file of ``poses`` moved to the original frame
    ``rec_frame^-1 * pose * lig_frame`` (frames as (R 3x3, v 3))."""
    lib = _lib.lib()
    poses = np.ascontiguousarray(poses, dtype=_lib.pose_dtype())
    rf, lf = _frame(rec_frame), _frame(lig_frame)
    rc = lib.fftdock_write_rigid(str(path).encode(), C.c_void_p(poses.ctypes.data), len(poses),
                                 C.c_void_p(rf.ctypes.data) if rf is not None else None,
                                 C.c_void_p(lf.ctypes.data) if lf is not None else None, 1 if text else 0)
    if rc:
        raise FFTDockError(rc, "writing %s" % path)
