"""Pre-scan frame set-up of a pair (``fftdock_frame_setup``): the frames the
reference's MolStruct moves the receptor and ligand into before the scan
(``include/PRODDL/docking_molstruct.hpp:199-252``), the padded box and the
grid size.  The returned frames are the ones ``gather.write_rigid`` undoes.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import FFTDockError


@dataclass
class PairFrame:
    rec_xyz: np.ndarray      # receptor atoms in the scan frame
    lig_xyz: np.ndarray      # ligand atoms, rotation centre at the origin
    rec_frame: tuple         # (R 3x3, v 3): original -> scan frame
    lig_frame: tuple
    lig_size: float
    min_box: np.ndarray      # (2, 3) padded receptor box
    fft_size: tuple          # per-axis FFT size (findBestSize)
    grid_n: int              # smallest built cubic edge covering it (0: none)


def frame_setup(rec_xyz, lig_xyz, grid_step=1.2, cut_off_fft=9.0, starting_spin=23.3734432, lig_mass=None,
                box=None, lig_diam=None):
    """``box``: None (axis-aligned receptor box), "min_volume" (the
    minimum-volume box, computed as the reference's Box does) or (directions
    3x3 rows, corner (0,0,0), corner (1,1,1)) in the original frame."""
    rec = np.ascontiguousarray(rec_xyz, dtype=np.float64).reshape(-1, 3)
    lig = np.ascontiguousarray(lig_xyz, dtype=np.float64).reshape(-1, 3)
    mass = None if lig_mass is None else np.ascontiguousarray(lig_mass, dtype=np.float64)
    a = _lib.FrameIn()
    a.n_rec, a.rec_xyz = len(rec), rec.ctypes.data
    a.n_lig, a.lig_xyz = len(lig), lig.ctypes.data
    a.lig_mass = mass.ctypes.data if mass is not None else None
    a.grid_step, a.cut_off_fft, a.starting_spin = float(grid_step), float(cut_off_fft), float(starting_spin)
    keep = []
    if box is None:
        a.box_mode = _lib.FFTDOCK_BOX_AXES
    elif isinstance(box, str):
        if box != "min_volume":
            raise ValueError("box: None, 'min_volume' or (dirs, corner0, corner1)")
        a.box_mode = _lib.FFTDOCK_BOX_MIN_VOLUME
    else:
        dirs = np.ascontiguousarray(box[0], dtype=np.float64).reshape(9)
        corners = np.ascontiguousarray(np.concatenate([np.ravel(box[1]), np.ravel(box[2])]), dtype=np.float64)
        keep += [dirs, corners]
        a.box_mode = _lib.FFTDOCK_BOX_GIVEN
        a.box_dirs, a.box_corners = dirs.ctypes.data, corners.ctypes.data
    if lig_diam is not None:
        dm = np.ascontiguousarray(np.concatenate([np.ravel(lig_diam[0]), np.ravel(lig_diam[1])]), dtype=np.float64)
        keep.append(dm)
        a.lig_diam = dm.ctypes.data
    rec_out = np.empty_like(rec)
    lig_out = np.empty_like(lig)
    f = _lib.Frame()
    rc = _lib.lib().fftdock_frame_setup(C.byref(a), C.c_void_p(rec_out.ctypes.data), C.c_void_p(lig_out.ctypes.data),
                                        C.byref(f))
    if rc:
        raise FFTDockError(rc, "frame set-up: bad input")
    fr = lambda t: (np.array(t[:9]).reshape(3, 3), np.array(t[9:12]))  # noqa: E731
    return PairFrame(rec_out, lig_out, fr(f.rec_frame), fr(f.lig_frame), float(f.lig_size),
                     np.array(f.min_box).reshape(2, 3), tuple(int(v) for v in f.fft_size), int(f.grid_n))


def min_volume_box(xyz, grid=5):
    """Minimum-volume bounding box of the points (``fftdock_min_volume_box``):
    (direction rows 3x3, corner (0,0,0), corner (1,1,1))."""
    pts = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    dirs = np.zeros(9)
    corners = np.zeros(6)
    rc = _lib.lib().fftdock_min_volume_box(len(pts), C.c_void_p(pts.ctypes.data), int(grid),
                                           C.c_void_p(dirs.ctypes.data), C.c_void_p(corners.ctypes.data))
    if rc:
        raise FFTDockError(rc, "minimum-volume box: bad input")
    return dirs.reshape(3, 3), corners[:3].copy(), corners[3:].copy()
