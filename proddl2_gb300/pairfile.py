"""Text pair file read by ``fftdock-scan`` in place of the reference's HDF5
molforce file (atoms, desolvation types, the desolvation matrix and the frame
transforms of the receptor and ligand)."""
from __future__ import annotations

import numpy as np


def _frame_line(name, frame):
    r, v = frame
    vals = list(np.asarray(r, dtype=np.float64).reshape(9)) + list(np.asarray(v, dtype=np.float64).reshape(3))
    return "%s %s\n" % (name, " ".join("%.17g" % x for x in vals))


def write_pair(path, rec_xyz, rec_type, lig_xyz, lig_type, ace=None, rec_frame=None, lig_frame=None,
               rec_lj=None, lig_lj=None):
    """``rec_lj`` (n, 3) sigma, eps, alpha and ``lig_lj`` (m, 2) sigma, eps: the
    per-atom parameters of the reference's LJ potentials (ljComp, ljAvg)."""
    out = ["# fftdock pair file\n"]
    for name, xyz, typ in (("receptor", rec_xyz, rec_type), ("ligand", lig_xyz, lig_type)):
        xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
        typ = np.zeros(len(xyz), dtype=np.int32) if typ is None else np.asarray(typ, dtype=np.int32)
        out.append("%s %d\n" % (name, len(xyz)))
        out.extend("%.17g %.17g %.17g %d\n" % (p[0], p[1], p[2], t) for p, t in zip(xyz, typ))
    if ace is not None:
        ace = np.asarray(ace, dtype=np.float64)
        out.append("ace %d\n" % ace.shape[0])
        out.extend(" ".join("%.17g" % x for x in row) + "\n" for row in ace)
    for name, arr in (("receptor_lj", rec_lj), ("ligand_lj", lig_lj)):
        if arr is not None:
            arr = np.asarray(arr, dtype=np.float64)
            out.append("%s %d\n" % (name, arr.shape[0]))
            out.extend(" ".join("%.17g" % x for x in row) + "\n" for row in arr)
    if rec_frame is not None:
        out.append(_frame_line("receptor_frame", rec_frame))
    if lig_frame is not None:
        out.append(_frame_line("ligand_frame", lig_frame))
    with open(path, "w") as f:
        f.writelines(out)


def write_angles(path, angles_deg):
    """Rotation file in the reference's ``ang*.dat`` layout: a count line,
    then one line of three Euler angles in degrees per rotation."""
    angles_deg = np.asarray(angles_deg, dtype=np.float64).reshape(-1, 3)
    with open(path, "w") as f:
        f.write("%d   Scan angles\n" % len(angles_deg))
        f.writelines("%.17g %.17g %.17g\n" % tuple(a) for a in angles_deg)
