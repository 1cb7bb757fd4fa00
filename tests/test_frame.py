"""Pre-scan frame set-up (fftdock_frame_setup) against its FP64 restatement
(bit-exact), and against the reference's own gdiam library compiled from the
reference tree (oracle/_ref, built where the tree exists): the diameter end
points with eps = 0 and the frame built on the reference's minimum-volume
box."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from oracle import fftdock_oracle as O

REF = Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "libgdiam_ref.so"


def _gdiam():
    if not REF.exists():
        pytest.skip("the reference's gdiam is not built here (no reference tree)")
    lib = C.CDLL(str(REF))
    lib.ref_diam_pair.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_void_p]
    lib.ref_mvbb.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    return lib


def _pair(seed, n_rec=900, n_lig=150):
    from proddl2_gb300 import synth
    rec = synth.molecule(n_rec, seed)
    lig = synth.molecule(n_lig, seed + 1)
    # an arbitrary original frame: rotate and shift both
    R = synth.quaternion_rotations(1, seed + 2)[0]
    return rec.xyz @ R.T + np.array([10.0, -4.0, 7.0]), lig.xyz @ R.T + np.array([40.0, 3.0, -9.0])


def _check_same(a, b):
    rec, lig, trr, trl, size, box, fft = b
    assert np.array_equal(a.rec_xyz, rec) and np.array_equal(a.lig_xyz, lig)
    assert np.array_equal(a.rec_frame[0], trr[0]) and np.array_equal(a.rec_frame[1], trr[1])
    assert np.array_equal(a.lig_frame[0], trl[0]) and np.array_equal(a.lig_frame[1], trl[1])
    assert a.lig_size == size and np.array_equal(a.min_box, box) and list(a.fft_size) == list(fft)


@pytest.mark.parametrize("seed", [1, 2])
def test_axis_box_frame_matches_restatement(built_lib, seed):
    from proddl2_gb300.frame import frame_setup
    rec, lig = _pair(seed)
    mass = np.linspace(12.0, 32.0, len(lig))
    a = frame_setup(rec, lig, 1.2, 9.0, lig_mass=mass)
    _check_same(a, O.frame_setup(rec, lig, mass, 1.2, 9.0))
    # the frames map the original atoms onto the moved ones
    for xyz, out, fr in ((rec, a.rec_xyz, a.rec_frame), (lig, a.lig_xyz, a.lig_frame)):
        assert np.allclose(xyz @ fr[0].T + fr[1], out, atol=1e-9)
    # receptor box centred on the origin; ligand diameter centre at the origin
    assert np.allclose(a.rec_xyz.min(0) + a.rec_xyz.max(0), 0.0, atol=1e-9)
    assert a.grid_n >= max(a.fft_size)


def test_frames_round_trip_through_write_rigid(built_lib, tmp_path):
    """A pose found in the scan frame, written by write_rigid with these
    frames, moves the original ligand onto the moved-and-posed ligand seen
    from the original receptor frame (MolStruct::toOriginalFrame)."""
    from proddl2_gb300 import _lib
    from proddl2_gb300.frame import frame_setup
    from proddl2_gb300.gather import write_rigid
    rec, lig = _pair(3)
    a = frame_setup(rec, lig, 1.2, 9.0)
    pose = np.zeros(1, dtype=_lib.pose_dtype())
    pose[0]["value"] = -5.0
    pose[0]["rot"] = O.euler_to_matrix((0.3, -0.2, 0.9)).reshape(9)
    pose[0]["t"] = (2.4, -1.2, 3.6)
    path = tmp_path / "r.bin"
    write_rigid(str(path), pose, rec_frame=a.rec_frame, lig_frame=a.lig_frame)
    ref = O.pack_rigid([(-5.0, O.euler_to_matrix((0.3, -0.2, 0.9)), np.array([2.4, -1.2, 3.6]))],
                       a.rec_frame, a.lig_frame)
    assert path.read_bytes() == ref


def test_diameter_matches_reference_gdiam(built_lib):
    lib = _gdiam()
    from proddl2_gb300 import synth
    for seed in (4, 5, 6):
        xyz = np.ascontiguousarray(synth.molecule(300, seed).xyz)
        out = np.zeros(6)
        lib.ref_diam_pair(xyz.ctypes.data, len(xyz), 0.0, out.ctypes.data)
        p, q = O.farthest_pair(xyz)
        d_ref = np.linalg.norm(out[3:] - out[:3])
        assert abs(d_ref - np.linalg.norm(q - p)) <= 1e-12 * d_ref
        assert {tuple(out[:3]), tuple(out[3:])} == {tuple(p), tuple(q)}


@pytest.mark.parametrize("seed,n,stretch", [(7, 900, (1.0, 1.0, 1.0)), (9, 1500, (1.5, 1.0, 0.8)),
                                            (10, 2000, (2.0, 1.2, 0.7))])
def test_min_volume_box_matches_reference_gdiam(built_lib, seed, n, stretch):
    """The library's minimum-volume box against the reference's own gdiam
    (grid 5, every point, as Geom::Bounding::Box calls it): the same volume
    to 1e-4 (never larger by more), the same three axes up to their order and
    sign, every point inside."""
    lib = _gdiam()
    from proddl2_gb300 import synth
    from proddl2_gb300.frame import min_volume_box
    x = synth.molecule(n, seed).xyz * np.array(stretch)
    R = synth.quaternion_rotations(1, seed + 50)[0]
    x = np.ascontiguousarray(x @ R.T)
    D, c0, c1 = min_volume_box(x)
    corners, dirs = np.zeros(6), np.zeros(9)
    lib.ref_mvbb(x.ctypes.data, len(x), 5, len(x), corners.ctypes.data, dirs.ctypes.data)
    Dr = dirs.reshape(3, 3)
    vol = lambda d, a, b: abs(np.prod(d @ (b - a)))  # noqa: E731
    v, vr = vol(D, c0, c1), vol(Dr, corners[:3], corners[3:])
    assert abs(v / vr - 1.0) <= 1e-4 and v <= vr * (1.0 + 1e-9), (v, vr)
    assert np.allclose(D @ D.T, np.eye(3), atol=1e-12)
    match = np.abs(D @ Dr.T)
    assert np.all(np.sort(match.max(axis=1)) >= 0.999), match
    proj = x @ D.T
    lo, hi = D @ c0, D @ c1
    assert np.all(proj >= lo - 1e-9) and np.all(proj <= hi + 1e-9)
    # no larger than the axis-aligned box
    assert v <= np.prod(x.max(0) - x.min(0)) * (1.0 + 1e-12)


def test_frame_on_the_library_minimum_volume_box(built_lib):
    """box='min_volume' is the frame built on the library's own minimum-volume
    box (the same as passing that box in)."""
    from proddl2_gb300.frame import frame_setup, min_volume_box
    rec, lig = _pair(8, n_rec=600)
    a = frame_setup(rec, lig, 1.2, 9.0, box="min_volume")
    b = frame_setup(rec, lig, 1.2, 9.0, box=min_volume_box(rec))
    assert np.array_equal(a.rec_xyz, b.rec_xyz) and np.array_equal(a.min_box, b.min_box)
    assert np.array_equal(a.rec_frame[0], b.rec_frame[0]) and list(a.fft_size) == list(b.fft_size)
    vol = lambda f: np.prod(f.min_box[1] - f.min_box[0])  # noqa: E731
    assert vol(a) <= vol(frame_setup(rec, lig, 1.2, 9.0)) * 1.0001


def test_frame_on_the_reference_minimum_volume_box(built_lib):
    """Box directions and corners from the reference's own gdiam MVBB (grid
    5, every point sampled, as Geom::Bounding::Box does) give the same frame
    in the library and in the restatement; the box frame is orthonormal and
    centres the receptor."""
    lib = _gdiam()
    from proddl2_gb300.frame import frame_setup
    rec, lig = _pair(7)
    rc = np.ascontiguousarray(rec)
    corners, dirs = np.zeros(6), np.zeros(9)
    lib.ref_mvbb(rc.ctypes.data, len(rc), 5, len(rc), corners.ctypes.data, dirs.ctypes.data)
    D = dirs.reshape(3, 3)
    assert np.allclose(D @ D.T, np.eye(3), atol=1e-9)
    box = (D, corners[:3], corners[3:])
    a = frame_setup(rec, lig, 1.2, 9.0, box=box)
    _check_same(a, O.frame_setup(rec, lig, None, 1.2, 9.0, box=box))
    lo, hi = a.rec_xyz.min(0), a.rec_xyz.max(0)
    assert np.all(lo >= a.min_box[0]) and np.all(hi <= a.min_box[1])
    # the minimum-volume box is no larger than the axis-aligned one
    ax = frame_setup(rec, lig, 1.2, 9.0)
    vol = lambda f: np.prod(f.min_box[1] - f.min_box[0])  # noqa: E731
    assert vol(a) <= vol(ax) * 1.0001
