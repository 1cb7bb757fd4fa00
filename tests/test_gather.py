"""Gather and pose output (C ABI, no GPU needed) against the oracle's
restatement of Foreman::run / writeResults and the reference formats."""
import struct

import numpy as np
import pytest

from oracle import fftdock_oracle as O


def _records(rng, n_rec):
    recs = []
    for _ in range(n_rec):
        rot = O.euler_to_matrix(rng.uniform(-3, 3, 3))
        n = int(rng.integers(0, 6))
        recs.append((rot, rng.normal(scale=10, size=(n, 3)), rng.normal(scale=50, size=n)))
    return recs


def _write(path, recs):
    path.write_bytes(b"".join(O.pack_record(r, t, v) for r, t, v in recs))


def _frame(rng):
    return O.euler_to_matrix(rng.uniform(-3, 3, 3)), rng.normal(scale=5, size=3)


def test_gather_matches_oracle_over_files_and_list(built_lib, tmp_path):
    from proddl2_gb300 import gather
    rng = np.random.default_rng(8)
    a, b = _records(rng, 20), _records(rng, 15)
    # duplicate values across files: ties keep file order
    b[0] = (b[0][0], b[0][1][:1], np.array([a[1][2][0]])) if len(a[1][2]) else b[0]
    _write(tmp_path / "s1.bin", a)
    _write(tmp_path / "s2.bin", b)
    for k in (1, 7, 50, 1000):
        ref = O.gather_records(a + b, k)
        got = gather.gather_records([tmp_path / "s1.bin", tmp_path / "s2.bin"], k)
        assert len(got) == len(ref)
        for g, (v, r, t) in zip(got, ref):
            assert g["value"] == v
            assert np.array_equal(g["rot"].reshape(3, 3), r)
            assert np.array_equal(g["t"], t)
    lst = tmp_path / "list.tab"
    lst.write_text("%s\n%s\n" % (tmp_path / "s1.bin", tmp_path / "s2.bin"))
    got = gather.gather_list(lst, 30)
    assert np.array_equal(got["value"], [v for v, _, _ in O.gather_records(a + b, 30)])


def test_truncated_record_ends_its_file_and_bad_signature_fails(built_lib, tmp_path):
    from proddl2_gb300 import gather, FFTDockError, _lib
    rng = np.random.default_rng(9)
    a = _records(rng, 5)
    blob = b"".join(O.pack_record(r, t, v) for r, t, v in a)
    (tmp_path / "t.bin").write_bytes(blob + O.pack_record(*a[0])[:-8])
    got = gather.gather_records([tmp_path / "t.bin"], 100)
    assert len(got) == sum(len(v) for _, _, v in a)
    (tmp_path / "bad.bin").write_bytes(struct.pack("<i", 7) + blob[4:])
    with pytest.raises(FFTDockError) as ei:
        gather.gather_records([tmp_path / "bad.bin"], 10)
    assert ei.value.code == _lib.FFTDOCK_EIO


def test_rigid_file_matches_oracle(built_lib, tmp_path):
    from proddl2_gb300 import gather
    rng = np.random.default_rng(10)
    recs = _records(rng, 30)
    poses = O.gather_records(recs, 40)
    from proddl2_gb300 import _lib
    arr = np.zeros(len(poses), dtype=_lib.pose_dtype())
    for i, (v, r, t) in enumerate(poses):
        arr[i]["value"], arr[i]["rot"], arr[i]["t"] = v, r.reshape(9), t
    rf, lf = _frame(rng), _frame(rng)
    gather.write_rigid(tmp_path / "out.rigid", arr, rf, lf)
    assert (tmp_path / "out.rigid").read_bytes() == O.pack_rigid(poses, rf, lf)
    gather.write_rigid(tmp_path / "out.txt", arr, rf, lf, text=True)
    lines = (tmp_path / "out.txt").read_text().splitlines()
    assert int(lines[0]) == len(poses)
    bin_vals = np.frombuffer(O.pack_rigid(poses, rf, lf)[8:], dtype="<f4").reshape(-1, 7)
    txt_vals = np.array([[float(x) for x in ln.split("\t")] for ln in lines[1:]])
    assert np.allclose(txt_vals, bin_vals, rtol=1e-9, atol=0)
