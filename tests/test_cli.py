"""fftdock-scan, the rot-scan/gather command-line front end."""
import json
import math
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import fftdock_oracle as O

ROOT = Path(__file__).resolve().parents[1]
CLI = ROOT / "proddl2_gb300" / "fftdock-scan"
GOLDEN = Path(__file__).resolve().parent / "golden"


def _opts(tmp_path, **kw):
    d = {"scan": dict(dict(gridStep=1.2, maxNTrans=4, maxNTransInp=10000, maxValCorr=1e300,
                           maxNRigidMatches=25), **kw)}
    p = tmp_path / "scan.json"
    p.write_text(json.dumps(d, indent=2))
    return p


def _pair(tmp_path, f, frames=None):
    from proddl2_gb300.pairfile import write_pair
    p = tmp_path / "pair.txt"
    rf, lf = frames if frames else (None, None)
    write_pair(p, f["rec_xyz"], f["rec_type"], f["lig_xyz"], f["lig_type"], f["ace"], rf, lf)
    return p


def test_cli_gather_matches_oracle(built_lib, tmp_path):
    rng = np.random.default_rng(3)
    recs = [(O.euler_to_matrix(rng.uniform(-3, 3, 3)), rng.normal(size=(3, 3)), rng.normal(size=3))
            for _ in range(12)]
    (tmp_path / "a.dat").write_bytes(b"".join(O.pack_record(*r) for r in recs[:7]))
    (tmp_path / "b.dat").write_bytes(b"".join(O.pack_record(*r) for r in recs[7:]))
    (tmp_path / "list.tab").write_text("%s\n%s\n" % (tmp_path / "a.dat", tmp_path / "b.dat"))
    f = np.load(GOLDEN / "scan_shape_ace_n32.npz")
    frames = ((O.euler_to_matrix([0.3, -0.2, 1.0]), np.array([1.0, -2.0, 0.5])),
              (O.euler_to_matrix([-1.1, 0.4, 0.2]), np.array([0.25, 3.0, -1.0])))
    pair = _pair(tmp_path, f, frames)
    r = subprocess.run([str(CLI), "--task", "gather", "--options", str(_opts(tmp_path)), "--fft-rot-scan-list",
                        str(tmp_path / "list.tab"), "--fft-res", str(tmp_path / "out.rigid"),
                        "--molforce-params", str(pair)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    expect = O.pack_rigid(O.gather_records(recs, 25), *frames)
    assert (tmp_path / "out.rigid").read_bytes() == expect


def test_cli_rot_scan_without_gpu_fails_loudly(built_lib, tmp_path):
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    from proddl2_gb300.pairfile import write_angles
    f = np.load(GOLDEN / "scan_shape_ace_n32.npz")
    write_angles(tmp_path / "ang.dat", [[0, 0, 0], [10, 20, 30]])
    r = subprocess.run([str(CLI), "--task", "rot-scan", "--options", str(_opts(tmp_path, gridN=32,
                        anglesFile=str(tmp_path / "ang.dat"))), "--molforce-params", str(_pair(tmp_path, f)),
                        "--fft-rot-grid-start", "0", "--fft-rot-grid-end", "2",
                        "--fft-rot-scan-res", str(tmp_path / "o.dat")], capture_output=True, text=True)
    assert r.returncode == 2 and "no CUDA device" in r.stderr
    assert not (tmp_path / "o.dat").exists()


@pytest.mark.gpu
def test_cli_rot_scan_ranges_match_the_c_abi(tmp_path):
    from proddl2_gb300 import FFTScan, ScanConfig
    from proddl2_gb300.pairfile import write_angles
    f = np.load(GOLDEN / "scan_shape_ace_n32.npz")
    rng = np.random.default_rng(12)
    ang = rng.uniform(-180, 180, size=(10, 3))
    write_angles(tmp_path / "ang.dat", ang)
    opts = _opts(tmp_path, gridN=32, anglesFile=str(tmp_path / "ang.dat"))
    pair = _pair(tmp_path, f)
    outs = []
    for lo, hi in ((0, 6), (6, 10)):
        out = tmp_path / ("scan_res.%04d-%04d.dat" % (lo, hi))
        r = subprocess.run([str(CLI), "--task", "rot-scan", "--options", str(opts), "--molforce-params", str(pair),
                            "--fft-rot-grid-start", str(lo), "--fft-rot-grid-end", str(hi),
                            "--fft-rot-scan-res", str(out)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        outs.append(out)
    recs = O.unpack_records(b"".join(p.read_bytes() for p in outs))
    rots = np.stack([O.euler_to_matrix(np.asarray(a) * (math.pi / 180.0)) for a in ang])
    with FFTScan(ScanConfig(grid_n=32, term_set="shape_ace", ace_matrix=f["ace"])) as s:
        s.set_receptor(f["rec_xyz"], f["rec_type"])
        s.set_ligand(f["lig_xyz"], f["lig_type"])
        res = s.scan(rots)
    assert len(recs) == 10
    for i, (rot, t, v) in enumerate(recs):
        assert np.array_equal(rot, rots[i])
        _, tt, sc = res.rotation(i)
        assert np.array_equal(t, tt) and np.array_equal(v, sc)


@pytest.mark.gpu
def test_cli_rot_scan_with_the_reference_ljcomp_potential(tmp_path):
    """potentialName "ljComp" with per-atom sigma/eps/alpha in the pair file
    gives the records of the C ABI's fftdock_set_pair_lj scan."""
    from proddl2_gb300 import FFTScan, ScanConfig, synth
    from proddl2_gb300.pairfile import write_angles, write_pair
    pair = synth.make_pair(300, 60, 1, seed=77)
    rng = np.random.default_rng(5)
    rl = np.stack([rng.uniform(3.0, 3.9, 300), rng.uniform(0.05, 0.6, 300), np.full(300, 0.4)], axis=1)
    ll = np.stack([rng.uniform(3.0, 3.9, 60), rng.uniform(0.05, 0.6, 60)], axis=1)
    pf = tmp_path / "pair.txt"
    write_pair(pf, pair.receptor.xyz, pair.receptor.ace_type, pair.ligand.xyz, pair.ligand.ace_type,
               rec_lj=rl, lig_lj=ll)
    ang = rng.uniform(-180, 180, size=(5, 3))
    write_angles(tmp_path / "ang.dat", ang)
    opts = _opts(tmp_path, gridN=48, anglesFile=str(tmp_path / "ang.dat"), potentialName="ljComp", cutOffFft=9.0)
    out = tmp_path / "o.dat"
    r = subprocess.run([str(CLI), "--task", "rot-scan", "--options", str(opts), "--molforce-params", str(pf),
                        "--fft-rot-grid-start", "0", "--fft-rot-grid-end", "5", "--fft-rot-scan-res", str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    recs = O.unpack_records(out.read_bytes())
    rots = np.stack([O.euler_to_matrix(np.asarray(a) * (math.pi / 180.0)) for a in ang])
    with FFTScan(ScanConfig(grid_n=48, term_set="lj_comp", lj_cut=9.0, peaks_per_rot=4, max_val_corr=1e300)) as s:
        s.set_pair_lj(pair.receptor.xyz, rl[:, 0], rl[:, 1], rl[:, 2], pair.ligand.xyz, ll[:, 0], ll[:, 1])
        res = s.scan(rots)
    for i, (rot, t, v) in enumerate(recs):
        _, tt, sc = res.rotation(i)
        assert np.array_equal(t, tt) and np.array_equal(v, sc)
