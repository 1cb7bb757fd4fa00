"""Many pairs in one CUDA graph (fftdock_scan_pairs): the grid-edge rule on
the CPU; on the GPU, results identical to scanning each pair through the
single-pair entry points, with and without the autotuner."""
import math

import numpy as np
import pytest

from oracle import fftdock_oracle as O


def _radius(xyz, centre):
    t = np.asarray(xyz) - centre
    return float(np.sqrt((t * t).sum(axis=1)).max())


def test_pair_grid_rule(built_lib):
    from proddl2_gb300 import synth
    from proddl2_gb300.pairs import pair_grid
    built = [48, 64, 80, 96, 112, 128, 144]
    for rec, lig in synth.uneven_pairs(12, seed=5):
        rr = _radius(rec.xyz, 0.5 * (rec.xyz.min(0) + rec.xyz.max(0)))
        rl = _radius(lig.xyz, np.zeros(3))
        need = math.ceil((2 * rr + 2 * rl + 12.0) / 1.2)
        assert pair_grid(rec.xyz, lig.xyz) == min(n for n in built if n >= need)


def _inputs(n_pairs, seed, n_rot):
    from proddl2_gb300 import synth
    from proddl2_gb300.pairs import PairInput
    rot = synth.quaternion_rotations(n_rot, seed=seed)
    out = []
    for rec, lig in synth.uneven_pairs(n_pairs, seed=seed, rec_range=(300, 2500), lig_range=(60, 400)):
        out.append(PairInput(rec.xyz, lig.xyz, rot, rec.ace_type, lig.ace_type))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("tune", [False, True])
def test_pair_graph_matches_single_pair_scans(tune):
    from proddl2_gb300 import FFTScan, ScanConfig, synth
    from proddl2_gb300.pairs import scan_pairs
    ace = synth.ace_matrix(18, 3)
    pairs = _inputs(7, 21, 150)
    base = ScanConfig(term_set="shape_ace", ace_matrix=ace, peaks_per_rot=4, rot_batch=48)
    res, rep = scan_pairs(base, pairs, tune=tune)
    assert rep["rotations"] == 7 * 150
    assert len(set(rep["grid_n"])) >= 2, rep["grid_n"]
    if tune:
        assert rep["n_streams"] in (1, 2, 4)
        assert set(rep["rot_batch"].values()) <= {32, 64, 128, 256}
        # the tuner chose a pencil form per edge (a tensor-form edge takes
        # rotations in multiples of 128)
        assert set(rep["pencil_form"]) == set(rep["rot_batch"])
        assert all(rep["rot_batch"][n] % 128 == 0 for n, f in rep["pencil_form"].items() if f == "tensor")
        # the tuned plan, reused without tuning, gives the same peaks
        res2, rep2 = scan_pairs(base, pairs, tune=False, plan=rep)
        assert rep2["n_streams"] == rep["n_streams"] and rep2["rot_batch"] == rep["rot_batch"]
        assert rep2["pencil_form"] == rep["pencil_form"]
        for a, b in zip(res, res2):
            assert np.array_equal(a.n_peaks, b.n_peaks) and np.array_equal(a.peaks, b.peaks)
    else:
        # grid edges up to 128 run the tensor form, which takes rotations in
        # whole groups (the requested 48 is rounded up to a multiple of 128)
        assert rep["n_streams"] == 1
        assert all((b >= 128 and b % 128 == 0) if int(n) <= 128 else b == 48
                   for n, b in rep["rot_batch"].items()), rep["rot_batch"]
        assert all(f == ("tensor" if n <= 128 else "fft") for n, f in rep["pencil_form"].items())
    # each pair against a single-pair scan with the pencil form its edge ran
    for p, r, n in zip(pairs, res, rep["grid_n"]):
        cfg = ScanConfig(grid_n=n, term_set="shape_ace", ace_matrix=ace, peaks_per_rot=4,
                         pencil_mode=rep["pencil_form"][n])
        with FFTScan(cfg) as s:
            s.set_receptor(p.rec_xyz, p.rec_type)
            s.set_ligand(p.lig_xyz, p.lig_type)
            ref = s.scan(p.rotations)
        assert np.array_equal(r.n_peaks, ref.n_peaks)
        for i in range(len(p.rotations)):
            k = r.n_peaks[i]
            assert np.array_equal(r.peaks[i, :k], ref.peaks[i, :k])


@pytest.mark.gpu
def test_pair_graph_reports_out_of_grid_and_bad_input():
    from proddl2_gb300 import FFTDockError, ScanConfig, _lib
    from proddl2_gb300.pairs import PairInput, scan_pairs
    rot = np.eye(3)[None]
    lig = np.array([[0.0, 0.0, 0.0], [40.0, 0.0, 0.0]])   # the far atom leaves a 48^3 grid
    rec = np.zeros((5, 3))
    res, rep = scan_pairs(ScanConfig(term_set="shape"), [PairInput(rec, lig, rot, grid_n=48)],
                          tune=False, raise_out_of_grid=False)
    assert rep["n_out_of_grid"] == 1 and res[0].n_peaks[0] == 0
    assert res[0].status == _lib.FFTDOCK_EOUT_OF_GRID
    with pytest.raises(FFTDockError) as ei:
        scan_pairs(ScanConfig(term_set="shape"), [PairInput(rec, lig, rot, grid_n=50)], tune=False)
    assert ei.value.code == _lib.FFTDOCK_EUNSUPPORTED
