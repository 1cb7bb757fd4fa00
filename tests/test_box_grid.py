"""Box grids: FFT sizes chosen per axis, as the reference sizes its grid
(findBestSize<N_dim> per axis over the padded receptor box,
include/PRODDL/docking_fft.hpp:541-553), and cubic edges without compiled
plans.  GPU receptor grids, correlation grids and peaks against the FP64
oracle on the same per-axis geometry, through the C ABI."""
import numpy as np
import pytest

from oracle import fftdock_oracle as O

pytestmark = pytest.mark.gpu

REL = 1e-4
NAMES = {O.TERMS_SHAPE: "shape", O.TERMS_SHAPE_ACE: "shape_ace"}


def _ctx(dims, term_set, ace, k=4, **kw):
    from proddl2_gb300 import FFTScan, ScanConfig
    return FFTScan(ScanConfig(grid_dims=tuple(dims), grid_step=1.2, term_set=NAMES[term_set], peaks_per_rot=k,
                              ace_matrix=ace, **kw))


def _oracle(dims, term_set, ace, rec_xyz, rec_type, lig_type):
    geom = O.Geometry.centred(1.2, dims)
    tp = O.TermParams(term_set=term_set, ace_matrix=ace)
    return geom, O.receptor_terms(geom, rec_xyz, rec_type, tp), O.ligand_term_weights(lig_type, tp)


def _peaks_match(res, i, geom, rg, rs, lig_xyz, w, rot, k, cand=None):
    """One rotation's peaks tie-aware against the oracle; every reported
    score is the FP64 direct-space energy of its cell."""
    ref = O.scan_rotation(geom, rg, rs, lig_xyz, w, rot, k, workers=8)
    assert ref.in_grid
    cells, _ = O.bin_ligand(geom, rot, lig_xyz)
    nx, ny, nz = geom.dims
    cell, t, score = res.rotation(i)
    assert len(score) == len(ref.scores)
    assert np.array_equal(t, O.translation(cell, geom))
    scale = np.maximum(np.abs(ref.scores), 1.0)
    assert np.all(np.abs(score - ref.scores) <= REL * scale), (score, ref.scores)
    off = (cell[:, 0] * ny + cell[:, 1]) * nz + cell[:, 2]
    last = ref.scores[-1]
    tie = REL * max(abs(last), 1.0)
    got = set(int(o) for o in off)
    for o, s in zip(ref.offsets, ref.scores):
        if s < last - tie:
            assert int(o) in got, ("missing strict peak", o, s)
    for o, c, s in zip(off, cell, score):
        e = O.direct_score(rg, cells, w, c)
        assert abs(e - s) <= 1e-9 * max(1.0, abs(e))
        if int(o) not in set(int(v) for v in ref.offsets):
            assert abs(e - last) <= tie, ("extra peak that is not a tie", o, e, last)
    if cand is not None:
        vals, offs = cand
        for v, o in zip(vals[i][:k], offs[i][:k]):
            e = O.direct_score(rg, cells, w, O.offsets_to_cells([int(o)], geom.dims)[0])
            assert abs(v - e) <= REL * max(1.0, abs(ref.scores[0]))


@pytest.mark.parametrize("dims", [(40, 48, 36), (45, 42, 50)])
def test_box_grid_receptor_and_correlation_grids(dims):
    from proddl2_gb300 import synth
    pair = synth.make_pair(300, 60, 2, seed=71)
    geom, rg, w = _oracle(dims, O.TERMS_SHAPE_ACE, pair.ace, pair.receptor.xyz, pair.receptor.ace_type,
                          pair.ligand.ace_type)
    rs = O.receptor_spectra(rg, workers=8)
    with _ctx(dims, O.TERMS_SHAPE_ACE, pair.ace) as s:
        assert s.grid_dims == tuple(dims)
        s.set_receptor(pair.receptor.xyz, pair.receptor.ace_type)
        s.set_ligand(pair.ligand.xyz, pair.ligand.ace_type)
        for t in range(rg.shape[0]):
            assert np.allclose(s.receptor_grid(t), rg[t], rtol=1e-12, atol=1e-12)
        corr = s.correlation_grid(pair.rotations[0]).astype(np.float64)
    ref = O.scan_rotation(geom, rg, rs, pair.ligand.xyz, w, pair.rotations[0], 4, keep_corr=True, workers=8).corr
    assert corr.shape == ref.shape
    err = np.abs(corr - ref).max()
    assert err <= REL * np.abs(ref).max(), (err, np.abs(ref).max())


@pytest.mark.parametrize("mode", ["fft", "tensor"])
@pytest.mark.parametrize("dims,term_set", [((90, 96, 100), O.TERMS_SHAPE), ((84, 90, 78), O.TERMS_SHAPE_ACE),
                                           ((100, 100, 100), O.TERMS_SHAPE), ((88, 104, 91), O.TERMS_SHAPE),
                                           ((126, 112, 120), O.TERMS_SHAPE_ACE)])
def test_box_grid_peaks_vs_live_oracle(dims, term_set, mode):
    """Peaks of uneven grids at the sizes findBestSize returns (including
    factors 11 and 13, 88 = 8 x 11, 104 = 8 x 13, 91 = 7 x 13) and of a cubic
    edge without compiled plans, against the live FP64 oracle, through both
    pencil-stage forms."""
    from proddl2_gb300 import synth
    pair = synth.make_pair(1500, 400, 3, seed=81 + dims[2])
    geom, rg, w = _oracle(dims, term_set, pair.ace, pair.receptor.xyz, pair.receptor.ace_type, pair.ligand.ace_type)
    rs = O.receptor_spectra(rg, workers=8)
    with _ctx(dims, term_set, pair.ace, pencil_mode=mode) as s:
        s.set_receptor(pair.receptor.xyz, pair.receptor.ace_type)
        s.set_ligand(pair.ligand.xyz, pair.ligand.ace_type)
        assert s.info()["pencil_path"] == mode
        res = s.scan(pair.rotations)
        cand = s.candidates(pair.rotations)
    assert np.all(res.n_peaks == 4)
    for i, rot in enumerate(pair.rotations):
        _peaks_match(res, i, geom, rg, rs, pair.ligand.xyz, w, rot, 4, cand)


def test_box_grid_at_the_frame_setup_sizes():
    """The drop-in sizing: the pre-scan frame set-up's per-axis FFT sizes
    (findBestSize over the padded receptor box) used as they are, the atoms
    in the frames it returns, against the oracle on the same geometry."""
    from proddl2_gb300 import FFTScan, ScanConfig, synth
    from proddl2_gb300.frame import frame_setup
    from proddl2_gb300.scan import supported_dims
    pair = synth.make_pair(1200, 300, 3, seed=91)
    # an elongated receptor, so that the three sizes differ (77 x 63 x 55)
    rec = pair.receptor.xyz * np.array([1.5, 1.0, 0.8])
    fr = frame_setup(rec, pair.ligand.xyz, grid_step=1.2, cut_off_fft=6.0)
    dims = fr.fft_size
    assert len(set(dims)) == 3 and supported_dims(dims)
    geom, rg, w = _oracle(dims, O.TERMS_SHAPE_ACE, pair.ace, fr.rec_xyz, pair.receptor.ace_type,
                          pair.ligand.ace_type)
    rs = O.receptor_spectra(rg, workers=8)
    with FFTScan(ScanConfig(grid_dims=dims, grid_step=1.2, term_set="shape_ace", peaks_per_rot=4,
                            ace_matrix=pair.ace)) as s:
        s.set_receptor(fr.rec_xyz, pair.receptor.ace_type)
        s.set_ligand(fr.lig_xyz, pair.ligand.ace_type)
        res = s.scan(pair.rotations)
    for i, rot in enumerate(pair.rotations):
        _peaks_match(res, i, geom, rg, rs, fr.lig_xyz, w, rot, 4)


def test_box_grid_ljcomp_vs_oracle():
    """The reference's default potential (ljComp, weighted ligand entries) on
    an uneven grid."""
    from proddl2_gb300 import FFTScan, ScanConfig, synth
    dims = (48, 54, 50)
    pair = synth.make_pair(500, 120, 3, seed=101)
    rng = np.random.Generator(np.random.PCG64(5))
    lj = O.LjParams(rec_sigma=rng.uniform(3.0, 3.9, 500), rec_eps=rng.uniform(0.05, 0.6, 500),
                    rec_alpha=np.full(500, 0.4), lig_sigma=rng.uniform(3.0, 3.9, 120),
                    lig_eps=rng.uniform(0.05, 0.6, 120), mix=1, cut=9.0)
    geom = O.Geometry.centred(1.2, dims)
    rg = O.lj_receptor_terms(geom, pair.receptor.xyz, lj, O.TERMS_LJ_COMP)
    w = O.lj_ligand_weights(lj, O.TERMS_LJ_COMP)
    rs = O.receptor_spectra(rg, workers=8)
    with FFTScan(ScanConfig(grid_dims=dims, grid_step=1.2, term_set="lj_comp", peaks_per_rot=4, lj_cut=9.0)) as s:
        s.set_pair_lj(pair.receptor.xyz, lj.rec_sigma, lj.rec_eps, lj.rec_alpha, pair.ligand.xyz, lj.lig_sigma,
                      lj.lig_eps)
        for t in range(2):
            assert np.allclose(s.receptor_grid(t), rg[t], rtol=1e-12, atol=1e-9)
        res = s.scan(pair.rotations)
    for i, rot in enumerate(pair.rotations):
        _peaks_match(res, i, geom, rg, rs, pair.ligand.xyz, w, rot, 4)


def test_box_grid_out_of_grid_and_batches():
    """Out-of-grid rotations are reported per rotation; batch size does not
    change the peaks."""
    from proddl2_gb300 import FFTDockError, _lib, synth
    dims = (36, 40, 45)
    pair = synth.make_pair(250, 50, 5, seed=111)
    outs = []
    for batch in (1, 3, 64):
        with _ctx(dims, O.TERMS_SHAPE_ACE, pair.ace, rot_batch=batch) as s:
            s.set_receptor(pair.receptor.xyz, pair.receptor.ace_type)
            s.set_ligand(pair.ligand.xyz, pair.ligand.ace_type)
            outs.append(s.scan(pair.rotations))
    for r in outs[1:]:
        assert np.array_equal(r.peaks, outs[0].peaks)
    geom = O.Geometry.centred(1.2, dims)
    lig = np.array(pair.ligand.xyz) + np.array([0.0, 0.0, geom.spatial_domain()[1][2] - 1.0])
    with _ctx(dims, O.TERMS_SHAPE_ACE, pair.ace) as s:
        s.set_receptor(pair.receptor.xyz, pair.receptor.ace_type)
        s.set_ligand(lig, pair.ligand.ace_type)
        with pytest.raises(FFTDockError) as ei:
            s.scan(pair.rotations)
        assert ei.value.code == _lib.FFTDOCK_EOUT_OF_GRID


def test_box_grid_forms_agree_over_many_sizes():
    """Both pencil-stage forms on 15 box grids drawn from the sizes findBestSize
    can return (x from 10 to 128, including odd and 11/13-factor lengths, and
    three with x above 128, up to 250, where the tensor stage takes two
    128-row output tiles), 48 rotations each: wherever the top-4 lists differ, every cell of either list
    is adjudicated with its FP64 direct-space energy (each form must hold
    every cell of the union's best four below the 4th by more than the tie
    tolerance), and every reported score is the exact energy of its cell."""
    from proddl2_gb300 import FFTScan, ScanConfig, synth
    from proddl2_gb300.scan import supported_dims
    rng = np.random.Generator(np.random.PCG64(2024))
    sizes = [n for n in range(10, 129) if supported_dims((n, n, n))]
    checked = 0
    for case in range(15):
        dims = tuple(int(v) for v in rng.choice([n for n in sizes if n >= 40], size=3))
        dims = (int(rng.choice(sizes[:8])) if case < 2 else dims[0],) + dims[1:]
        if case >= 12:
            dims = ((150, 52, 44), (176, 60, 65), (250, 40, 42))[case - 12]
        # molecules that fit the smallest axis (the first two grids are thin)
        pair = synth.make_pair(600, 120, 48, seed=300 + case) if case >= 2 else \
            synth.make_pair(150, 12, 48, seed=300 + case)
        geom, rg, w = _oracle(dims, O.TERMS_SHAPE_ACE, pair.ace, pair.receptor.xyz, pair.receptor.ace_type,
                              pair.ligand.ace_type)
        res = {}
        for mode in ("fft", "tensor"):
            with FFTScan(ScanConfig(grid_dims=dims, grid_step=1.2, term_set="shape_ace", peaks_per_rot=4,
                                    ace_matrix=pair.ace, pencil_mode=mode)) as s:
                s.set_receptor(pair.receptor.xyz, pair.receptor.ace_type)
                s.set_ligand(pair.ligand.xyz, pair.ligand.ace_type)
                assert s.info()["pencil_path"] == mode, dims
                res[mode] = s.scan(pair.rotations, raise_out_of_grid=False)
        ok = (res["fft"].n_peaks == 4) & (res["tensor"].n_peaks == 4)
        nx, ny, nz = dims
        for i in np.nonzero(ok)[0]:
            cells, _ = O.bin_ligand(geom, pair.rotations[i], pair.ligand.xyz)
            lists, exact = {}, {}
            for mode in ("fft", "tensor"):
                cell, _, score = res[mode].rotation(i)
                offs = [int((c[0] * ny + c[1]) * nz + c[2]) for c in cell]
                lists[mode] = set(offs)
                if mode == "tensor" or np.any(res["fft"].peaks["cell"][i] != res["tensor"].peaks["cell"][i]):
                    for o, c, sc in zip(offs, cell, score):
                        e = O.direct_score(rg, cells, w, c)
                        assert abs(e - sc) <= 1e-9 * max(1.0, abs(e)), (dims, mode, i, sc, e)
                        exact[o] = e
            if lists["fft"] == lists["tensor"]:
                checked += 1
                continue
            best = sorted(exact.items(), key=lambda t: (t[1], t[0]))[:4]
            last = best[-1][1]
            tie = REL * max(1.0, abs(last))
            for mode in ("fft", "tensor"):
                for o, e in best:
                    if e < last - tie:
                        assert o in lists[mode], (dims, mode, i, o, e, last)
            checked += 1
    assert checked >= 15 * 24, checked
