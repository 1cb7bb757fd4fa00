"""The reference's own FFT potentials ("ljComp", "ljAvg"): the restated
fields against the identity the reference states for them (with alpha = 0,
SoftCoreLJRep x sqrt(eps) sigma^6 + SoftCoreLJAttr x sqrt(eps) sigma^3 is the
pairwise LJ with geometric sigma mixing, potentials_inc.hpp:260-268) and the
force-shifted cutoff of SoftCoreLJ; on the GPU, receptor fields, correlation
grids and peaks against the FP64 oracle through fftdock_set_pair_lj."""
import math

import numpy as np
import pytest

from oracle import fftdock_oracle as O

REL = 1e-4


def _lj_inputs(n_rec, n_lig, seed, alpha=0.4):
    rng = np.random.Generator(np.random.PCG64(seed))
    return O.LjParams(rec_sigma=rng.uniform(3.0, 3.9, n_rec), rec_eps=rng.uniform(0.05, 0.6, n_rec),
                      rec_alpha=np.full(n_rec, alpha), lig_sigma=rng.uniform(3.0, 3.9, n_lig),
                      lig_eps=rng.uniform(0.05, 0.6, n_lig), mix=1, cut=9.0)


def test_ljcomp_halves_make_the_pairwise_lj_at_zero_alpha():
    lj = _lj_inputs(5, 7, 1, alpha=0.0)
    c = O.lj_atom_constants(lj, O.TERMS_LJ_COMP)
    w = O.lj_ligand_weights(lj, O.TERMS_LJ_COMP)
    for i in range(5):
        for j in range(7):
            for r in (3.1, 4.0, 6.5):
                r2 = r * r
                got = O.lj_field(c[i], r2, 0) * w[j, 0] + O.lj_field(c[i], r2, 1) * w[j, 1]
                s = math.sqrt(lj.rec_sigma[i] * lj.lig_sigma[j])
                e = math.sqrt(lj.rec_eps[i] * lj.lig_eps[j])
                ref = 4 * e * ((s / r) ** 12 - (s / r) ** 6)
                assert abs(got - ref) <= 1e-12 * max(1.0, abs(ref)), (got, ref)


def test_ljavg_energy_and_force_vanish_at_the_cutoff():
    lj = _lj_inputs(4, 6, 2)
    c = O.lj_atom_constants(lj, O.TERMS_LJ_AVG)
    cut2 = lj.cut * lj.cut
    for ci in c:
        f_cut = O.lj_field(ci, cut2, "avg")
        scale = abs(O.lj_field(ci, 16.0, "avg"))
        assert abs(f_cut) <= 1e-12 * max(scale, 1.0)
        d = 1e-4
        slope = (O.lj_field(ci, (lj.cut - d) ** 2, "avg") - O.lj_field(ci, (lj.cut - 2 * d) ** 2, "avg")) / d
        assert abs(slope) <= 1e-6 * max(scale, 1.0)


def test_reference_potential_names_select_the_lj_sets():
    from proddl2_gb300 import ScanConfig
    c = ScanConfig.from_options({"potentialName": "ljComp", "cutOffFft": 8.0})
    assert c.term_set == "lj_comp" and c.lj_cut == 8.0
    assert ScanConfig.from_options({"potentialName": "ljAvg"}).term_set == "lj_avg"


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def _case(term_set, n, n_rec, n_lig, n_rot, seed):
    from proddl2_gb300 import synth
    pair = synth.make_pair(n_rec, n_lig, n_rot, seed=seed)
    lj = _lj_inputs(n_rec, n_lig, seed + 7)
    geom = O.Geometry.centred(1.2, n)
    rg = O.lj_receptor_terms(geom, pair.receptor.xyz, lj, term_set)
    w = O.lj_ligand_weights(lj, term_set)
    return pair, lj, geom, rg, w


def _ctx(term_set, n, k=4, **kw):
    from proddl2_gb300 import FFTScan, ScanConfig
    name = {O.TERMS_LJ_COMP: "lj_comp", O.TERMS_LJ_AVG: "lj_avg"}[term_set]
    return FFTScan(ScanConfig(grid_n=n, grid_step=1.2, term_set=name, peaks_per_rot=k, lj_cut=9.0, **kw))


def _load(s, pair, lj):
    s.set_pair_lj(pair.receptor.xyz, lj.rec_sigma, lj.rec_eps, lj.rec_alpha, pair.ligand.xyz, lj.lig_sigma, lj.lig_eps)


@pytest.mark.gpu
@pytest.mark.parametrize("term_set", [O.TERMS_LJ_COMP, O.TERMS_LJ_AVG])
def test_lj_receptor_fields_and_correlation_grid(term_set):
    pair, lj, geom, rg, w = _case(term_set, 32, 250, 50, 2, 31)
    with _ctx(term_set, 32) as s:
        _load(s, pair, lj)
        assert s.n_terms == rg.shape[0]
        for t in range(rg.shape[0]):
            g = s.receptor_grid(t)
            assert np.allclose(g, rg[t], rtol=1e-12, atol=1e-12 * np.abs(rg[t]).max())
        c = s.correlation_grid(pair.rotations[0]).astype(np.float64)
    cells, _ = O.bin_ligand(geom, pair.rotations[0], pair.ligand.xyz)
    ref = O.correlate(O.receptor_spectra(rg), O.ligand_grids(geom, cells, w))
    assert np.abs(c - ref).max() <= REL * np.abs(ref).max()


@pytest.mark.gpu
@pytest.mark.parametrize("term_set,n", [(O.TERMS_LJ_COMP, 32), (O.TERMS_LJ_COMP, 48), (O.TERMS_LJ_AVG, 48)])
def test_lj_peaks_match_the_oracle(term_set, n):
    from test_gpu_parity import assert_peaks_match
    pair, lj, geom, rg, w = _case(term_set, n, {32: 250, 48: 600}[n], {32: 50, 48: 120}[n], 5, 40 + n)
    rs = O.receptor_spectra(rg, workers=8)
    with _ctx(term_set, n) as s:
        _load(s, pair, lj)
        res = s.scan(pair.rotations)
    for i, rot in enumerate(pair.rotations):
        ref = O.scan_rotation(geom, rg, rs, pair.ligand.xyz, w, rot, 4, workers=8)
        cells, _ = O.bin_ligand(geom, rot, pair.ligand.xyz)
        cell, _, score = res.rotation(i)
        off = (cell[:, 0] * n + cell[:, 1]) * n + cell[:, 2]
        exact = lambda o: O.direct_score(rg, cells, w, O.offsets_to_cells([o], n)[0])  # noqa: E731
        assert_peaks_match(off, score, ref.offsets, ref.scores, exact)


@pytest.mark.gpu
def test_lj_argument_rules():
    from proddl2_gb300 import FFTDockError, _lib
    pair, lj, _, _, _ = _case(O.TERMS_LJ_COMP, 32, 50, 20, 1, 3)
    with _ctx(O.TERMS_LJ_COMP, 32) as s:
        with pytest.raises(FFTDockError) as ei:
            s.set_receptor(pair.receptor.xyz)
        assert ei.value.code == _lib.FFTDOCK_EINVAL
        with pytest.raises(FFTDockError) as ei:
            s.set_pair_lj(pair.receptor.xyz, -lj.rec_sigma, lj.rec_eps, lj.rec_alpha, pair.ligand.xyz,
                          lj.lig_sigma, lj.lig_eps)
        assert ei.value.code == _lib.FFTDOCK_EINVAL
    with pytest.raises(FFTDockError) as ei:
        _ctx(O.TERMS_LJ_COMP, 32, lj_mix=0)
    assert ei.value.code == _lib.FFTDOCK_EINVAL
    with pytest.raises(FFTDockError) as ei:
        _ctx(O.TERMS_LJ_COMP, 32, precision="bf16")
    assert ei.value.code == _lib.FFTDOCK_EUNSUPPORTED
