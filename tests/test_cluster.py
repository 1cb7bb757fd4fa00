"""Translational clustering of each rotation's queue (TranClust,
``include/PRODDL/docking_fft.hpp:30-140`` over ``ClusterMatrix``,
``include/PRODDL/Geom/cluster.hpp:121-477``).

CPU: the oracle's leader clustering against the reference's own clustering
test (``src/PRODDL/Geom/test_cluster.cpp``: ten well separated sphere clusters
in nine columns must come out as ten clusters) and the walk-order rules.

GPU: the clustering scan through the C ABI.
* exact: given the FP32 correlation grid the GPU computes
  (``fftdock_correlation_grid``), the queue (lowest ``maxNTransInp`` cells
  below ``maxValCorr``, ties by offset) and the leaders are recomputed on the
  CPU with the oracle's clustering; cells and order must be identical;
* against the FP64 oracle: identical leaders for every rotation whose FP64
  queue has no two values (nor the queue bound) within the 1e-4 tolerance of
  each other; reported scores equal the exact FP64 energies to 1e-9;
* degenerate grids (all values equal, so the queue is decided by offsets
  alone) and queues with fewer cells than the bound.
"""
import math

import numpy as np
import pytest

from oracle import fftdock_oracle as O

REL = 1e-4


# ---------------------------------------------------------------------------
# CPU: oracle pins
# ---------------------------------------------------------------------------
def _sphere_clusters(seed, n_rows=1000, n_cols=9, n_clust=10, radius=1.0, min_dist=5.0, max_dist=7.0):
    """The generator of test_cluster.cpp:38-103, seeded: cluster centres in a
    cube of side max_dist * n_clust^(1/n_cols) at least min_dist apart, rows
    uniform in a ball of ``radius`` around their centre."""
    rng = np.random.Generator(np.random.PCG64(seed))
    box = max_dist * n_clust ** (1.0 / n_cols)
    centres = []
    while len(centres) < n_clust:
        c = rng.random(n_cols) * box
        if all(((c - o) ** 2).sum() >= min_dist ** 2 for o in centres):
            centres.append(c)
    rows = []
    for c in centres:
        for _ in range(n_rows // n_clust):
            while True:
                r = (rng.random(n_cols) - 0.5) * 2 * radius
                if (r * r).sum() <= radius * radius:
                    rows.append(r + c)
                    break
    return np.array(rows)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_oracle_finds_the_reference_tests_ten_clusters(seed):
    # test_cluster.cpp:105-131: weights 1, cutoff 2 * radius, 10 clusters
    m = _sphere_clusters(seed)
    leaders = O.cluster_leaders(m, 2.0, 10 ** 6, range(len(m) - 1, -1, -1))
    assert len(leaders) == 10
    # one leader per generated cluster
    assert sorted(int(i) // 100 for i in leaders) == list(range(10))


def test_neighbour_radius_is_sqrt3_times_the_option():
    # three clustered columns: cutoff2 = r^2 * 3 (cluster.hpp:153-156)
    r = 5.0
    assert O.cluster_radius2(r) == math.sqrt(75.0) ** 2
    t = np.array([[0.0, 0.0, 0.0], [8.6, 0.0, 0.0], [8.7, 0.0, 0.0]])
    v = np.array([-3.0, -2.0, -1.0])
    # walk from the worst: 8.7 leads, 8.6 joins it, 0 is 8.7 > sqrt(75) away and leads
    assert list(O.tran_cluster(t, v, r, 10)) == [2, 0]
    # best first: 0 leads, 8.6 <= 8.66 joins, 8.7 > 8.66 leads
    assert list(O.tran_cluster(t, v, r, 10, O.CLUSTER_ORDER_BEST_FIRST)) == [0, 2]


def test_reference_walk_starts_from_the_worst_value():
    # weights = -value sorted ascending (cluster.hpp:238-253): the queue's
    # last (worst) entry is the first leader
    t = np.array([[0, 0, 0], [1.2, 0, 0], [30, 0, 0], [31.2, 0, 0], [60, 0, 0]], dtype=float)
    v = np.array([-50.0, -40.0, -30.0, -20.0, -10.0])
    assert list(O.tran_cluster(t, v, 1.0, 10)) == [4, 3, 1]
    assert list(O.tran_cluster(t, v, 1.0, 2)) == [4, 3]
    assert list(O.tran_cluster(t, v, 1.0, 10, O.CLUSTER_ORDER_BEST_FIRST)) == [0, 2, 4]
    assert list(O.tran_cluster(t[:0], v[:0], 1.0, 10)) == []


def test_cluster_options_from_reference_names():
    from proddl2_gb300 import ScanConfig
    c = ScanConfig.from_options({"doClusterTranslations": True, "clusterRadiusTrans": 0.5, "maxNTransInp": 300})
    assert c.cluster_trans and c.cluster_radius == 0.5 and c.max_trans_inp == 300


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def _ctx(n, term_set, ace, m, radius, order="reference", k=4, max_val=float("inf"), batch=64):
    from proddl2_gb300 import FFTScan, ScanConfig
    return FFTScan(ScanConfig(grid_n=int(n), grid_step=1.2, term_set=term_set, peaks_per_rot=k, rot_batch=batch,
                              ace_matrix=ace, max_trans_inp=m, max_val_corr=max_val, cluster_trans=True,
                              cluster_radius=radius, cluster_order=order))


def _queue_from_grid(grid, m, max_val):
    """Lowest m cells of an FP32 grid below max_val, ties by offset."""
    flat = grid.reshape(-1)
    idx = np.nonzero(flat.astype(np.float64) < max_val)[0]
    vals = flat[idx]
    order = np.lexsort((idx, vals))[:m]
    return idx[order], vals[order]


def _expected_from_grid(grid, n, m, radius, k, order, max_val):
    geom = O.Geometry.centred(1.2, n)
    offs, vals = _queue_from_grid(grid, m, max_val)
    t = O.translation(O.offsets_to_cells(offs, n), geom)
    o = O.CLUSTER_ORDER_BEST_FIRST if order == "best_first" else O.CLUSTER_ORDER_REFERENCE
    keep = O.tran_cluster(t, vals, radius, k, o)
    return offs[keep]


def _peak_offsets(res, i, n):
    cell, _, _ = res.rotation(i)
    return (cell[:, 0] * n + cell[:, 1]) * n + cell[:, 2]


@pytest.mark.gpu
@pytest.mark.parametrize("m,radius,order,max_val", [
    (50, 2.0, "reference", float("inf")),
    (300, 5.0, "reference", float("inf")),
    (300, 5.0, "best_first", float("inf")),
    (2000, 1.0, "reference", -5.0),
])
def test_cluster_scan_exact_given_the_gpu_grid(m, radius, order, max_val):
    f = np.load(__import__("pathlib").Path(__file__).resolve().parent / "golden" / "scan_shape_ace_n32.npz")
    n = int(f["grid_n"])
    with _ctx(n, "shape_ace", f["ace"], m, radius, order, k=8, max_val=max_val) as s:
        s.set_receptor(f["rec_xyz"], f["rec_type"])
        s.set_ligand(f["lig_xyz"], f["lig_type"])
        res = s.scan(f["rotations"])
        grids = [s.correlation_grid(r) for r in f["rotations"]]
    geom, rg, w = _setup(n, f)
    for i, rot in enumerate(f["rotations"]):
        exp = _expected_from_grid(grids[i], n, m, radius, 8, order, max_val)
        got = _peak_offsets(res, i, n)
        assert list(got) == list(exp), (i, got, exp)
        cells, _ = O.bin_ligand(geom, rot, f["lig_xyz"])
        for o, sc in zip(got, res.rotation(i)[2]):
            e = O.direct_score(rg, cells, w, O.offsets_to_cells([o], n)[0])
            assert abs(sc - e) <= 1e-9 * max(1.0, abs(e))


def _setup(n, f):
    geom = O.Geometry.centred(1.2, n)
    tp = O.TermParams(term_set=int(f["term_set"]), ace_matrix=f["ace"])
    return geom, O.receptor_terms(geom, f["rec_xyz"], f["rec_type"], tp), O.ligand_term_weights(f["lig_type"], tp)


@pytest.mark.gpu
def test_cluster_scan_vs_fp64_oracle():
    from proddl2_gb300 import synth
    n, m, radius, k = 48, 40, 3.0, 4
    pair = synth.make_pair(700, 150, 12, seed=321)
    tp = O.TermParams(term_set=O.TERMS_SHAPE_ACE, ace_matrix=pair.ace)
    geom = O.Geometry.centred(1.2, n)
    rg = O.receptor_terms(geom, pair.receptor.xyz, pair.receptor.ace_type, tp)
    w = O.ligand_term_weights(pair.ligand.ace_type, tp)
    rs = O.receptor_spectra(rg, workers=8)
    with _ctx(n, "shape_ace", pair.ace, m, radius, k=k) as s:
        s.set_receptor(pair.receptor.xyz, pair.receptor.ace_type)
        s.set_ligand(pair.ligand.xyz, pair.ligand.ace_type)
        res = s.scan(pair.rotations)
    rad2 = O.cluster_radius2(radius)
    checked = 0
    for i, rot in enumerate(pair.rotations):
        cells, _ = O.bin_ligand(geom, rot, pair.ligand.xyz)
        got = _peak_offsets(res, i, n)
        _, t_got, sc_got = res.rotation(i)
        for o, sc in zip(got, sc_got):
            e = O.direct_score(rg, cells, w, O.offsets_to_cells([o], n)[0])
            assert abs(sc - e) <= 1e-9 * max(1.0, abs(e))
        for a in range(len(t_got)):
            for b in range(a):
                assert ((t_got[a] - t_got[b]) ** 2).sum() > rad2 * (1 - 1e-12)
        full = O.scan_rotation(geom, rg, rs, pair.ligand.xyz, w, rot, m + 1, workers=8)
        tol = REL * max(1.0, np.abs(full.scores).max())
        if np.any(np.diff(full.scores) <= tol):
            continue  # a near-tie inside the queue or at its bound can reorder the walk
        checked += 1
        ref = O.scan_rotation_clustered(geom, rg, rs, pair.ligand.xyz, w, rot, m, k, radius, workers=8)
        assert list(got) == list(ref.offsets), (i, got, ref.offsets)
        assert np.allclose(sc_got, ref.scores, rtol=REL, atol=REL)
    assert checked >= len(pair.rotations) // 3, checked


@pytest.mark.gpu
def test_cluster_scan_all_equal_values_resolved_by_offset():
    # empty receptor: every correlation value is 0; the queue is the m lowest
    # offsets and the radix select has to resolve all of it in the offset bits
    n, m, radius, k = 32, 700, 2.0, 16
    geom = O.Geometry.centred(1.2, n)
    with _ctx(n, "shape", None, m, radius, k=k) as s:
        s.set_receptor(np.zeros((0, 3)))
        s.set_ligand(np.zeros((1, 3)))
        res = s.scan(np.eye(3)[None])
    offs = np.arange(m)
    t = O.translation(O.offsets_to_cells(offs, n), geom)
    exp = offs[O.tran_cluster(t, np.zeros(m), radius, k)]
    assert list(_peak_offsets(res, 0, n)) == list(exp)
    assert list(res.rotation(0)[2]) == [0.0] * len(exp)


@pytest.mark.gpu
def test_cluster_context_rejects_candidate_pool_and_noalloc():
    import torch
    from proddl2_gb300 import FFTDockError, _lib
    f = np.load(__import__("pathlib").Path(__file__).resolve().parent / "golden" / "scan_shape_ace_n32.npz")
    with _ctx(32, "shape_ace", f["ace"], 100, 5.0) as s:
        s.set_receptor(f["rec_xyz"], f["rec_type"])
        s.set_ligand(f["lig_xyz"], f["lig_type"])
        with pytest.raises(FFTDockError) as ei:
            s.candidates(f["rotations"])
        assert ei.value.code == _lib.FFTDOCK_EUNSUPPORTED
        rot = torch.as_tensor(f["rotations"].reshape(-1, 9), device="cuda")
        pk = torch.zeros((rot.shape[0], 4 * 48), dtype=torch.uint8, device="cuda")
        npk = torch.zeros(rot.shape[0], dtype=torch.int32, device="cuda")
        with pytest.raises(FFTDockError) as ei:
            s.scan_device_noalloc(rot.data_ptr(), rot.shape[0], pk.data_ptr(), npk.data_ptr())
        assert ei.value.code == _lib.FFTDOCK_EUNSUPPORTED


@pytest.mark.gpu
def test_cluster_queue_bound_checks():
    from proddl2_gb300 import FFTDockError, _lib
    with pytest.raises(FFTDockError) as ei:
        _ctx(32, "shape", None, _lib.FFTDOCK_MAX_QUEUE_CLUSTERED + 1, 5.0)
    assert ei.value.code == _lib.FFTDOCK_EINVAL


@pytest.mark.gpu
@pytest.mark.parametrize("m,k", [(10000, 10), (400, 4)])
def test_cluster_full_size_128_reference_options(m, k):
    """shape_ace128 inputs with the reference's option values (maxNTransInp
    10000 with maxNTrans 10 from its option generator, and its default
    maxNTrans * 100; clusterRadiusTrans 5): exact against the queue
    recomputed from the GPU grid for two rotations, leaders separated for
    all."""
    from proddl2_gb300 import synth
    n, radius = 128, 5.0
    pair = synth.make_pair(4000, 1500, 64, seed=11)
    with _ctx(n, "shape_ace", pair.ace, m, radius, k=k) as s:
        s.set_receptor(pair.receptor.xyz, pair.receptor.ace_type)
        s.set_ligand(pair.ligand.xyz, pair.ligand.ace_type)
        res = s.scan(pair.rotations)
        grids = [s.correlation_grid(pair.rotations[i]) for i in (0, 37)]
    for g, i in zip(grids, (0, 37)):
        exp = _expected_from_grid(g, n, m, radius, k, "reference", float("inf"))
        assert list(_peak_offsets(res, i, n)) == list(exp)
    rad2 = O.cluster_radius2(radius)
    for i in range(len(pair.rotations)):
        _, t, _ = res.rotation(i)
        assert len(t) == k
        d2 = ((t[:, None, :] - t[None, :, :]) ** 2).sum(-1)
        assert np.all(d2[~np.eye(len(t), dtype=bool)] > rad2 * (1 - 1e-12))
