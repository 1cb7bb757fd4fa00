"""The CPU oracle checked against the vectors of the reference's own unit tests.

These pin the parts of the scan path the reference tests do cover: the
bounded priority queue, the FFT size rule, grid domain conventions, the scan
record format and the rotation-file loader.  Score parity itself is unpinned
(the reference ships no score fixtures and cannot be built here); the last
tests check the oracle's FFT correlation against its independent exact
direct-space scorer.
"""
import math
import os

import numpy as np
import pytest

from oracle import fftdock_oracle as O


def test_queue_semantics_match_reference_test():
    # src/PRODDL/Common/test_queue.cpp:21-99
    q = O.BoundPriorityQueue(4, 10)
    for x in (1, 5, 11, 12, 4, 3, -5, 2):
        q.push(x)
    assert q.size() == 4
    assert q.top() == 3
    assert q.sort() == [-5, 1, 2, 3]
    q.clear()
    assert q.size() == 0
    q.push(2)
    assert q.top() == 2
    q.pop()
    assert q.size() == 0
    for x in (5, 4, 12, 1, 2):
        q.push(x)
    assert q.size() == 4


def _sieve(n_numbers, primes):
    # numbers[i] != 0 iff i factors completely over `primes` (test_pfactors.cpp)
    out = [0] * n_numbers
    for i in range(2, n_numbers):
        r = i
        for p in primes:
            while r % p == 0:
                r //= p
        out[i] = 1 if r == 1 else 0
    return out


def test_find_first_prime_factoring_matches_sieve():
    # src/PRODDL/Math/test_pfactors.cpp:73-132
    primes = (2, 3, 5, 7, 11, 13)
    n_numbers = 1024
    numbers = _sieve(n_numbers, primes)
    for i in range(n_numbers):
        nxt = next((j for j in range(i, n_numbers) if numbers[j]), n_numbers)
        ok, n, exps = O.find_first_prime_factoring(i, n_numbers, primes)
        if nxt < n_numbers:
            assert ok and n == nxt
            assert math.prod(p ** e for p, e in zip(primes, exps)) == n
            if exps[4] + exps[5] <= 1:
                assert O.find_best_size(i) == n
        else:
            assert not ok


def test_find_best_size_skips_11_13_products():
    # 143 = 11 * 13 is not an FFTW-friendly size; 121 = 11^2 neither
    assert O.find_best_size(143) == 144
    assert O.find_best_size(121) == 125
    assert O.find_best_size(97) == 98


def test_grid_domain_conventions():
    # src/PRODDL/Grid/test_grid.cpp:65-76: step 20, shape (50,51,51)
    # -> spatial domain [-500, 500] x [-510, 510]^2
    for n, lo in ((50, -500.0), (51, -510.0)):
        g = O.Geometry.centred(20.0, n)
        assert g.spatial_domain() == (lo, -lo)
        # cell centres, and the truncating toLogical on them and at the edges
        assert g.to_spatial(0) == lo + 10.0
        assert int(g.to_logical(g.to_spatial(7))) == 7
        assert int(g.to_logical(lo + 1e-9)) == 0
        assert int(g.to_logical(-lo - 1e-9)) == n - 1
        assert int(g.to_logical(lo - 1e-9)) < 0
        assert int(g.to_logical(-lo + 1e-9)) >= n


def test_box_grid_domain_conventions():
    # src/PRODDL/Grid/test_grid.cpp:65-76 itself: step 20, shape (50, 51, 51)
    # -> spatial domain [-500, 500] x [-510, 510] x [-510, 510]
    g = O.Geometry.centred(20.0, (50, 51, 51))
    lo, hi = g.spatial_domain()
    assert list(lo) == [-500.0, -510.0, -510.0] and list(hi) == [500.0, 510.0, 510.0]
    p = np.array([[-500 + 1e-9, -510 + 1e-9, 510 - 1e-9], [500 - 1e-9, 0.0, -510 - 1e-9]])
    assert g.to_logical(p).tolist() == [[0, 0, 50], [49, 25, -1]]
    assert g.to_spatial(0, 1) == -500.0 and g.to_spatial(0, 0) == -490.0


def test_box_grid_fft_correlation_equals_direct_scores():
    """On a grid whose three sizes differ (FFT sizes chosen per axis), the
    oracle's FFT correlation equals its exact direct-space energies, and a
    translation stands for h * unwrap(cell) per axis."""
    from proddl2_gb300 import synth
    pair = synth.make_pair(220, 50, 2, seed=61)
    geom = O.Geometry.centred(1.2, (24, 30, 28))
    tp = O.TermParams(term_set=O.TERMS_SHAPE_ACE, ace_matrix=pair.ace)
    rg = O.receptor_terms(geom, pair.receptor.xyz, pair.receptor.ace_type, tp)
    assert rg.shape == (18, 24, 30, 28)
    rs = O.receptor_spectra(rg)
    w = O.ligand_term_weights(pair.ligand.ace_type, tp)
    for rot in pair.rotations:
        res = O.scan_rotation(geom, rg, rs, pair.ligand.xyz, w, rot, 6, keep_corr=True)
        assert res.in_grid
        cells, _ = O.bin_ligand(geom, rot, pair.ligand.xyz)
        for off, c, s in zip(res.offsets, res.cells, res.scores):
            assert np.array_equal(O.offsets_to_cells([off], geom.dims)[0], c)
            assert abs(O.direct_score(rg, cells, w, c) - s) <= 1e-9 * max(1.0, abs(s))
        # a few arbitrary cells of the whole correlation grid
        rng = np.random.default_rng(1)
        for c in rng.integers(0, [24, 30, 28], size=(5, 3)):
            assert abs(O.direct_score(rg, cells, w, c) - res.corr[tuple(c)]) <= 1e-9 * max(1.0, abs(res.corr[tuple(c)]))
        t = O.translation(res.cells, geom)
        assert np.all(t / 1.2 >= -np.array([12, 15, 14])) and np.all(t / 1.2 < np.array([12, 15, 14]))


def test_scan_record_roundtrip():
    # src/PRODDL/IO/test_dock_io_bin.cpp:41-104 (identity rotation, 2 records)
    rot = np.eye(3)
    t = np.array([[2.0, 2.0, 2.0], [0.0, 0.0, 0.0]])
    data = O.pack_record(rot, t, [1.0, 2.0]) + O.pack_record(rot, t, [1.0, 3.0])
    recs = O.unpack_records(data)
    assert len(recs) == 2
    assert recs[0][2][1] == 2.0 and recs[1][2][1] == 3.0
    assert np.array_equal(recs[0][0], rot)
    # one record: 4 + 72 + 8 + n*32 bytes
    assert len(O.pack_record(rot, t, [1.0, 2.0])) == 4 + 72 + 8 + 2 * 32
    with pytest.raises(ValueError):
        O.unpack_records(b"\x00\x00\x00\x00" + data[4:])


def test_rotation_file_loader_tolerates_short_final_read():
    text = "3   Scan angles\n 0 0 0\n 90 0 0\n"
    mats = O.load_rotational_grid(text)
    assert mats.shape == (3, 3, 3)
    assert np.allclose(mats[0], np.eye(3))
    assert np.allclose(mats[1], [[0, 1, 0], [-1, 0, 0], [0, 0, 1]], atol=1e-12)
    assert np.array_equal(mats[2], mats[1])


def test_euler_matrix_is_orthonormal():
    rng = np.random.default_rng(0)
    for _ in range(10):
        m = O.euler_to_matrix(rng.uniform(-3, 3, 3))
        assert np.allclose(m @ m.T, np.eye(3), atol=1e-12)
        assert abs(np.linalg.det(m) - 1) < 1e-12


def test_unwrap_matches_reference_rule():
    # WrappedIndex::unwrap (Math/fft.hpp:199-206): y = -x; y += n if y < -(n/2)
    for n in (7, 8, 48, 128):
        x = np.arange(n)
        y = O.unwrap(x, n)
        assert y.min() == -(n // 2)
        assert y.max() == n - n // 2 - 1
        assert np.all((y + x) % n == 0)
        assert np.all(y >= -(n // 2)) and np.all(y < n - n // 2)


def _small_pair(seed, n_rec=250, n_lig=60):
    from proddl2_gb300 import synth
    return synth.make_pair(n_rec, n_lig, 3, seed=seed)


@pytest.mark.parametrize("term_set", [O.TERMS_SHAPE, O.TERMS_SHAPE_ACE])
def test_fft_correlation_equals_direct_space(term_set):
    pair = _small_pair(11)
    geom = O.Geometry.centred(1.2, 32)
    tp = O.TermParams(term_set=term_set, ace_matrix=pair.ace)
    rg = O.receptor_terms(geom, pair.receptor.xyz, pair.receptor.ace_type, tp)
    rs = O.receptor_spectra(rg)
    w = O.ligand_term_weights(pair.ligand.ace_type, tp)
    rng = np.random.default_rng(5)
    for rot in pair.rotations:
        res = O.scan_rotation(geom, rg, rs, pair.ligand.xyz, w, rot, 4, keep_corr=True)
        cells, ok = O.bin_ligand(geom, rot, pair.ligand.xyz)
        assert ok
        for c in list(res.cells) + [rng.integers(0, 32, 3) for _ in range(4)]:
            d = O.direct_score(rg, cells, w, c)
            v = res.corr[tuple(c)]
            assert abs(v - d) <= 1e-9 * max(1.0, abs(d))


def test_folded_terms_equal_unfolded():
    pair = _small_pair(12)
    geom = O.Geometry.centred(1.2, 32)
    tp = O.TermParams(term_set=O.TERMS_SHAPE_ACE, ace_matrix=pair.ace)
    rf = O.receptor_terms(geom, pair.receptor.xyz, pair.receptor.ace_type, tp, folded=True)
    ru = O.receptor_terms(geom, pair.receptor.xyz, pair.receptor.ace_type, tp, folded=False)
    wf = O.ligand_term_weights(pair.ligand.ace_type, tp, folded=True)
    wu = O.ligand_term_weights(pair.ligand.ace_type, tp, folded=False)
    cells, _ = O.bin_ligand(geom, pair.rotations[0], pair.ligand.xyz)
    for s in ([0, 0, 0], [3, 30, 7], [16, 16, 16]):
        a = O.direct_score(rf, cells, wf, s)
        b = O.direct_score(ru, cells, wu, s)
        assert abs(a - b) <= 1e-9 * max(1.0, abs(a))


def test_select_minima_queue_semantics():
    rng = np.random.default_rng(3)
    c = rng.integers(-5, 5, size=(6, 6, 6)).astype(float)
    offs, vals = O.select_minima(c, 7, max_val=-2.5)
    # the reference's queue compares values only; the key adds the oracle's offset tie-break
    q = O.BoundPriorityQueue(7, (-2.5, -1), key=lambda i: (c.reshape(-1)[i], i))
    for i in range(c.size):
        q.push(i)
    assert list(offs) == q.sort()
    assert np.all(vals < -2.5)
    assert np.all(np.diff(vals) >= 0)


def test_transform_algebra_matches_reference_test():
    # src/PRODDL/Geom/test_transformation.cpp:20-50
    cm = np.array([5.0, 4.0, 3.0])
    v_trans = np.array([1.0, 2.0, 3.0])
    m1 = np.array([[0, 1, 1], [0.2, 0.3, 0.4], [1, 0.3, 0.5]])
    m2 = np.array([[0.4, 1.7, 1.8], [0.7, 0.9, 0.3], [1.3, 0.1, 0.9]])
    ident = np.eye(3)
    zero = np.zeros(3)
    # Rot(m2) * Tran(cm + v) * (Rot(m1) * Tran(0 - cm)), then inverse
    inner = O.rt_compose((m1, zero), (ident, 0.0 - cm))
    rt = O.rt_compose((m2, zero), O.rt_compose((ident, cm + v_trans), inner))
    r, v = O.rt_inverse(rt)
    assert np.allclose(r, [[2.14, 0.48, 0.92], [1.45, 1.06, 1.6], [1.98, 1.21, 1.79]])
    assert np.allclose(v, [-0.2324, 1.5222, 1.3322])


def test_euler_round_trip():
    rng = np.random.default_rng(2)
    for _ in range(20):
        ang = rng.uniform(-1.4, 1.4, 3)
        m = O.euler_to_matrix(ang)
        # rotMatrToEulerAng inverts eulerAngToRotMatr (with its angle order swap)
        m2 = O.euler_to_matrix(O.matrix_to_euler(m))
        assert np.allclose(m, m2, atol=1e-12)


def test_gather_keeps_smallest_ascending():
    rng = np.random.default_rng(4)
    recs = []
    for i in range(6):
        rot = O.euler_to_matrix(rng.uniform(-1, 1, 3))
        n = int(rng.integers(0, 5))
        recs.append((rot, rng.normal(size=(n, 3)), rng.normal(size=n)))
    allv = sorted(v for _, _, vals in recs for v in vals)
    out = O.gather_records(recs, 7)
    assert [p[0] for p in out] == allv[:7]
    blob = O.pack_rigid(out, (np.eye(3), np.zeros(3)), (np.eye(3), np.zeros(3)))
    assert len(blob) == 8 + 28 * len(out)
