"""CPU FP64 oracle for the PRODDL2 FFT rotational/translational correlation scan.

TEST INFRASTRUCTURE ONLY.  This module is the checker: the parity tests, the
smoke check and the CPU-baseline leg of ``bench.py`` import it.  The product
path (``proddl2_gb300`` + ``libfftdock.so``) never imports or calls it.

It restates, in numpy float64, the reference's ``rot-scan`` worker path
(``include/PRODDL/docking_app.hpp:450-466`` ``Worker::scanRotation`` ->
``findTranslationalMinima`` at ``:417-447``) with the reference's conventions:

* centred grid geometry and the truncating ``toLogical`` used for ligand
  binning (``include/PRODDL/Grid/gridcoord.hpp:127-191``,
  ``include/PRODDL/Grid/grid.hpp:442-451``);
* receptor radial-field projection on cell centres inside the cropped
  ``toLogical(c +- cut)`` box, with ``r^2`` clamped to ``(h/4)^2``
  (``include/PRODDL/Grid/project.hpp:51-176``,
  ``include/PRODDL/docking_molforce.hpp:298-320``);
* ligand point scatter ``grid(cell(p')) += w`` after ``p' = R p``
  (``docking_molforce.hpp:351-368``, ``Geom/transformation.hpp:206-222``,
  matrix-vector order of ``Blitz/bztinyvec.hpp:52-65``);
* per-term correlation ``C = IFFT(conj(FFT R) * FFT L) / V`` summed over the
  terms in real space (``docking_fft.hpp:622-633``, ``:812-819``,
  ``docking_molforce.hpp:249-269``);
* selection of the ``k`` smallest values below ``maxValCorr`` in ascending
  order (``docking_fft.hpp:316-345,452-468``, ``Common/queue.hpp:221-251``),
  ties broken by the cell's flat offset;
* offset -> translation through ``WrappedIndex::unwrap`` and ``toSpatialDiff``
  (``docking_fft.hpp:368-389``, ``Math/fft.hpp:199-206``,
  ``Grid/gridcoord.hpp:150``).

Parity status.  The reference cannot be built or run here (FFTW3, Blitz++,
Boost and HDF5 are absent) and ships no golden vectors for correlation scores,
so score parity is *unpinned*: it rests on this restatement and on the
independent exact direct-space scorer :func:`direct_score`.  The parts the
reference's own unit tests do pin -- queue semantics
(``src/PRODDL/Common/test_queue.cpp:21-99``), the FFT size rule
(``src/PRODDL/Math/test_pfactors.cpp:73-132``), grid domain conventions
(``src/PRODDL/Grid/test_grid.cpp:65-76``) and the scan record format
(``src/PRODDL/IO/test_dock_io_bin.cpp:41-104``) -- are checked against those
tests' vectors in ``tests/test_oracle_pins.py``.

The shape (surface +1 / core -15) and 18-type ACE-style desolvation terms are
not in the reference's FFT path; they are this project's plug-in terms built
with the reference's radial-field projection mechanism, and this module is
their definition: receptor grid ``S`` (set, not summed), ``D_t`` sums of the
``PotAce`` sigmoid (``include/PRODDL/potentials_inc.hpp:357-406``, no cut
shift), ligand grids of unit weights, total score
``-corr(S, L) + sum_t corr(D_t, L_t)``, folded to ``sum_t corr(D_t - S, L_t)``.
"""
from __future__ import annotations

import heapq
import math
import struct
from dataclasses import dataclass, field

import numpy as np

# ----------------------------------------------------------------------------
# Term sets (mirrors the C ABI enum in include/fftdock.h)
# ----------------------------------------------------------------------------
TERMS_SHAPE = 1        # K = 1: -S correlated with all ligand atoms
TERMS_SHAPE_ACE = 2    # K = n_types (folded): D_t - S correlated with type-t atoms
TERMS_LJ_COMP = 3      # "ljComp": soft-core LJ repulsion + attraction, K = 2
TERMS_LJ_AVG = 4       # "ljAvg": soft-core LJ with ligand-averaged parameters, K = 1

SHAPE_SURFACE = 1.0
SHAPE_CORE = -15.0


# ----------------------------------------------------------------------------
# FFT size rule: Math/pfactors.hpp:29-57, Math/fft.hpp:82-168, Math/fft.cc:8
# ----------------------------------------------------------------------------
FFTW_PRIMES = (2, 3, 5, 7, 11, 13)


def find_first_prime_factoring(start_n, end_n, primes=FFTW_PRIMES):
    """First N in [max(start_n, 2), end_n) that factors over ``primes``.

    Returns ``(found, N, exponents)`` (``Math/pfactors.hpp:29-57``)."""
    n0 = 2 if start_n <= 1 else start_n
    for n_cand in range(n0, end_n):
        rem = n_cand
        exps = []
        for p in primes:
            e = 0
            while rem % p == 0:
                rem //= p
                e += 1
            exps.append(e)
            if rem == 1:
                exps += [0] * (len(primes) - len(exps))
                return True, n_cand, exps
    return False, None, None


def find_best_size(start_n, end_n=2**31 - 1):
    """``FFTW_Size::findBestSize`` (``Math/fft.hpp:82-115,141-151``): first size
    >= start_n over {2,3,5,7,11,13} with exp(11) + exp(13) <= 1."""
    while True:
        ok, n, exps = find_first_prime_factoring(start_n, end_n)
        if not ok:
            return None
        if exps[4] + exps[5] <= 1:
            return n
        start_n = n + 1


# ----------------------------------------------------------------------------
# BoundPriorityQueue: Common/queue.hpp:49-280
# ----------------------------------------------------------------------------
class _MaxItem:
    """Heap entry ordered so that heapq's min-heap keeps the largest key on top."""
    __slots__ = ("key", "seq", "item")

    def __init__(self, key, seq, item):
        self.key, self.seq, self.item = key, seq, item

    def __lt__(self, other):
        return other.key < self.key or (not self.key < other.key and self.seq > other.seq)


class BoundPriorityQueue:
    """Keeps at most ``size_limit`` smallest items whose key is < ``max_val``.

    Same push/sort semantics as the reference (``queue.hpp:221-251,184-193``):
    an item is dropped unless ``key(x) < max_val``; when full, it replaces the
    current largest only if strictly smaller.  ``sort()`` returns ascending."""

    def __init__(self, size_limit, max_val, key=lambda x: x):
        if size_limit <= 0:
            raise ValueError("size_limit must be > 0")
        self.size_limit = size_limit
        self.max_val = max_val
        self.key = key
        self._heap = []
        self._seq = 0

    def push(self, x):
        k = self.key(x)
        if not (k < self.max_val):
            return
        e = _MaxItem(k, self._seq, x)
        self._seq += 1
        if len(self._heap) >= self.size_limit:
            if k < self._heap[0].key:
                heapq.heapreplace(self._heap, e)
            return
        heapq.heappush(self._heap, e)

    def top(self):
        return self._heap[0].item

    def pop(self):
        heapq.heappop(self._heap)

    def size(self):
        return len(self._heap)

    def clear(self):
        self._heap = []

    def sort(self):
        return [e.item for e in sorted(self._heap, key=lambda e: (e.key, e.seq))]


# ----------------------------------------------------------------------------
# Grid geometry: Grid/gridcoord.hpp:127-191
# ----------------------------------------------------------------------------
@dataclass(frozen=True)
class Geometry:
    """Centred grid of cubic cells; the logical size may differ per axis
    (``fftSize`` is a 3-vector, ``docking_fft.hpp:541-553``).  For a cubic
    grid the scalar fields describe every axis; ``dims``/``zeros`` always
    hold the per-axis sizes and low corners."""
    h: float
    n: int            # the edge of a cubic grid (the x size of a box grid)
    zero: float       # spatial coordinate of the grid's low corner (x axis)
    zero_h: float     # zero - h, used by toLogical (x axis)
    center0: float    # centre of cell 0 (x axis)
    dims: tuple = ()  # (nx, ny, nz)
    zeros: tuple = ()  # per-axis low corner

    @staticmethod
    def centred(h, n):
        """``UniformCubicGeometry(step, logicalSize)`` (gridcoord.hpp:127-142),
        per axis: zero = -(toSpatialRight(n - 1) - toSpatialLeft(0)) / 2;
        ``n`` is one edge or (nx, ny, nz)."""
        h = float(h)
        dims = (int(n),) * 3 if np.ndim(n) == 0 else tuple(int(v) for v in n)
        zeros = []
        for nd in dims:
            s_upper = h + h * float(nd - 1)   # toSpatialRight(n-1) with zero 0
            s_size = s_upper - 0.0
            zeros.append((-1.0 * s_size) / 2.0)
        z = zeros[0]
        return Geometry(h=h, n=dims[0], zero=z, zero_h=z - h, center0=z + h / 2.0, dims=dims, zeros=tuple(zeros))

    @property
    def cubic(self):
        return self.dims[0] == self.dims[1] == self.dims[2]

    @property
    def volume(self):
        return self.dims[0] * self.dims[1] * self.dims[2]

    def to_logical(self, x):
        """``toLogical``: int((x - (zero - h)) / h) - 1, C truncation toward 0;
        on a box grid ``x`` is (..., 3) points."""
        x = np.asarray(x, dtype=np.float64)
        zh = self.zero_h if self.cubic else np.array(self.zeros) - self.h
        v = (x - zh) / self.h
        return np.trunc(v).astype(np.int64) - 1

    def to_spatial(self, i, axis=0):
        c0 = self.center0 if self.cubic else self.zeros[axis] + self.h / 2.0
        return c0 + self.h * np.asarray(i, dtype=np.float64)

    def spatial_domain(self):
        if self.cubic:
            return self.zero, self.zero + self.h * self.n
        z = np.array(self.zeros)
        return z, z + self.h * np.array(self.dims)


# ----------------------------------------------------------------------------
# Rotations: Geom/euler.hpp:38-52, Geom/rotational_grid.hpp:25-64
# ----------------------------------------------------------------------------
def euler_to_matrix(angles):
    """``Eu_xyz::eulerAngToRotMatr`` (euler.hpp:38-52), radians in."""
    a, b, g = (float(v) for v in angles)
    sa, ca, sb, cb, sg, cg = math.sin(a), math.cos(a), math.sin(b), math.cos(b), math.sin(g), math.cos(g)
    return np.array([
        [cg * ca, cg * sa, -sg],
        [sb * sg * ca - cb * sa, sb * sg * sa + cb * ca, cg * sb],
        [cb * sg * ca + sb * sa, cb * sg * sa - sb * ca, cg * cb],
    ], dtype=np.float64)


def load_rotational_grid(text):
    """``loadRotationalGrid`` (rotational_grid.hpp:25-64): header count, then
    Euler triples in degrees; a short final read is tolerated (the shipped
    files' header counts are one more than their data rows)."""
    lines = text.splitlines()
    n = int(lines[0].split()[0])
    pi = 4.0 * math.atan(1.0)
    deg = pi / 180.0
    rows = []
    for ln in lines[1:]:
        parts = ln.split()
        if len(parts) >= 3:
            rows.append([float(p) for p in parts[:3]])
    mats = []
    for i in range(n):
        if i < len(rows):
            ang = [v * deg for v in rows[i]]
        else:
            ang = [v * deg for v in rows[-1]]   # failed read leaves the last value
        mats.append(euler_to_matrix(ang))
    return np.stack(mats)


def rotate_points(rot, xyz):
    """p' = R p with the reference's accumulation order (bztinyvec.hpp:52-65):
    y_i = ((0 + m_i0 x0) + m_i1 x1) + m_i2 x2, each product rounded."""
    rot = np.asarray(rot, dtype=np.float64)
    x = np.asarray(xyz, dtype=np.float64)
    out = np.empty_like(x)
    for i in range(3):
        acc = rot[i, 0] * x[:, 0]
        acc = acc + rot[i, 1] * x[:, 1]
        acc = acc + rot[i, 2] * x[:, 2]
        out[:, i] = acc
    return out


# ----------------------------------------------------------------------------
# Receptor radial-field projection: Grid/project.hpp:51-176
# ----------------------------------------------------------------------------
def _projection_boxes(geom, center, cut):
    lo = geom.to_logical(center - cut)
    hi = geom.to_logical(center + cut)
    lo = np.maximum(lo, 0)
    hi = np.minimum(hi, np.array(geom.dims) - 1)
    return lo, hi


def _cells_in_box(geom, center, cut):
    """Cells of the cropped toLogical box around ``center`` and their r^2
    (project.hpp:87-98,150-152), r^2 summed x, y, z in that order."""
    lo, hi = _projection_boxes(geom, center, cut)
    if np.any(lo > hi):
        return None
    ix = np.arange(lo[0], hi[0] + 1)
    iy = np.arange(lo[1], hi[1] + 1)
    iz = np.arange(lo[2], hi[2] + 1)
    dx = geom.to_spatial(ix, 0) - center[0]
    dy = geom.to_spatial(iy, 1) - center[1]
    dz = geom.to_spatial(iz, 2) - center[2]
    r2 = (dx[:, None, None] * dx[:, None, None] + dy[None, :, None] * dy[None, :, None]) \
        + dz[None, None, :] * dz[None, None, :]
    return (slice(lo[0], hi[0] + 1), slice(lo[1], hi[1] + 1), slice(lo[2], hi[2] + 1)), r2


def shape_grid(geom, rec_xyz, r_core, width):
    """Plug-in shape term: +1 on surface cells (centre within r_core+width of
    an atom, not core), -15 on core cells (within r_core)."""
    flag = np.zeros(geom.dims, dtype=np.int8)
    cut = float(r_core) + float(width)
    rc2 = float(r_core) * float(r_core)
    rs2 = cut * cut
    for c in np.asarray(rec_xyz, dtype=np.float64):
        got = _cells_in_box(geom, c, cut)
        if got is None:
            continue
        sl, r2 = got
        f = np.where(r2 <= rc2, 2, np.where(r2 <= rs2, 1, 0)).astype(np.int8)
        np.maximum(flag[sl], f, out=flag[sl])
    s = np.zeros(geom.dims, dtype=np.float64)
    s[flag == 1] = SHAPE_SURFACE
    s[flag == 2] = SHAPE_CORE
    return s


def ace_sigmoid(r2, b, k, a):
    """``PotAce::f2`` with no cut shift (potentials_inc.hpp:394-397)."""
    r = np.sqrt(r2)
    return 1.0 / (1.0 + np.exp(b * (k * r - a)))


def ace_type_density(geom, rec_xyz, rec_type, n_types, b, k, a, cut):
    """G_tau(x) = sum over type-tau atoms of the sigmoid at the cell centre,
    r^2 <= cut^2, r^2 clamped to (h/4)^2 (project.hpp:143-159,
    docking_molforce.hpp:307-310)."""
    g = np.zeros((n_types,) + tuple(geom.dims), dtype=np.float64)
    cut2 = float(cut) * float(cut)
    min_d = geom.h / 4.0
    min_d2 = min_d * min_d
    for c, t in zip(np.asarray(rec_xyz, dtype=np.float64), np.asarray(rec_type)):
        got = _cells_in_box(geom, c, cut)
        if got is None:
            continue
        sl, r2 = got
        inside = r2 <= cut2
        r2c = np.where(r2 < min_d2, min_d2, r2)
        val = np.where(inside, ace_sigmoid(r2c, b, k, a), 0.0)
        g[int(t)][sl] += val
    return g


@dataclass
class TermParams:
    term_set: int = TERMS_SHAPE
    shape_core_radius: float = 2.2
    shape_surface_width: float = 1.8
    n_types: int = 18
    ace_matrix: np.ndarray | None = None
    ace_b: float = 7.0
    ace_k: float = 0.15
    ace_a: float = 0.6
    ace_cut: float = 6.0


def receptor_terms(geom, rec_xyz, rec_type, tp: TermParams, folded=True):
    """Receptor grids R_t (float64, K x N^3).

    folded=True gives the K the GPU uses (shape: [-S]; shape+ACE:
    [D_t - S for t]).  folded=False gives the reference-style term list with
    one correlator per term ([-S] + [D_t]), paired with
    :func:`ligand_term_weights` (folded=False)."""
    s = shape_grid(geom, rec_xyz, tp.shape_core_radius, tp.shape_surface_width)
    if tp.term_set == TERMS_SHAPE:
        return (-s)[None]
    if tp.term_set != TERMS_SHAPE_ACE:
        raise ValueError("unknown term set")
    e = np.asarray(tp.ace_matrix, dtype=np.float64)
    g = ace_type_density(geom, rec_xyz, rec_type, tp.n_types, tp.ace_b, tp.ace_k, tp.ace_a, tp.ace_cut)
    d = np.einsum("ut,uxyz->txyz", e, g)
    if folded:
        return d - s[None]
    return np.concatenate([(-s)[None], d], axis=0)


def ligand_term_weights(lig_type, tp: TermParams, folded=True):
    """(n_atoms, K) weights of each ligand atom on each ligand grid."""
    lig_type = np.asarray(lig_type)
    n = lig_type.shape[0]
    if tp.term_set == TERMS_SHAPE:
        return np.ones((n, 1))
    w = np.zeros((n, tp.n_types))
    w[np.arange(n), lig_type] = 1.0
    if folded:
        return w
    return np.concatenate([np.ones((n, 1)), w], axis=1)


# ----------------------------------------------------------------------------
# The reference's own FFT potentials: MolForceLJComp / MolForceLJ
# (docking_molforce.hpp:375-600, docking_app.hpp:52-66) with SoftCoreLJ,
# SoftCoreLJRep, SoftCoreLJAttr (potentials_inc.hpp:142-354)
# ----------------------------------------------------------------------------
@dataclass
class LjParams:
    rec_sigma: np.ndarray
    rec_eps: np.ndarray
    rec_alpha: np.ndarray
    lig_sigma: np.ndarray
    lig_eps: np.ndarray
    mix: int = 1           # PotentialsT::LJ_MIX_0 / LJ_MIX_1
    cut: float = 9.0       # cutOffFft


def _pow3(x):
    return (x * x) * x


def _pow6(x):
    t = (x * x) * x
    return t * t


def _mean(v):
    t = 0.0
    for x in np.asarray(v, dtype=np.float64):
        t = t + float(x)
    return t / float(len(v))


def lj_atom_constants(lj: LjParams, term_set):
    """Per receptor atom (as6, 4es6, 4es12, fshift, gshift), computed in the
    reference's operation order.  ljComp: the constants shared by
    SoftCoreLJRep and SoftCoreLJAttr (no shift); ljAvg: SoftCoreLJ with
    CUT_POLICY_SHIFT_FORCE."""
    sig_l = _mean(lj.lig_sigma)
    out = []
    cut = float(lj.cut)
    cut2 = cut * cut
    for si, ei, ai in zip(np.asarray(lj.rec_sigma, float), np.asarray(lj.rec_eps, float),
                          np.asarray(lj.rec_alpha, float)):
        if term_set == TERMS_LJ_COMP:
            sigma = math.sqrt(si)
            sigma_alpha = math.sqrt(si * sig_l)
            eps = math.sqrt(ei)
            s6 = _pow6(sigma)
            as6 = ai * _pow6(sigma_alpha)
            e6 = 4.0 * eps * s6
            e12 = e6 * s6
            out.append((as6, e6, e12, 0.0, 0.0))
        else:
            eps_l = _mean(lj.lig_eps)
            sigma = (si + sig_l) / 2.0 if lj.mix == 0 else math.sqrt(si * sig_l)
            eps = math.sqrt(ei * eps_l)
            s6 = _pow6(sigma)
            as6 = ai * s6
            e6 = 4.0 * eps * s6
            e12 = e6 * s6
            # g2 at the cutoff with no shift yet (potentials_inc.hpp:226-234)
            r6 = _pow3(cut2)
            A = r6 + as6
            B = s6 / (r6 + as6) - 1.0
            C = -6.0 * (cut2 * cut2) * (e6 * A * B + e12) / _pow3(A)
            gcut = cut * C + cut * (0.0 / math.sqrt(cut2))
            fshift = -((e12 / A - e6) / A + 0.0 + 0.0 * math.sqrt(cut2))
            gshift = -gcut
            fshift = fshift - gshift * cut
            out.append((as6, e6, e12, fshift, gshift))
    return np.array(out)


def lj_field(c, r2, term):
    """f2(r^2) of one atom's constants c: term 0 = ljComp repulsion, 1 =
    ljComp attraction, 'avg' = ljAvg."""
    as6, e6, e12, fshift, gshift = c
    A = _pow3(r2) + as6
    if term == 0:
        return e12 / A / A
    if term == 1:
        return -e6 / A
    return (e12 / A - e6) / A + fshift + gshift * np.sqrt(r2)


def lj_receptor_terms(geom, rec_xyz, lj: LjParams, term_set):
    """K receptor grids of the reference's LJ potentials, projected like
    ProjectorRadialField::projectFields (atoms in order, r^2 clamped to
    (h/4)^2 inside the cropped box, r^2 <= cut^2)."""
    consts = lj_atom_constants(lj, term_set)
    k = 2 if term_set == TERMS_LJ_COMP else 1
    grids = np.zeros((k,) + tuple(geom.dims))
    md = geom.h / 4.0
    md2 = md * md
    cut = float(lj.cut)
    for c, cen in zip(consts, np.asarray(rec_xyz, dtype=np.float64)):
        got = _cells_in_box(geom, cen, cut)
        if got is None:
            continue
        sl, r2 = got
        inside = r2 <= cut * cut
        rr = np.where(r2 < md2, md2, r2)
        if term_set == TERMS_LJ_COMP:
            for t in range(2):
                grids[t][sl] += np.where(inside, lj_field(c, rr, t), 0.0)
        else:
            grids[0][sl] += np.where(inside, lj_field(c, rr, "avg"), 0.0)
    return grids


def lj_ligand_weights(lj: LjParams, term_set):
    """(n_atoms, K) ligand weights: ljComp sqrt(eps) sigma^6 and sqrt(eps)
    sigma^3 (docking_molforce.hpp:503-510,569-576); ljAvg 1 (:441-445)."""
    sig = np.asarray(lj.lig_sigma, dtype=np.float64)
    eps = np.asarray(lj.lig_eps, dtype=np.float64)
    if term_set == TERMS_LJ_AVG:
        return np.ones((len(sig), 1))
    w = np.zeros((len(sig), 2))
    for i, (s, e) in enumerate(zip(sig, eps)):
        w[i, 0] = math.sqrt(e) * _pow6(s)
        w[i, 1] = math.sqrt(e) * _pow3(s)
    return w


# ----------------------------------------------------------------------------
# Ligand scatter: docking_molforce.hpp:351-368
# ----------------------------------------------------------------------------
def bin_ligand(geom, rot, lig_xyz):
    """Rotated ligand cells (n, 3) int64 and an all-in-grid flag."""
    p = rotate_points(rot, lig_xyz)
    cells = geom.to_logical(p)
    ok = bool(np.all((cells >= 0) & (cells < np.array(geom.dims))))
    return cells, ok


def ligand_grids(geom, cells, weights):
    nx, ny, nz = geom.dims
    k = weights.shape[1]
    grids = np.zeros((k, nx, ny, nz), dtype=np.float64)
    flat = (cells[:, 0] * ny + cells[:, 1]) * nz + cells[:, 2]
    for t in range(k):
        np.add.at(grids[t].reshape(-1), flat, weights[:, t])
    return grids


# ----------------------------------------------------------------------------
# Correlation: docking_fft.hpp:622-633 (+ collectTotal, docking_molforce.hpp:249-269)
# ----------------------------------------------------------------------------
def receptor_spectra(rec_grids, workers=1):
    import scipy.fft as sfft
    return np.stack([sfft.rfftn(r, workers=workers) for r in rec_grids])


def correlate(rec_spectra, lig_grids, workers=1):
    """sum_t IFFT(conj(R^_t) * FFT(L_t)) (normalised by V), one forward and one
    inverse transform per term as the reference does."""
    import scipy.fft as sfft
    shape = lig_grids.shape[1:]
    total = None
    for rs, lg in zip(rec_spectra, lig_grids):
        lf = sfft.rfftn(lg, workers=workers)
        c = sfft.irfftn(np.conj(rs) * lf, s=shape, workers=workers)
        total = c if total is None else total + c
    return total


def select_minima(corr, k, max_val=np.inf):
    """k smallest cells with value < max_val, ascending, ties by flat offset."""
    flat = corr.reshape(-1)
    idx = np.nonzero(flat < max_val)[0]
    if idx.size == 0:
        return np.zeros(0, dtype=np.int64), np.zeros(0)
    vals = flat[idx]
    if idx.size > k:
        part = np.argpartition(vals, k - 1)[:k]
        kth = vals[part].max()
        pool = np.nonzero(vals <= kth)[0]
        idx, vals = idx[pool], vals[pool]
    order = np.lexsort((idx, vals))[:k]
    return idx[order], vals[order]


def unwrap(cell, n):
    """``WrappedIndex::unwrap`` (Math/fft.hpp:199-206): y = -x, +n if y < -(n/2),
    per axis (``n`` one edge or the three sizes)."""
    n = np.asarray(n, dtype=np.int64)
    y = -np.asarray(cell, dtype=np.int64)
    y = np.where(y < -(n // 2), y + n, y)
    return y


def offsets_to_cells(offsets, n):
    """Flat C-order offsets (z fastest) -> (x, y, z); ``n`` one edge or the
    three sizes."""
    offsets = np.asarray(offsets, dtype=np.int64)
    ny, nz = (n, n) if np.ndim(n) == 0 else (int(n[1]), int(n[2]))
    return np.stack([offsets // (ny * nz), (offsets // nz) % ny, offsets % nz], axis=-1)


def translation(cell, geom):
    """``toSpatialDiff(unwrap(cell))`` (gridcoord.hpp:150)."""
    return geom.h * unwrap(cell, geom.dims).astype(np.float64)


# ----------------------------------------------------------------------------
# Exact direct-space scorer (independent check of the FFT path)
# ----------------------------------------------------------------------------
def direct_score(rec_grids, cells, weights, shift_cell):
    """C(s) = sum_j sum_t w_jt R_t(cell_j - s mod N), summed with math.fsum.

    ``shift_cell`` is the correlation offset s (the FFT output index); the
    ligand translation it stands for is h * unwrap(s)."""
    dims = np.array(rec_grids.shape[1:], dtype=np.int64)
    s = np.asarray(shift_cell, dtype=np.int64)
    c = (np.asarray(cells, dtype=np.int64) - s[None, :]) % dims[None, :]
    terms = []
    for t in range(rec_grids.shape[0]):
        w = weights[:, t]
        nz = w != 0
        if not np.any(nz):
            continue
        vals = rec_grids[t][c[nz, 0], c[nz, 1], c[nz, 2]] * w[nz]
        terms.extend(vals.tolist())
    return math.fsum(terms)


# ----------------------------------------------------------------------------
# Whole-rotation scan (Worker::scanRotation)
# ----------------------------------------------------------------------------
@dataclass
class ScanResult:
    rot_id: int
    offsets: np.ndarray
    cells: np.ndarray
    scores: np.ndarray
    translations: np.ndarray
    in_grid: bool = True
    corr: np.ndarray | None = field(default=None, repr=False)


def scan_rotation(geom, rec_grids, rec_spectra, lig_xyz, lig_weights, rot, k, max_val=np.inf,
                  rot_id=0, keep_corr=False, workers=1):
    cells, ok = bin_ligand(geom, rot, lig_xyz)
    if not ok:
        return ScanResult(rot_id, np.zeros(0, np.int64), np.zeros((0, 3), np.int64), np.zeros(0),
                          np.zeros((0, 3)), in_grid=False)
    lg = ligand_grids(geom, cells, lig_weights)
    corr = correlate(rec_spectra, lg, workers=workers)
    offs, vals = select_minima(corr, k, max_val)
    pc = offsets_to_cells(offs, geom.dims)
    return ScanResult(rot_id, offs, pc, vals, translation(pc, geom), True, corr if keep_corr else None)


# ----------------------------------------------------------------------------
# Translational clustering: TranClust (docking_fft.hpp:30-140) over
# ClusterMatrix::cluster / getClusters (Geom/cluster.hpp:121-477)
# ----------------------------------------------------------------------------
CLUSTER_ORDER_REFERENCE = 0
CLUSTER_ORDER_BEST_FIRST = 1


def cluster_radius2(radius, n_cols=3):
    """Squared neighbour radius the reference ends up testing against:
    cutoff2 = r^2 * n_cols, cutoff = sqrt(cutoff2), and the sphere iterator
    compares with cutoff * cutoff (cluster.hpp:153-156,
    partpoints.hpp:551-562)."""
    c2 = (radius * radius) * float(n_cols)
    c = math.sqrt(c2)
    return c * c


def cluster_leaders(rows, radius, max_out, walk):
    """``ClusterMatrix::cluster`` leader pass (cluster.hpp:268-338) over the
    rows in ``walk`` order: a row within the neighbour radius (squared
    distance summed column by column, ``<= cluster_radius2``) of an earlier
    leader joins it, otherwise it becomes a leader.  Stops after ``max_out``
    leaders (the later leaders cannot change the earlier ones).  Returns the
    leaders' row indexes in walk order, as ``getClusters`` lists them."""
    m = np.asarray(rows, dtype=np.float64)
    if m.shape[0] == 0:
        return np.zeros(0, dtype=np.int64)
    m = m.reshape(m.shape[0], -1)
    rad2 = cluster_radius2(radius, m.shape[1])
    leaders = []
    for i in walk:
        if len(leaders) >= max_out:
            break
        covered = False
        for j in leaders:
            d2 = 0.0
            for c in range(m.shape[1]):
                d = m[i, c] - m[j, c]
                d2 = d2 + d * d
            if d2 <= rad2:
                covered = True
                break
        if not covered:
            leaders.append(int(i))
    return np.asarray(leaders, dtype=np.int64)


def tran_cluster(translations, values, radius, max_out, order=CLUSTER_ORDER_REFERENCE):
    """TranClust::process on one rotation's queue output.

    ``translations`` (n, 3) and ``values`` (n,) are the queue's entries in
    ascending (value, offset) order.  The reference sets every row's weight
    to ``-value`` and then its density to that weight (the ``dens = weights``
    override at cluster.hpp:238), sorts rows by ascending density -- the
    least negative value, i.e. the worst score, first -- and walks them in
    that order (:func:`cluster_leaders`); ``getClusters`` lists the leaders
    in walk order and ``TranClust::process`` keeps the first ``max_out``.
    The reference's ``std::sort`` leaves the order of equal densities
    unspecified; here equal values are walked from the higher queue position
    down (the queue list read backwards).  ``order=CLUSTER_ORDER_BEST_FIRST``
    walks the queue forwards instead.

    Returns the indexes (into the input) of the kept leaders, in output order.
    """
    t = np.asarray(translations, dtype=np.float64).reshape(-1, 3)
    n = t.shape[0]
    walk = range(n) if order == CLUSTER_ORDER_BEST_FIRST else range(n - 1, -1, -1)
    return cluster_leaders(t, radius, max_out, walk)


def scan_rotation_clustered(geom, rec_grids, rec_spectra, lig_xyz, lig_weights, rot, max_trans_inp, max_out,
                            radius, max_val=np.inf, order=CLUSTER_ORDER_REFERENCE, rot_id=0, workers=1):
    """``findTranslationalMinima`` with ``doClusterTranslations`` on
    (docking_app.hpp:417-447): the ``max_trans_inp`` queue, then TranClust,
    then the first ``max_out`` entries (``getTranValuesFilled``)."""
    res = scan_rotation(geom, rec_grids, rec_spectra, lig_xyz, lig_weights, rot, max_trans_inp, max_val,
                        rot_id=rot_id, workers=workers)
    if not res.in_grid:
        return res
    keep = tran_cluster(res.translations, res.scores, radius, max_out, order)
    return ScanResult(rot_id, res.offsets[keep], res.cells[keep], res.scores[keep], res.translations[keep], True)


# ----------------------------------------------------------------------------
# Scan record format: docking_io_bin.hpp:21-76 (RotFftScanIO_Bin)
# ----------------------------------------------------------------------------
SCAN_SIGNATURE = 2014011401


def pack_record(rot, translations, values):
    """[int32 signature][3x3 float64 rotation][size_t n][n x (3 float64, float64)]."""
    rot = np.asarray(rot, dtype=np.float64).reshape(9)
    buf = struct.pack("<i", SCAN_SIGNATURE) + struct.pack("<9d", *rot)
    n = len(values)
    buf += struct.pack("<Q", n)
    for t, v in zip(translations, values):
        buf += struct.pack("<4d", float(t[0]), float(t[1]), float(t[2]), float(v))
    return buf


def unpack_records(data):
    out = []
    pos = 0
    while pos + 4 <= len(data):
        (sig,) = struct.unpack_from("<i", data, pos)
        if sig != SCAN_SIGNATURE:
            raise ValueError("Signature mismatch for binary format")
        pos += 4
        if pos + 72 + 8 > len(data):
            break
        rot = np.array(struct.unpack_from("<9d", data, pos)).reshape(3, 3)
        pos += 72
        (n,) = struct.unpack_from("<Q", data, pos)
        pos += 8
        if pos + 32 * n > len(data):
            break
        vals = np.array(struct.unpack_from("<%dd" % (4 * n), data, pos)).reshape(n, 4)
        pos += 32 * n
        out.append((rot, vals[:, :3], vals[:, 3]))
    return out


# ----------------------------------------------------------------------------
# Rigid transforms: Geom/transformation.hpp:135-360 (row-major 3x3 + vector)
# ----------------------------------------------------------------------------
def mat_vec(m, v):
    """blitz_ext::product (Blitz/bztinyvec.hpp:52-65): ((0 + m0 v0) + m1 v1) + m2 v2."""
    return np.array([(m[i][0] * v[0] + m[i][1] * v[1]) + m[i][2] * v[2] for i in range(3)])


def mat_mat(a, b):
    """blitz_ext::product of two matrices, same accumulation order."""
    return np.array([[(a[i][0] * b[0][j] + a[i][1] * b[1][j]) + a[i][2] * b[2][j] for j in range(3)]
                     for i in range(3)])


def rt_compose(a, b):
    """RotationTranslation a * b = apply b, then a (transformation.hpp:300-305)."""
    (ra, va), (rb, vb) = a, b
    return mat_mat(ra, rb), mat_vec(ra, vb) + va


def rt_inverse(a):
    """RotationTranslation::inverse (transformation.hpp:336-338): the
    transpose as rotation, then the negated vector: (R^T, R^T (0 - v))."""
    r, v = a
    rt = np.array(r).T
    return rt, mat_vec(rt, 0.0 - np.asarray(v))


def matrix_to_euler(m):
    """Eu_xyz::rotMatrToEulerAng (Geom/euler.hpp:58-102), radians."""
    half_pi = 4.0 * math.atan(1.0) / 2.0
    if m[0][2] < 1.0:
        if m[0][2] > -1.0:
            a0 = math.atan2(-m[1][2], m[2][2])
            a1 = math.asin(m[0][2])
            a2 = math.atan2(-m[0][1], m[0][0])
        else:
            a0 = -math.atan2(m[1][0], m[1][1])
            a1 = -half_pi
            a2 = 0.0
    else:
        a0 = math.atan2(m[1][0], m[1][1])
        a1 = half_pi
        a2 = 0.0
    return np.array([-a2, -a0, -a1])


# ----------------------------------------------------------------------------
# Gather: Foreman::run (docking_app.hpp:174-220) + writeResults (:269-281)
# ----------------------------------------------------------------------------
def gather_records(records, max_matches):
    """records: iterable of (rot 3x3, translations (n,3), values (n,)) in file
    order.  Each translation t becomes Translation(t) * rot = (rot, t); the
    max_matches smallest values below 1e16 are kept and returned ascending
    as (value, rot, t) (ties in arrival order)."""
    q = BoundPriorityQueue(max_matches, (1e16, -1), key=lambda e: (e[0], e[3]))
    seq = 0
    for rot, trans, vals in records:
        for t, v in zip(trans, vals):
            q.push((float(v), np.asarray(rot, dtype=np.float64), np.asarray(t, dtype=np.float64), seq))
            seq += 1
    return [(v, r, t) for v, r, t, _ in q.sort()]


RIGID_SIGNATURE = 2005052501


def pack_rigid(poses, rec_frame, lig_frame):
    """IORigid::writeCoords binary form (IO/rigid.hpp:115-146) of poses moved
    to the original frame, tR^-1 * pose * tL (docking_molstruct.hpp:31-51):
    [int32 signature][int32 n][n x float32 {value, euler[3], xyz[3]}]."""
    inv_r = rt_inverse(rec_frame)
    out = struct.pack("<ii", RIGID_SIGNATURE, len(poses))
    for v, r, t in poses:
        rr, tt = rt_compose(rt_compose(inv_r, (r, t)), lig_frame)
        ang = matrix_to_euler(rr)
        out += struct.pack("<7f", v, *ang, *tt)
    return out


# ----------------------------------------------------------------------------
# Pre-scan frame set-up: MolStruct::moveIntoReferencePositions
# (docking_molstruct.hpp:199-252) with Geom/bounding.hpp:27-250 and the
# RotationTranslation algebra of Geom/transformation.hpp:135-345
# ----------------------------------------------------------------------------
def rt_apply(t, p):
    """RotationTranslation::operator()(Point): product(R, p) + v."""
    r, v = t
    return mat_vec(r, p) + np.asarray(v)


def centre_of_mass(xyz, mass):
    """MolStruct::centerOfMass (:112-126): x += p_i m_i, then x /= sum(m)."""
    x = np.zeros(3)
    tot = 0.0
    for m in mass:
        tot = tot + float(m)
    for p, m in zip(np.asarray(xyz, dtype=np.float64), mass):
        x = x + p * float(m)
    return x / tot


def farthest_pair(xyz):
    """Exact diameter end points: the first pair (i < j, row order) of
    largest ((dx^2 + dy^2) + dz^2)."""
    xyz = np.asarray(xyz, dtype=np.float64)
    best, pair = -1.0, (0, 0)
    for i in range(len(xyz)):
        d = xyz[i + 1:] - xyz[i]
        if len(d) == 0:
            continue
        d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        j = int(np.argmax(d2))
        if d2[j] > best:
            best, pair = float(d2[j]), (i, i + 1 + j)
    return xyz[pair[0]].copy(), xyz[pair[1]].copy()


def axis_box(xyz):
    """Box(points, fixedDirections=true) (bounding.hpp:166-182): min/max
    corners and identity directions."""
    xyz = np.asarray(xyz, dtype=np.float64)
    return np.eye(3), xyz.min(axis=0), xyz.max(axis=0)


def frame_setup(rec_xyz, lig_xyz, lig_mass, grid_step, cut_off_fft, starting_spin=23.3734432, box=None,
                lig_diam=None):
    """The scan frame of a pair.  ``box`` = (directions 3x3 rows, corner
    (0,0,0), corner (1,1,1)) in the original frame; None = axis-aligned box.
    ``lig_diam`` = the diameter's two end points; None = exact farthest pair.
    Returns (rec_out, lig_out, rec_frame, lig_frame, lig_size, min_box (2x3),
    fft_size per axis)."""
    rec = np.array(rec_xyz, dtype=np.float64).reshape(-1, 3)
    lig = np.array(lig_xyz, dtype=np.float64).reshape(-1, 3)
    mass = np.ones(len(lig)) if lig_mass is None else np.asarray(lig_mass, dtype=np.float64)
    ident = (np.eye(3), np.zeros(3))
    tr_rec, tr_lig = ident, ident
    # randomizeLigandOrientation (:213-225)
    s = float(starting_spin)
    spin = euler_to_matrix((s, s * 3.7877, s * (-4.513432)))
    cm = centre_of_mass(lig, mass)
    t = (spin, cm)                                   # Translation(cm) * Rotation
    t = (t[0], mat_vec(t[0], -1.0 * cm) + t[1])      # ... * Translation(-cm)
    lig = np.array([rt_apply(t, p) for p in lig])
    tr_lig = rt_compose(t, tr_lig)
    # moveIntoMinBox (:199-245)
    dirs, c0, c1 = axis_box(rec) if box is None else (np.asarray(box[0], dtype=np.float64).reshape(3, 3),
                                                       np.asarray(box[1], dtype=np.float64),
                                                       np.asarray(box[2], dtype=np.float64))
    centre = -(c0 + (c1 - c0) / 2.0)
    tb = (dirs, mat_vec(dirs, centre))               # Rotation(dirs) * Translation(-centre)
    d0, d1 = rt_apply(tb, c0), rt_apply(tb, c1)
    rec = np.array([rt_apply(tb, p) for p in rec])
    lig = np.array([rt_apply(tb, p) for p in lig])
    tr_rec = rt_compose(tb, tr_rec)
    tr_lig = rt_compose(tb, tr_lig)
    p, q = farthest_pair(lig) if lig_diam is None else (np.asarray(lig_diam[0], dtype=np.float64),
                                                         np.asarray(lig_diam[1], dtype=np.float64))
    tl = -((q + p) / 2.0)
    lig = np.array([tl + x for x in lig])
    tr_lig = (tr_lig[0], tr_lig[1] + tl)             # Translation * RotationTranslation
    dd = q - p
    lig_size = math.sqrt((dd[0] * dd[0] + dd[1] * dd[1]) + dd[2] * dd[2])
    pad = (grid_step * 2.0 + lig_size / 2.0) + cut_off_fft
    lo, hi = d0 - pad, d1 + pad
    # FFTCorrelator::init (docking_fft.hpp:535-553): toLogical of the upper
    # corner in a geometry whose zero is the lower corner, then findBestSize
    zero_h = lo - grid_step
    start = [int((hi[d] - zero_h[d]) / grid_step) - 1 for d in range(3)]
    fft = [find_best_size(v) for v in start]
    return rec, lig, tr_rec, tr_lig, lig_size, np.stack([lo, hi]), fft
