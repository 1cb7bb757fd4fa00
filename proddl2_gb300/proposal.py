"""Learned rotation proposal: host side (no counterpart in the reference).

``Proposal`` wraps the ``fftdock_proposal_*`` C ABI (network, training and
inference kernels on the GPU).  The helpers turn exhaustive scan results into
training targets, prune a rotation set with a trained network, and measure
what the pruning keeps: the top-k pose recall against the exhaustive scan,
which stays the fallback and the judge.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import FFTDockError

DESC = 128


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def receptor_descriptor(xyz, element):
    """Radial element histograms of a receptor (128 floats)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    el = np.ascontiguousarray(element, dtype=np.int32).reshape(-1)
    out = np.zeros(DESC, dtype=np.float32)
    rc = _lib.lib().fftdock_receptor_descriptor(len(xyz), _ptr(xyz), _ptr(el), _ptr(out))
    if rc:
        raise FFTDockError(rc, "receptor descriptor: element outside 0..3 or non-finite coordinate")
    return out


def receptor_descriptor_oriented(xyz):
    """Receptor occupancy in the scan frame (128 floats: 4^3 cells, all and
    outer atoms), so that the network sees both molecules in one frame."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    out = np.zeros(DESC, dtype=np.float32)
    rc = _lib.lib().fftdock_receptor_descriptor_oriented(len(xyz), _ptr(xyz), _ptr(out))
    if rc:
        raise FFTDockError(rc, "oriented receptor descriptor: non-finite coordinate")
    return out


class Proposal:
    """One network on one GPU."""

    def __init__(self, device=0, seed=0):
        self.lib = _lib.lib()
        h = C.c_void_p()
        rc = self.lib.fftdock_proposal_create(int(device), int(seed), C.byref(h))
        self._h = h
        if rc:
            msg = self._err()
            self.close()
            raise FFTDockError(rc, msg)

    def _err(self):
        m = self.lib.fftdock_proposal_last_error(self._h)
        return m.decode() if m else ""

    def _check(self, rc):
        if rc:
            raise FFTDockError(rc, self._err())

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self.lib.fftdock_proposal_destroy(self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def n_params(self):
        return int(self.lib.fftdock_proposal_n_params())

    @property
    def params(self):
        out = np.empty(self.n_params, dtype=np.float32)
        self._check(self.lib.fftdock_proposal_get_params(self._h, _ptr(out)))
        return out

    @params.setter
    def params(self, value):
        v = np.ascontiguousarray(value, dtype=np.float32).reshape(-1)
        if v.size != self.n_params:
            raise ValueError("expected %d parameters" % self.n_params)
        self._check(self.lib.fftdock_proposal_set_params(self._h, _ptr(v)))

    def add_pair(self, lig_xyz, rec_xyz=None, rec_element=None, desc=None):
        """Register a pair (ligand in the scan frame); returns its id."""
        lig = np.ascontiguousarray(lig_xyz, dtype=np.float64).reshape(-1, 3)
        if desc is None:
            desc = receptor_descriptor(rec_xyz, rec_element)
        d = np.ascontiguousarray(desc, dtype=np.float32).reshape(DESC)
        i = C.c_int32()
        self._check(self.lib.fftdock_proposal_add_ligand(self._h, len(lig), _ptr(lig), _ptr(d), C.byref(i)))
        return int(i.value)

    def add_samples(self, pair_id, rotations, targets):
        rot = np.ascontiguousarray(rotations, dtype=np.float64).reshape(-1, 9)
        t = np.ascontiguousarray(targets, dtype=np.float32).reshape(-1)
        if len(t) != len(rot):
            raise ValueError("one target per rotation")
        self._check(self.lib.fftdock_proposal_add_samples(self._h, int(pair_id), len(rot), _ptr(rot), _ptr(t)))

    def clear_samples(self):
        self._check(self.lib.fftdock_proposal_clear_samples(self._h))

    def train(self, steps, batch=256, lr=1e-3, seed=0):
        loss = C.c_float()
        self._check(self.lib.fftdock_proposal_train(self._h, int(steps), int(batch), float(lr), int(seed),
                                                    C.byref(loss)))
        return float(loss.value)

    def gradients(self, pair_ids, rotations, targets):
        ids = np.ascontiguousarray(pair_ids, dtype=np.int32).reshape(-1)
        rot = np.ascontiguousarray(rotations, dtype=np.float64).reshape(-1, 9)
        t = np.ascontiguousarray(targets, dtype=np.float32).reshape(-1)
        g = np.empty(self.n_params, dtype=np.float32)
        loss = C.c_float()
        self._check(self.lib.fftdock_proposal_gradients(self._h, len(ids), _ptr(ids), _ptr(rot), _ptr(t), _ptr(g),
                                                        C.byref(loss)))
        return g, float(loss.value)

    def predict(self, pair_id, rotations):
        rot = np.ascontiguousarray(rotations, dtype=np.float64).reshape(-1, 9)
        out = np.empty(len(rot), dtype=np.float32)
        self._check(self.lib.fftdock_proposal_predict(self._h, int(pair_id), len(rot), _ptr(rot), _ptr(out)))
        return out

    def predict_device(self, pair_id, d_rot_ptr, n, d_out_ptr, stream_ptr=None):
        self._check(self.lib.fftdock_proposal_predict_device(self._h, int(pair_id), int(n), C.c_void_p(d_rot_ptr),
                                                             C.c_void_p(d_out_ptr),
                                                             C.c_void_p(stream_ptr) if stream_ptr else None))

    def save(self, path):
        np.save(path, self.params)

    def load(self, path):
        self.params = np.load(path)


# ---------------------------------------------------------------------------
# targets, pruning and recall
# ---------------------------------------------------------------------------
def best_scores(result):
    """Best (lowest) score of each rotation of a ScanResult; +inf when none."""
    n = result.n_peaks
    best = np.where(n > 0, result.peaks["score"][:, 0], np.inf)
    return best.astype(np.float64)


def standardize(best):
    """Per-pair standardised targets (lower = better stays lower)."""
    b = np.asarray(best, dtype=np.float64)
    fin = np.isfinite(b)
    mu = b[fin].mean() if fin.any() else 0.0
    sd = b[fin].std() if fin.sum() > 1 else 1.0
    sd = sd if sd > 0 else 1.0
    z = np.where(fin, (b - mu) / sd, 3.0)
    return z.astype(np.float32)


def keep_best(pred, frac):
    """Indexes of the ceil(frac * n) rotations with the lowest prediction."""
    pred = np.asarray(pred)
    k = max(1, int(np.ceil(frac * len(pred))))
    return np.sort(np.argsort(pred, kind="stable")[:k])


def top_poses(result, rot_ids, k=100):
    """The k best poses (score, rotation id, cell) of a scan over rot_ids."""
    poses = []
    for i, rid in enumerate(rot_ids):
        for j in range(int(result.n_peaks[i])):
            p = result.peaks[i, j]
            poses.append((float(p["score"]), int(rid), tuple(int(c) for c in p["cell"])))
    poses.sort(key=lambda e: (e[0], e[1], e[2]))
    return poses[:k]


def recall(exhaustive_top, pruned_top):
    """Fraction of the exhaustive top poses that the pruned scan also ranks
    in its top list (a pose = rotation id + translation cell)."""
    ref = {(r, c) for _, r, c in exhaustive_top}
    got = {(r, c) for _, r, c in pruned_top}
    return len(ref & got) / max(1, len(ref))
