"""Many docking pairs of uneven grid sizes in one CUDA graph
(``fftdock_scan_pairs``; the reference runs one pair per process).

``scan_pairs`` takes a base :class:`ScanConfig` (everything but the grid
edge) and a list of :class:`PairInput`; it returns one ScanResult per pair and
the run's report (streams, rotations per launch chosen per grid edge, timings).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import FFTDockError
from .scan import ScanConfig, ScanResult, native_config


@dataclass
class PairInput:
    rec_xyz: np.ndarray
    lig_xyz: np.ndarray
    rotations: np.ndarray
    rec_type: np.ndarray | None = None
    lig_type: np.ndarray | None = None
    grid_n: int = 0            # 0: pair_grid(...)
    first_rot_id: int = 0


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def pair_grid(rec_xyz, lig_xyz, step=1.2, margin=6.0):
    """Smallest built grid edge >= 48 covering both molecules plus a margin."""
    r = np.ascontiguousarray(rec_xyz, dtype=np.float64).reshape(-1, 3)
    l_ = np.ascontiguousarray(lig_xyz, dtype=np.float64).reshape(-1, 3)
    n = C.c_int32()
    lib = _lib.lib()
    rc = lib.fftdock_pair_grid(len(r), _ptr(r), len(l_), _ptr(l_), float(step), float(margin), C.byref(n))
    if rc:
        raise FFTDockError(rc, lib.fftdock_pairs_last_error().decode())
    return int(n.value)


def scan_pairs(config: ScanConfig, pairs, tune=True, raise_out_of_grid=True, plan=None):
    """``plan``: the report of an earlier call, reused (streams, and per grid
    edge the rotations per launch and the pencil-stage form) when ``tune`` is
    false."""
    lib = _lib.lib()
    cfg, ace = native_config(config)
    P = config.peaks_per_rot
    keep, results = [], []
    descs = (_lib.PairDesc * max(1, len(pairs)))()
    for i, p in enumerate(pairs):
        rec = np.ascontiguousarray(p.rec_xyz, dtype=np.float64).reshape(-1, 3)
        lig = np.ascontiguousarray(p.lig_xyz, dtype=np.float64).reshape(-1, 3)
        rot = np.ascontiguousarray(p.rotations, dtype=np.float64).reshape(-1, 9)
        rt = None if p.rec_type is None else np.ascontiguousarray(p.rec_type, dtype=np.int32)
        lt = None if p.lig_type is None else np.ascontiguousarray(p.lig_type, dtype=np.int32)
        n = p.grid_n or pair_grid(rec, lig, config.grid_step)
        peaks = np.zeros((len(rot), P), dtype=_lib.peak_dtype())
        npk = np.zeros(len(rot), dtype=np.int32)
        keep += [rec, lig, rot, rt, lt]
        results.append(ScanResult(peaks, npk))
        d = descs[i]
        d.grid_n = n
        d.n_rec, d.rec_xyz, d.rec_type = len(rec), rec.ctypes.data, (rt.ctypes.data if rt is not None else None)
        d.n_lig, d.lig_xyz, d.lig_type = len(lig), lig.ctypes.data, (lt.ctypes.data if lt is not None else None)
        d.n_rot, d.rot, d.first_rot_id = len(rot), rot.ctypes.data, int(p.first_rot_id)
        d.peaks, d.n_peaks = peaks.ctypes.data, npk.ctypes.data
    rep = _lib.PairsReport()
    if plan is not None and not tune:
        rep.n_streams = int(plan["n_streams"])
        forms = {"fft": _lib.FFTDOCK_PENCIL_FFT, "tensor": _lib.FFTDOCK_PENCIL_TENSOR}
        for k in range(_lib.N_SIZES):
            rep.rot_batch[k] = int(plan["rot_batch"].get(int(_lib.BUILT_SIZES[k]), 0))
            rep.pencil_form[k] = forms.get(plan.get("pencil_form", {}).get(int(_lib.BUILT_SIZES[k])), 0)
    rc = lib.fftdock_scan_pairs(C.byref(cfg), len(pairs), descs, 1 if tune else 0, C.byref(rep))
    msg = lib.fftdock_pairs_last_error().decode() if rc else ""
    report = {
        "n_streams": rep.n_streams,
        "rot_batch": {int(rep.grid_sizes[k]): int(rep.rot_batch[k]) for k in range(_lib.N_SIZES) if rep.rot_batch[k]},
        "pencil_form": {int(rep.grid_sizes[k]): ("tensor" if rep.pencil_form[k] == _lib.FFTDOCK_PENCIL_TENSOR else "fft")
                        for k in range(_lib.N_SIZES) if rep.rot_batch[k]},
        "setup_ms": rep.setup_ms, "tune_ms": rep.tune_ms, "capture_ms": rep.capture_ms, "run_ms": rep.run_ms,
        "rotations": int(rep.rotations), "n_out_of_grid": int(rep.n_out_of_grid),
        "grid_n": [int(descs[i].grid_n) for i in range(len(pairs))],
    }
    if rc and not (rc == _lib.FFTDOCK_EOUT_OF_GRID and not raise_out_of_grid):
        raise FFTDockError(rc, msg)
    for r in results:
        r.status, r.message = rc, msg
    return results, report
