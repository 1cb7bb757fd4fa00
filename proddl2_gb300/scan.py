"""Host-side interface of the GPU correlation scan.

Mirrors the reference's rot-scan worker for one receptor/ligand pair
(``include/PRODDL/docking_app.hpp:316-513``): options with the reference's
names (``gridStep``, ``maxNTrans``, ``maxNTransInp``, ``maxValCorr``,
``potentialName``), receptor preparation once per pair, then a scan over a
rotation set that returns, per rotation, the ``maxNTrans`` lowest-energy
translations in ascending order.  Errors the reference raises as C++
exceptions surface as :class:`FFTDockError`; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import FFTDockError

TERM_SETS = {"shape": _lib.FFTDOCK_TERMS_SHAPE, "shape_ace": _lib.FFTDOCK_TERMS_SHAPE_ACE,
             "lj_comp": _lib.FFTDOCK_TERMS_LJ_COMP, "lj_avg": _lib.FFTDOCK_TERMS_LJ_AVG}
# the reference's potentialName values
POTENTIAL_NAMES = {"ljComp": "lj_comp", "ljAvg": "lj_avg"}
PENCIL_MODES = {"auto": _lib.FFTDOCK_PENCIL_AUTO, "fft": _lib.FFTDOCK_PENCIL_FFT, "tensor": _lib.FFTDOCK_PENCIL_TENSOR}


@dataclass
class ScanConfig:
    grid_n: int = 128               # FFT grid edge (the configs fix N directly)
    grid_step: float = 1.2          # gridStep
    term_set: str = "shape_ace"     # potentialName
    peaks_per_rot: int = 4          # maxNTrans
    max_trans_inp: int = 10000      # maxNTransInp
    max_val_corr: float = float("inf")  # maxValCorr
    rot_batch: int = 64
    n_types: int = 18
    ace_matrix: np.ndarray | None = None
    shape_core_radius: float = 2.2
    shape_surface_width: float = 1.8
    ace_b: float = 7.0
    ace_k: float = 0.15
    ace_a: float = 0.6
    ace_cut: float = 6.0
    device: int = 0
    pencil_mode: str = "auto"       # "auto", "fft" (CUDA-core x-FFTs) or "tensor" (tcgen05 GEMM form)
    precision: str = "fp32"         # receptor spectra: "fp32" or "bf16"
    cluster_trans: bool = False     # doClusterTranslations
    cluster_radius: float = 5.0     # clusterRadiusTrans
    cluster_order: str = "reference"  # leader walk: "reference" (worst value first) or "best_first"
    lj_mix: int = 1                 # LJ sets: sigma rule (0 arithmetic, 1 geometric; ljComp needs 1)
    lj_cut: float = 9.0             # LJ sets: cutOffFft
    tc_terms_per_sum: int = 0       # tensor form: terms per tensor-memory sum (0: library default)
    grid_dims: tuple | None = None  # FFT sizes per axis (the reference's fftSize); None: grid_n on every axis

    @classmethod
    def from_options(cls, opts: dict, **kw):
        """Build from a reference-style options dict (``config/noarch/proddl.json.in``)."""
        names = {"gridStep": "grid_step", "maxNTrans": "peaks_per_rot", "maxNTransInp": "max_trans_inp",
                 "maxValCorr": "max_val_corr", "doClusterTranslations": "cluster_trans",
                 "clusterRadiusTrans": "cluster_radius"}
        args = {names[k]: v for k, v in opts.items() if k in names}
        if "potentialName" in opts and opts["potentialName"] in POTENTIAL_NAMES:
            args["term_set"] = POTENTIAL_NAMES[opts["potentialName"]]
        if "cutOffFft" in opts:
            args["lj_cut"] = opts["cutOffFft"]
        args.update(kw)
        return cls(**args)


@dataclass
class ScanResult:
    peaks: np.ndarray       # (n_rot, peaks_per_rot) structured fftdock_peak
    n_peaks: np.ndarray     # (n_rot,) int32
    status: int = 0
    message: str = ""

    def rotation(self, i):
        """(cells (n,3), translations (n,3), scores (n,)) of rotation i."""
        k = int(self.n_peaks[i])
        p = self.peaks[i, :k]
        return p["cell"], p["t"], p["score"]


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def native_config(config: ScanConfig):
    """The C ``fftdock_config`` of a ScanConfig (and the array it points to)."""
    cfg = _lib.Config()
    _lib.lib().fftdock_config_init(C.byref(cfg))
    cfg.grid_n = int(config.grid_n)
    cfg.grid_step = float(config.grid_step)
    cfg.term_set = TERM_SETS[config.term_set]
    cfg.peaks_per_rot = int(config.peaks_per_rot)
    cfg.max_trans_inp = int(config.max_trans_inp)
    cfg.max_val_corr = float(config.max_val_corr)
    cfg.rot_batch = int(config.rot_batch)
    cfg.n_types = int(config.n_types)
    ace = None
    if config.ace_matrix is not None:
        ace = np.ascontiguousarray(config.ace_matrix, dtype=np.float64)
        cfg.ace_matrix = ace.ctypes.data_as(C.POINTER(C.c_double))
    cfg.shape_core_radius = float(config.shape_core_radius)
    cfg.shape_surface_width = float(config.shape_surface_width)
    cfg.ace_b, cfg.ace_k, cfg.ace_a, cfg.ace_cut = (float(config.ace_b), float(config.ace_k),
                                                    float(config.ace_a), float(config.ace_cut))
    cfg.device = int(config.device)
    cfg.pencil_mode = PENCIL_MODES[config.pencil_mode]
    cfg.precision = {"fp32": _lib.FFTDOCK_PREC_FP32, "bf16": _lib.FFTDOCK_PREC_BF16_SPECTRA}[config.precision]
    cfg.cluster_trans = 1 if config.cluster_trans else 0
    cfg.cluster_radius = float(config.cluster_radius)
    cfg.cluster_order = {"reference": 0, "best_first": 1}[config.cluster_order]
    cfg.lj_mix = int(config.lj_mix)
    cfg.lj_cut = float(config.lj_cut)
    cfg.tc_terms_per_sum = int(config.tc_terms_per_sum)
    if config.grid_dims is not None:
        cfg.grid_nx, cfg.grid_ny, cfg.grid_nz = (int(v) for v in config.grid_dims)
        cfg.grid_n = int(config.grid_dims[0])
    return cfg, ace


class FFTScan:
    """One receptor/ligand pair on one GPU (C ABI ``fftdock_ctx``)."""

    def __init__(self, config: ScanConfig):
        self.lib = _lib.lib()
        self.config = config
        cfg, self._ace = native_config(config)
        h = C.c_void_p()
        rc = self.lib.fftdock_create(C.byref(cfg), C.byref(h))
        self._h = h
        if rc != 0:
            msg = self._err()
            self.close()
            raise FFTDockError(rc, msg)

    # -- plumbing -------------------------------------------------------------
    def _err(self):
        m = self.lib.fftdock_last_error(self._h)
        return m.decode() if m else ""

    def _check(self, rc):
        if rc != 0:
            raise FFTDockError(rc, self._err())

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self.lib.fftdock_destroy(self._h)
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
    def grid_n(self):
        return self.lib.fftdock_grid_n(self._h)

    @property
    def grid_dims(self):
        """FFT sizes (nx, ny, nz)."""
        d = (C.c_int32 * 3)()
        self._check(self.lib.fftdock_grid_dims(self._h, d))
        return tuple(int(v) for v in d)

    @property
    def n_terms(self):
        return self.lib.fftdock_n_terms(self._h)

    def info(self):
        """Grid, terms, the pencil-stage form that runs, batch and ligand window."""
        st = _lib.ScanInfo()
        self._check(self.lib.fftdock_get_scan_info(self._h, C.byref(st)))
        path = {_lib.FFTDOCK_PENCIL_FFT: "fft", _lib.FFTDOCK_PENCIL_TENSOR: "tensor"}[st.pencil_path]
        return dict(grid_n=st.grid_n, n_terms=st.n_terms, pencil_path=path, rot_batch=st.rot_batch,
                    n_entries=st.n_entries, window_x0=st.window_x0, window_w=st.window_w)

    # -- the scan -------------------------------------------------------------
    def set_receptor(self, xyz, types=None):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        t = None if types is None else np.ascontiguousarray(types, dtype=np.int32)
        self._check(self.lib.fftdock_set_receptor(self._h, xyz.shape[0], _ptr(xyz), _ptr(t)))

    def set_pair_lj(self, rec_xyz, rec_sigma, rec_eps, rec_alpha, lig_xyz, lig_sigma, lig_eps):
        """Both molecules with their LJ parameters (the LJ term sets)."""
        r = np.ascontiguousarray(rec_xyz, dtype=np.float64).reshape(-1, 3)
        l_ = np.ascontiguousarray(lig_xyz, dtype=np.float64).reshape(-1, 3)
        arr = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
               for a in (rec_sigma, rec_eps, rec_alpha, lig_sigma, lig_eps)]
        self._check(self.lib.fftdock_set_pair_lj(self._h, len(r), _ptr(r), _ptr(arr[0]), _ptr(arr[1]), _ptr(arr[2]),
                                                 len(l_), _ptr(l_), _ptr(arr[3]), _ptr(arr[4])))

    def set_ligand(self, xyz, types=None):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        t = None if types is None else np.ascontiguousarray(types, dtype=np.int32)
        self._check(self.lib.fftdock_set_ligand(self._h, xyz.shape[0], _ptr(xyz), _ptr(t)))

    def scan(self, rotations, first_rot_id=0, raise_out_of_grid=True) -> ScanResult:
        rot = np.ascontiguousarray(rotations, dtype=np.float64).reshape(-1, 9)
        n = rot.shape[0]
        P = self.config.peaks_per_rot
        peaks = np.zeros((n, P), dtype=_lib.peak_dtype())
        npk = np.zeros(n, dtype=np.int32)
        rc = self.lib.fftdock_scan(self._h, n, _ptr(rot), int(first_rot_id), _ptr(peaks), _ptr(npk))
        res = ScanResult(peaks, npk, rc, self._err() if rc else "")
        if rc == _lib.FFTDOCK_EOUT_OF_GRID and not raise_out_of_grid:
            return res
        self._check(rc)
        return res

    def scan_device(self, d_rot_ptr, n_rot, d_peaks_ptr, d_npeaks_ptr, first_rot_id=0, stream_ptr=None):
        """Queue a scan on device buffers (raw CUDA pointers, e.g. torch
        ``tensor.data_ptr()``); returns without synchronising."""
        self._check(self.lib.fftdock_scan_device(self._h, int(n_rot), C.c_void_p(d_rot_ptr), int(first_rot_id),
                                                 C.c_void_p(d_peaks_ptr), C.c_void_p(d_npeaks_ptr),
                                                 C.c_void_p(stream_ptr) if stream_ptr else None))

    def scan_device_noalloc(self, d_rot_ptr, n_rot, d_peaks_ptr, d_npeaks_ptr, first_rot_id=0, stream_ptr=None):
        """Like :meth:`scan_device`, but the library allocates nothing: its
        work memory is a fixed 16 MiB array inside the library, for callers
        whose host owns all device memory or forbids allocation while running.
        Calls that overlap on the GPU share that array and race."""
        self._check(self.lib.fftdock_scan_device_noalloc(
            self._h, int(n_rot), C.c_void_p(d_rot_ptr), int(first_rot_id), C.c_void_p(d_peaks_ptr),
            C.c_void_p(d_npeaks_ptr), C.c_void_p(stream_ptr) if stream_ptr else None))

    # -- diagnostics ----------------------------------------------------------
    def profile(self, enable=True):
        """Record CUDA events around every scan kernel (starting clears the record)."""
        self._check(self.lib.fftdock_profile(self._h, 1 if enable else 0))

    def kernel_stats(self):
        """{kernel: (launches, total_ms)} of the recorded launches."""
        st = _lib.KernelStats()
        self._check(self.lib.fftdock_get_kernel_stats(self._h, C.byref(st)))
        return {name: (int(st.launches[i]), float(st.total_ms[i])) for i, name in enumerate(_lib.KERNEL_NAMES)}

    def receptor_grid(self, term):
        out = np.empty(self.grid_dims, dtype=np.float64)
        self._check(self.lib.fftdock_get_receptor_grid(self._h, int(term), _ptr(out)))
        return out

    def correlation_grid(self, rotation):
        rot = np.ascontiguousarray(rotation, dtype=np.float64).reshape(9)
        out = np.empty(self.grid_dims, dtype=np.float32)
        self._check(self.lib.fftdock_correlation_grid(self._h, _ptr(rot), _ptr(out)))
        return out

    def candidates(self, rotations):
        rot = np.ascontiguousarray(rotations, dtype=np.float64).reshape(-1, 9)
        n = rot.shape[0]
        v = np.empty((n, _lib.KC), dtype=np.float32)
        o = np.empty((n, _lib.KC), dtype=np.int32)
        self._check(self.lib.fftdock_scan_candidates(self._h, n, _ptr(rot), _ptr(v), _ptr(o)))
        return v, o


def supported_grid(n):
    """A cubic edge with compiled plans."""
    return bool(_lib.lib().fftdock_supported_grid(int(n)))


def supported_dims(dims):
    """Per-axis FFT sizes the library scans (a compiled cubic edge or box-grid sizes)."""
    nx, ny, nz = (int(v) for v in dims)
    return bool(_lib.lib().fftdock_supported_dims(nx, ny, nz))


def find_best_size(start_n):
    out = C.c_int32()
    rc = _lib.lib().fftdock_find_best_size(int(start_n), C.byref(out))
    if rc:
        raise FFTDockError(rc, "no FFT size found")
    return out.value


def write_scan_records(path, rotations, result: ScanResult, append=False):
    """Write RotFftScanIO_Bin records (docking_io_bin.hpp:55-71)."""
    rot = np.ascontiguousarray(rotations, dtype=np.float64).reshape(-1, 9)
    peaks = np.ascontiguousarray(result.peaks)
    npk = np.ascontiguousarray(result.n_peaks, dtype=np.int32)
    rc = _lib.lib().fftdock_write_scan_records(str(path).encode(), rot.shape[0], _ptr(rot), peaks.shape[1],
                                               _ptr(peaks), _ptr(npk), 1 if append else 0)
    if rc:
        raise FFTDockError(rc, "writing %s" % path)
