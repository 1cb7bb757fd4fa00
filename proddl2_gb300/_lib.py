"""ctypes binding of libfftdock.so (include/fftdock.h).

The library is built in-tree by ``proddl2_gb300.build``; importing this
module does not build it.  :func:`lib` raises if the shared object is missing
so that no caller can silently fall back to a CPU path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libfftdock.so"

FFTDOCK_OK = 0
FFTDOCK_EINVAL = 1
FFTDOCK_EOUT_OF_GRID = 2
FFTDOCK_ECUDA = 3
FFTDOCK_ENOMEM = 4
FFTDOCK_ESTATE = 5
FFTDOCK_EUNSUPPORTED = 6
FFTDOCK_EIO = 7

STATUS_NAMES = {
    0: "FFTDOCK_OK", 1: "FFTDOCK_EINVAL", 2: "FFTDOCK_EOUT_OF_GRID", 3: "FFTDOCK_ECUDA",
    4: "FFTDOCK_ENOMEM", 5: "FFTDOCK_ESTATE", 6: "FFTDOCK_EUNSUPPORTED", 7: "FFTDOCK_EIO",
}

FFTDOCK_TERMS_SHAPE = 1
FFTDOCK_TERMS_SHAPE_ACE = 2
FFTDOCK_TERMS_LJ_COMP = 3
FFTDOCK_TERMS_LJ_AVG = 4
FFTDOCK_PREC_FP32 = 0
FFTDOCK_PREC_BF16_SPECTRA = 1
FFTDOCK_PENCIL_AUTO = 0
FFTDOCK_PENCIL_FFT = 1
FFTDOCK_PENCIL_TENSOR = 2
FFTDOCK_CLUSTER_ORDER_REFERENCE = 0
FFTDOCK_CLUSTER_ORDER_BEST_FIRST = 1
FFTDOCK_MAX_QUEUE_CLUSTERED = 16384
KC = 16


class Config(C.Structure):
    _fields_ = [
        ("struct_size", C.c_int32),
        ("grid_n", C.c_int32),
        ("grid_step", C.c_double),
        ("term_set", C.c_int32),
        ("peaks_per_rot", C.c_int32),
        ("max_trans_inp", C.c_int32),
        ("max_val_corr", C.c_double),
        ("rot_batch", C.c_int32),
        ("precision", C.c_int32),
        ("device", C.c_int32),
        ("n_types", C.c_int32),
        ("ace_matrix", C.POINTER(C.c_double)),
        ("shape_core_radius", C.c_double),
        ("shape_surface_width", C.c_double),
        ("ace_b", C.c_double),
        ("ace_k", C.c_double),
        ("ace_a", C.c_double),
        ("ace_cut", C.c_double),
        ("pencil_mode", C.c_int32),
        ("cluster_trans", C.c_int32),
        ("cluster_order", C.c_int32),
        ("cluster_radius", C.c_double),
        ("lj_mix", C.c_int32),
        ("lj_cut", C.c_double),
        ("tc_terms_per_sum", C.c_int32),
        ("grid_nx", C.c_int32),
        ("grid_ny", C.c_int32),
        ("grid_nz", C.c_int32),
    ]


FFTDOCK_BOX_AXES = 0
FFTDOCK_BOX_GIVEN = 1
FFTDOCK_BOX_MIN_VOLUME = 2


class FrameIn(C.Structure):
    _fields_ = [
        ("n_rec", C.c_int32), ("rec_xyz", C.c_void_p),
        ("n_lig", C.c_int32), ("lig_xyz", C.c_void_p), ("lig_mass", C.c_void_p),
        ("grid_step", C.c_double), ("cut_off_fft", C.c_double), ("starting_spin", C.c_double),
        ("box_mode", C.c_int32), ("box_dirs", C.c_void_p), ("box_corners", C.c_void_p), ("lig_diam", C.c_void_p),
    ]


class Frame(C.Structure):
    _fields_ = [
        ("rec_frame", C.c_double * 12), ("lig_frame", C.c_double * 12), ("lig_size", C.c_double),
        ("min_box", C.c_double * 6), ("fft_size", C.c_int32 * 3), ("grid_n", C.c_int32),
    ]


N_SIZES = 10
BUILT_SIZES = (16, 24, 32, 48, 64, 80, 96, 112, 128, 144)


class PairDesc(C.Structure):
    _fields_ = [
        ("grid_n", C.c_int32),
        ("n_rec", C.c_int32),
        ("rec_xyz", C.c_void_p),
        ("rec_type", C.c_void_p),
        ("n_lig", C.c_int32),
        ("lig_xyz", C.c_void_p),
        ("lig_type", C.c_void_p),
        ("n_rot", C.c_int32),
        ("rot", C.c_void_p),
        ("first_rot_id", C.c_int32),
        ("peaks", C.c_void_p),
        ("n_peaks", C.c_void_p),
    ]


class PairsReport(C.Structure):
    _fields_ = [
        ("n_streams", C.c_int32),
        ("grid_sizes", C.c_int32 * N_SIZES),
        ("rot_batch", C.c_int32 * N_SIZES),
        ("setup_ms", C.c_double),
        ("tune_ms", C.c_double),
        ("capture_ms", C.c_double),
        ("run_ms", C.c_double),
        ("rotations", C.c_int64),
        ("n_out_of_grid", C.c_int32),
        ("pencil_form", C.c_int32 * N_SIZES),
    ]


class Peak(C.Structure):
    _fields_ = [
        ("rot_id", C.c_int32),
        ("cell", C.c_int32 * 3),
        ("t", C.c_double * 3),
        ("score", C.c_double),
    ]


class KernelStats(C.Structure):
    _fields_ = [("launches", C.c_int64 * 4), ("total_ms", C.c_double * 4)]


KERNEL_NAMES = ("ligand_prep", "pencil", "plane", "finalize")


class ScanInfo(C.Structure):
    _fields_ = [("grid_n", C.c_int32), ("n_terms", C.c_int32), ("pencil_path", C.c_int32),
                ("rot_batch", C.c_int32), ("n_entries", C.c_int32), ("window_x0", C.c_int32),
                ("window_w", C.c_int32)]


class Pose(C.Structure):
    _fields_ = [("value", C.c_double), ("rot", C.c_double * 9), ("t", C.c_double * 3)]


def pose_dtype():
    import numpy as np
    return np.dtype([("value", "<f8"), ("rot", "<f8", (9,)), ("t", "<f8", (3,))])


# numpy view of fftdock_peak
def peak_dtype():
    import numpy as np
    return np.dtype([("rot_id", "<i4"), ("cell", "<i4", (3,)), ("t", "<f8", (3,)), ("score", "<f8")], align=True)


# symbol -> (restype, argtypes); the exported surface of include/fftdock.h
_P = C.c_void_p
SIGNATURES = {
    "fftdock_config_init": (None, [C.POINTER(Config)]),
    "fftdock_supported_grid": (C.c_int, [C.c_int32]),
    "fftdock_supported_dims": (C.c_int, [C.c_int32, C.c_int32, C.c_int32]),
    "fftdock_grid_dims": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "fftdock_find_best_size": (C.c_int, [C.c_int32, C.POINTER(C.c_int32)]),
    "fftdock_create": (C.c_int, [C.POINTER(Config), C.POINTER(_P)]),
    "fftdock_destroy": (None, [_P]),
    "fftdock_last_error": (C.c_char_p, [_P]),
    "fftdock_set_pair_lj": (C.c_int, [_P, C.c_int32, _P, _P, _P, _P, C.c_int32, _P, _P, _P]),
    "fftdock_set_receptor": (C.c_int, [_P, C.c_int32, _P, _P]),
    "fftdock_set_ligand": (C.c_int, [_P, C.c_int32, _P, _P]),
    "fftdock_scan": (C.c_int, [_P, C.c_int32, _P, C.c_int32, _P, _P]),
    "fftdock_scan_device": (C.c_int, [_P, C.c_int32, _P, C.c_int32, _P, _P, _P]),
    "fftdock_scan_device_noalloc": (C.c_int, [_P, C.c_int32, _P, C.c_int32, _P, _P, _P]),
    "fftdock_grid_n": (C.c_int, [_P]),
    "fftdock_n_terms": (C.c_int, [_P]),
    "fftdock_get_scan_info": (C.c_int, [_P, C.POINTER(ScanInfo)]),
    "fftdock_get_receptor_grid": (C.c_int, [_P, C.c_int32, _P]),
    "fftdock_correlation_grid": (C.c_int, [_P, _P, _P]),
    "fftdock_scan_candidates": (C.c_int, [_P, C.c_int32, _P, _P, _P]),
    "fftdock_profile": (C.c_int, [_P, C.c_int32]),
    "fftdock_get_kernel_stats": (C.c_int, [_P, C.POINTER(KernelStats)]),
    "fftdock_gather_records": (C.c_int, [C.POINTER(C.c_char_p), C.c_int32, C.c_int32, _P, C.POINTER(C.c_int32)]),
    "fftdock_gather_list": (C.c_int, [C.c_char_p, C.c_int32, _P, C.POINTER(C.c_int32)]),
    "fftdock_write_rigid": (C.c_int, [C.c_char_p, _P, C.c_int32, _P, _P, C.c_int32]),
    "fftdock_write_scan_records": (C.c_int, [C.c_char_p, C.c_int32, _P, C.c_int32, _P, _P, C.c_int32]),
    "fftdock_frame_setup": (C.c_int, [C.POINTER(FrameIn), _P, _P, C.POINTER(Frame)]),
    "fftdock_min_volume_box": (C.c_int, [C.c_int32, _P, C.c_int32, _P, _P]),
    "fftdock_scan_pairs": (C.c_int, [C.POINTER(Config), C.c_int32, C.POINTER(PairDesc), C.c_int32,
                                     C.POINTER(PairsReport)]),
    "fftdock_pairs_last_error": (C.c_char_p, []),
    "fftdock_pair_grid": (C.c_int, [C.c_int32, _P, C.c_int32, _P, C.c_double, C.c_double, C.POINTER(C.c_int32)]),
    "fftdock_proposal_create": (C.c_int, [C.c_int32, C.c_uint64, C.POINTER(_P)]),
    "fftdock_proposal_destroy": (None, [_P]),
    "fftdock_proposal_last_error": (C.c_char_p, [_P]),
    "fftdock_proposal_n_params": (C.c_int32, []),
    "fftdock_proposal_get_params": (C.c_int, [_P, _P]),
    "fftdock_proposal_set_params": (C.c_int, [_P, _P]),
    "fftdock_proposal_add_ligand": (C.c_int, [_P, C.c_int32, _P, _P, C.POINTER(C.c_int32)]),
    "fftdock_proposal_add_samples": (C.c_int, [_P, C.c_int32, C.c_int32, _P, _P]),
    "fftdock_proposal_clear_samples": (C.c_int, [_P]),
    "fftdock_proposal_train": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_float, C.c_uint64, C.POINTER(C.c_float)]),
    "fftdock_proposal_gradients": (C.c_int, [_P, C.c_int32, _P, _P, _P, _P, C.POINTER(C.c_float)]),
    "fftdock_proposal_predict": (C.c_int, [_P, C.c_int32, C.c_int32, _P, _P]),
    "fftdock_proposal_predict_device": (C.c_int, [_P, C.c_int32, C.c_int32, _P, _P, _P]),
    "fftdock_receptor_descriptor": (C.c_int, [C.c_int32, _P, _P, _P]),
    "fftdock_receptor_descriptor_oriented": (C.c_int, [C.c_int32, _P, _P]),
}

_lib = None


def lib():
    """Load libfftdock.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            "libfftdock.so is not built (%s); run `python -m proddl2_gb300.build` -- "
            "there is no CPU fallback" % LIB_PATH)
    h = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(h, name)
        fn.restype = res
        fn.argtypes = args
    _lib = h
    return h


class FFTDockError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS_NAMES.get(code, str(code)), msg))
        self.code = code
