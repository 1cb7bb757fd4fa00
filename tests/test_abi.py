"""C ABI surface of libfftdock.so, checked without a GPU.

The library must load, export every function include/fftdock.h declares, and
answer the host-only calls (defaults, size rule, record writer) exactly like
the oracle.  Calls that need a GPU must fail loudly where there is none.
"""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import fftdock_oracle as O

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "fftdock.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fftdock_[a-z_]+)\s*\(", text)))


def test_header_declares_expected_surface():
    names = declared_functions()
    from proddl2_gb300 import _lib
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(str(built_lib))
    for name in declared_functions():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", str(built_lib)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (fftdock_\w+)", out))
    assert set(declared_functions()) <= exported


def test_config_defaults(built_lib):
    from proddl2_gb300 import _lib
    cfg = _lib.Config()
    _lib.lib().fftdock_config_init(C.byref(cfg))
    assert cfg.struct_size == C.sizeof(_lib.Config)
    assert (cfg.grid_n, cfg.grid_step, cfg.peaks_per_rot, cfg.rot_batch) == (128, 1.2, 4, 64)
    assert cfg.term_set == _lib.FFTDOCK_TERMS_SHAPE_ACE and cfg.n_types == 18
    assert np.isinf(cfg.max_val_corr)
    assert (cfg.ace_b, cfg.ace_k, cfg.ace_a, cfg.ace_cut) == (7.0, 0.15, 0.6, 6.0)


def test_peak_struct_layout():
    from proddl2_gb300 import _lib
    assert C.sizeof(_lib.Peak) == 48
    assert _lib.peak_dtype().itemsize == 48
    assert _lib.Peak.t.offset == 16 and _lib.Peak.score.offset == 40


def test_supported_grids(built_lib):
    from proddl2_gb300 import supported_grid
    for n in (16, 24, 32, 48, 64, 80, 96, 112, 128, 144):
        assert supported_grid(n)
    for n in (0, 8, 100, 120, 256):
        assert not supported_grid(n)


def test_find_best_size_matches_oracle(built_lib):
    from proddl2_gb300 import find_best_size
    for n in list(range(0, 400)) + [1000, 1021, 2047, 4097]:
        assert find_best_size(n) == O.find_best_size(n), n


def test_scan_records_writer_matches_reference_layout(built_lib, tmp_path):
    from proddl2_gb300 import ScanResult, write_scan_records, _lib
    rng = np.random.default_rng(1)
    n_rot, P = 3, 4
    rot = rng.normal(size=(n_rot, 3, 3))
    peaks = np.zeros((n_rot, P), dtype=_lib.peak_dtype())
    peaks["t"] = rng.normal(size=(n_rot, P, 3))
    peaks["score"] = rng.normal(size=(n_rot, P))
    npk = np.array([4, 0, 2], dtype=np.int32)
    path = tmp_path / "scan.bin"
    write_scan_records(path, rot, ScanResult(peaks, npk))
    write_scan_records(path, rot[:1], ScanResult(peaks[:1], npk[:1]), append=True)
    data = path.read_bytes()
    expect = b"".join(O.pack_record(rot[i], peaks["t"][i, :npk[i]], peaks["score"][i, :npk[i]])
                      for i in range(n_rot))
    expect += O.pack_record(rot[0], peaks["t"][0, :4], peaks["score"][0, :4])
    assert data == expect
    recs = O.unpack_records(data)
    assert [len(r[2]) for r in recs] == [4, 0, 2, 4]


def test_create_fails_loudly_without_gpu(built_lib):
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    from proddl2_gb300 import FFTScan, ScanConfig, FFTDockError, _lib
    with pytest.raises(FFTDockError) as ei:
        FFTScan(ScanConfig(grid_n=32, term_set="shape"))
    assert ei.value.code == _lib.FFTDOCK_ECUDA


def test_create_rejects_bad_config(built_lib):
    from proddl2_gb300 import FFTScan, ScanConfig, FFTDockError, _lib
    bad = [
        (dict(grid_n=97), _lib.FFTDOCK_EUNSUPPORTED),           # prime: no FFT plan
        (dict(grid_n=300), _lib.FFTDOCK_EUNSUPPORTED),          # beyond the box-grid sizes
        (dict(grid_dims=(90, 96, 100), precision="bf16"), _lib.FFTDOCK_EUNSUPPORTED),  # box grids keep FP32
        (dict(grid_dims=(90, 96, 100), cluster_trans=True), _lib.FFTDOCK_EUNSUPPORTED),
        (dict(grid_dims=(90, 96, 100), peaks_per_rot=17), _lib.FFTDOCK_EUNSUPPORTED),
        (dict(grid_dims=(90, 96, 102)), _lib.FFTDOCK_EUNSUPPORTED),  # 102 = 2 * 3 * 17
        (dict(grid_n=32, peaks_per_rot=0), _lib.FFTDOCK_EINVAL),
        (dict(grid_n=32, peaks_per_rot=257), _lib.FFTDOCK_EINVAL),
        (dict(grid_n=32, grid_step=0.0), _lib.FFTDOCK_EINVAL),
        (dict(grid_n=32, rot_batch=0), _lib.FFTDOCK_EINVAL),
        (dict(grid_n=32, term_set="shape_ace", ace_matrix=None), _lib.FFTDOCK_EINVAL),
    ]
    for kw, code in bad:
        with pytest.raises(FFTDockError) as ei:
            FFTScan(ScanConfig(**kw))
        assert ei.value.code == code, kw
