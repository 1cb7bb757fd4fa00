"""GB300-native FFT rotational/translational correlation scan (PRODDL2 rot-scan).

The compute path is ``libfftdock.so`` (hand-written sm_103a CUDA behind the C
ABI of ``include/fftdock.h``); this package is its host-side interface.
"""
from .scan import FFTScan, ScanConfig, ScanResult, find_best_size, supported_grid, write_scan_records  # noqa: F401
from ._lib import FFTDockError  # noqa: F401

__all__ = ["FFTScan", "ScanConfig", "ScanResult", "FFTDockError", "find_best_size", "supported_grid",
           "write_scan_records"]
