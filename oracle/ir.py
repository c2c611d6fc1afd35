"""ctypes wrapper of the oracle's C restatement of the impulse-response
analysis (analysis.rs; oracle/ir_oracle.c).  Test infrastructure only (see
oracle/__init__.py)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import fdtd as _fdtd

OCTAVES = (63.0, 125.0, 250.0, 500.0, 1000.0, 2000.0, 4000.0, 8000.0)
PARAMS = ("edt", "t20", "t30", "c80", "d50", "ts")


def _lib():
    L = _fdtd.lib()
    if not getattr(L, "_ir_ready", False):
        dp, i64 = C.POINTER(C.c_double), C.c_int64
        L.wo_ir_params.argtypes = [dp, i64, C.c_double, dp, C.c_int, C.c_int, C.c_int, dp]
        L.wo_ir_params.restype = None
        L.wo_octave_filter.argtypes = [dp, i64, C.c_double, C.c_double]
        L.wo_octave_filter.restype = None
        L.wo_onset.argtypes = [dp, i64]
        L.wo_onset.restype = i64
        L.wo_params_from.argtypes = [dp, i64, C.c_double, C.c_double, dp]
        L.wo_params_from.restype = None
        L._ir_ready = True
    return L


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def octave_filter(x, fc: float, fs: float) -> np.ndarray:
    y = np.ascontiguousarray(x, dtype=np.float64).copy()
    _lib().wo_octave_filter(_dp(y), len(y), float(fc), float(fs))
    return y


def onset(x) -> int:
    a = np.ascontiguousarray(x, dtype=np.float64)
    return int(_lib().wo_onset(_dp(a), len(a)))


def noise_free_params(e, fs: float) -> np.ndarray:
    a = np.ascontiguousarray(e, dtype=np.float64)
    out = np.empty(6)
    _lib().wo_params_from(_dp(a), len(a), 0.0, float(fs), _dp(out))
    return out


def ir_params(p, fs: float, bands=OCTAVES, integrate: bool = True, lundeby: bool = True) -> np.ndarray:
    """[n_bands][6] = edt, t20, t30, c80, d50, ts of one time series."""
    a = np.ascontiguousarray(p, dtype=np.float64)
    b = np.ascontiguousarray(bands, dtype=np.float64)
    out = np.empty((len(b), 6))
    _lib().wo_ir_params(_dp(a), len(a), float(fs), _dp(b), len(b), int(integrate), int(lundeby), _dp(out))
    return out
