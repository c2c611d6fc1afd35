"""ctypes wrapper of the oracle's C restatement of run_cpu (fdtd.rs:644-725).

Test infrastructure only (see oracle/__init__.py).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        dp, i64p, u32p, u8p = (C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_uint32),
                               C.POINTER(C.c_uint8))
        args = [C.c_int64, C.c_int64, C.c_int64, C.c_double, u8p, u32p, C.c_int64, u32p, u32p, dp, i64p, dp,
                C.c_int64, dp, C.c_int64, i64p, C.c_int64, dp, C.c_int64, dp, dp, C.c_int]
        for name in ("wo_run_f64", "wo_run_f32"):
            f = getattr(L, name)
            f.restype = C.c_int
            f.argtypes = args
        L.wo_max_threads.restype = C.c_int
        L.wo_last_loop_seconds.restype = C.c_double
        L.wo_run_f16.restype = C.c_int
        L.wo_run_f16.argtypes = [C.c_int64, C.c_int64, C.c_int64, C.c_double, u8p, u32p, C.c_int64, u32p, dp,
                                 C.c_int64, i64p, i64p, dp, dp, C.c_int64, i64p, C.c_int64, dp, C.c_int]
        _lib = L
    return _lib


def max_threads() -> int:
    return lib().wo_max_threads()


def last_loop_seconds() -> float:
    """Seconds of the step loop of the last FP64 run, without its allocation
    and first touch of the fields."""
    return float(lib().wo_last_loop_seconds())


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def run(grid, taps, signal, receivers, freqs, precision: str = "f64", ir: bool = False, threads: int = 0):
    """Receiver spectra [n_recv, nf] (complex) of the reference's CPU run,
    and the time series [n_recv, steps] when ir=True.

    precision "f64": fdtd::run_cpu_with (fdtd.rs:644-725);
    precision "f32": the same loop in the shader's FP32 order (fdtd.wgsl).
    """
    flags = np.ascontiguousarray(grid.flags, dtype=np.uint8)
    bidx = np.ascontiguousarray(grid.bidx, dtype=np.uint32)
    bcell = np.ascontiguousarray(grid.bcell, dtype=np.uint32)
    bstart = np.ascontiguousarray(grid.bstart, dtype=np.uint32)
    slots = np.ascontiguousarray(grid.slots, dtype=np.float64).reshape(-1)
    if len(bcell) == 0:
        bcell = np.zeros(1, np.uint32)
    if len(slots) == 0:
        slots = np.zeros(4)
    tc = np.ascontiguousarray([int(c) for c, _ in taps] or [0], dtype=np.int64)
    tw = np.ascontiguousarray([float(w) for _, w in taps] or [0.0], dtype=np.float64)
    sig = np.ascontiguousarray(signal, dtype=np.float64)
    rx = np.ascontiguousarray(receivers if len(receivers) else [0], dtype=np.int64)
    fr = np.ascontiguousarray(freqs if len(freqs) else [0.0], dtype=np.float64)
    nr, nf = len(receivers), len(freqs)
    out = np.zeros(max(nr * nf, 1) * 2, dtype=np.float64)
    irb = np.zeros(max(nr * len(sig), 1), dtype=np.float64) if ir else None
    f = lib().wo_run_f64 if precision == "f64" else lib().wo_run_f32
    st = f(grid.n[0], grid.n[1], grid.n[2], grid.dt, _p(flags, C.c_uint8), _p(bidx, C.c_uint32),
           len(grid.bstart) - 1, _p(bcell, C.c_uint32), _p(bstart, C.c_uint32), _p(slots, C.c_double),
           _p(tc, C.c_int64), _p(tw, C.c_double), len(taps), _p(sig, C.c_double), len(sig), _p(rx, C.c_int64), nr,
           _p(fr, C.c_double), nf, _p(out, C.c_double), _p(irb, C.c_double) if ir else None, int(threads))
    if st != 0:
        raise MemoryError("oracle allocation failed")
    spec = out[: 2 * nr * nf].view(np.complex128).reshape(nr, nf)
    if ir:
        return spec, irb[: nr * len(sig)].reshape(nr, len(sig))
    return spec


def run_f16(grid, sources, signal, receivers, shift: int = 14):
    """Receiver time series [S, n_recv, steps] of the FP16-storage form
    (fp16_oracle.c): the right-hand sides in chunks of V lanes as the CUDA
    plan packs them (V = 1, 2 or 4; a 3-source batch is one 4-lane chunk),
    each chunk sharing its slab scales.  signal: one row for every source or
    one row per source."""
    S = len(sources)
    V = 4 if S >= 4 else (1 if S == 1 else (2 if S == 2 else 4))
    sig = np.asarray(signal, dtype=np.float64)
    steps = sig.shape[-1]
    rows = sig if sig.ndim == 2 else np.broadcast_to(sig, (S, steps))
    flags = np.ascontiguousarray(grid.flags, dtype=np.uint8)
    bidx = np.ascontiguousarray(grid.bidx, dtype=np.uint32)
    bstart = np.ascontiguousarray(grid.bstart, dtype=np.uint32)
    slots = np.ascontiguousarray(grid.slots, dtype=np.float64).reshape(-1)
    if len(slots) == 0:
        slots = np.zeros(4)
    rx = np.ascontiguousarray(receivers if len(receivers) else [0], dtype=np.int64)
    nr = len(receivers)
    out = np.zeros((S, nr, steps))
    for c0 in range(0, S, V):
        chunk = sources[c0:c0 + V]
        starts, cells, weights = [0], [], []
        for taps in chunk:
            cells += [int(c) for c, _ in taps]
            weights += [float(w) for _, w in taps]
            starts.append(len(cells))
        starts += [len(cells)] * (V - len(chunk))  # padding lanes: no taps
        lane_sig = np.zeros((V, steps))
        lane_sig[:len(chunk)] = rows[c0:c0 + len(chunk)]
        ts = np.ascontiguousarray(starts, dtype=np.int64)
        tc = np.ascontiguousarray(cells or [0], dtype=np.int64)
        tw = np.ascontiguousarray(weights or [0.0], dtype=np.float64)
        ls = np.ascontiguousarray(lane_sig)
        irb = np.zeros(max(V * nr * steps, 1))
        st = lib().wo_run_f16(grid.n[0], grid.n[1], grid.n[2], grid.dt, _p(flags, C.c_uint8), _p(bidx, C.c_uint32),
                              len(grid.bstart) - 1, _p(bstart, C.c_uint32), _p(slots, C.c_double), V,
                              _p(ts, C.c_int64), _p(tc, C.c_int64), _p(tw, C.c_double), _p(ls, C.c_double), steps,
                              _p(rx, C.c_int64), nr, _p(irb, C.c_double), int(shift))
        if st == 2:
            raise FloatingPointError("a value left the FP16 range of its slab scale")
        if st != 0:
            raise MemoryError("oracle allocation failed")
        out[c0:c0 + len(chunk)] = irb[:V * nr * steps].reshape(V, nr, steps)[:len(chunk)]
    return out
