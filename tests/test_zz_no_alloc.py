"""wavey_cuda_receiver_dft_noalloc: receiver spectra without device allocation.

This entry point serves callers that cannot allocate device memory when they
need the spectra (a real-time audio thread, where cudaMalloc can stall the
device; a host whose pool allocator owns all device memory).  The test gives
it receiver time series already on the device and compares its spectra with
those of the regular entry point (wavey_cuda_fdtd_run) for the same run, on
two calls in a row, since every call reuses the same fixed scratch array.

Kept in a file of its own, collected after every other test file.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from scenes import branch_room, spread_source, worst_relative
from wavey_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _noalloc(series: np.ndarray, freqs: np.ndarray, dt: float) -> np.ndarray:
    import torch

    d_series = torch.as_tensor(np.ascontiguousarray(series, dtype=np.float32), device="cuda")
    d_freqs = torch.as_tensor(np.ascontiguousarray(freqs, dtype=np.float64), device="cuda")
    n_recv, steps = series.shape
    nf = len(freqs)
    d_out = torch.full((n_recv, nf, 2), float("nan"), dtype=torch.float64, device="cuda")
    err = C.create_string_buffer(256)
    torch.cuda.synchronize()
    st = N.cuda().wavey_cuda_receiver_dft_noalloc(
        0, C.cast(d_series.data_ptr(), C.POINTER(C.c_float)), n_recv, steps,
        C.cast(d_freqs.data_ptr(), C.POINTER(C.c_double)), nf, float(dt),
        C.cast(d_out.data_ptr(), C.POINTER(C.c_double)), None, err, 256)
    torch.cuda.synchronize()
    assert st == N.WAVEY_OK, err.value.decode()
    out = d_out.cpu().numpy()
    return out[..., 0] + 1j * out[..., 1]


def test_noalloc_dft_matches_regular_entry_point_twice(backend, library):
    runs = [spread_source(), branch_room(library, 0.2)]
    for g, taps, sig, rcv, freqs in runs:
        spec, ir = backend.run_fdtd(g, taps, sig, rcv, freqs, ir=True)
        got = _noalloc(ir, freqs, g.dt)
        assert got.shape == spec.shape
        assert worst_relative(spec, got) < 1e-6


def test_noalloc_rejects_too_many_frequencies():
    err = C.create_string_buffer(256)
    st = N.cuda().wavey_cuda_receiver_dft_noalloc(0, None, 4, 100, None, 4096, 1e-4, None, None, err, 256)
    assert st == N.WAVEY_E_LIMIT
    assert b"2048" in err.value
