"""wavey_cuda_receiver_dft_noalloc: receiver spectra without device allocation.

This entry point serves callers that cannot allocate device memory when they
need the spectra (a real-time audio thread, where cudaMalloc can stall the
device; a host whose pool allocator owns all device memory).  The tests give
it receiver time series already on the device and compare its spectra with
those of the regular entry point (wavey_cuda_fdtd_run) for the same run, on
two calls in a row, since every call reuses the same fixed scratch array;
they check that a warmed-up call leaves the device's free memory unchanged,
and they call it on a side stream and at its frequency limit.

Kept in a file of its own, collected after every other test file.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from scenes import branch_room, spread_source, worst_relative
from wavey_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _device_inputs(series: np.ndarray, freqs: np.ndarray):
    import torch

    d_series = torch.as_tensor(np.ascontiguousarray(series, dtype=np.float32), device="cuda")
    d_freqs = torch.as_tensor(np.ascontiguousarray(freqs, dtype=np.float64), device="cuda")
    d_out = torch.full((series.shape[0], len(freqs), 2), float("nan"), dtype=torch.float64, device="cuda")
    return d_series, d_freqs, d_out


def _call(d_series, d_freqs, d_out, dt: float, stream=None) -> None:
    """One call of the entry point; everything it touches is allocated by the caller."""
    n_recv, steps = d_series.shape
    err = C.create_string_buffer(256)
    st = N.cuda().wavey_cuda_receiver_dft_noalloc(
        0, C.cast(d_series.data_ptr(), C.POINTER(C.c_float)), n_recv, steps,
        C.cast(d_freqs.data_ptr(), C.POINTER(C.c_double)), d_freqs.shape[0], float(dt),
        C.cast(d_out.data_ptr(), C.POINTER(C.c_double)), stream, err, 256)
    assert st == N.WAVEY_OK, err.value.decode()


def _spectra(d_out) -> np.ndarray:
    out = d_out.cpu().numpy()
    return out[..., 0] + 1j * out[..., 1]


def _noalloc(series: np.ndarray, freqs: np.ndarray, dt: float) -> np.ndarray:
    import torch

    d_series, d_freqs, d_out = _device_inputs(series, freqs)
    torch.cuda.synchronize()
    _call(d_series, d_freqs, d_out, dt)
    torch.cuda.synchronize()
    return _spectra(d_out)


def test_noalloc_dft_matches_regular_entry_point_twice(backend, library):
    runs = [spread_source(), branch_room(library, 0.2)]
    for g, taps, sig, rcv, freqs in runs:
        spec, ir = backend.run_fdtd(g, taps, sig, rcv, freqs, ir=True)
        got = _noalloc(ir, freqs, g.dt)
        assert got.shape == spec.shape
        assert worst_relative(spec, got) < 1e-6


def test_noalloc_call_leaves_device_memory_unchanged(backend, library):
    """After one warm-up call (which may load the library's module and with it
    the fixed scratch array), further calls must not change the device's free
    memory: they allocate nothing."""
    import torch

    g, taps, sig, rcv, freqs = spread_source()
    spec, ir = backend.run_fdtd(g, taps, sig, rcv, freqs, ir=True)
    d_series, d_freqs, d_out = _device_inputs(ir, freqs)
    torch.cuda.synchronize()
    _call(d_series, d_freqs, d_out, g.dt)
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        _call(d_series, d_freqs, d_out, g.dt)
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before, f"device free memory changed by {free_before - free_after} bytes"
    assert worst_relative(spec, _spectra(d_out)) < 1e-6


def test_noalloc_on_a_side_stream_at_the_frequency_limit(backend, library):
    """A call on a non-default stream, with the maximum number of frequencies
    and a step count that is not a multiple of the 128-step chunk, against the
    regular entry point's spectra of the same run."""
    import torch

    g, taps, sig, rcv, _ = spread_source()
    steps = 300
    sig = sig[:steps]
    nf = N.WAVEY_NOALLOC_MAX_FREQS
    freqs = np.linspace(20.0, 400.0, nf)
    spec, ir = backend.run_fdtd(g, taps, sig, rcv, freqs, ir=True)
    d_series, d_freqs, d_out = _device_inputs(ir, freqs)
    side = torch.cuda.Stream()
    torch.cuda.synchronize()
    for _ in range(2):
        d_out.fill_(float("nan"))
        torch.cuda.synchronize()
        _call(d_series, d_freqs, d_out, g.dt, C.c_void_p(side.cuda_stream))
        side.synchronize()
        assert worst_relative(spec, _spectra(d_out)) < 1e-6


def test_noalloc_rejects_too_many_frequencies():
    err = C.create_string_buffer(256)
    st = N.cuda().wavey_cuda_receiver_dft_noalloc(0, None, 4, 100, None, 4096, 1e-4, None, None, err, 256)
    assert st == N.WAVEY_E_LIMIT
    assert b"2048" in err.value


def test_noalloc_rejects_an_overflowing_size():
    err = C.create_string_buffer(256)
    st = N.cuda().wavey_cuda_receiver_dft_noalloc(0, None, 2**62, 100, None, 2048, 1e-4, None, None, err, 256)
    assert st == N.WAVEY_E_LIMIT
