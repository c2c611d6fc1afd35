"""Failure handling of the CUDA backend, made on the host.

The reference checks its limits before it touches the device
(core/wavey-solver/src/gpu_fdtd.rs:56-66), returns Ok(None) when cancelled
(gpu_fdtd.rs:202-204) and an Err otherwise.  Here every bad input is
rejected by the C-ABI before any kernel runs, with a negative status and a
message; cancellation returns WAVEY_CANCELLED at the next 128-step chunk.
Nothing in these tests faults, traps or hangs a GPU: the failures are bad
arguments and a host flag.
"""
from __future__ import annotations

import numpy as np
import pytest

from scenes import spread_source
from wavey_gb300 import _native as N
from wavey_gb300.backend import CancelFlag, WaveyError

pytestmark = pytest.mark.gpu


class _Grid:
    """A grid whose arrays a test may corrupt."""

    def __init__(self, g):
        self.n, self.dx, self.dt = g.n, g.dx, g.dt
        self.flags, self.bidx = g.flags.copy(), g.bidx.copy()
        self.bstart, self.slots = g.bstart.copy(), g.slots.copy()


def test_cancel_from_progress_returns_none(backend):
    g, taps, sig, rcv, freqs = spread_source()
    flag = CancelFlag()
    seen = []

    def progress(f):
        seen.append(f)
        if f > 0.3:
            flag.set()

    assert backend.run_fdtd(g, taps, sig, rcv, freqs, cancel=flag, progress=progress) is None
    assert 0.3 < seen[-1] < 1.0
    # The same backend runs again normally afterwards.
    flag.clear()
    assert backend.run_fdtd(g, taps, sig[:300], rcv, freqs, cancel=flag) is not None


def test_progress_reaches_one(backend):
    g, taps, sig, rcv, freqs = spread_source()
    seen = []
    backend.run_fdtd(g, taps, sig, rcv, freqs, progress=seen.append)
    assert seen == sorted(seen) and seen[-1] == 1.0


def _expect(backend, code, match, *args, **kw):
    with pytest.raises(WaveyError, match=match) as e:
        backend.run_batch(*args, **kw)
    assert e.value.code == code


def test_bad_taps_and_receivers_are_rejected(backend):
    g, taps, sig, rcv, freqs = spread_source()
    cells = g.n[0] * g.n[1] * g.n[2]
    _expect(backend, N.WAVEY_E_INVALID, "out of range", g, [[(cells, 1.0)]], sig, rcv, freqs)
    _expect(backend, N.WAVEY_E_INVALID, "out of range", g, [[(-1, 1.0)]], sig, rcv, freqs)
    _expect(backend, N.WAVEY_E_INVALID, "not air", g, [[(0, 1.0)]], sig, rcv, freqs)
    _expect(backend, N.WAVEY_E_INVALID, "receiver", g, [taps], sig, [cells + 5], freqs)
    _expect(backend, N.WAVEY_E_INVALID, "no sources", g, [], sig, rcv, freqs)
    _expect(backend, N.WAVEY_E_INVALID, "precision", g, [taps], sig, rcv, freqs, precision=7)


def test_grid_without_solid_border_is_rejected(backend):
    g, taps, sig, rcv, freqs = spread_source()
    bad = _Grid(g)
    bad.flags[0] = 64  # an air cell on the border: its neighbours would leave the grid
    _expect(backend, N.WAVEY_E_INVALID, "border", bad, [taps], sig, rcv, freqs)


def test_corrupt_boundary_tables_are_rejected(backend):
    g, taps, sig, rcv, freqs = spread_source()
    bad = _Grid(g)
    i = int(np.flatnonzero(bad.bidx != 0xFFFFFFFF)[0])
    bad.bidx[i] = len(bad.bstart) + 10
    _expect(backend, N.WAVEY_E_INVALID, "boundary index", bad, [taps], sig, rcv, freqs)
    bad = _Grid(g)
    bad.bstart[1], bad.bstart[2] = bad.bstart[2], bad.bstart[1]
    _expect(backend, N.WAVEY_E_INVALID, "ascending", bad, [taps], sig, rcv, freqs)


def test_limits_are_errors(backend):
    g, taps, sig, rcv, freqs = spread_source()
    huge = _Grid(g)
    huge.n = (1000, 1000, 1000)  # 1e9 cells > MAX_CELLS (fdtd.rs:140)
    _expect(backend, N.WAVEY_E_LIMIT, "M cells", huge, [taps], sig, rcv, freqs)
    many = _Grid(g)
    b = int(np.flatnonzero(np.diff(many.bstart.astype(np.int64)) > 0)[0])
    many.bstart = many.bstart.astype(np.int64)
    many.bstart[b + 1:] += 40  # one node with more than 31 slots
    many.bstart = many.bstart.astype(np.uint32)
    many.slots = np.concatenate([many.slots, np.zeros((40, 4))])
    _expect(backend, N.WAVEY_E_LIMIT, "slots", many, [taps], sig, rcv, freqs)


def test_backend_survives_rejected_calls(backend):
    g, taps, sig, rcv, freqs = spread_source()
    with pytest.raises(WaveyError):
        backend.run_batch(g, [[(-1, 1.0)]], sig, rcv, freqs)
    out = backend.run_fdtd(g, taps, sig[:256], rcv, freqs)
    assert np.all(np.isfinite(out))
