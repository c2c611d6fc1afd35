"""Degenerate and ragged inputs through the C-ABI, against the oracle where
there is something to compare: no receivers, no frequencies, no steps, a
step count that is not a multiple of the 128-step chunk and one shorter than
a chunk, taps repeated within a source (the reference sums them per cell,
gpu_fdtd.rs:67-75), identical sources in one batch, a zero-weight source,
and receivers on special cells (boundary nodes and the tap cell itself)."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import fdtd as ofd
from scenes import branch_room, spread_source
from wavey_gb300.backend import FP16_STORAGE, FP32, FP64

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [FP32, FP64, FP16_STORAGE], ids=["fp32", "fp64", "fp16"])
def test_no_receivers_no_freqs_no_steps(backend, precision):
    g, taps, sig, rcv, freqs = spread_source()
    out = backend.run_batch(g, [taps], sig[:300], [], freqs, precision=precision)
    assert out.shape == (1, 0, len(freqs))
    out = backend.run_batch(g, [taps], sig[:300], rcv, [], precision=precision)
    assert out.shape == (1, len(rcv), 0)
    spec, ir = backend.run_batch(g, [taps], sig[:0], rcv, freqs, precision=precision, ir=True)
    assert spec.shape == (1, len(rcv), len(freqs)) and not np.any(spec) and ir.shape == (1, len(rcv), 0)


@pytest.mark.parametrize("steps", [1, 77, 128, 129, 300])
def test_ragged_step_counts_match_the_oracle(backend, steps):
    g, taps, sig, rcv, freqs = spread_source()
    _, ref_ir = ofd.run(g, taps, sig[:steps], rcv, freqs, "f32", ir=True)
    _, ir = backend.run_fdtd(g, taps, sig[:steps], rcv, freqs, ir=True)
    assert ir.shape == (len(rcv), steps)
    assert np.array_equal(ir, ref_ir)


def test_repeated_taps_are_summed_per_cell(backend):
    g, taps, sig, rcv, freqs = spread_source()
    split = []
    for cell, w in taps:
        split += [(cell, 0.25 * w), (cell, 0.75 * w)]  # same cell twice, weights summing to w
    _, a = backend.run_fdtd(g, taps, sig[:400], rcv, freqs, ir=True)
    _, b = backend.run_fdtd(g, split, sig[:400], rcv, freqs, ir=True)
    # The merged weight 0.25 w + 0.75 w is w exactly for these weights.
    assert np.array_equal(a, b)


def test_identical_and_zero_sources_in_one_batch(backend):
    g, taps, sig, rcv, freqs = spread_source()
    zero = [(c, 0.0) for c, _ in taps]
    spec, ir = backend.run_batch(g, [taps, zero, taps, taps, zero], sig[:400], rcv, freqs, ir=True)
    assert np.array_equal(ir[0], ir[2]) and np.array_equal(ir[0], ir[3]) and np.array_equal(ir[2], ir[3])
    assert not np.any(ir[1]) and not np.any(ir[4]) and not np.any(spec[1])


def test_receivers_on_special_cells(backend, library):
    g, taps, sig, rcv, freqs = branch_room(library, 0.1)
    boundary = [int(g.bcell[k]) for k in (0, len(g.bcell) // 2, len(g.bcell) - 1)]
    rx = boundary + [taps[0][0]] + list(rcv)
    _, ref_ir = ofd.run(g, taps, sig, rx, freqs, "f32", ir=True)
    _, ir = backend.run_fdtd(g, taps, sig, rx, freqs, ir=True)
    assert np.array_equal(ir, ref_ir)
    assert np.any(ir[3])  # the tap cell itself carries the injected signal
