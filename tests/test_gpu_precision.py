"""The reduced-precision storage form against the FP64 oracle.

FP16 field storage (WAVEY_FP16_STORAGE) rounds every stored field value to
11 significant bits, so it cannot match the FP64 scheme bit for bit; these
tests state the error it is kept under on the reference's own test grids.
Measured on a GB300 (room_pillars, 8661 steps, 4 right-hand sides, against
the FP64 GPU run): octave-band levels within 0.16 dB (99 % within 0.07 dB),
receiver time series within 1.6 % of their peak.  On the branch-material
room the late time series carries a slowly varying (near-DC) component in
which FP16 rounding accumulates to about 5 % of the peak; its spectra stay
within 2 %.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import fdtd as ofd
from scenes import branch_room, pillar_room, spread_source, worst_relative
from wavey_gb300.backend import FP16_STORAGE, FP64

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("scene", ["spread", "pillar", "branches"])
def test_fp16_storage_within_stated_error(backend, library, scene):
    g, taps, sig, rcv, freqs = {"spread": spread_source, "pillar": pillar_room,
                                "branches": lambda: branch_room(library)}[scene]()
    ref, ref_ir = ofd.run(g, taps, sig, rcv, freqs, "f64", ir=True)
    spec, ir = backend.run_batch(g, [taps], sig, rcv, freqs, precision=FP16_STORAGE, ir=True)
    assert worst_relative(ref, spec[0]) < 2e-2
    peak = np.abs(ref_ir).max(axis=1, keepdims=True)
    assert float((np.abs(ir[0] - ref_ir) / peak).max()) < (8e-2 if scene == "branches" else 3e-2)


def test_fp16_batch_of_components(backend):
    """A directional source's four components in one FP16 chunk."""
    from scenes import directional_components

    g, taps, sig, rcv, freqs = spread_source()
    comps = directional_components(g, (3.0, 2.0, 1.5))
    ref = np.stack([ofd.run(g, c, sig, rcv, freqs, "f64") for c in comps])
    spec = backend.run_batch(g, comps, sig, rcv, freqs, precision=FP16_STORAGE)
    for s in range(4):
        assert worst_relative(ref[s], spec[s]) < 2e-2


def test_fp64_gpu_matches_oracle_spectra(backend, library):
    g, taps, sig, rcv, freqs = pillar_room(0.3)
    ref = ofd.run(g, taps, sig, rcv, freqs, "f64")
    spec = backend.run_batch(g, [taps], sig, rcv, freqs, precision=FP64)
    assert worst_relative(ref, spec[0]) < 1e-9


def test_fp64_receiver_accumulation_option(backend):
    """WAVEY_DFT_FP64=1: FP32 fields with the receiver DFT folded in FP64
    (FP64 twiddles, FP64 sums over each 128-step chunk).  The time series are
    the FP32 run's bit for bit (only the fold changes); the spectra stay
    within the reference's 1e-3 bar of the FP64 oracle and move by no more
    than FP32 chunk-sum rounding from the FP32-fold spectra."""
    import os

    from wavey_gb300.backend import FP32

    g, taps, sig, rcv, freqs = spread_source()
    ref_spec, ref_ir = backend.run_batch(g, [taps], sig, rcv, freqs, precision=FP32, ir=True)
    os.environ["WAVEY_DFT_FP64"] = "1"
    try:
        plan = backend.plan(g, [taps], sig, rcv, freqs, precision=FP32, ir=True)
        assert plan.info()["dft_fp64"] == 1
        plan.run()
        spec, ir = plan.read()
        plan.close()
    finally:
        del os.environ["WAVEY_DFT_FP64"]
    assert np.array_equal(ir, ref_ir)
    ora = ofd.run(g, taps, sig, rcv, freqs, "f64")
    assert worst_relative(ora, spec[0]) < 1e-3
    assert worst_relative(ref_spec, spec) < 1e-5
