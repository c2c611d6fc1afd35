"""The CUDA path against the oracle, through the C-ABI.

Bars:
  * spectra, FP32 GPU vs the FP64 CPU restatement of run_cpu: worst
    |a - b| / max |a| < 1e-3, the reference's own GPU-vs-CPU bar
    (core/wavey-solver/tests/fdtd.rs:168, 203, 374);
  * receiver time series, FP32 GPU vs the FP32 restatement in the shader's
    operation order: bit-identical;
  * receiver time series, FP64 GPU vs the FP64 restatement: bit-identical;
  * a batched run's lanes vs single-source runs: bit-identical time series.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import fdtd as ofd
from scenes import branch_room, directional_components, pillar_room, spread_source, worst_relative
from wavey_gb300.backend import FP64

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("scene", ["spread", "pillar", "branches"])
def test_spectra_match_fp64_oracle(backend, library, scene):
    g, taps, sig, rcv, freqs = {"spread": spread_source, "pillar": pillar_room,
                                "branches": lambda: branch_room(library)}[scene]()
    ref = ofd.run(g, taps, sig, rcv, freqs, "f64")
    got = backend.run_fdtd(g, taps, sig, rcv, freqs)
    assert got.shape == (len(rcv), len(freqs))
    w = worst_relative(ref, got)
    assert w < 1e-3, f"{scene}: worst relative difference {w:.2e}"


@pytest.mark.parametrize("scene", ["spread", "branches"])
def test_fp32_time_series_bit_identical(backend, library, scene):
    g, taps, sig, rcv, freqs = {"spread": spread_source, "branches": lambda: branch_room(library, 0.2)}[scene]()
    _, ref_ir = ofd.run(g, taps, sig, rcv, freqs, "f32", ir=True)
    _, got_ir = backend.run_fdtd(g, taps, sig, rcv, freqs, ir=True)
    assert got_ir.shape == ref_ir.shape
    diff = np.flatnonzero(got_ir.reshape(-1) != ref_ir.reshape(-1))
    assert diff.size == 0, f"{diff.size} samples differ, first at {diff[0]}"


def test_fp64_time_series_bit_identical(backend, library):
    g, taps, sig, rcv, freqs = branch_room(library, 0.15)
    ref, ref_ir = ofd.run(g, taps, sig, rcv, freqs, "f64", ir=True)
    spec, ir = backend.run_batch(g, [taps], sig, rcv, freqs, precision=FP64, ir=True)
    assert np.array_equal(ir[0], ref_ir)
    assert worst_relative(ref, spec[0]) < 1e-9


def test_batched_lanes_equal_single_runs(backend):
    """Five right-hand sides (one full chunk of four plus a padded one):
    every lane's time series equals its own single-source run."""
    g, taps, sig, rcv, freqs = spread_source()
    sig = sig[:600]
    comps = directional_components(g, (3.0, 2.0, 1.5))
    sources = comps + [taps]
    spec, ir = backend.run_batch(g, sources, sig, rcv, freqs, ir=True)
    assert spec.shape == (5, len(rcv), len(freqs))
    for s, t in enumerate(sources):
        one_spec, one_ir = backend.run_fdtd(g, t, sig, rcv, freqs, ir=True)
        assert np.array_equal(ir[s], one_ir), f"lane {s}"
        assert worst_relative(one_spec, spec[s]) < 1e-6


def test_per_source_signals(backend):
    """Each right-hand side with its own signal: lane s equals a run of s alone."""
    g, taps, sig, rcv, freqs = spread_source()
    sig = sig[:400]
    sigs = np.stack([sig, -0.5 * sig, np.roll(sig, 7)])
    sources = [taps, taps, taps]
    _, ir = backend.run_batch(g, sources, sigs, rcv, freqs, ir=True)
    for s in range(3):
        _, one = backend.run_fdtd(g, taps, sigs[s], rcv, freqs, ir=True)
        assert np.array_equal(ir[s], one)


def test_autotuned_plan_gives_identical_results(backend):
    """The autotuner only changes the interior kernel's shape and the launch
    form of the special-cell branch, never the arithmetic: results before and
    after tuning are identical."""
    g, taps, sig, rcv, freqs = spread_source()
    plan = backend.plan(g, [taps, taps], sig[:700], rcv, freqs, ir=True)
    plan.run()
    before = plan.read()
    res = plan.autotune()
    assert res["candidates"] and res["step_us"] > 0
    # The winner is one of the candidates, and among the four fastest of the
    # first timing (the confirmation stage re-times those four).
    firsts = sorted(res["candidates"], key=lambda c: c[3])[:4]
    assert (res["cfg"], res["zt"], res["branch"]) in [(c[0], c[1], c[2]) for c in firsts]
    plan.run()
    after = plan.read()
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])
    assert plan.info()["tma_zt"] == res["zt"] and plan.info()["branch"] == res["branch"]
    plan.close()
