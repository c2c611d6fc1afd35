"""The benchmark configurations that run whole in seconds, against the oracle.

* The small shoebox (6 x 4 x 3 m, seeded wall absorption 0.05-0.4, 250 Hz,
  one monopole, 8 receivers, the full 0.5 s): spectra within the reference's
  GPU-vs-CPU bar of 1e-3 (core/wavey-solver/tests/fdtd.rs:168, 203, 374) of
  the FP64 oracle (fdtd::run_cpu), receiver time series bit-identical to the
  FP32 restatement in the shader's order, and the FP64 path bit-identical to
  the FP64 oracle.
* The multi-room batch (the small shoebox with 32 seeded speakers, plus four
  seeded shoeboxes of 5-25 x 4-20 x 3-10 m, all in one launch per step):
  every room's every right-hand side against the oracle over the full 0.5 s.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from oracle import fdtd as ofd
from scenes import worst_relative
from wavey_gb300 import workloads
from wavey_gb300.backend import FP64, RoomJob

pytestmark = pytest.mark.gpu


def test_small_shoebox_full_run_matches_oracle(backend):
    sc = workloads.room_small()
    taps = sc.sources[0]
    assert sc.steps == math.ceil(0.5 / sc.grid.dt)
    spec, ir = backend.run_fdtd(sc.grid, taps, sc.signal, sc.receivers, sc.freqs, ir=True)
    ref64, ref64_ir = ofd.run(sc.grid, taps, sc.signal, sc.receivers, sc.freqs, "f64", ir=True)
    _, ref32_ir = ofd.run(sc.grid, taps, sc.signal, sc.receivers, sc.freqs, "f32", ir=True)
    assert worst_relative(ref64, spec) < 1e-3
    assert np.array_equal(ir, ref32_ir), "FP32 time series differ from the shader-order restatement"
    spec64, ir64 = backend.run_batch(sc.grid, [taps], sc.signal, sc.receivers, sc.freqs, precision=FP64, ir=True)
    assert np.array_equal(ir64[0], ref64_ir), "FP64 time series differ from the FP64 oracle"
    assert worst_relative(ref64, spec64[0]) < 1e-12


def test_multi_room_batch_matches_oracle(backend):
    scenes = workloads.rooms_batch()
    jobs = [RoomJob(sc.grid, sc.sources, sc.signal, sc.receivers, sc.freqs) for sc in scenes]
    res = backend.run_rooms(jobs, ir=True)
    assert len(jobs[0].sources) >= 64
    for r, j in enumerate(jobs):
        spec, ir = res[r]
        assert spec.shape == (len(j.sources), len(j.receivers), len(j.freqs))
        for s, taps in enumerate(j.sources):
            _, ref32_ir = ofd.run(j.grid, taps, j.signal, j.receivers, j.freqs, "f32", ir=True)
            assert np.array_equal(ir[s], ref32_ir), f"room {r}, right-hand side {s}: time series differ"
        # The FP64 spectra of the first and last right-hand side of each room.
        for s in sorted({0, len(j.sources) - 1}):
            ref64 = ofd.run(j.grid, j.sources[s], j.signal, j.receivers, j.freqs, "f64")
            assert worst_relative(ref64, spec[s]) < 1e-3, f"room {r}, right-hand side {s}"
