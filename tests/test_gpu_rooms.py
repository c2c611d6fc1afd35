"""Several rooms in one launch per step (wavey_cuda_fdtd_run_rooms).

Each room of a multi-room run must give exactly what it gives alone: the
rooms share launches, not arithmetic.  The rooms differ in size, number of
right-hand sides (so lanes per chunk), receivers, frequencies and step
count (a room that stops early must stop cleanly inside a chunk).
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import fdtd as ofd
from scenes import branch_room, directional_components, pillar_room, spread_source, worst_relative
from wavey_gb300.backend import FP32, FP64, RoomJob

pytestmark = pytest.mark.gpu


def _jobs(library):
    g1, t1, s1, r1, f1 = spread_source()
    g2, t2, s2, r2, f2 = branch_room(library, 0.25)
    g3, t3, s3, r3, f3 = pillar_room(0.1)
    comps = directional_components(g1, (3.0, 2.0, 1.5))
    return [
        RoomJob(g1, comps + [t1], s1[:900], r1, f1),   # 5 right-hand sides: a chunk of 4 and a padded one
        RoomJob(g2, [t2, t2], s2, r2, f2[:11]),        # 2 lanes, another step count
        RoomJob(g3, [t3], s3, r3 + r3[:1], f3),        # 1 lane, stops after 1 chunk + 101 steps
    ]


@pytest.mark.parametrize("precision", [FP32, FP64])
def test_each_room_equals_its_own_run(backend, library, precision):
    jobs = _jobs(library)
    res = backend.run_rooms(jobs, precision=precision, ir=True)
    for r, j in enumerate(jobs):
        spec, ir = backend.run_batch(j.grid, j.sources, j.signal, j.receivers, j.freqs, precision=precision, ir=True)
        assert np.array_equal(res[r][1], ir), f"room {r}: time series differ"
        assert worst_relative(spec, res[r][0]) < 1e-12, f"room {r}"


def test_rooms_match_oracle(backend, library):
    jobs = _jobs(library)
    res = backend.run_rooms(jobs)
    for r, j in enumerate(jobs):
        for s, taps in enumerate(j.sources[:2]):
            ref = ofd.run(j.grid, taps, j.signal, j.receivers, j.freqs, "f64")
            assert worst_relative(ref, res[r][s]) < 1e-3


def test_rooms_plan_repeats(backend, library):
    jobs = _jobs(library)
    plan = backend.rooms_plan(jobs)
    plan.run()
    a = [plan.read(r) for r in range(3)]
    st = plan.run(stats=True)
    assert st["chunks"] == max(int(np.ceil(len(j.signal) / 128)) for j in jobs)
    for r in range(3):
        assert np.array_equal(plan.read(r), a[r])
    plan.close()
