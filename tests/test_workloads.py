"""The seeded benchmark scenes that bench.py measures, checked on the host:
the mixed-precision configuration's speakers (right-hand sides and their
combination weights) and the multi-room configuration's rooms."""
from __future__ import annotations

import math

import numpy as np

from wavey_gb300 import workloads as W
from wavey_gb300.fdtd import component_weights, fit_first_order


def test_pillar_room_with_32_speakers():
    sc = W.room_pillars_speakers(32)
    kinds, rhs, weights = sc.notes["speakers"], sc.notes["speaker_rhs"], sc.notes["speaker_weights"]
    assert len(kinds) == len(rhs) == len(weights) == 32
    # Right-hand sides laid out speaker after speaker, no gaps.
    assert rhs[0][0] == 0
    for (a, n), (b, _m) in zip(rhs, rhs[1:]):
        assert b == a + n
    assert rhs[-1][0] + rhs[-1][1] == len(sc.sources)
    nf = len(sc.freqs)
    for kind, (a, n), w in zip(kinds, rhs, weights):
        w = np.asarray(w)
        if kind == "monopole":
            assert n == 1 and np.all(w == 1.0)
        else:
            assert kind == "cardioid" and n == 4 and w.shape == (nf, 4)
            assert np.all(np.isfinite(w))
    # The receivers start with the 64 mics (the IR comparison uses them).
    assert sc.notes["mics"] == 64 and len(sc.receivers) > 64
    # The weights are the reference's first-order fit of a cardioid: the
    # monopole part a0 of D = 0.5 + 0.5 d.x is 0.5 at every frequency.
    k = next(i for i, kind in enumerate(kinds) if kind == "cardioid")
    f = float(sc.freqs[0])
    a0, a, _res = fit_first_order(W.cardioid, np.eye(3), f)
    assert abs(a0 - 0.5) < 1e-9
    assert len(component_weights(a0, a, 2.0 * math.pi * f / W.C_AIR, sc.grid.dx)) == 4
    assert np.asarray(weights[k]).shape == (nf, 4)


def test_many_rooms_configuration():
    rooms = W.rooms_batch()
    assert len(rooms) == 5
    assert sum(len(r.sources) for r in rooms) == 81
    assert len({r.steps for r in rooms}) == 1
    for r in rooms[1:]:
        assert 2e5 < r.grid.cells < 2.1e6
