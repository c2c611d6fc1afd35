"""Two steps per pass over the fields (WAVEY_TBLOCK=1: interior_tb2 beside the
special-cell kernel, then tb2_second) give the one-step path's results bit
for bit: every update is the same arithmetic on the same values.  Covered:
both kernel shapes, tile heights from 1 to 22 output rows, z-runs of 1, 3
and 64 planes, rooms with branch materials, a rigid pillar and interior
source taps, two chunks of four sources, and a step count that leaves a
remainder after the last 128-step chunk (run as single steps)."""
from __future__ import annotations

import os

import numpy as np
import pytest

from scenes import branch_room, directional_components, pillar_room, spread_source

pytestmark = pytest.mark.gpu


def _run(backend, env, *args, **kw):
    """Spectra and time series of a plan created with env set; the plan must
    take the two-step path exactly when WAVEY_TBLOCK is set."""
    old = {k: os.environ.get(k) for k in env}
    os.environ.update({k: str(v) for k, v in env.items()})
    try:
        plan = backend.plan(*args, ir=True, **kw)
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v
    try:
        info = plan.info()
        assert info["two_step"] == (1 if "WAVEY_TBLOCK" in env else 0)
        if "WAVEY_TB_ROWS" in env:
            assert (info["two_step_rows"], info["two_step_zt"]) == (env["WAVEY_TB_ROWS"], env["WAVEY_TB_ZT"])
        plan.run()
        return plan.read()
    finally:
        plan.close()


@pytest.mark.parametrize("cfg,rows,zt", [(0, 22, 64), (0, 15, 3), (0, 6, 1), (1, 14, 3), (1, 1, 64), (1, 9, 7)])
def test_two_step_pass_matches_single_steps(backend, library, cfg, rows, zt):
    g, taps, sig, rcv, freqs = branch_room(library, 0.1)
    sources = (directional_components(g, (1.6, 1.3, 1.1)) + [taps])[:4]
    sig = sig[:301]
    ref = _run(backend, {}, g, sources, sig, rcv, freqs)
    got = _run(backend, {"WAVEY_TBLOCK": 1, "WAVEY_TB_CFG": cfg, "WAVEY_TB_ROWS": rows, "WAVEY_TB_ZT": zt},
               g, sources, sig, rcv, freqs)
    assert np.array_equal(got[1], ref[1])
    assert np.array_equal(got[0], ref[0])


def test_two_step_pass_in_the_pillar_room_with_two_chunks(backend):
    """The reference's pillar room (fdtd.rs:171-204, rigid pillar faces) with
    eight right-hand sides (two chunks of four) and the default two-step
    shape."""
    g, taps, sig, rcv, freqs = pillar_room(0.1)
    comps = directional_components(g, (1.5, 3.0, 1.5))
    other = directional_components(g, (6.0, 4.5, 2.0))
    sources = comps + other
    ref = _run(backend, {}, g, sources, sig, rcv, freqs)
    got = _run(backend, {"WAVEY_TBLOCK": 1}, g, sources, sig, rcv, freqs)
    assert np.array_equal(got[1], ref[1])
    assert np.array_equal(got[0], ref[0])


def test_two_step_pass_with_spread_taps(backend):
    """A source spread over many interior taps: every tap cell is special, so
    its neighbours join the shell."""
    g, taps, sig, rcv, freqs = spread_source()
    sources = [taps, taps[:3], taps[::2], [taps[0]]]
    sig = sig[:260]
    ref = _run(backend, {}, g, sources, sig, rcv, freqs)
    got = _run(backend, {"WAVEY_TBLOCK": 1, "WAVEY_TB_ROWS": 5, "WAVEY_TB_ZT": 4}, g, sources, sig, rcv, freqs)
    assert np.array_equal(got[1], ref[1])
    assert np.array_equal(got[0], ref[0])
