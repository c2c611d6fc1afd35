"""Band parameters of receiver time series computed on the device
(wavey_cuda_plan_band_params) against the oracle's restatement of the
reference's analysis (analysis.rs) run on the same series read back from the
plan.  Both are FP64 in the same operation order; the filter coefficients'
cos/sin and the log10 of the decay curves come from different math
libraries, so the bar is 1e-6 relative (NaN where both are undefined)."""
from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import C_AIR
from oracle import ir as oir
from wavey_gb300.backend import FP64, WaveyError
from wavey_gb300.fdtd import BoxRoom, FdtdGrid, source_signal
from wavey_gb300.materials import fit_surfaces, scalar_material

pytestmark = pytest.mark.gpu

BANDS = (63.0, 125.0, 250.0, 500.0)


def _room_plan(backend, precision=None):
    room = BoxRoom(6.0, 4.5, 3.2)
    fits = fit_surfaces([scalar_material(a) for a in (0.1, 0.3, 0.15, 0.2, 0.25, 0.12)], (20.0, 707.0))
    g = FdtdGrid.build(room, fits, C_AIR, 500.0, 10.0)
    src = g.taps_at((1.7, 1.3, 1.4))
    rx = [g.nearest_air(p) for p in [(4.5, 3.1, 1.2), (2.9, 2.2, 1.6), (5.2, 0.8, 2.5), (0.9, 3.6, 0.9)]]
    steps = math.ceil(1.0 / g.dt)
    sig = source_signal(500.0, g.dt, steps)
    kw = {} if precision is None else {"precision": precision}
    plan = backend.plan(g, [src, src], np.stack([sig, 0.5 * sig]), rx, np.array([100.0]), ir=True, **kw)
    plan.run()
    return g, plan


@pytest.mark.parametrize("lundeby", [False, True])
@pytest.mark.parametrize("integrate", [True, False])
def test_device_band_params_match_the_oracle(backend, integrate, lundeby):
    g, plan = _room_plan(backend)
    dev = plan.band_params(BANDS, integrate=integrate, lundeby=lundeby)
    _, series = plan.read()
    plan.close()
    assert dev.shape == (2, 4, len(BANDS), 6)
    for s in range(2):
        for r in range(4):
            ref = oir.ir_params(series[s, r], 1.0 / g.dt, BANDS, integrate=integrate, lundeby=lundeby)
            assert np.allclose(dev[s, r], ref, rtol=1e-6, atol=1e-12, equal_nan=True), (s, r, dev[s, r], ref)
    # A decaying room: finite decay times of a plausible size in every band.
    assert np.all(np.isfinite(dev[..., 2])) and np.all((dev[..., 2] > 0.05) & (dev[..., 2] < 5.0))


def test_fp64_plan_series(backend):
    g, plan = _room_plan(backend, FP64)
    dev = plan.band_params(BANDS[1:3], integrate=True, lundeby=False)
    _, series = plan.read()
    plan.close()
    ref = oir.ir_params(series[1, 2], 1.0 / g.dt, BANDS[1:3], integrate=True, lundeby=False)
    assert np.allclose(dev[1, 2], ref, rtol=1e-6, atol=1e-12, equal_nan=True)


def test_band_params_reject_bad_requests(backend):
    g, plan = _room_plan(backend)
    with pytest.raises(WaveyError, match="fs / 2"):
        plan.band_params((0.6 / g.dt,))
    plan.close()
    from scenes import spread_source

    g, taps, sig, rcv, freqs = spread_source()
    p2 = backend.plan(g, [taps], sig[:300], rcv, freqs)  # no time series recorded
    p2.run()
    with pytest.raises(WaveyError, match="time series"):
        p2.band_params(BANDS)
    p2.close()
