"""The batched wave stage on the GPU (wavey_gb300/wave.py over the CUDA
backend): one batched run for all speakers' components and one multi-room
run for all calibration pairs, against

  * the same stage over the FP64 oracle: within the reference's GPU-vs-CPU
    bar, 1e-3 of the largest value (core/wavey-solver/tests/fdtd.rs:168);
  * the reference's loop of one GPU run per speaker and component: bit-identical
    (batched lanes are bit-identical to single runs);
  * the reference's directional known-answer test (tests/fdtd.rs:446-518)
    driven through the stage: a cardioid speaker reproduces its fitted
    directivity within 0.05.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from oracle_backend import OracleBackend
from wave_scenes import c, per_component_reference, small_solve, worst_relative
from wavey_gb300.fdtd import BoxRoom, FdtdGrid, fit_first_order, speaker_rotation
from wavey_gb300.materials import fit_surfaces, scalar_material
from wavey_gb300.wave import Speaker, calibrate_cabinets, wave_stage
from wavey_gb300.workloads import cardioid

pytestmark = pytest.mark.gpu


def test_wave_stage_matches_oracle_and_per_component_runs(backend):
    room, g, speakers, rx, freqs, steps, cab = small_solve(with_cabinet=True)
    cal = calibrate_cabinets(backend, [cab], c, 354.0, 8.0, 2.0, freqs)
    cal_o = calibrate_cabinets(OracleBackend(), [cab], c, 354.0, 8.0, 2.0, freqs)
    assert worst_relative(cal_o[0].on_axis, cal[0].on_axis) < 2e-3
    assert worst_relative(cal_o[0].directivity, cal[0].directivity) < 2e-3
    cals = {"boxed": cal[0]}
    got = wave_stage(backend, g, speakers, rx, freqs, c, 354.0, steps, calibrations=cals)
    ora = wave_stage(OracleBackend(), g, speakers, rx, freqs, c, 354.0, steps, calibrations=cals)
    loop = per_component_reference(backend, g, speakers, rx, freqs, steps, 354.0, calibrations=cals)
    for sp, t, to, tl in zip(speakers, got.transfers, ora.transfers, loop):
        assert worst_relative(to, t) < 1e-3, sp.name
        assert np.array_equal(t, tl), sp.name


def test_calibration_pairs_in_one_launch_equal_separate_runs(backend):
    _, _, _, _, freqs, _, cab = small_solve()
    from wavey_gb300.wave import _calibration_from, _calibration_setup

    cal = calibrate_cabinets(backend, [cab, cab], c, 354.0, 8.0, 4.0, freqs)
    s = _calibration_setup(cab, c, 354.0, 8.0, 4.0)
    sw = backend.run_fdtd(s["grids"][0], s["taps"][0], s["signal"], s["rx"][0], freqs)
    sb = backend.run_fdtd(s["grids"][1], s["taps"][1], s["signal"], s["rx"][1], freqs)
    one = _calibration_from(sw, sb, freqs, s["f_cab"], s["angles"])
    for k in range(2):
        assert np.array_equal(cal[k].on_axis, one.on_axis)
        assert np.array_equal(cal[k].directivity, one.directivity)


def test_cardioid_speaker_reproduces_its_directivity(backend):
    """tests/fdtd.rs:446-518 through the stage: the cardioid speaker's
    transfer over the omnidirectional one's follows the first-order fit
    (with the dipoles' near-field term) within 0.05."""
    room = BoxRoom(14.0, 12.0, 10.0)
    f_max = 500.0
    g = FdtdGrid.build(room, fit_surfaces([scalar_material(0.2)] * 6, (20.0, f_max)), c, f_max, 12.0)
    node = g.nearest_air((7.0, 6.0, 5.0))
    centre = g.pos(node)
    rot = speaker_rotation(90.0, 0.0, 0.0)
    speakers = [Speaker("cardioid", tuple(centre), rotation=rot, directivity=cardioid),
                Speaker("omni", tuple(centre))]
    r = 1.6
    angles = [0.0, 60.0, 90.0, 135.0, 180.0, 270.0]
    rx = [g.nearest_air(centre + r * np.array([math.cos(math.radians(a)), math.sin(math.radians(a)), 0.0]))
          for a in angles]
    rx.append(g.nearest_air(centre + np.array([0.0, 0.0, r])))
    freqs = np.array([120.0, 200.0, 300.0])
    res = wave_stage(backend, g, speakers, rx, freqs, c, f_max, int(0.018 / g.dt))
    assert res.right_hand_sides == 5
    card, omni = res.transfers
    worst = 0.0
    for fi, f in enumerate(freqs):
        a0, a, _ = fit_first_order(cardioid, rot, f)
        k = 2 * math.pi * f / c
        for ri, cell in enumerate(rx):
            d = g.pos(cell) - centre
            dist = float(np.linalg.norm(d))
            fit = a0 + (a[0] * d[0] + a[1] * d[1] + a[2] * d[2]) / dist * (1.0 + 1.0 / (1j * k * dist))
            worst = max(worst, abs(card[ri, fi] / omni[ri, fi] - fit))
    assert worst < 0.05, worst


def test_transfer_section_from_device_spectra(backend):
    """wave_stage_results combines on the device and reads back complex64 in
    the results.bin layout: equal to the host combination laid out the same
    way, to complex64 rounding."""
    from wavey_gb300.wave import layout_transfers, wave_stage_results

    room, g, speakers, rx, freqs, steps, cab = small_solve(with_cabinet=True)
    cals = {"boxed": calibrate_cabinets(backend, [cab], c, 354.0, 8.0, 2.0, freqs)[0]}
    n_mics, planes = 1, [2, 1]  # receivers: one mic, then planes of two and one points
    host = wave_stage(backend, g, speakers, rx, freqs, c, 354.0, steps, calibrations=cals)
    want = layout_transfers(host.transfers, n_mics, planes)
    got = wave_stage_results(backend, g, speakers, rx, n_mics, planes, freqs, c, 354.0, steps, calibrations=cals)
    assert got.dtype == np.complex64 and got.shape == want.shape
    assert np.abs(got - want).max() <= 1e-6 * np.abs(want).max()


def test_transfer_layout_is_checked(backend):
    from wavey_gb300.backend import WaveyError

    room, g, speakers, rx, freqs, steps, _ = small_solve()
    plan = backend.plan(g, [g.taps_at(speakers[0].position)], np.zeros(200), rx, freqs)
    plan.run()
    fac = np.ones((1, len(freqs)), complex)
    with pytest.raises(WaveyError, match="receivers"):
        plan.transfers([0], fac, 1, [1])  # 2 receivers laid out, the plan has 4
    with pytest.raises(WaveyError, match="speaker"):
        plan.transfers([-2], fac, 4)
    out = plan.transfers([0], fac, 4)
    assert out.shape == (4 * len(freqs),)
    plan.close()
