"""The batched wave stage (wavey_gb300/wave.py) on the CPU, with the FP64
oracle behind the backend interface: all speakers' components go through
ONE batched call and all cabinet calibration pairs through ONE multi-room
call, and the result equals the reference's loop of one run per speaker and
component (run.rs:631-660, fdtd.rs:890-955)."""
from __future__ import annotations

import math

import numpy as np
import pytest

from oracle_backend import OracleBackend
from wave_scenes import c, per_component_reference, small_solve, worst_relative
from wavey_gb300.wave import (CabinetCalibration, Speaker, WaveStageError, _calibration_from, _calibration_setup,
                              calibrate_cabinets, plan_speaker, wave_stage)


def test_one_batched_run_equals_the_per_component_loop():
    room, g, speakers, rx, freqs, steps, _ = small_solve()
    b = OracleBackend()
    res = wave_stage(b, g, speakers, rx, freqs, c, 354.0, steps)
    assert b.calls == [("batch", 5)]  # 1 omni + 4 cardioid components, one call
    assert res.right_hand_sides == 5
    ref = per_component_reference(OracleBackend(), g, speakers, rx, freqs, steps, 354.0)
    for got, want in zip(res.transfers, ref):
        assert got.shape == (len(rx), len(freqs))
        assert np.array_equal(got, want)
    assert any("fitted to first order" in n for n in res.notes)


def test_speaker_plans_follow_the_reference_rules():
    room, g, speakers, rx, freqs, steps, cab = small_solve(with_cabinet=True)
    omni, card, boxed = (plan_speaker(g, sp, freqs, c, 1, sp.cabinet is not None) for sp in speakers)
    assert len(omni.components) == 1 and np.all(omni.weights == 1)
    assert len(card.components) == 4 and card.weights.shape == (len(freqs), 4)
    # A calibrated cabinet radiates from the baffle point as one component (run.rs:611-619).
    assert len(boxed.components) == 1
    bp = g.baffle_point(speakers[2].position, speakers[2].axis)
    assert boxed.components[0] == g.taps_at(bp)
    # Order 0 turns a directional speaker into one component.
    p0 = plan_speaker(g, speakers[1], freqs, c, 0, False)
    assert len(p0.components) == 1


def test_speaker_outside_the_grid_is_an_error():
    room, g, speakers, rx, freqs, steps, _ = small_solve()
    with pytest.raises(WaveStageError, match="not inside"):
        plan_speaker(g, Speaker("far", (50.0, 50.0, 50.0)), freqs, c, 1, False)


def test_calibration_ratio_fade_and_directivity():
    """fdtd.rs:944-954 on synthetic spectra."""
    freqs = np.array([20.0, 50.0, 100.0, 200.0])
    f_cab = 100.0
    rng = np.random.default_rng(4)
    s_bare = rng.normal(size=(12, 4)) + 1j * rng.normal(size=(12, 4))
    m = 1.5 * np.exp(1j * 0.7) * np.ones((12, 4))
    m[3] *= 0.5
    cal = _calibration_from(s_bare * m, s_bare, freqs, f_cab, np.arange(12) * 30.0)
    w = np.minimum((freqs / f_cab) ** 2, 1.0)
    want = 1.5 ** w * np.exp(1j * 0.7 * w)
    assert np.allclose(cal.on_axis, want)
    assert np.allclose(cal.directivity[0], 1.0)
    assert np.allclose(np.abs(cal.directivity[3]), 0.5 ** w)
    assert cal.on_axis[-1] == pytest.approx(1.5 * np.exp(0.7j))  # above f_cab: the measured ratio


def test_calibration_setup_follows_the_reference_geometry():
    room, g, speakers, rx, freqs, steps, cab = small_solve()
    s = _calibration_setup(cab, c, 354.0, 10.0, 6.0)
    g_with, g_bare = s["grids"]
    assert g_with.dx == g_bare.dx and g_with.n == g_bare.n
    assert g_with.air < g_bare.air  # the cabinet's cells are solid
    reach = max(np.linalg.norm(cab.corners() - np.asarray(cab.acoustic_center), axis=1))
    assert s["f_cab"] == pytest.approx(0.5 * c / (2 * math.pi * reach))
    assert len(s["rx"][0]) == 12 and list(s["angles"]) == [30.0 * k for k in range(12)]
    # Duration: twice the box diagonal plus 12 source widths (fdtd.rs:936).
    side = g_bare.n[0] * g_bare.dx  # about 2 * half plus the border
    assert len(s["signal"]) * g_with.dt > 2 * math.sqrt(3) * (side - 4 * g_bare.dx) / c


def test_calibrations_run_as_one_multi_room_call():
    room, g, speakers, rx, freqs, steps, cab = small_solve(with_cabinet=True)
    b = OracleBackend()
    cal = calibrate_cabinets(b, [cab], c, 150.0, 12.0, 1.0, freqs)  # a coarse grid: the oracle is slow
    assert b.calls == [("rooms", 2)]
    assert isinstance(cal[0], CabinetCalibration)
    assert cal[0].directivity.shape == (12, len(freqs))
    # Below the cabinet's ka = 0.5 the ratio fades to 1.
    assert abs(cal[0].on_axis[0] - 1) < 0.05
    res = wave_stage(b, g, speakers, rx, freqs, c, 354.0, steps, calibrations={"boxed": cal[0]})
    ref = per_component_reference(OracleBackend(), g, speakers, rx, freqs, steps, 354.0,
                                  calibrations={"boxed": cal[0]})
    assert worst_relative(ref[2], res.transfers[2]) == 0.0


def _save_layout_like_reference(transfers, n_mics, plane_points):
    """result.rs:444-456 written out: every mic's transfer per speaker, then
    every plane's transfer per speaker, each a run of Complex32."""
    out = []
    for m in range(n_mics):
        for s in range(len(transfers)):
            out.extend(np.asarray(transfers[s][m], dtype=np.complex64))
    r0 = n_mics
    for pts in plane_points:
        for s in range(len(transfers)):
            out.extend(np.asarray(transfers[s][r0:r0 + pts], dtype=np.complex64).reshape(-1))
        r0 += pts
    return np.array(out, dtype=np.complex64)


def test_transfer_section_layout_matches_results_bin(tmp_path):
    from wavey_gb300.wave import layout_transfers, write_transfer_section

    rng = np.random.default_rng(7)
    S, n_mics, planes, nf = 3, 2, [4, 5], 6
    R = n_mics + sum(planes)
    t = rng.normal(size=(S, R, nf)) + 1j * rng.normal(size=(S, R, nf))
    sec = layout_transfers(t, n_mics, planes)
    assert np.array_equal(sec, _save_layout_like_reference(t, n_mics, planes))
    write_transfer_section(tmp_path / "t.bin", sec)
    raw = np.fromfile(tmp_path / "t.bin", dtype="<f4")
    assert np.array_equal(raw[0::2], sec.real) and np.array_equal(raw[1::2], sec.imag)


def test_transfer_factors_reproduce_the_host_combination():
    """The device combination's inputs: sum over lanes of factor x spectrum
    equals the wave stage's host combination."""
    from wavey_gb300.fdtd import source_signal
    from wavey_gb300.wave import transfer_factors

    room, g, speakers, rx, freqs, steps, _ = small_solve()
    b = OracleBackend()
    host = wave_stage(b, g, speakers, rx, freqs, c, 354.0, steps)
    plans = [plan_speaker(g, sp, freqs, c, 1, False) for sp in speakers]
    sig = source_signal(354.0, g.dt, steps)
    lanes, fac = transfer_factors(g, speakers, plans, freqs, c, sig)
    spectra = b.run_batch(g, [t for p in plans for t in p.components], sig, rx, freqs)
    for s in range(len(speakers)):
        dev = sum(fac[k][None, :] * spectra[k] for k in range(len(lanes)) if lanes[k] == s)
        assert worst_relative(host.transfers[s], dev) < 1e-12
