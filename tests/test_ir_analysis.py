"""The oracle's restatement of the reference's impulse-response analysis
(analysis.rs; oracle/ir_oracle.c), pinned by known answers: the reference
stores no golden vectors for it, so closed forms of a sampled exponential
decay, a band-centre sinusoid and a delayed pulse stand in."""
from __future__ import annotations

import math

import numpy as np
import pytest

from oracle import ir

FS = 8000.0


def test_noise_free_params_of_an_exponential_decay():
    """Energy r^i decays 60 dB in T seconds: the Schroeder curve is the same
    exponential (minus its truncation), so T20, T30 and EDT are T; D50, C80
    and the centre time are geometric sums."""
    T, n = 1.1, 20000
    r = 10.0 ** (-6.0 / (T * FS))
    e = r ** np.arange(n)
    edt, t20, t30, c80, d50, ts = ir.noise_free_params(e, FS)
    for v in (edt, t20, t30):
        assert v == pytest.approx(T, rel=5e-3)
    geo = lambda k: (1 - r ** k) / (1 - r)
    i50, i80 = int(0.05 * FS), int(0.08 * FS)
    assert d50 == pytest.approx(geo(i50) / geo(n), rel=1e-9)
    assert c80 == pytest.approx(10 * math.log10(geo(i80) / (geo(n) - geo(i80))), rel=1e-9)
    assert ts == pytest.approx(float(np.sum(np.arange(n) / FS * e) / np.sum(e)), rel=1e-9)


def test_octave_filter_passes_its_band_with_zero_phase():
    t = np.arange(16000) / FS
    for fc in (125.0, 500.0, 1000.0):
        x = np.sin(2 * math.pi * fc * t)
        y = ir.octave_filter(x, fc, FS)
        mid = slice(4000, 12000)
        amp = np.sqrt(2 * np.mean(y[mid] ** 2))
        # At fc each 6th-order Butterworth side has |H|^2 = 1 / (1 + (1/sqrt2)^12) = 64/65, and the
        # forward-backward pass squares the magnitude: (64/65)^2.
        assert amp == pytest.approx((64 / 65) ** 2, abs=0.015), fc  # (bilinear warping near fs / 8)
        # Zero phase: the output lines up with the input (no lag).
        lag = np.argmax(np.correlate(y[mid], x[mid], "full")) - (len(x[mid]) - 1)
        assert lag == 0, fc
        far = ir.octave_filter(np.sin(2 * math.pi * 4 * fc * t), fc, FS)
        assert np.sqrt(2 * np.mean(far[mid] ** 2)) < 0.02, fc


def test_onset_is_the_first_sample_within_20_db_of_the_peak():
    x = np.zeros(3000)
    x[700:710] = np.linspace(0.05, 1.0, 10)
    assert ir.onset(x) == 701  # 0.1556^2 >= 0.01 first at index 701
    assert ir.onset(np.zeros(10)) == 0


def test_lundeby_recovers_the_decay_under_a_noise_floor():
    rng = np.random.default_rng(3)
    T, n = 0.8, 24000
    t = np.arange(n) / FS
    p = rng.normal(size=n) * 10 ** (-3.0 * t / T) + 10 ** (-50 / 20) * rng.normal(size=n)
    with_l = ir.ir_params(p, FS, bands=(1000.0,), integrate=False, lundeby=True)[0]
    without = ir.ir_params(p, FS, bands=(1000.0,), integrate=False, lundeby=False)[0]
    assert with_l[2] == pytest.approx(T, rel=0.08)       # T30 with truncation and compensation
    assert abs(with_l[2] - T) < abs(without[2] - T)        # the noise tail biases the plain integration


def test_band_decay_times_of_a_diffuse_decay():
    rng = np.random.default_rng(5)
    T, n = 1.2, 20000
    t = np.arange(n) / FS
    p = rng.normal(size=n) * 10 ** (-3.0 * t / T)
    out = ir.ir_params(p, FS, bands=(250.0, 500.0, 1000.0, 2000.0), integrate=False, lundeby=False)
    assert out.shape == (4, 6)
    assert np.all(np.abs(out[:, 1] / T - 1) < 0.06)   # T20
    assert np.all(np.abs(out[:, 2] / T - 1) < 0.06)   # T30
