"""The reference's unit tests of the boundary admittance fit and the
absorption helpers (core/wavey-materials/src/impedance_fit.rs:237-283,
material.rs:113-157, spectrum.rs:229-247), against the host library."""
from __future__ import annotations

import math

import numpy as np
import pytest

from wavey_gb300.materials import Spectrum, fit_admittance, fit_real_impedance

MAX_Q = 2.0


def _paris_real(z):
    n = 256
    h = math.pi / 2 / n
    s = 0.0
    for i in range(n):
        th = (i + 0.5) * h
        r = (z * math.cos(th) - 1) / (z * math.cos(th) + 1)
        s += (1 - r * r) * math.sin(2 * th) * h
    return s


def test_log_interpolation():
    s = Spectrum.bands([100.0, 1000.0], [0.0, 1.0])
    assert s.eval(50.0) == 0.0 and s.eval(5000.0) == 1.0
    assert abs(s.eval(316.227766) - 0.5) < 1e-6
    assert Spectrum.bands([125.0, 250.0], [0.1, 0.2]).eval(125.0) == 0.1


@pytest.mark.parametrize("alpha", [0.02, 0.1, 0.3, 0.6, 0.9])
def test_impedance_fit_reproduces_absorption(alpha):
    z = fit_real_impedance(alpha)
    assert abs(_paris_real(z) - alpha) < 1e-6


@pytest.fixture(scope="module")
def low_band_fits(library):
    return {mid: fit_admittance(m, (20.0, 424.0), 2) for mid, m in library.items()}


def test_library_materials_fit_over_low_band(low_band_fits):
    for mid, fit in low_band_fits.items():
        assert fit.max_error < 0.05, f"{mid}: max error {fit.max_error}"
        assert fit.rms_error < 0.02, f"{mid}: rms error {fit.rms_error}"


def test_branches_are_broad(library):
    for mid, m in library.items():
        for b in fit_admittance(m, (20.0, 707.0), 2).branches:
            assert math.sqrt(b.m * b.k) / b.r <= MAX_Q + 1e-9, mid


def test_passive_admittance(low_band_fits):
    for mid, fit in low_band_fits.items():
        for i in range(200):
            assert fit.admittance(1.0 + i * 25.0).real >= 0.0, mid


def test_audience_is_nearly_transparent_at_low_frequency(library):
    fit = fit_admittance(library["audience-standing"], (20.0, 424.0), 2)
    assert fit.absorption(40.0) < 0.08
    assert fit.absorption(300.0) > 0.3


def test_rigid_material_fits_rigid(library):
    fit = fit_admittance(library["rigid"], (20.0, 300.0), 2)
    assert fit.is_rigid()
