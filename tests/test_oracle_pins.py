"""Pins the oracle to the reference's own known answers.

The reference stores no golden vectors for its FDTD path; its tests
(core/wavey-solver/tests/fdtd.rs) check the CPU solver against analytic
results.  The same checks, with the same thresholds, run here against the
oracle's FP64 restatement of run_cpu, so the oracle that the CUDA path is
compared with is itself tied to the reference's accepted behaviour.
"""
from __future__ import annotations

import numpy as np
import pytest

import analytic
from oracle import fdtd as ofd
from wavey_gb300.fdtd import blend


def run(g, taps, sig, rcv, freqs):
    return ofd.run(g, taps, sig, rcv, freqs, "f64")


def run_ir(g, taps, sig, rcv):
    return ofd.run(g, taps, sig, rcv, [], "f64", ir=True)[1]


def run_batch(g, sources, sig, rcv, freqs):
    return np.stack([run(g, t, sig, rcv, freqs) for t in sources])


def test_direct_sound_is_calibrated():
    analytic.direct_sound_is_calibrated(run)


def test_rigid_box_eigenfrequencies():
    analytic.rigid_box_eigenfrequencies(run)


@pytest.mark.slow
def test_rigid_cube_modes_to_800_hz():
    analytic.rigid_cube_modes_to_800_hz(run)


def test_tube_reflection_matches_fitted_impedance(library):
    analytic.tube_reflection_matches_fitted_impedance(run, library)


@pytest.mark.slow
def test_branch_boundaries_are_stable(library):
    analytic.branch_boundaries_are_stable(run_ir, library)


@pytest.mark.slow
def test_directional_source_reproduces_directivity():
    analytic.directional_source_reproduces_directivity(run_batch)


def test_oblique_reflection_matches_spherical_wave_theory():
    analytic.oblique_reflection_matches_spherical_wave_theory(run)


def test_spherical_reflection_limits():
    """reflection.rs tests: the Faddeeva values the reference checks, and the
    spherical factor tending to the plane-wave one far from the source and
    to 1 at grazing incidence close to it."""
    from scipy.special import wofz

    assert abs(wofz(1j) - 0.427583576155807) < 1e-12
    assert abs(wofz(1.0) - complex(0.367879441171442, 0.607157705841394)) < 1e-12
    assert abs(wofz(2 + 1j) - complex(0.140239581366278, 0.222213440179899)) < 1e-12
    zeta = complex(3.0, -1.5)
    far = analytic.spherical_reflection(zeta, 0.8, 50.0, 1e4)
    assert abs(far - analytic.plane_reflection(zeta, 0.8)) < 1e-3
    grazing = analytic.spherical_reflection(zeta, 0.0, 1.0, 0.01)
    assert abs(grazing - 1.0) < 0.2


def test_crossover_blend_is_power_complementary():
    """fdtd.rs:593-616"""
    a = 2.0 * np.exp(0.3j)
    for w in [0.0, 0.25, 0.5, 0.75, 1.0]:
        assert abs(blend(a, a, w) - a) < 1e-12
    n = 360
    e_blend = e_plain = 0.0
    for i in range(n):
        b = np.exp(2j * np.pi * i / n)
        e_blend += abs(blend(a, b, 0.5)) ** 2
        e_plain += abs(a * 0.5 + b * 0.5) ** 2
    want = 0.5 * 4.0 + 0.5 * 1.0
    assert abs(e_blend / n - want) < 1e-9
    assert e_plain / n < 0.6 * want
    assert abs(abs(blend(a, -a, 0.5)) ** 2 - 4.0) < 1e-9


def test_fp32_order_restatement_tracks_fp64():
    """The oracle's two precisions agree to the reference's GPU bar."""
    from scenes import branch_room, worst_relative
    import json, pathlib
    from wavey_gb300.materials import Material, Spectrum

    data = json.loads((pathlib.Path(__file__).parent / "golden" / "materials.json").read_text())
    lib = {k: Material(k, Spectrum.bands(v["freqs_hz"], v["values"]) if isinstance(v, dict) else Spectrum(v))
           for k, v in data.items()}
    g, taps, sig, rcv, freqs = branch_room(lib, 0.3)
    a = ofd.run(g, taps, sig, rcv, freqs, "f64")
    b = ofd.run(g, taps, sig, rcv, freqs, "f32")
    assert worst_relative(a, b) < 1e-3
