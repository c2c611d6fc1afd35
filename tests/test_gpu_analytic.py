"""The reference's analytic FDTD tests (core/wavey-solver/tests/fdtd.rs) run
through the CUDA path, FP32, with the reference's thresholds."""
from __future__ import annotations

import pytest

import numpy as np

import analytic
from oracle import fdtd as ofd
from wavey_gb300.backend import FP64

pytestmark = pytest.mark.gpu


@pytest.fixture
def runners(backend):
    def run(g, taps, sig, rcv, freqs):
        return backend.run_fdtd(g, taps, sig, rcv, freqs)

    def run_ir(g, taps, sig, rcv):
        # The reference runs this 200 k-step test on its FP64 CPU solver; the
        # GPU counterpart is the FP64 path.  FP32 (the reference shader's
        # arithmetic) drifts at DC over runs this long; see
        # test_fp32_boundary_drift_is_the_shader_arithmetic.
        return backend.run_batch(g, [taps], sig, rcv, [], precision=FP64, ir=True)[1][0]

    def run_batch(g, sources, sig, rcv, freqs):
        return backend.run_batch(g, sources, sig, rcv, freqs)

    return run, run_ir, run_batch


def test_direct_sound_is_calibrated(runners):
    analytic.direct_sound_is_calibrated(runners[0])


def test_rigid_box_eigenfrequencies(runners):
    analytic.rigid_box_eigenfrequencies(runners[0])


def test_rigid_cube_modes_to_800_hz(runners):
    analytic.rigid_cube_modes_to_800_hz(runners[0])


def test_tube_reflection_matches_fitted_impedance(runners, library):
    analytic.tube_reflection_matches_fitted_impedance(runners[0], library)


def test_branch_boundaries_are_stable(runners, library):
    analytic.branch_boundaries_are_stable(runners[1], library)


def test_directional_source_reproduces_directivity(runners):
    analytic.directional_source_reproduces_directivity(runners[2])


def test_fp32_boundary_drift_is_the_shader_arithmetic(backend, library):
    """Over 30 k steps the FP32 path's receiver series equals the FP32
    restatement of the reference shader bit for bit, drift included, so
    the long-run DC drift is the reference GPU arithmetic's, not a defect
    of this port."""
    g, taps, sig, rcv, freqs = __import__("scenes").branch_room(library, 5.0)
    sig = sig[:30000]
    _, ref = ofd.run(g, taps, sig, rcv, [], "f32", ir=True)
    _, got = backend.run_fdtd(g, taps, sig, rcv, [], ir=True)
    assert np.array_equal(got, ref)


def test_oblique_reflection_matches_spherical_wave_theory(runners):
    analytic.oblique_reflection_matches_spherical_wave_theory(runners[0])
