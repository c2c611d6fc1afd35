"""The reference's analytic FDTD tests (core/wavey-solver/tests/fdtd.rs) run
through the CUDA path, FP32, with the reference's thresholds."""
from __future__ import annotations

import pytest

import analytic

pytestmark = pytest.mark.gpu


@pytest.fixture
def runners(backend):
    def run(g, taps, sig, rcv, freqs):
        return backend.run_fdtd(g, taps, sig, rcv, freqs)

    def run_ir(g, taps, sig, rcv):
        return backend.run_fdtd(g, taps, sig, rcv, [], ir=True)[1]

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
