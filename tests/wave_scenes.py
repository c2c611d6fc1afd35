"""Scenes and checks of the batched wave stage, shared by the CPU tests
(oracle behind the backend interface) and the GPU tests (CUDA backend)."""
from __future__ import annotations

import math

import numpy as np

from conftest import C_AIR
from wavey_gb300.fdtd import BoxRoom, FdtdGrid, speaker_rotation, to_transfer
from wavey_gb300.materials import fit_surfaces, scalar_material
from wavey_gb300.wave import Cabinet, Speaker, plan_speaker
from wavey_gb300.workloads import cardioid

c = C_AIR


def small_solve(with_cabinet: bool = False):
    """A 5 x 4 x 3 m room at 250 Hz with three speakers: an omnidirectional
    one, a cardioid aimed into the room and (optionally) one in a box
    cabinet drawn into the grid as a rigid solid."""
    cab = Cabinet((0.3, 0.25, 0.4), (0.1, 0.0, 0.05))
    cab_pos = np.array([1.0, 2.6, 1.2])  # box centre; acoustic centre = cab_pos + cab.acoustic_center
    solids = []
    if with_cabinet:
        h = 0.5 * np.asarray(cab.size)
        solids.append(tuple(np.concatenate([cab_pos - h, cab_pos + h])))
    room = BoxRoom(5.0, 4.0, 3.0, solids=solids)
    fits = fit_surfaces([scalar_material(a) for a in (0.1, 0.15, 0.2, 0.25, 0.3, 0.35)], (20.0, 354.0))
    # The cabinet drawn on the band's grid (run.rs:446-448, Draft/Standard), not resolved cell by cell.
    g = FdtdGrid.build_dx(room, fits, c, c / (250.0 * 10.0))
    speakers = [
        Speaker("omni", (3.6, 1.1, 1.4), h0=lambda f: complex(1.0, 0.1 * f / 250.0)),
        Speaker("cardioid", (2.2, 2.1, 1.6), rotation=speaker_rotation(30.0, 10.0, 0.0), directivity=cardioid,
                reference_distance=1.0),
    ]
    if with_cabinet:
        speakers.append(Speaker("boxed", tuple(cab_pos + np.asarray(cab.acoustic_center)), cabinet=cab))
    rx = [g.nearest_air(p) for p in [(4.2, 3.1, 1.2), (0.8, 0.7, 2.1), (2.5, 2.0, 0.6), (4.0, 0.6, 2.4)]]
    freqs = 30.0 + np.arange(24) * 12.0
    steps = math.ceil(0.35 / g.dt)
    return room, g, speakers, rx, freqs, steps, cab


def per_component_reference(backend, g, speakers, rx, freqs, steps, grid_fmax, calibrations=None):
    """The reference's loop (run.rs:631-660): one single-source run per
    speaker and component, combined per speaker."""
    from wavey_gb300.fdtd import source_signal

    calibrations = calibrations or {}
    sig = source_signal(grid_fmax, g.dt, steps)
    out = []
    for sp in speakers:
        p = plan_speaker(g, sp, freqs, c, 1, sp.name in calibrations)
        h0 = np.array([complex(sp.h0(f)) if callable(sp.h0) else complex(sp.h0) for f in freqs])
        t = np.zeros((len(rx), len(freqs)), complex)
        for ci, taps in enumerate(p.components):
            spec = backend.run_fdtd(g, taps, sig, rx, freqs)
            tc = to_transfer(spec, sig, g, freqs, c, sp.reference_distance, h0)
            if sp.name in calibrations:
                tc = tc / calibrations[sp.name].on_axis[None, :]
            t += p.weights[None, :, ci] * tc
        out.append(t)
    return out


def worst_relative(ref, got):
    ref, got = np.asarray(ref), np.asarray(got)
    return float(np.abs(ref - got).max() / np.abs(ref).max())
