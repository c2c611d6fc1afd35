"""Test set-ups restated from the reference's FDTD tests
(core/wavey-solver/tests/fdtd.rs).  Each returns the grid and run inputs."""
from __future__ import annotations

import numpy as np

from conftest import C_AIR
from wavey_gb300.fdtd import BoxRoom, FdtdGrid, source_signal, source_components
from wavey_gb300.materials import fit_surfaces, scalar_material


def spread_source():
    """gpu_matches_cpu_with_a_source_spread_over_many_cells (fdtd.rs:147-169)."""
    room = BoxRoom(6.0, 4.0, 3.0)
    fits = fit_surfaces([scalar_material(0.2)] * room.n_surfaces, (20.0, 200.0))
    g = FdtdGrid.build(room, fits, C_AIR, 200.0, 12.0)
    taps = g.taps_at((1.53, 1.27, 1.41))
    rcv = [g.nearest_air(p) for p in [(4.5, 3.0, 1.2), (5.0, 1.0, 2.0)]]
    steps = int(0.4 / g.dt)
    sig = source_signal(200.0, g.dt, steps)
    freqs = 30.0 + np.arange(20) * 8.0
    return g, taps, sig, rcv, freqs


def pillar_room(duration=0.8):
    """gpu_matches_cpu (fdtd.rs:171-204): 8 x 6 x 3 m with a 1 m pillar."""
    room = BoxRoom(8.0, 6.0, 3.0, pillars=[(3.5, 2.5, 4.5, 3.5)])
    mats = [scalar_material(0.1 if i % 2 == 0 else 0.4) for i in range(room.n_surfaces)]
    fits = fit_surfaces(mats, (20.0, 300.0))
    g = FdtdGrid.build(room, fits, C_AIR, 300.0, 12.0)
    src = g.nearest_air((1.5, 3.0, 1.5))
    rcv = [g.nearest_air(p) for p in [(6.5, 3.0, 1.2), (6.0, 1.0, 2.0), (2.0, 5.0, 0.5)]]
    steps = int(duration / g.dt)
    sig = source_signal(300.0, g.dt, steps)
    freqs = 30.0 + np.arange(40) * 6.0
    return g, [(src, 1.0)], sig, rcv, freqs


BRANCH_MATERIALS = ["audience-standing", "mineral-wool-50", "plaster-rough", "carpet-heavy", "wood-panel",
                    "ceiling-industrial"]


def branch_room(library, duration=0.6):
    """gpu_matches_cpu_with_branches (fdtd.rs:352-375)."""
    room = BoxRoom(5.0, 4.0, 3.0)
    mats = [library[BRANCH_MATERIALS[i % 6]] for i in range(room.n_surfaces)]
    fits = fit_surfaces(mats, (20.0, 300.0))
    g = FdtdGrid.build(room, fits, C_AIR, 300.0, 12.0)
    src = g.nearest_air((1.2, 1.1, 1.3))
    rcv = [g.nearest_air(p) for p in [(4.1, 3.2, 1.5), (2.5, 0.5, 2.6)]]
    steps = int(duration / g.dt)
    sig = source_signal(300.0, g.dt, steps)
    freqs = 30.0 + np.arange(30) * 9.0
    return g, [(src, 1.0)], sig, rcv, freqs


def directional_components(g, at):
    """Monopole + three dipoles at the air node nearest `at` (fdtd.rs:730-743)."""
    return source_components(g, g.nearest_air(at), 1)


def worst_relative(ref, got):
    """The reference's GPU-vs-CPU measure: max |a - b| / max |a|."""
    ref = np.asarray(ref)
    return float(np.abs(ref - np.asarray(got)).max() / np.abs(ref).max())
