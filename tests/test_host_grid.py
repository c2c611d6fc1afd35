"""The host library's voxeliser, taps and signals.

The product's C++ grid builder is compared bit for bit with the oracle's
independent numpy restatement of FdtdGrid::build_dx (fdtd.rs:289-378), and
the reference's own assertions about grids are restated.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import C_AIR
from oracle import voxel
from wavey_gb300.fdtd import (AIR, BoxRoom, FdtdGrid, frequency_grid, source_components, source_signal,
                              band_edges, FdtdSettings)
from wavey_gb300.materials import fit_surfaces, scalar_material


def _compare(room, fits, dx):
    g = FdtdGrid.build_dx(room, fits, C_AIR, dx)
    o = voxel.build_dx(room, fits, C_AIR, dx)
    assert g.n == o.n
    assert np.array_equal(g.origin, o.origin)
    assert g.dt == o.dt
    assert np.array_equal(g.flags, o.flags)
    assert np.array_equal(g.bidx, o.bidx)
    assert np.array_equal(g.bcell, o.bcell)
    assert np.array_equal(g.bstart, o.bstart)
    assert np.array_equal(g.slots, o.slots)
    return g


ROOMS = {
    "shoebox": BoxRoom(6.0, 4.0, 3.0),
    "pillar": BoxRoom(8.0, 6.0, 3.0, pillars=[(3.5, 2.5, 4.5, 3.5)]),
    "pillars_offset": BoxRoom(7.3, 5.1, 2.9, x0=-1.2, y0=0.4, pillars=[(1.05, 1.33, 1.71, 2.02), (3.3, 3.0, 3.9, 3.6)]),
    "balcony": BoxRoom(9.0, 7.0, 5.0, blocks=[(0.0, 5.0, 2.5, 9.0, 7.0, 2.9), (0.0, 5.8, 2.9, 9.0, 7.0, 3.3)]),
    "cabinet": BoxRoom(5.0, 4.0, 3.0, solids=[(2.0, 1.5, 1.0, 2.4, 1.8, 1.6)]),
}


@pytest.mark.parametrize("name", list(ROOMS))
def test_grid_matches_numpy_restatement(name, library):
    room = ROOMS[name]
    mats = [library[["audience-standing", "mineral-wool-50", "wood-panel", "carpet-heavy"][i % 4]]
            if i % 3 else scalar_material(0.1 * (1 + i % 4)) for i in range(room.n_surfaces)]
    fits = fit_surfaces(mats, (20.0, 300.0))
    g = _compare(room, fits, C_AIR / (300.0 * 10.0))
    assert g.n_boundary > 0
    # Boundary numbering follows the cell index (fdtd.rs:368-375).
    assert np.all(np.diff(g.bcell.astype(np.int64)) > 0)
    assert np.all(g.bidx[g.bcell] == np.arange(g.n_boundary))


def test_padding_layer_and_spacing():
    """fdtd.rs:290-299: origin lo - dx/2, ceil(size/dx) + 2 cells, solid border."""
    room = BoxRoom(3.0, 2.5, 2.0)
    fits = fit_surfaces([scalar_material(0.0)] * 6, (20.0, C_AIR))
    g = FdtdGrid.build(room, fits, C_AIR, C_AIR, 10.0)
    assert abs(g.dx - 0.1) < 1e-12  # tests/fdtd.rs:58
    # ceil(size/dx) + 2 in FP64: 3.0/0.1 is 30.000000000000004, so x gets an
    # extra (solid) cell, exactly as the reference's grid does.
    assert g.n == tuple(math.ceil(s / g.dx) + 2 for s in (3.0, 2.5, 2.0))
    assert np.allclose(g.origin, [-0.05, -0.05, -0.05])
    f = g.flags.reshape(g.n[2], g.n[1], g.n[0])
    for sl in [f[0], f[-1], f[:, 0], f[:, -1], f[:, :, 0], f[:, :, -1]]:
        assert not np.any(sl & AIR)
    # Rigid walls (alpha 0) give no boundary slots: the fit is rigid.
    assert g.n_boundary == 0
    assert g.air == 30 * 25 * 20


def test_max_cells_is_an_error():
    room = BoxRoom(100.0, 100.0, 100.0)
    fits = fit_surfaces([scalar_material(0.1)] * 6, (20.0, 100.0))
    with pytest.raises(ValueError, match="MAX_CELLS"):
        FdtdGrid.build_dx(room, fits, C_AIR, 0.1)


def test_taps_spread_over_eight_cells():
    """tests/fdtd.rs:159-160: a point between nodes gives eight taps."""
    room = BoxRoom(6.0, 4.0, 3.0)
    fits = fit_surfaces([scalar_material(0.2)] * 6, (20.0, 200.0))
    g = FdtdGrid.build(room, fits, C_AIR, 200.0, 12.0)
    taps = g.taps_at((1.53, 1.27, 1.41))
    assert len(taps) == 8
    assert abs(sum(w for _, w in taps) - 1.0) < 1e-12
    # Trilinear weights reproduce the position.
    p = sum(w * g.pos(c) for c, w in taps)
    assert np.allclose(p, [1.53, 1.27, 1.41], atol=1e-9)


def test_nearest_air_and_components():
    room = BoxRoom(6.0, 4.0, 3.0, pillars=[(2.0, 1.0, 3.0, 2.0)])
    fits = fit_surfaces([scalar_material(0.2)] * room.n_surfaces, (20.0, 200.0))
    g = FdtdGrid.build(room, fits, C_AIR, 200.0, 12.0)
    inside_pillar = (2.5, 1.5, 1.0)
    i = g.nearest_air(inside_pillar)
    assert g.flags[i] & AIR
    assert not room.contains(inside_pillar) and room.contains(g.pos(i))
    c = g.nearest_air((4.5, 3.0, 1.5))
    comps = source_components(g, c, 1)
    nx, nxy = g.n[0], g.n[0] * g.n[1]
    assert comps == [[(c, 1.0)], [(c + 1, 1.0), (c - 1, -1.0)], [(c + nx, 1.0), (c - nx, -1.0)],
                     [(c + nxy, 1.0), (c - nxy, -1.0)]]
    corner = g.nearest_air((0.01, 0.01, 0.01))
    assert source_components(g, corner, 1) is None
    assert source_components(g, corner, 0) == [[(corner, 1.0)]]


def test_source_signal_formula():
    dt, f_max = 1e-4, 300.0
    s = source_signal(f_max, dt, 50)
    sigma = 0.342 / f_max
    t = np.arange(50) * dt - 6 * sigma
    assert np.allclose(s, -t / sigma**2 * np.exp(-t * t / (2 * sigma * sigma)) * dt, rtol=1e-13, atol=0)


def test_frequency_grid_matches_reference_tests():
    """freq.rs:41-47: 31 third-octave bands 19.69 Hz ... 20158.7 Hz."""
    g = frequency_grid(20.0, 20000.0, 3)
    assert len(g) == 31
    assert np.any(np.abs(g - 1000.0) < 1e-9)
    assert abs(g[0] - 19.69) < 0.01 and abs(g[30] - 20158.7) < 0.1
    lo, hi = band_edges(1000.0, 1.0)
    assert abs(lo * hi - 1e6) < 1e-6 and abs(hi / lo - 2.0) < 1e-12


def test_crossover_weight():
    s = FdtdSettings(crossover_hz=250.0)
    assert s.weight(100.0) == 1.0 and s.weight(1000.0) == 0.0
    assert abs(s.weight(250.0) - 0.5) < 1e-12
    assert abs(s.f_max() - 250.0 * math.sqrt(2.0)) < 1e-12
