"""The BRAS room CR2 on the host: the fixture (tests/golden/cr2.json) builds
a closed mesh room, every source and microphone lies inside it, and the
700 Hz grid of the reference's bras_wave run (FdtdGrid::build at 10 points
per wavelength, c at the comparison's 19.5 C) has its sources and
microphones on air nodes next to their positions."""
from __future__ import annotations

import math

import numpy as np
import pytest

from cr2_scene import cr2_spec
from wavey_gb300 import room_ir


def test_cr2_room_is_closed_and_holds_its_positions():
    spec, published, temperature_c = cr2_spec()
    room = spec.room
    assert temperature_c == 19.5
    assert len(room.groups) == 5 and room.n_surfaces > len(room.groups)
    # Every surface takes its group's material.
    for s, g in enumerate(room.surface_groups):
        assert spec.surface_materials[s] is spec.group_materials[room.groups[g]]
    lo, hi = room.bounds()
    assert np.all(hi - lo > 2.9)
    # A closed mesh: the volume from the divergence theorem lies inside its box.
    assert 0.0 < room.volume() < np.prod(hi - lo)
    for name, p in spec.speakers + spec.mics:
        assert room.contains(p), name
    assert published["bands_hz"] == [63, 125, 250]


def test_cr2_grid_and_nodes():
    spec, _, temperature_c = cr2_spec()
    c = room_ir.speed_of_sound(temperature_c)
    assert c == pytest.approx(342.92, abs=0.01)
    run = room_ir.prepare(spec, f_max=700.0, duration=2.5, c=c)
    g = run.grid
    assert g.dx == pytest.approx(c / 7000.0)
    assert run.steps == math.ceil(2.5 / g.dt)
    assert run.bands == [63.0, 125.0, 250.0]
    # Air fills the room's volume to within a surface layer of cells.
    assert g.air * g.dx ** 3 == pytest.approx(spec.room.volume(), rel=0.05)
    for node, (_, p) in zip(run.sources + run.receivers, spec.speakers + spec.mics):
        assert np.linalg.norm(g.pos(node) - np.array(p)) <= g.dx * math.sqrt(3) / 2 + 1e-12
