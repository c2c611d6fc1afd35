"""FdtdGrid.build_dx on the device (wavey_cuda_grid_build) against the host
builder (wh_grid_build, itself pinned to the numpy restatement of the
reference's voxeliser in tests/test_host_grid.py): every array identical --
flags, boundary indices, node cells, slot ranges and slot constants -- for
rooms with pillars, absorbing blocks, rigid solids and branch materials."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import C_AIR
from wavey_gb300.fdtd import FdtdGrid
from wavey_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _same(a: FdtdGrid, b: FdtdGrid):
    assert a.n == b.n and a.dx == b.dx and a.dt == b.dt and np.array_equal(a.origin, b.origin)
    assert a.air == b.air and a.n_boundary == b.n_boundary
    for name in ("flags", "bidx", "bcell", "bstart", "slots"):
        x, y = getattr(a, name), getattr(b, name)
        assert x.shape == y.shape, name
        assert np.array_equal(x, y), name


def test_pillar_room(backend):
    sc = W.room_small(seed=1)
    dev = backend.build_grid(sc.room, sc.fits, W.C_AIR, sc.grid.dx)  # the workloads' speed of sound
    _same(sc.grid, dev)


def test_hall_with_pillars_and_balcony(backend):
    sc = W.room_hall(crossover=150.0, speakers=1, n_mics=4, plane_spacing=2.0)
    dev = backend.build_grid(sc.room, sc.fits, W.C_AIR, sc.grid.dx)  # the workloads' speed of sound
    _same(sc.grid, dev)


def test_branch_materials_and_a_cabinet(backend, library):
    from scenes import BRANCH_MATERIALS
    from wavey_gb300.fdtd import BoxRoom
    from wavey_gb300.materials import fit_surfaces

    room = BoxRoom(5.0, 4.0, 3.0, pillars=[(3.0, 1.0, 3.4, 1.5)], solids=[(1.0, 2.4, 1.0, 1.3, 2.7, 1.4)])
    fits = fit_surfaces([library[BRANCH_MATERIALS[i % 6]] for i in range(room.n_surfaces)], (20.0, 300.0))
    host = FdtdGrid.build_dx(room, fits, C_AIR, 0.05)
    dev = backend.build_grid(room, fits, C_AIR, 0.05)
    _same(host, dev)
    assert host.n_boundary > 0 and np.any(np.diff(host.bstart.astype(np.int64)) > 2)


def test_grid_build_limits(backend):
    from wavey_gb300.backend import WaveyError
    from wavey_gb300.fdtd import BoxRoom
    from wavey_gb300.materials import AdmittanceFit

    room = BoxRoom(400.0, 400.0, 100.0)
    with pytest.raises(WaveyError, match="MAX_CELLS"):
        backend.build_grid(room, [AdmittanceFit(0.1)] * 6, C_AIR, 0.05)


def test_mesh_room_cr2(backend):
    """The BRAS room CR2 (an OBJ mesh) at the 700 Hz grid of the reference's
    bras_wave run: column_fill and the triangle face lookup on the device
    give the host builder's arrays."""
    from cr2_scene import cr2_spec
    from wavey_gb300 import room_ir
    from wavey_gb300.materials import fit_surfaces

    spec, _, temperature_c = cr2_spec()
    c = room_ir.speed_of_sound(temperature_c)
    fits = fit_surfaces(spec.surface_materials, (20.0, 700.0))
    host = FdtdGrid.build(spec.room, fits, c, 700.0, 10.0)
    dev = backend.build_grid(spec.room, fits, c, host.dx)
    _same(host, dev)
    assert host.air > 1_000_000


def test_mesh_room_with_overhang_and_a_cabinet(backend):
    """A room swept from a stepped profile with an overhanging slab (the
    reference's column_fill test room), every surface its own material, and
    a rigid box inside."""
    from test_mesh_rooms import swept
    from wavey_gb300.materials import fit_surfaces, scalar_material

    profile = [(0.0, 0.0), (6.0, 0.0), (6.0, 1.0), (10.0, 1.0), (10.0, 4.0), (0.0, 4.0), (0.0, 2.6), (3.0, 2.6),
               (3.0, 2.2), (0.0, 2.2)]
    room = swept(profile, [list(range(10))], 5.0)
    fits = fit_surfaces([scalar_material(0.05 + 0.03 * i) for i in range(room.n_surfaces)], (20.0, 200.0))
    solids = [(7.0, 2.0, 1.5, 7.6, 2.5, 2.3)]
    host = FdtdGrid.build_dx(room, fits, 343.0, 0.08, solids=solids)
    dev = backend.build_grid(room, fits, 343.0, 0.08, solids=solids)
    _same(host, dev)
    assert host.n_boundary > 10_000
