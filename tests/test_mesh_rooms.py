"""Mesh rooms on the host: room_from_mesh, column_fill and the face lookup.

* column_fill_matches_the_inside_test (core/wavey-solver/tests/
  mesh_rooms.rs:74-99): a room swept from a stepped profile with an
  overhanging slab; every interior cell's air flag equals the room's own
  inside test at the cell centre.
* A mesh copy of a box room (one material group per surface, in the box
  room's surface order) voxelises to exactly the box builder's grid: flags,
  boundary indices and slots (the reference's mesh copy of an extruded room,
  mesh_rooms.rs:12-15).
* The OBJ reader (wavey-project/src/import/obj.rs:8-45) and the CSV
  material reader (wavey-cli/src/build.rs, csv_material).
"""
from __future__ import annotations

import numpy as np
import pytest

from wavey_gb300.fdtd import AIR, BoxRoom, FdtdGrid
from wavey_gb300.materials import fit_surfaces, scalar_material
from wavey_gb300.mesh import MeshRoom, read_csv_material


def swept(profile, caps, w):
    """A profile in (x, z) swept along y from 0 to w (mesh_rooms.rs:18-31):
    side face i has group i, the caps groups n and n + 1."""
    n = len(profile)
    v = [(x, 0.0, z) for x, z in profile] + [(x, w, z) for x, z in profile]
    faces = [([i, (i + 1) % n, n + (i + 1) % n, n + i], i) for i in range(n)]
    for c in caps:
        faces.append((list(c), n))
        faces.append(([n + i for i in c], n + 1))
    return MeshRoom(v, faces)


def test_column_fill_matches_the_inside_test():
    profile = [(0.0, 0.0), (6.0, 0.0), (6.0, 1.0), (10.0, 1.0), (10.0, 4.0), (0.0, 4.0), (0.0, 2.6), (3.0, 2.6),
               (3.0, 2.2), (0.0, 2.2)]
    room = swept(profile, [list(range(10))], 5.0)
    fits = fit_surfaces([scalar_material(0.1)] * room.n_surfaces, (20.0, 200.0))
    g = FdtdGrid.build_dx(room, fits, 343.0, 0.1)
    nx, ny, nz = g.n
    flags = g.flags.reshape(nz, ny, nx)
    air = mismatch = 0
    for z in range(1, nz - 1):
        for y in range(1, ny - 1):
            for x in range(1, nx - 1):
                a = bool(flags[z, y, x] & AIR)
                b = room.contains(g.center(x, y, z))
                air += b
                mismatch += a != b
    assert air > 100_000
    assert mismatch == 0


def test_swept_room_surfaces_face_into_the_room():
    profile = [(0.0, 0.0), (6.0, 0.0), (6.0, 1.0), (10.0, 1.0), (10.0, 4.0), (0.0, 4.0)]
    room = swept(profile, [list(range(6))], 5.0)
    # 6 side faces + 2 caps, each its own group and plane.
    assert room.n_surfaces == 8
    assert room.surface_kinds[0] == "floor" and room.surface_kinds[4] == "ceiling"
    assert np.allclose(room.surface_normals[0], [0, 0, 1]) and np.allclose(room.surface_normals[1], [-1, 0, 0])
    area = 6 * 4 + 4 * 3
    assert room.volume() == pytest.approx(area * 5.0, rel=1e-12)
    assert room.contains((2.0, 2.5, 0.5)) and not room.contains((8.0, 2.5, 0.5))


def _box_as_mesh(x1, y1, h, pillar):
    """The surfaces of BoxRoom(x1, y1, h, pillars=[pillar]) in its surface
    order (floor, ceiling, walls y=0, x=x1, y=y1, x=0, pillar faces y=py0,
    x=px0, y=py1, x=px1) as polygons, one group per surface; floor and
    ceiling are cut into rectangles around the pillar."""
    px0, py0, px1, py1 = pillar
    verts, faces = [], []

    def quad(pts, g):
        base = len(verts)
        verts.extend(pts)
        faces.append(([base, base + 1, base + 2, base + 3], g))

    def plan_tiles(z, g):
        for (a0, b0, a1, b1) in [(0, 0, px0, y1), (px1, 0, x1, y1), (px0, 0, px1, py0), (px0, py1, px1, y1)]:
            quad([(a0, b0, z), (a1, b0, z), (a1, b1, z), (a0, b1, z)], g)

    plan_tiles(0.0, 0)
    plan_tiles(h, 1)
    quad([(0, 0, 0), (x1, 0, 0), (x1, 0, h), (0, 0, h)], 2)
    quad([(x1, 0, 0), (x1, y1, 0), (x1, y1, h), (x1, 0, h)], 3)
    quad([(x1, y1, 0), (0, y1, 0), (0, y1, h), (x1, y1, h)], 4)
    quad([(0, y1, 0), (0, 0, 0), (0, 0, h), (0, y1, h)], 5)
    quad([(px0, py0, 0), (px1, py0, 0), (px1, py0, h), (px0, py0, h)], 6)
    quad([(px0, py0, 0), (px0, py1, 0), (px0, py1, h), (px0, py0, h)], 7)
    quad([(px0, py1, 0), (px1, py1, 0), (px1, py1, h), (px0, py1, h)], 8)
    quad([(px1, py0, 0), (px1, py1, 0), (px1, py1, h), (px1, py0, h)], 9)
    return MeshRoom(verts, faces)


def test_mesh_copy_of_a_box_room_gives_the_same_grid():
    pillar = (3.5, 2.5, 4.5, 3.5)
    box = BoxRoom(8.0, 6.0, 3.0, pillars=[pillar])
    mesh = _box_as_mesh(8.0, 6.0, 3.0, pillar)
    assert mesh.n_surfaces == box.n_surfaces == 10
    assert mesh.surface_groups == list(range(10))
    mats = [scalar_material(0.05 + 0.04 * i) for i in range(10)]
    fits = fit_surfaces(mats, (20.0, 300.0))
    a = FdtdGrid.build(box, fits, 343.0, 300.0, 10.0)
    b = FdtdGrid.build(mesh, fits, 343.0, 300.0, 10.0)
    assert a.n == b.n and a.dx == b.dx and np.array_equal(a.origin, b.origin)
    assert np.array_equal(a.flags, b.flags)
    assert np.array_equal(a.bidx, b.bidx)
    assert np.array_equal(a.bstart, b.bstart)
    assert np.array_equal(a.slots, b.slots)
    assert a.n_boundary > 1000


OBJ = """# unit-scaled box, two material groups
v 0 0 0
v 4 0 0
v 4 3 0
v 0 3 0
v 0 0 2.5
v 4 0 2.5
v 4 3 2.5
v 0 3 2.5
usemtl Floor
f 1/1/1 2/2/1 3/3/1 4/4/1
usemtl Walls
f 5 6 7 8
f 1 2 6 5
f -7 -6 -2 -3
f 3 4 8 7
f 4 1 5 8
"""


def test_obj_reader_groups_and_room():
    room = MeshRoom.from_obj(OBJ)
    assert room.groups == ["Floor", "Walls"]
    assert len(room.faces) == 6
    assert room.faces[3] == ([1, 2, 6, 5], 1)  # negative indices count back from the last vertex
    assert room.volume() == pytest.approx(30.0, rel=1e-12)
    lo, hi = room.bounds()
    assert np.allclose(lo, 0) and np.allclose(hi, [4, 3, 2.5])
    # Floor group: one surface; walls group: the ceiling and four walls.
    assert room.n_surfaces == 6
    assert room.surface_groups.count(0) == 1
    mm = "\n".join(f"v {1000 * x} {1000 * y} {1000 * z}" for x, y, z in room.vertices)
    mm += "\n" + "\n".join(line for line in OBJ.splitlines() if not line.startswith("v "))
    room_mm = MeshRoom.from_obj(mm, 0.001)
    assert room_mm.volume() == pytest.approx(30.0, rel=1e-12)


def test_csv_material():
    m = read_csv_material("c", "concrete", "freq;63;125;250\nabs;0.1;0.2;0.3\nsct;0.05;0.05;0.05\n")
    assert m.absorption.freqs_hz == (63.0, 125.0, 250.0)
    assert m.absorption_at(125.0) == pytest.approx(0.2)
    with pytest.raises(ValueError):
        read_csv_material("c", "c", "freq;63;125\nabs;0.1\n")
