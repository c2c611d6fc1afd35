"""Rooms imported as polygon meshes, and the reference's room description
format for them, over libwavey_host.so.

  MeshRoom            wavey-geom/src/room.rs:399-461 (room_from_mesh), the
                      room's surfaces per (material group, plane), its
                      inside test (room.rs:151-157, 355-367) and volume
  MeshRoom.from_obj   wavey-project/src/import/obj.rs:8-45 and
                      import/mod.rs:220-231 (v, f, usemtl; no repair)
  read_csv_material   wavey-cli/src/build.rs: csv_material (freq / abs / sct
                      rows, separated by ';' or ',')
  load_room_spec      wavey-cli/src/build.rs: `wavey build <spec.json>` for a
                      mesh room ({"mesh": {"obj", "scale", "groups"},
                      "material_csv", "speakers", "mics"}): the room, each
                      surface's material (its group's), the speakers'
                      acoustic centres and the microphones

FdtdGrid.build / build_dx accept a MeshRoom wherever they accept a BoxRoom.
"""
from __future__ import annotations

import ctypes as C
import json
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _native as N
from .materials import Material, Spectrum


def _vec3(p):
    return (C.c_double * 3)(*[float(v) for v in p])


class MeshRoom:
    """A closed room given as polygons with a material group each.

    vertices: [n][3] metres; faces: list of (vertex indices, group index);
    groups: the group names (material slots), indexed by a face's group.
    """

    def __init__(self, vertices, faces, groups=None):
        self.vertices = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3)
        self.faces = [([int(i) for i in f], int(g)) for f, g in faces]
        n_groups = 1 + max((g for _, g in self.faces), default=-1)
        self.groups = list(groups) if groups is not None else [f"group{i}" for i in range(n_groups)]
        idx = np.ascontiguousarray([i for f, _ in self.faces for i in f] or [0], dtype=np.uint32)
        start = np.zeros(len(self.faces) + 1, dtype=np.int64)
        start[1:] = np.cumsum([len(f) for f, _ in self.faces])
        grp = np.ascontiguousarray([g for _, g in self.faces] or [0], dtype=np.int32)
        h = C.c_void_p()
        st = N.host().wh_mesh_room_build(N.ptr(self.vertices, C.c_double), len(self.vertices),
                                         N.ptr(idx, C.c_uint32), N.ptr(start, C.c_int64),
                                         N.ptr(grp, C.c_int32), len(self.faces), C.byref(h))
        if st != N.WAVEY_OK:
            raise ValueError(f"not a room mesh ({st})")
        self._h = h
        self.n_surfaces = int(N.host().wh_mesh_room_surface_count(h))
        self.surface_groups, self.surface_kinds, self.surface_normals, self.surface_areas = [], [], [], []
        for s in range(self.n_surfaces):
            g, k = C.c_int32(), C.c_int32()
            n = (C.c_double * 3)()
            d, a = C.c_double(), C.c_double()
            N.host().wh_mesh_room_surface(h, s, C.byref(g), C.byref(k), n, C.byref(d), C.byref(a))
            self.surface_groups.append(int(g.value))
            self.surface_kinds.append(("wall", "floor", "ceiling")[k.value])
            self.surface_normals.append(np.array(n[:]))
            self.surface_areas.append(float(a.value))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            N.host().wh_mesh_room_free(h)
            self._h = None

    @staticmethod
    def from_obj(text: str, scale: float = 1.0) -> "MeshRoom":
        """Wavefront OBJ: `v` lines, `f` polygons (1-based or negative
        indices, `v/vt/vn` forms), groups from `usemtl` names, or from `g` /
        `o` names when the file has no `usemtl`; faces before any group go to
        group "default" (obj.rs:8-45)."""
        has_materials = any(line.lstrip().startswith("usemtl") for line in text.splitlines())
        verts, faces, names = [], [], []
        group = None

        def group_of(name):
            if name not in names:
                names.append(name)
            return names.index(name)

        for ln, line in enumerate(text.splitlines()):
            p = line.split()
            if not p:
                continue
            if p[0] == "v" and len(p) >= 4:
                verts.append([float(x) * scale for x in p[1:4]])
            elif p[0] == "usemtl" and len(p) >= 2:
                group = group_of(" ".join(p[1:]))
            elif p[0] in ("g", "o") and len(p) >= 2 and not has_materials:
                group = group_of(" ".join(p[1:]))
            elif p[0] == "f" and len(p) >= 4:
                if group is None:
                    group = group_of("default")
                n = len(verts)
                idx = []
                for t in p[1:]:
                    i = int(t.split("/")[0])
                    i = n + i if i < 0 else i - 1
                    if i < 0 or i >= n:
                        raise ValueError(f"line {ln + 1}: vertex {i + 1} out of range")
                    idx.append(i)
                faces.append((idx, group))
        if not faces:
            raise ValueError("no faces in OBJ")
        return MeshRoom(verts, faces, names)

    # ------------------------------------------------------------ queries
    def materials_for(self, group_materials: dict) -> list:
        """Each surface's material: its group's (build.rs: mesh surfaces take
        their group's material)."""
        return [group_materials[self.groups[g]] for g in self.surface_groups]

    def contains(self, p) -> bool:
        return bool(N.host().wh_mesh_room_contains(self._h, _vec3(p)))

    def bounds(self):
        lo, hi = (C.c_double * 3)(), (C.c_double * 3)()
        N.host().wh_mesh_room_bounds(self._h, lo, hi)
        return np.array(lo[:]), np.array(hi[:])

    def volume(self) -> float:
        return float(N.host().wh_mesh_room_volume(self._h))

    def triangles(self):
        """(positions [T][3][3], surface of each triangle [T])."""
        t = int(N.host().wh_mesh_room_triangle_count(self._h))
        pos = np.zeros((t, 3, 3))
        srf = np.zeros(t, dtype=np.uint32)
        N.host().wh_mesh_room_triangles(self._h, N.ptr(pos, C.c_double), N.ptr(srf, C.c_uint32))
        return pos, srf


def read_csv_material(mid: str, name: str, text: str) -> Material:
    """A material from `freq;...` / `abs;...` (/ `sct;...`) rows; scattering
    is not used on the FDTD path."""
    rows = {}
    for line in text.splitlines():
        cells = [c.strip() for c in line.replace(",", ";").split(";")]
        if len(cells) < 2:
            continue
        vals = []
        for c in cells[1:]:
            try:
                vals.append(float(c))
            except ValueError:
                pass
        rows[cells[0].lower()] = vals
    if "freq" not in rows:
        raise ValueError("no freq row")
    f = rows["freq"]
    a = rows.get("abs")
    if a is None or len(a) != len(f):
        raise ValueError("no abs row matching freq")
    return Material(id=mid, absorption=Spectrum.bands(f, a), name=name)


@dataclass
class RoomSpec:
    """A mesh room as `wavey build` reads it: the room, each surface's
    material, speakers (name, acoustic centre) and microphones (name,
    position)."""

    room: MeshRoom
    surface_materials: list
    speakers: list = field(default_factory=list)
    mics: list = field(default_factory=list)
    group_materials: dict = field(default_factory=dict)


def load_room_spec(path) -> RoomSpec:
    """Reads a mesh-room description (the reference's `wavey build` JSON with
    a "mesh" entry).  Speakers are taken at their given centre (x, y, z); the
    acoustic centre of the omnidirectional sample model is its centre."""
    path = Path(path)
    spec = json.loads(path.read_text())
    ms = spec.get("mesh")
    if not ms:
        raise ValueError("only mesh rooms are read here (no \"mesh\" entry)")
    base = path.parent
    room = MeshRoom.from_obj((base / ms["obj"]).read_text(), float(ms.get("scale", 1.0)))
    mats = {}
    for c in spec.get("material_csv", []):
        m = read_csv_material(c["id"], c.get("name") or c["id"], (base / c["file"]).read_text())
        k = c.get("absorption_scale")
        if k is not None:
            m = Material(id=m.id, name=m.name, absorption=Spectrum.bands(
                m.absorption.freqs_hz, [min(v * float(k), 0.99) for v in m.absorption.values]))
        mats[m.id] = m
    group_materials = {}
    for g in room.groups:
        mid = ms.get("groups", {}).get(g)
        if mid is None or mid not in mats:
            raise ValueError(f"group {g!r} has no material")
        group_materials[g] = mats[mid]
    speakers = [(s["name"], (float(s["x"]), float(s["y"]), float(s.get("z", 1.5)))) for s in spec.get("speakers", [])]
    mics = [(m["name"], (float(m["x"]), float(m["y"]), float(m["z"]))) for m in spec.get("mics", [])]
    return RoomSpec(room, room.materials_for(group_materials), speakers, mics, group_materials)
