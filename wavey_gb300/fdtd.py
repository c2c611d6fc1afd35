"""Grids, sources and post-processing of the FDTD wave solver
(wavey-solver/src/fdtd.rs), over libwavey_host.so.

  BoxRoom                    box-shaped rooms as wavey-geom's build_room makes
                             them from a rectangular plan (room.rs:281-349),
                             with pillars, absorbing blocks and rigid solids
  FdtdGrid.build / build_dx  fdtd.rs:276-378
  FdtdGrid.nearest_air       fdtd.rs:245-272
  FdtdGrid.taps_at           fdtd.rs:467-492
  source_components          fdtd.rs:730-743
  source_signal              fdtd.rs:601-610
  to_transfer                fdtd.rs:819-840
  fit_first_order            fdtd.rs:749-807
  component_weights          fdtd.rs:812-815
  FdtdSettings               fdtd.rs:85-176
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from .materials import AdmittanceFit

COURANT = 0.5773502691896257
MAX_CELLS = 600_000_000
NO_BOUNDARY = 0xFFFFFFFF
AIR = 64


def _vec3(p) -> "C.Array":
    return (C.c_double * 3)(*[float(v) for v in p])


@dataclass
class BoxRoom:
    """A rectangular plan [x0, x1] x [y0, y1] extruded to `height`.

    pillars: floor-to-ceiling rectangles (x0, y0, x1, y1), holes of the plan.
    blocks:  axis-aligned absorbing boxes (x0, y0, z0, x1, y1, z1), e.g.
             balcony steps; their six faces are room surfaces.
    solids:  rigid boxes (cabinets): cells inside are not air and their faces
             carry no admittance (fdtd.rs:355-356).
    Surfaces: floor, ceiling, walls y=y0, x=x1, y=y1, x=x0, then 4 faces per
    pillar (y=py0, x=px0, y=py1, x=px1), then 6 faces per block.
    """

    x1: float
    y1: float
    height: float
    x0: float = 0.0
    y0: float = 0.0
    pillars: list = field(default_factory=list)
    blocks: list = field(default_factory=list)
    solids: list = field(default_factory=list)

    def _c(self):
        keep = []

        def arr(rows, w):
            if not rows:
                return 0, None
            a = np.ascontiguousarray(np.asarray(rows, dtype=np.float64).reshape(-1, w))
            keep.append(a)
            return len(a), N.ptr(a, C.c_double)

        np_, pp = arr(self.pillars, 4)
        nb_, bp = arr(self.blocks, 6)
        ns_, sp = arr(self.solids, 6)
        r = N.WhRoom(self.x0, self.y0, self.x1, self.y1, self.height, np_, pp, nb_, bp, ns_, sp)
        return r, keep

    @property
    def n_surfaces(self) -> int:
        return 6 + 4 * len(self.pillars) + 6 * len(self.blocks)

    def contains(self, p) -> bool:
        r, keep = self._c()
        return bool(N.host().wh_room_contains(C.byref(r), _vec3(p)))

    def bounds(self):
        return np.array([self.x0, self.y0, 0.0]), np.array([self.x1, self.y1, self.height])


class FdtdGrid:
    """Voxelised room (FdtdGrid, fdtd.rs:196-209).  Arrays are numpy views
    of the host library's buffers, alive as long as this object."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)
        v = N.WhGridView()
        N.host().wh_grid_view_of(self._h, C.byref(v))
        self.n = (int(v.nx), int(v.ny), int(v.nz))
        self.origin = np.array(v.origin[:])
        self.dx = float(v.dx)
        self.dt = float(v.dt)
        cells = self.n[0] * self.n[1] * self.n[2]
        self.flags = np.ctypeslib.as_array(v.flags, shape=(cells,))
        self.bidx = np.ctypeslib.as_array(v.bidx, shape=(cells,))
        nb = int(v.n_boundary)
        self.n_boundary = nb
        self.bcell = np.ctypeslib.as_array(v.bcell, shape=(nb,)) if nb else np.zeros(0, np.uint32)
        self.bstart = np.ctypeslib.as_array(v.bstart, shape=(nb + 1,))
        ns = int(v.n_slots)
        self.slots = np.ctypeslib.as_array(v.slots, shape=(ns, 4)) if ns else np.zeros((0, 4))
        self.air = int(v.air_cells)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            N.host().wh_grid_free(h)
            self._h = None

    # -------------------------------------------------------------- build
    @staticmethod
    def build_dx(room, fits: list, c: float, dx: float, solids=()) -> "FdtdGrid":
        """room: a BoxRoom, or a MeshRoom (with optional rigid boxes
        `solids`, (x0, y0, z0, x1, y1, z1) each)."""
        if len(fits) != room.n_surfaces:
            raise ValueError(f"{len(fits)} fits for {room.n_surfaces} surfaces")
        arr = (N.WhFit * len(fits))(*[f._c() for f in fits])
        out = C.c_void_p()
        if hasattr(room, "_h"):  # MeshRoom
            sol = np.ascontiguousarray(np.asarray(solids, dtype=np.float64).reshape(-1, 6))
            st = N.host().wh_grid_build_mesh(room._h, N.ptr(sol, C.c_double) if len(sol) else None, len(sol), arr,
                                             len(fits), float(c), float(dx), C.byref(out))
        else:
            r, keep = room._c()
            st = N.host().wh_grid_build(C.byref(r), arr, len(fits), float(c), float(dx), C.byref(out))
        if st == N.WAVEY_E_LIMIT:
            raise ValueError("the wave solver grid would exceed MAX_CELLS; lower the crossover frequency")
        if st != 0:
            raise ValueError(f"grid build failed ({st})")
        return FdtdGrid(out.value)

    @staticmethod
    def build(room, fits: list, c: float, f_max: float, ppw: float, solids=()) -> "FdtdGrid":
        """FdtdGrid::build / build_with (fdtd.rs:276-286): dx = c / (f_max
        ppw), at most the smallest solid side / 8."""
        if hasattr(room, "_h"):  # MeshRoom
            dx = float(c) / (float(f_max) * float(ppw))
            for s in solids:
                dx = min(dx, min(s[3] - s[0], s[4] - s[1], s[5] - s[2]) / 8.0)
            return FdtdGrid.build_dx(room, fits, c, dx, solids)
        r, keep = room._c()
        dx = N.host().wh_grid_spacing(C.byref(r), float(c), float(f_max), float(ppw))
        return FdtdGrid.build_dx(room, fits, c, dx)

    # -------------------------------------------------------------- queries
    @property
    def cells(self) -> int:
        return self.n[0] * self.n[1] * self.n[2]

    def air_cells(self) -> int:
        return self.air

    def index(self, x: int, y: int, z: int) -> int:
        return (z * self.n[1] + y) * self.n[0] + x

    def center(self, x: int, y: int, z: int) -> np.ndarray:
        return self.origin + np.array([x, y, z], dtype=np.float64) * self.dx

    def pos(self, i: int) -> np.ndarray:
        nx, ny = self.n[0], self.n[1]
        z, r = divmod(int(i), nx * ny)
        y, x = divmod(r, nx)
        return self.center(x, y, z)

    def nearest_air(self, p):
        i = N.host().wh_nearest_air(self._h, _vec3(p))
        return None if i < 0 else int(i)

    def taps_at(self, p):
        cells = (C.c_int64 * 8)()
        w = (C.c_double * 8)()
        n = N.host().wh_taps_at(self._h, _vec3(p), cells, w)
        if n < 0:
            return None
        return [(int(cells[k]), float(w[k])) for k in range(n)]

    def baffle_point(self, p, axis) -> np.ndarray:
        out = (C.c_double * 3)()
        N.host().wh_baffle_point(self._h, _vec3(p), _vec3(axis), out)
        return np.array(out[:])

    def air_along(self, p, axis):
        i = N.host().wh_air_along(self._h, _vec3(p), _vec3(axis))
        return None if i < 0 else int(i)

    def boundary_slots_of(self, b: int) -> np.ndarray:
        return self.slots[self.bstart[b]:self.bstart[b + 1]]


def source_components(g: FdtdGrid, c: int, order: int):
    cells = (C.c_int64 * 8)()
    w = (C.c_double * 8)()
    n = (C.c_int32 * 4)()
    k = N.host().wh_source_components(g._h, int(c), int(order), cells, w, n)
    if k < 0:
        return None
    return [[(int(cells[2 * i + j]), float(w[2 * i + j])) for j in range(n[i])] for i in range(k)]


def source_signal(f_max: float, dt: float, steps: int) -> np.ndarray:
    out = np.empty(int(steps), dtype=np.float64)
    N.host().wh_source_signal(float(f_max), float(dt), int(steps), N.ptr(out, C.c_double))
    return out


def frequency_grid(f_min: float, f_max: float, n: int) -> np.ndarray:
    count = N.host().wh_frequency_grid(float(f_min), float(f_max), int(n), None, 0)
    out = np.empty(max(count, 0), dtype=np.float64)
    N.host().wh_frequency_grid(float(f_min), float(f_max), int(n), N.ptr(out, C.c_double), count)
    return out


def band_edges(f: float, fraction: float):
    """freq.rs:32-35"""
    h = 2.0 ** (0.5 / fraction)
    return f / h, f * h


@dataclass
class FdtdSettings:
    crossover_hz: float = 250.0
    duration_s: float = 0.0
    points_per_wavelength: float = 15.0
    source_order: int = 1
    headroom: float = 2.0  # WaveAccuracy::High

    def f_max(self) -> float:
        return self.crossover_hz * math.sqrt(2.0)

    def weight(self, f: float) -> float:
        return N.host().wh_crossover_weight(float(self.crossover_hz), float(f))

    def grid_fmax(self, freqs) -> float:
        top = max([f for f in freqs if self.weight(f) > 0.0], default=0.0)
        return min(top * self.headroom, self.f_max()) if top > 0.0 else self.f_max()

    @staticmethod
    def phase_error_deg_per_m(f: float, c: float, dx: float) -> float:
        return N.host().wh_phase_error_deg_per_m(float(f), float(c), float(dx))


def auto_duration(rt) -> float:
    a = np.ascontiguousarray(rt, dtype=np.float64)
    return N.host().wh_auto_duration(N.ptr(a, C.c_double), len(a))


def to_transfer(spectra: np.ndarray, signal: np.ndarray, g: FdtdGrid, freqs, c: float, r_ref: float, h0) -> np.ndarray:
    """spectra: complex [n_recv * nf] or [n_recv, nf]; returns the same shape."""
    sp = np.ascontiguousarray(np.asarray(spectra, dtype=np.complex128))
    shape = sp.shape
    sp = sp.reshape(-1)
    fr = np.ascontiguousarray(freqs, dtype=np.float64)
    nf = len(fr)
    h = np.ascontiguousarray(np.broadcast_to(np.asarray(h0, dtype=np.complex128), (nf,)))
    sig = np.ascontiguousarray(signal, dtype=np.float64)
    out = np.empty_like(sp)
    N.host().wh_to_transfer(N.ptr(sp.view(np.float64), C.c_double), len(sp) // max(nf, 1), N.ptr(sig, C.c_double),
                            len(sig), g.dt, g.dx, N.ptr(fr, C.c_double), nf, float(c), float(r_ref),
                            N.ptr(h.view(np.float64), C.c_double), N.ptr(out.view(np.float64), C.c_double))
    return out.reshape(shape)


def blend(ism: complex, wave: complex, w: float) -> complex:
    a = (C.c_double * 2)(ism.real, ism.imag)
    b = (C.c_double * 2)(wave.real, wave.imag)
    o = (C.c_double * 2)()
    N.host().wh_blend(a, b, float(w), o)
    return complex(o[0], o[1])


def fit_directions() -> np.ndarray:
    out = np.empty((N.WH_FIT_DIRECTIONS, 3), dtype=np.float64)
    N.host().wh_fit_directions(N.ptr(out, C.c_double))
    return out


def speaker_rotation(yaw_deg: float = 0.0, pitch_deg: float = 0.0, roll_deg: float = 0.0) -> np.ndarray:
    """Column-major 3x3 local-to-room rotation, returned as a (3, 3) matrix
    whose [:, k] is column k."""
    out = (C.c_double * 9)()
    N.host().wh_speaker_rotation(float(yaw_deg), float(pitch_deg), float(roll_deg), out)
    return np.array(out[:]).reshape(3, 3).T


def fit_first_order(directivity, to_room: np.ndarray, f: float):
    """directivity(f, local_dir) -> complex.  Returns (a0, [ax, ay, az], residual)."""
    dirs = fit_directions()
    d = np.array([complex(directivity(f, v)) for v in dirs], dtype=np.complex128)
    dax = complex(directivity(f, np.array([1.0, 0.0, 0.0])))
    m = np.ascontiguousarray(np.asarray(to_room, dtype=np.float64).T.reshape(-1))  # column-major
    axis = (C.c_double * 2)(dax.real, dax.imag)
    out = (C.c_double * 8)()
    res = C.c_double()
    N.host().wh_fit_first_order(N.ptr(d.view(np.float64), C.c_double), axis, N.ptr(m, C.c_double), out, C.byref(res))
    a = [complex(out[2 * i], out[2 * i + 1]) for i in range(4)]
    return a[0], a[1:], float(res.value)


def component_weights(a0: complex, a, k: float, dx: float) -> list:
    x = (C.c_double * 2)(a0.real, a0.imag)
    y = (C.c_double * 6)(*[v for c in a for v in (c.real, c.imag)])
    o = (C.c_double * 8)()
    N.host().wh_component_weights(x, y, float(k), float(dx), o)
    return [complex(o[2 * i], o[2 * i + 1]) for i in range(4)]
