"""numpy restatement of the voxeliser for box-shaped rooms.

Test infrastructure only (see oracle/__init__.py).  Follows
FdtdGrid::build_dx (wavey-solver/src/fdtd.rs:289-378): one solid padding
layer (origin lo - dx/2, n = ceil(size/dx) + 2), air where the room contains
the cell centre strictly inside the prism (room.rs:151-157, with the
even-odd plan test of regions.rs:237-249, which holds a rectangle as
[x0, x1) x [y0, y1)), neighbour flags, the surface behind each missing
face within 1.5 dx along the axis (the BVH query of fdtd.rs:360-362), and
boundary_slots (fdtd.rs:539-571).  Written independently of the product's
C++ builder, vectorised over cells, so the two can be compared bit for bit.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

COURANT = 0.5773502691896257
AIR = 64
NO_BOUNDARY = 0xFFFFFFFF


@dataclass
class Grid:
    n: tuple
    origin: np.ndarray
    dx: float
    dt: float
    flags: np.ndarray
    bidx: np.ndarray
    bcell: np.ndarray
    bstart: np.ndarray
    slots: np.ndarray


def _rects(room):
    """(axis, c, lo[3], hi[3]) per surface, in the room's surface order."""
    h = room.height
    R = []

    def add(axis, c, lo, hi):
        R.append((axis, c, np.array(lo, float), np.array(hi, float)))

    add(2, 0.0, [room.x0, room.y0, 0], [room.x1, room.y1, 0])
    add(2, h, [room.x0, room.y0, 0], [room.x1, room.y1, 0])
    add(1, room.y0, [room.x0, 0, 0], [room.x1, 0, h])
    add(0, room.x1, [0, room.y0, 0], [0, room.y1, h])
    add(1, room.y1, [room.x0, 0, 0], [room.x1, 0, h])
    add(0, room.x0, [0, room.y0, 0], [0, room.y1, h])
    for (x0, y0, x1, y1) in room.pillars:
        add(1, y0, [x0, 0, 0], [x1, 0, h])
        add(0, x0, [0, y0, 0], [0, y1, h])
        add(1, y1, [x0, 0, 0], [x1, 0, h])
        add(0, x1, [0, y0, 0], [0, y1, h])
    for (x0, y0, z0, x1, y1, z1) in room.blocks:
        add(0, x0, [0, y0, z0], [0, y1, z1])
        add(0, x1, [0, y0, z0], [0, y1, z1])
        add(1, y0, [x0, 0, z0], [x1, 0, z1])
        add(1, y1, [x0, 0, z0], [x1, 0, z1])
        add(2, z0, [x0, y0, 0], [x1, y1, 0])
        add(2, z1, [x0, y0, 0], [x1, y1, 0])
    return R


def _fit_key(f):
    return (f.beta0, tuple((b.r, b.m, b.k) for b in f.branches), tuple(f.band), f.rms_error, f.max_error)


def _slots(faces, fits, dt):
    counts = []  # [surface, count]
    for s in faces:
        for c in counts:
            if _fit_key(fits[c[0]]) == _fit_key(fits[s]):
                c[1] += 1
                break
        else:
            counts.append([s, 1])
    out = []
    for s, count in counts:
        fit = fits[s]
        n = float(count)

        def add(r, m, k):
            r, m, k = r / n, m / n, k / n
            if m > 0.0:
                d, cv, w = m / dt + r / 2.0 + k * dt / 4.0, m / dt - r / 2.0 - k * dt / 4.0, 0.25
            else:
                d, cv, w = r + k * dt / 2.0, -k * dt / 2.0, 0.0
            out.append((1.0 / d, cv, k, w))

        if fit.beta0 > 0.0:
            add(1.0 / fit.beta0, 0.0, 0.0)
        for b in fit.branches:
            add(b.r, b.m, b.k)
    return out


def build_dx(room, fits, c: float, dx: float) -> Grid:
    dt = COURANT * dx / c
    lo = np.array([room.x0, room.y0, 0.0])
    hi = np.array([room.x1, room.y1, room.height])
    origin = lo - dx * 0.5
    n = tuple(int(math.ceil((hi[a] - lo[a]) / dx)) + 2 for a in range(3))
    nx, ny, nz = n
    xs = origin[0] + np.arange(nx, dtype=np.float64) * dx
    ys = origin[1] + np.arange(ny, dtype=np.float64) * dx
    zs = origin[2] + np.arange(nz, dtype=np.float64) * dx
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    solid = np.zeros((nz, ny, nx), bool)
    for (x0, y0, z0, x1, y1, z1) in room.solids:
        solid |= (X >= x0) & (Y >= y0) & (Z >= z0) & (X <= x1) & (Y <= y1) & (Z <= z1)
    inside = (Z > 0.0) & (Z < room.height) & (X >= room.x0) & (X < room.x1) & (Y >= room.y0) & (Y < room.y1)
    for (x0, y0, x1, y1) in room.pillars:
        inside &= ~((X >= x0) & (X < x1) & (Y >= y0) & (Y < y1))
    for (x0, y0, z0, x1, y1, z1) in room.blocks:
        inside &= ~((X >= x0) & (Y >= y0) & (Z >= z0) & (X <= x1) & (Y <= y1) & (Z <= z1))
    air = ~solid & inside
    air[0, :, :] = air[-1, :, :] = False
    air[:, 0, :] = air[:, -1, :] = False
    air[:, :, 0] = air[:, :, -1] = False
    flags = np.where(air, AIR, 0).astype(np.uint8)
    shifts = [(2, -1), (2, 1), (1, -1), (1, 1), (0, -1), (0, 1)]  # array axis (z, y, x order), step
    nb_air = []
    for k, (ax, st) in enumerate(shifts):
        a = np.zeros_like(air)
        src = [slice(None)] * 3
        dst = [slice(None)] * 3
        if st < 0:
            dst[ax], src[ax] = slice(1, None), slice(None, -1)
        else:
            dst[ax], src[ax] = slice(None, -1), slice(1, None)
        a[tuple(dst)] = air[tuple(src)]
        nb_air.append(a)
        flags |= np.where(air & a, 1 << k, 0).astype(np.uint8)
    rects = _rects(room)
    bidx = np.full(nx * ny * nz, NO_BOUNDARY, dtype=np.uint32)
    bcell, bstart, slots = [], [], []
    cand = np.flatnonzero((air & ((flags & 63) != 63)).reshape(-1))
    ff = flags.reshape(-1)
    sol = solid.reshape(-1)
    for i in cand:
        z, r = divmod(int(i), nx * ny)
        y, x = divmod(r, nx)
        p = np.array([xs[x], ys[y], zs[z]])
        faces = []
        for k in range(6):
            if ff[i] & (1 << k):
                continue
            off = [-1, 1, -nx, nx, -nx * ny, nx * ny][k]
            if sol[i + off]:
                continue
            axis, sgn = k // 2, (1.0 if k & 1 else -1.0)
            best, tbest = -1, dx * 1.5
            for q, (ra, rc, rlo, rhi) in enumerate(rects):
                if ra != axis:
                    continue
                t = (rc - p[axis]) * sgn
                if not (t > 0.0 and t < tbest):
                    continue
                if all(rlo[a] <= p[a] <= rhi[a] for a in range(3) if a != axis):
                    best, tbest = q, t
            if best >= 0:
                faces.append(best)
        sl = _slots(faces, fits, dt)
        if sl:
            bidx[i] = len(bcell)
            bcell.append(i)
            bstart.append(len(slots))
            slots.extend(sl)
    bstart.append(len(slots))
    return Grid(n, origin, dx, dt, flags.reshape(-1), bidx, np.array(bcell, np.uint32), np.array(bstart, np.uint32),
                np.array(slots, np.float64).reshape(-1, 4))
