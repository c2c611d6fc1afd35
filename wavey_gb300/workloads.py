"""Seeded synthetic scenes with the shapes of the wave solver's benchmark
configurations (no measured rooms or speaker data are needed).

  room_small      6 x 4 x 3 m shoebox at 250 Hz, frequency-independent walls
                  (alpha ~ U(0.05, 0.4) per surface), one monopole, 8 receivers,
                  0.5 s                                   (~26 k air cells)
  room_pillars    20 x 15 x 8 m with four 0.6 x 0.6 m pillars at 500 Hz, five
                  materials with octave-band alpha ~ U(0.02, 0.6) at
                  63..1000 Hz fitted to the boundary filter form, one cardioid
                  (monopole + 3 dipoles = 4 right-hand sides), 64 receivers
                  plus a 1.2 m cut plane at 0.25 m spacing, 1.0 s (~7 M cells)
  rooms_batch     room_small's room with 32 speakers (seeded monopoles and
                  cardioids, one right-hand side or four each) plus four
                  shoeboxes of U(5,25) x U(4,20) x U(3,10) m at 250 Hz with one
                  monopole each, all in one launch per step
  room_hall       40 x 25 x 15 m with 12 pillars and a stepped balcony at
                  1 kHz (~370 M cells), 8 materials

Grid spacing follows the reference's points-per-wavelength rule at ppw 10
(dx = c / (10 f_c)), the form its FDTD tests and `bras_wave` use
(FdtdGrid::build, fdtd.rs:276-286).  Receivers are mapped to nodes with
nearest_air (wavey-solver/src/run.rs:464); frequencies are the 1/12-octave
grid with a non-zero crossover weight (run.rs:463).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .fdtd import (BoxRoom, FdtdGrid, FdtdSettings, component_weights, fit_first_order, frequency_grid,
                   source_components, source_signal, speaker_rotation)
from .materials import Material, Spectrum, fit_surfaces

C_AIR = 343.0
OCTAVES = [63.0, 125.0, 250.0, 500.0, 1000.0]


def cardioid(_f, d):
    """D = 0.5 + 0.5 d.x in the speaker frame (tests/fdtd.rs:485)."""
    return complex(0.5 + 0.5 * d[0], 0.0)


@dataclass
class Scene:
    name: str
    room: BoxRoom
    grid: FdtdGrid
    fits: list
    sources: list          # right-hand sides: lists of (cell, weight) taps
    signal: np.ndarray
    receivers: list
    freqs: np.ndarray
    crossover: float
    weights: list = field(default_factory=list)   # per frequency, per component complex weight
    notes: dict = field(default_factory=dict)

    @property
    def steps(self) -> int:
        return len(self.signal)


def _pillars(rng, n, room_x, room_y, size=0.6, gap=1.0, margin=1.0):
    out = []
    while len(out) < n:
        x = rng.uniform(margin, room_x - margin - size)
        y = rng.uniform(margin, room_y - margin - size)
        if all(abs(x - p[0]) > size + gap or abs(y - p[1]) > size + gap for p in out):
            out.append((x, y, x + size, y + size))
    return out


def _random_points(rng, room, n, margin=0.5):
    pts = []
    while len(pts) < n:
        p = (rng.uniform(room.x0 + margin, room.x1 - margin), rng.uniform(room.y0 + margin, room.y1 - margin),
             rng.uniform(margin, room.height - margin))
        if room.contains(p):
            pts.append(p)
    return pts


def plane_points(room, z, spacing):
    """Inside points of a horizontal cut plane (receivers.rs:108-140)."""
    nu = max(1, math.ceil((room.x1 - room.x0) / spacing))
    nv = max(1, math.ceil((room.y1 - room.y0) / spacing))
    u0 = (room.x0 + room.x1) / 2.0 - (nu - 1.0) / 2.0 * spacing
    v0 = (room.y0 + room.y1) / 2.0 - (nv - 1.0) / 2.0 * spacing
    pts = []
    for iv in range(nv):
        for iu in range(nu):
            p = (u0 + iu * spacing, v0 + iv * spacing, z)
            if room.contains(p):
                pts.append(p)
    return pts


def wave_freqs(crossover):
    s = FdtdSettings(crossover_hz=crossover)
    return np.array([f for f in frequency_grid(20.0, 20000.0, 12) if s.weight(f) > 0.0])


def _materials(rng, n):
    return [Material(id=f"m{i}", absorption=Spectrum.bands(OCTAVES, rng.uniform(0.02, 0.6, len(OCTAVES))))
            for i in range(n)]


def room_small(seed: int = 1) -> Scene:
    rng = np.random.default_rng(seed)
    fc = 250.0
    room = BoxRoom(6.0, 4.0, 3.0)
    mats = [Material(id=f"a{i}", absorption=Spectrum(float(rng.uniform(0.05, 0.4)))) for i in range(6)]
    fits = fit_surfaces(mats, (20.0, fc * math.sqrt(2.0)))
    g = FdtdGrid.build(room, fits, C_AIR, fc, 10.0)
    src = _random_points(rng, room, 1, margin=2 * g.dx + 0.3)[0]
    taps = g.taps_at(src)
    rx = [g.nearest_air(p) for p in _random_points(rng, room, 8)]
    steps = math.ceil(0.5 / g.dt)
    return Scene("room_small", room, g, fits, [taps], source_signal(fc, g.dt, steps), rx, wave_freqs(fc), fc,
                 notes={"seed": seed, "source": src})


def room_pillars(seed: int = 2, duration: float = 1.0, n_materials: int = 5, plane_spacing: float = 0.25,
                 n_mics: int = 64, reference_grid: bool = False) -> Scene:
    """reference_grid: the grid `wavey simulate --fdtd 500` builds by default
    (FdtdSettings::default, fdtd.rs:119-156: 15 points per wavelength at
    grid_fmax = f_c sqrt 2, 2.12 times finer per axis, ~72 M cells) and the
    signal band of run.rs:612, instead of the benchmark configurations'
    ppw-10 rule at f_c; the room, materials, source and receivers are the
    same."""
    rng = np.random.default_rng(seed)
    fc = 500.0
    pillars = _pillars(rng, 4, 20.0, 15.0)
    room = BoxRoom(20.0, 15.0, 8.0, pillars=pillars)
    mats = _materials(rng, n_materials)
    assign = [mats[int(k)] for k in rng.integers(0, n_materials, room.n_surfaces)]
    fits = fit_surfaces(assign, (20.0, fc * math.sqrt(2.0)))
    if reference_grid:
        settings = FdtdSettings(crossover_hz=fc)
        f_grid = settings.grid_fmax(wave_freqs(fc))
        g = FdtdGrid.build(room, fits, C_AIR, f_grid, settings.points_per_wavelength)
    else:
        f_grid = fc
        g = FdtdGrid.build(room, fits, C_AIR, fc, 10.0)
    pos = _random_points(rng, room, 1, margin=2.0)[0]
    yaw, pitch = float(rng.uniform(0, 360)), float(rng.uniform(-30, 30))
    node = g.nearest_air(pos)
    comps = source_components(g, node, 1)
    if comps is None:
        raise RuntimeError("source too close to a surface for a directional source")
    mics = [g.nearest_air(p) for p in _random_points(rng, room, n_mics)]
    plane = [g.nearest_air(p) for p in plane_points(room, 1.2, plane_spacing)]
    freqs = wave_freqs(fc)
    steps = math.ceil(duration / g.dt)
    rot = speaker_rotation(yaw, pitch, 0.0)
    weights = []
    for f in freqs:
        a0, a, _res = fit_first_order(cardioid, rot, f)
        weights.append(component_weights(a0, a, 2.0 * math.pi * f / C_AIR, g.dx))
    return Scene("room_pillars_reference_grid" if reference_grid else "room_pillars", room, g, fits, comps,
                 source_signal(f_grid, g.dt, steps), mics + plane, freqs, fc, weights=weights,
                 notes={"seed": seed, "pillars": pillars, "source": pos, "yaw": yaw, "pitch": pitch,
                        "mics": len(mics), "plane_points": len(plane), "grid_fmax": f_grid,
                        "ppw": 15.0 if reference_grid else 10.0})


def room_pillars_shard(rank: int, world: int, seed: int = 7) -> Scene:
    """room_pillars split by source over `world` GPUs: one cardioid speaker
    (four right-hand sides) per rank, on the same grid.  Speaker 0 is
    room_pillars' own source, so one rank runs exactly room_pillars; speakers
    1..world-1 are seeded cardioids at seeded yaw and pitch.  No rank needs
    another's data: the only exchange is gathering the spectra afterwards."""
    if not 0 <= rank < world:
        raise ValueError("rank outside the world")
    base = room_pillars(seed=2)
    if rank == 0:
        base.notes = dict(base.notes, shard=f"speaker 0 of {world}")
        return base
    rng = np.random.default_rng([seed, rank])
    g = base.grid
    while True:
        pos = _random_points(rng, base.room, 1, margin=2.0)[0]
        comps = source_components(g, g.nearest_air(pos), 1)
        if comps is not None:
            break
    yaw, pitch = float(rng.uniform(0, 360)), float(rng.uniform(-30, 30))
    rot = speaker_rotation(yaw, pitch, 0.0)
    weights = []
    for f in base.freqs:
        a0, a, _res = fit_first_order(cardioid, rot, f)
        weights.append(component_weights(a0, a, 2.0 * math.pi * f / C_AIR, g.dx))
    base.sources = comps
    base.weights = weights
    base.notes = dict(base.notes, source=pos, yaw=yaw, pitch=pitch, shard=f"speaker {rank} of {world}")
    return base


def room_pillars_speakers(n_speakers: int, seed: int = 4, duration: float = 1.0) -> Scene:
    """room_pillars' room and materials with n seeded speakers; each speaker
    is a monopole or a cardioid (4 right-hand sides) at a seeded yaw and
    pitch.  notes["speaker_rhs"] holds each speaker's (first right-hand side,
    count) and notes["speaker_weights"] its per-frequency component weights
    ([nf][count]; 1 for a monopole), which combine its right-hand sides into
    the speaker's transfer function as the reference's wave stage does
    (run.rs:626-660)."""
    base = room_pillars(seed=2, duration=duration)
    rng = np.random.default_rng(seed)
    g = base.grid
    sources, kinds, rhs, weights = [], [], [], []
    for _ in range(n_speakers):
        pos = _random_points(rng, base.room, 1, margin=1.5)[0]
        node = g.nearest_air(pos)
        first = len(sources)
        if rng.uniform() < 0.5:
            sources.append(g.taps_at(pos))
            kinds.append("monopole")
            weights.append([[1.0 + 0.0j] for _f in base.freqs])
        else:
            sources.extend(source_components(g, node, 1))
            kinds.append("cardioid")
            rot = speaker_rotation(float(rng.uniform(0, 360)), float(rng.uniform(-30, 30)), 0.0)
            w = []
            for f in base.freqs:
                a0, a, _res = fit_first_order(cardioid, rot, f)
                w.append(component_weights(a0, a, 2.0 * math.pi * f / C_AIR, g.dx))
            weights.append(w)
        rhs.append((first, len(sources) - first))
    base.name = f"room_pillars_{n_speakers}spk"
    base.sources = sources
    base.weights = []
    base.notes = dict(base.notes, speakers=kinds, speaker_rhs=rhs, speaker_weights=weights)
    return base


def octave_levels(transfer: np.ndarray, freqs: np.ndarray, centres) -> np.ndarray:
    """10 log10 of the mean |H|^2 over the bins of each octave band
    (band_edges(f, 1), freq.rs:32-35); transfer [..., nf]."""
    out = []
    for fc in centres:
        lo, hi = fc / 2 ** 0.5, fc * 2 ** 0.5
        sel = (freqs >= lo) & (freqs < hi)
        out.append(10.0 * np.log10(np.mean(np.abs(transfer[..., sel]) ** 2, axis=-1)))
    return np.stack(out, axis=-1)


def rooms_batch(seed: int = 3, speakers: int = 32, extra_rooms: int = 4):
    """The multi-room batch: a list of Scenes sharing one launch per step."""
    rng = np.random.default_rng(seed)
    fc = 250.0
    first = room_small(seed=1)
    g = first.grid
    sources, kinds = [], []
    for _ in range(speakers):
        pos = _random_points(rng, first.room, 1, margin=2 * g.dx + 0.2)[0]
        if rng.uniform() < 0.5:
            sources.append(g.taps_at(pos))
            kinds.append("monopole")
        else:
            comps = source_components(g, g.nearest_air(pos), 1)
            if comps is None:
                sources.append(g.taps_at(pos))
                kinds.append("monopole")
            else:
                sources.extend(comps)
                kinds.append("cardioid")
    first.sources = sources
    first.name = f"room_small_{speakers}spk"
    first.notes = dict(first.notes, speakers=kinds)
    scenes = [first]
    for r in range(extra_rooms):
        dims = (float(rng.uniform(5, 25)), float(rng.uniform(4, 20)), float(rng.uniform(3, 10)))
        room = BoxRoom(*dims)
        mats = [Material(id=f"r{r}a{i}", absorption=Spectrum(float(rng.uniform(0.05, 0.4)))) for i in range(6)]
        fits = fit_surfaces(mats, (20.0, fc * math.sqrt(2.0)))
        gr = FdtdGrid.build(room, fits, C_AIR, fc, 10.0)
        src = _random_points(rng, room, 1, margin=1.0)[0]
        rx = [gr.nearest_air(p) for p in _random_points(rng, room, 8)]
        steps = math.ceil(0.5 / gr.dt)
        scenes.append(Scene(f"shoebox_{r}", room, gr, fits, [gr.taps_at(src)], source_signal(fc, gr.dt, steps), rx,
                            wave_freqs(fc), fc, notes={"dims": dims}))
    return scenes


def plane_points_axis(room, axis: str, offset: float, spacing: float):
    """Inside points of a vertical cut plane (receivers.rs:118-140): axis "x"
    is x = offset (u = y, v = z), axis "y" is y = offset (u = x, v = z)."""
    if axis == "x":
        ulo, uhi = room.y0, room.y1
    else:
        ulo, uhi = room.x0, room.x1
    vlo, vhi = 0.0, room.height
    nu = max(1, math.ceil((uhi - ulo) / spacing))
    nv = max(1, math.ceil((vhi - vlo) / spacing))
    u0 = (ulo + uhi) / 2.0 - (nu - 1.0) / 2.0 * spacing
    v0 = (vlo + vhi) / 2.0 - (nv - 1.0) / 2.0 * spacing
    pts = []
    for iv in range(nv):
        for iu in range(nu):
            u, v = u0 + iu * spacing, v0 + iv * spacing
            p = (offset, u, v) if axis == "x" else (u, offset, v)
            if room.contains(p):
                pts.append(p)
    return pts


def room_hall(seed: int = 5, speakers: int = 16, duration: float = 2.0, crossover: float = 1000.0,
              n_mics: int = 256, plane_spacing: float = 0.25) -> Scene:
    """40 x 25 x 15 m hall with 12 pillars and a stepped balcony (three
    absorbing steps along the back wall), eight fitted materials, directional
    speakers (monopole + 3 dipoles each), 256 mics and three cut planes."""
    rng = np.random.default_rng(seed)
    fc = crossover
    pillars = _pillars(rng, 12, 40.0, 25.0, gap=2.0, margin=2.0)
    z0 = float(rng.uniform(5.0, 6.0))
    blocks = [(1.0, 19.0, z0, 39.0, 25.0, z0 + 0.4), (1.0, 21.0, z0 + 0.4, 39.0, 25.0, z0 + 0.8),
              (1.0, 23.0, z0 + 0.8, 39.0, 25.0, z0 + 1.2)]
    room = BoxRoom(40.0, 25.0, 15.0, pillars=pillars, blocks=blocks)
    mats = _materials(rng, 8)
    assign = [mats[int(k)] for k in rng.integers(0, 8, room.n_surfaces)]
    fits = fit_surfaces(assign, (20.0, fc * math.sqrt(2.0)))
    g = FdtdGrid.build(room, fits, C_AIR, fc, 10.0)
    sources = []
    for _ in range(speakers):
        for _try in range(100):
            pos = _random_points(rng, room, 1, margin=2.0)[0]
            comps = source_components(g, g.nearest_air(pos), 1)
            if comps is not None:
                sources.extend(comps)
                break
    mics = [g.nearest_air(p) for p in _random_points(rng, room, n_mics)]
    planes = (plane_points(room, 1.2, plane_spacing) + plane_points(room, z0 + 1.2 + 1.2, plane_spacing)
              + plane_points_axis(room, "y", 12.5, plane_spacing))
    rx = mics + [g.nearest_air(p) for p in planes]
    steps = math.ceil(duration / g.dt)
    return Scene("room_hall", room, g, fits, sources, source_signal(fc, g.dt, steps), rx, wave_freqs(fc), fc,
                 notes={"seed": seed, "pillars": len(pillars), "balcony_z": z0, "speakers": speakers,
                        "mics": len(mics), "plane_points": len(planes)})
