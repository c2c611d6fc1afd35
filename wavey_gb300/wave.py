"""The wave stage of a solve as batched launches.

The reference's wave stage (core/wavey-solver/src/run.rs:519-662) runs the
FDTD solver once per speaker *and* per source component (run.rs:649: a
directional speaker is a monopole plus three dipoles), and each cabinet's
calibration as two more runs (fdtd.rs:941-942) -- every one a separate GPU
job over the same grid.  Here:

  * every component of every speaker is one right-hand side of ONE batched
    run over the room's grid (one launch per time step for all of them), and
  * every cabinet calibration pair ("with" and "bare" grids) is one room of
    ONE multi-room run,

and the per-speaker combination is the reference's (run.rs:596-660):
source node and driver point, component taps, first-order directivity fit,
to_transfer, calibration, weighted sum.  The GPU does the time stepping; the
host keeps the per-frequency algebra, which is small.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .backend import FP32, RoomJob
from .fdtd import (BoxRoom, FdtdGrid, component_weights, fit_first_order, source_components, source_signal,
                   to_transfer)
from .materials import AdmittanceFit


@dataclass(frozen=True)
class Cabinet:
    """A speaker cabinet as a rigid box: its size along the local axes (x on
    axis) and its acoustic centre relative to the box centre.  The reference
    takes the cabinet mesh (verts/tris); a box is the mesh this restatement
    supports."""
    size: tuple
    acoustic_center: tuple = (0.0, 0.0, 0.0)

    def corners(self) -> np.ndarray:
        h = 0.5 * np.asarray(self.size, dtype=np.float64)
        return np.array([[sx * h[0], sy * h[1], sz * h[2]] for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)])


@dataclass
class CabinetCalibration:
    """fdtd.rs:874-882: on-axis gain of cabinet + driver relative to the bare
    monopole per frequency, horizontal angles, and directivity re on-axis
    [angle][freq]."""
    on_axis: np.ndarray
    angles_deg: np.ndarray
    directivity: np.ndarray


@dataclass
class Speaker:
    """One source of a solve.
    position:  acoustic centre in room coordinates
    rotation:  local-to-room 3x3 matrix (speaker_rotation); +x local is the axis
    h0:        on-axis free-field response, callable f -> complex or an array over freqs
    directivity: callable (f, local_direction) -> complex (the balloon), or None (omnidirectional)
    reference_distance: the response's reference distance in m
    cabinet:   a Cabinet whose grid cells the room grid already holds as a rigid solid, or None
    """
    name: str
    position: tuple
    rotation: np.ndarray = field(default_factory=lambda: np.eye(3))
    h0: object = 1.0
    directivity: object = None
    reference_distance: float = 1.0
    cabinet: Cabinet | None = None

    @property
    def axis(self) -> np.ndarray:
        return np.asarray(self.rotation, dtype=np.float64) @ np.array([1.0, 0.0, 0.0])


class WaveStageError(ValueError):
    pass


def _h0(sp: Speaker, freqs) -> np.ndarray:
    if callable(sp.h0):
        return np.array([complex(sp.h0(float(f))) for f in freqs], dtype=np.complex128)
    return np.broadcast_to(np.asarray(sp.h0, dtype=np.complex128), (len(freqs),)).copy()


# ------------------------------------------------------------------ calibration
def _calibration_setup(cab: Cabinet, c: float, f_max: float, ppw: float, cells_across: float):
    """Grids, taps, receivers and signal of one calibration pair
    (fdtd.rs:898-940)."""
    ac = np.asarray(cab.acoustic_center, dtype=np.float64)
    verts = cab.corners()
    reach = max(0.1, float(np.max(np.linalg.norm(verts - ac, axis=1))))
    # The cabinet matters from about ka = 0.5: the absorbing box spans half a
    # wavelength there (capped by cell count) so its walls do not dominate.
    f_cab = 0.5 * c / (2.0 * math.pi * reach)
    lo, hi = verts.min(axis=0), verts.max(axis=0)
    dx = min(c / (f_max * ppw), float((hi - lo).min()) / cells_across)
    max_half = 0.5 * dx * 160.0  # at most 160^3 cells
    r_m = max(reach + 1.0, 3.0)  # far enough that the detour behind the box costs no level
    half = max(min(0.5 * c / f_cab, max_half), r_m + 1.5)
    side = 2.0 * half
    absorber = AdmittanceFit(1.0, (), (1.0, f_max))  # matched (rho c) walls
    p0 = np.array([half, half, half])
    shift = p0 - ac  # the box centre, so that the acoustic centre is at p0
    solid = tuple(float(v) for v in np.concatenate([lo + shift, hi + shift]))
    room_with = BoxRoom(side, side, side, solids=[solid])
    room_bare = BoxRoom(side, side, side)
    fits = [absorber] * room_bare.n_surfaces
    g_with = FdtdGrid.build_dx(room_with, fits, c, dx)
    g_bare = FdtdGrid.build_dx(room_bare, fits, c, dx)
    src = g_with.baffle_point(p0, (1.0, 0.0, 0.0))
    taps_with, taps_bare = g_with.taps_at(src), g_bare.taps_at(src)
    if taps_with is None or taps_bare is None:
        raise WaveStageError("calibration source is not in air")
    angles = np.arange(12) * 30.0
    pts = [p0 + np.array([math.cos(math.radians(a)), math.sin(math.radians(a)), 0.0]) * r_m for a in angles]
    rx_with = [g_with.nearest_air(p) for p in pts]
    rx_bare = [g_bare.nearest_air(p) for p in pts]
    if any(r is None for r in rx_with + rx_bare):
        raise WaveStageError("calibration receiver is not in air")
    duration = side * math.sqrt(3.0) * 2.0 / c + 12.0 * 0.342 / f_max
    steps = math.ceil(duration / g_with.dt)
    signal = source_signal(f_max, g_with.dt, steps)
    return dict(f_cab=f_cab, angles=angles, grids=(g_with, g_bare), taps=(taps_with, taps_bare),
                rx=(rx_with, rx_bare), signal=signal)


def _calibration_from(s_with: np.ndarray, s_bare: np.ndarray, freqs, f_cab: float, angles) -> CabinetCalibration:
    """fdtd.rs:944-954: the with/bare ratio, faded towards 1 as (f / f_cab)^2
    below f_cab, where the box is too small to measure its effect."""
    fr = np.asarray(freqs, dtype=np.float64)
    w = np.minimum((fr / f_cab) ** 2, 1.0)
    m = s_with / s_bare  # [angle][freq]
    ratio = np.abs(m) ** w * np.exp(1j * np.angle(m) * w)
    on_axis = ratio[0].copy()
    return CabinetCalibration(on_axis, np.asarray(angles, dtype=np.float64), ratio / on_axis[None, :])


def calibrate_cabinets(backend, cabinets, c: float, f_max: float, ppw: float, cells_across: float, freqs,
                       precision=FP32, cancel=None, progress=None):
    """Calibrates every cabinet (fdtd.rs:890-955) in ONE multi-room run: two
    rooms per cabinet, with and without it.  Returns a CabinetCalibration per
    cabinet, or None if cancelled."""
    setups = [_calibration_setup(cab, c, f_max, ppw, cells_across) for cab in cabinets]
    if not setups:
        return []
    jobs = []
    for s in setups:
        for k in range(2):
            jobs.append(RoomJob(s["grids"][k], [s["taps"][k]], s["signal"], s["rx"][k], freqs))
    out = backend.run_rooms(jobs, precision=precision, cancel=cancel, progress=progress)
    if out is None:
        return None
    cals = []
    for i, s in enumerate(setups):
        s_with, s_bare = out[2 * i][0], out[2 * i + 1][0]  # [rx][nf] of the one right-hand side
        cals.append(_calibration_from(s_with, s_bare, freqs, s["f_cab"], s["angles"]))
    return cals


# ------------------------------------------------------------------ wave stage
@dataclass
class SpeakerPlan:
    """How one speaker enters the batched run: its component taps, per-frequency
    component weights [nf][n_components], and notes."""
    components: list
    weights: np.ndarray
    notes: list


def plan_speaker(grid: FdtdGrid, sp: Speaker, freqs, c: float, source_order: int,
                 calibrated: bool) -> SpeakerPlan:
    """run.rs:596-630 for one speaker: source node, driver point, components
    and their weights."""
    notes = []
    center = np.asarray(sp.position, dtype=np.float64)
    axis = sp.axis
    # With a cabinet the driver radiates from the baffle in front of the
    # acoustic centre; a centre deep inside the cabinet also falls back to it.
    node = grid.air_along(center, axis) if calibrated else None
    if node is None:
        node = grid.nearest_air(center)
    if node is None:
        node = grid.air_along(center, axis)
    if node is None:
        raise WaveStageError(f"speaker `{sp.name}` is not inside the wave-solver grid")
    driver = grid.baffle_point(center, axis) if calibrated else center
    order = min(source_order, 1) if (sp.directivity is not None and not calibrated) else 0
    if calibrated or order == 0:
        comps = [grid.taps_at(driver) or [(node, 1.0)]]
    else:
        comps = source_components(grid, node, order)
        if comps is None:
            notes.append(f"wave solver: `{sp.name}` is too close to a surface for a directional source; "
                         "used omnidirectional")
            comps = [[(node, 1.0)]]
    nf = len(freqs)
    if len(comps) == 1:
        weights = np.ones((nf, 1), dtype=np.complex128)
    else:
        weights = np.empty((nf, len(comps)), dtype=np.complex128)
        worst = 0.0
        for k, f in enumerate(freqs):
            a0, a, res = fit_first_order(sp.directivity, sp.rotation, float(f))
            worst = max(worst, res)
            weights[k] = component_weights(a0, a, 2.0 * math.pi * float(f) / c, grid.dx)
        notes.append(f"wave solver: `{sp.name}` directivity fitted to first order "
                     f"(worst residual {worst * 100:.0f} % of the balloon)")
    return SpeakerPlan(comps, weights, notes)


@dataclass
class WaveStageResult:
    transfers: list          # per speaker: complex [n_receivers][nf]
    notes: list
    right_hand_sides: int    # components over all speakers, all in one run
    signal: np.ndarray


def wave_stage(backend, grid: FdtdGrid, speakers, receivers, freqs, c: float, grid_fmax: float, steps: int,
               source_order: int = 1, calibrations: dict | None = None, precision=FP32, cancel=None,
               progress=None):
    """All speakers of a solve through ONE batched run (run.rs:593-662).

    receivers:    air-node indices (nearest_air of the receiver points)
    calibrations: {speaker name: CabinetCalibration} for speakers with cabinets
    Returns a WaveStageResult, or None if cancelled.
    """
    calibrations = calibrations or {}
    freqs = np.asarray(freqs, dtype=np.float64)
    signal = source_signal(grid_fmax, grid.dt, steps)
    plans = [plan_speaker(grid, sp, freqs, c, source_order, sp.name in calibrations) for sp in speakers]
    sources = [t for p in plans for t in p.components]
    if not sources:
        return WaveStageResult([], [], 0, signal)
    spectra = backend.run_batch(grid, sources, signal, receivers, freqs, precision=precision, cancel=cancel,
                                progress=progress)
    if spectra is None:
        return None
    transfers, notes, lane = [], [], 0
    for sp, p in zip(speakers, plans):
        h0 = _h0(sp, freqs)
        cal = calibrations.get(sp.name)
        t = np.zeros((len(receivers), len(freqs)), dtype=np.complex128)
        for ci in range(len(p.components)):
            tc = to_transfer(spectra[lane], signal, grid, freqs, c, sp.reference_distance, h0)
            if cal is not None:
                tc = tc / cal.on_axis[None, :]
            t += p.weights[None, :, ci] * tc
            lane += 1
        transfers.append(t)
        notes.extend(p.notes)
    return WaveStageResult(transfers, notes, len(sources), signal)


# ------------------------------------------------------------------ results.bin
def transfer_factors(grid: FdtdGrid, speakers, plans, freqs, c: float, signal, calibrations=None):
    """Per right-hand side (in the batched run's order): its speaker and the
    complex factor per frequency that maps its spectrum to its share of the
    speaker's transfer -- component weight x to_transfer's scale
    (fdtd.rs:819-840, evaluated on a unit spectrum) / cabinet calibration."""
    calibrations = calibrations or {}
    freqs = np.asarray(freqs, dtype=np.float64)
    lane_speaker, factors = [], []
    for s, (sp, p) in enumerate(zip(speakers, plans)):
        unit = to_transfer(np.ones((1, len(freqs)), dtype=np.complex128), signal, grid, freqs, c,
                           sp.reference_distance, _h0(sp, freqs))[0]
        cal = calibrations.get(sp.name)
        if cal is not None:
            unit = unit / cal.on_axis
        for ci in range(len(p.components)):
            lane_speaker.append(s)
            factors.append(p.weights[:, ci] * unit)
    return np.array(lane_speaker, dtype=np.int32), np.array(factors, dtype=np.complex128)


def layout_transfers(transfers, n_mics: int, plane_points) -> np.ndarray:
    """Host-side form of the results.bin transfer section (result.rs:444-456)
    from per-speaker transfers [speaker][receiver][f]: mics [mic][speaker][f],
    then per plane [speaker][point][f], flattened complex64."""
    t = np.asarray(transfers)
    parts = [np.transpose(t[:, :n_mics, :], (1, 0, 2)).reshape(-1)]
    r0 = n_mics
    for pts in plane_points:
        parts.append(t[:, r0:r0 + pts, :].reshape(-1))
        r0 += pts
    return np.concatenate(parts).astype(np.complex64)


def wave_stage_results(backend, grid: FdtdGrid, speakers, receivers, n_mics: int, plane_points, freqs, c: float,
                       grid_fmax: float, steps: int, source_order: int = 1, calibrations: dict | None = None,
                       precision=FP32, cancel=None, progress=None, autotune: bool = False):
    """The wave stage straight to the results.bin transfer section: the
    batched run stays on the device as a plan, the per-speaker combination
    runs on the device (wavey_cuda_plan_transfers) and only the complex64
    result is read back.  receivers: the mics' nodes then every plane's
    inside points' nodes, in plane order.  Returns the flattened section (see
    layout_transfers), or None if cancelled."""
    calibrations = calibrations or {}
    freqs = np.asarray(freqs, dtype=np.float64)
    signal = source_signal(grid_fmax, grid.dt, steps)
    plans = [plan_speaker(grid, sp, freqs, c, source_order, sp.name in calibrations) for sp in speakers]
    sources = [t for p in plans for t in p.components]
    lane_speaker, factors = transfer_factors(grid, speakers, plans, freqs, c, signal, calibrations)
    plan = backend.plan(grid, sources, signal, receivers, freqs, precision)
    try:
        if autotune:
            plan.autotune()
        if plan.run(cancel=cancel, progress=progress) is None:
            return None
        return plan.transfers(lane_speaker, factors, n_mics, plane_points)
    finally:
        plan.close()


def write_transfer_section(path, section: np.ndarray) -> None:
    """Writes the transfer section as results.bin stores it: interleaved
    little-endian f32 (re, im) pairs."""
    np.ascontiguousarray(section, dtype=np.complex64).astype("<c8").tofile(path)
