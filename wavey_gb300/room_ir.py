"""The wave solver alone on a room: impulse responses of every source-
microphone pair from the FDTD grid, analysed like measured room impulse
responses (ISO 3382-1) in the octave bands the grid resolves.  This is the
reference's bras_wave example (core/wavey-cli/examples/bras_wave.rs:15-60)
on the CUDA backend, step by step:

  fits     fit_surfaces(surface materials, (20, f_max))        bras_wave.rs:24
  grid     FdtdGrid.build(room, fits, c, f_max, ppw 10)         bras_wave.rs:26
  steps    ceil(duration / dt)                                  bras_wave.rs:27
  signal   source_signal(2 f_max, dt, steps): a wider pulse band than the
           grid's, so the analysed bands see a flat source       bras_wave.rs:35
  sources  one node each, nearest_air(acoustic centre), weight 1  bras_wave.rs:43
  series   run_cpu_ir per source; here every source is one right-hand side
           of a single IR plan                                  bras_wave.rs:45
  analysis running sum of each series (the response to the pulse's
           integral), onset, octave_filter, band_params with Lundeby's
           truncation -- on the device (wavey_cuda_plan_band_params)
                                                                bras_wave.rs:46-58
  bands    OCTAVES[b] * sqrt(2) <= 0.75 f_max                   bras_wave.rs:18
  means    per band over all pairs, finite values only          bras_wave.rs:88-91
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .backend import FP32
from .fdtd import FdtdGrid, source_signal
from .materials import fit_surfaces

# analysis.rs: OCTAVES
OCTAVES = (63.0, 125.0, 250.0, 500.0, 1000.0, 2000.0, 4000.0, 8000.0)


def speed_of_sound(temperature_c: float = 20.0) -> float:
    """Medium::speed_of_sound (wavey-materials/src/medium.rs:22-24)."""
    return 331.3 * math.sqrt(1.0 + temperature_c / 273.15)


# Speed of sound of Medium::default() (20 C).
C_DEFAULT = speed_of_sound(20.0)
# Columns of wavey_cuda_plan_band_params' output.
EDT, T20, T30, C80, D50, TS = range(6)


def analysed_bands(f_max: float) -> list:
    """bras_wave.rs:18: the octaves whose upper edge lies below 0.75 f_max."""
    return [b for b in OCTAVES if b * math.sqrt(2.0) <= f_max * 0.75]


@dataclass
class RoomRun:
    grid: FdtdGrid
    steps: int
    signal: np.ndarray
    sources: list        # one node per source
    receivers: list      # one node per microphone
    bands: list
    fits: list


def prepare(spec, f_max: float = 700.0, duration: float = 2.5, c: float = C_DEFAULT, ppw: float = 10.0) -> RoomRun:
    """Grid, signal and nodes of a RoomSpec (wavey_gb300.mesh) as bras_wave
    builds them."""
    fits = fit_surfaces(spec.surface_materials, (20.0, f_max))
    g = FdtdGrid.build(spec.room, fits, c, f_max, ppw)
    steps = math.ceil(duration / g.dt)
    signal = source_signal(2.0 * f_max, g.dt, steps)
    src = []
    for name, p in spec.speakers:
        node = g.nearest_air(p)
        if node is None:
            raise ValueError(f"source {name} outside grid")
        src.append(node)
    rx = []
    for name, p in spec.mics:
        node = g.nearest_air(p)
        if node is None:
            raise ValueError(f"mic {name} outside grid")
        rx.append(node)
    return RoomRun(g, steps, signal, src, rx, analysed_bands(f_max), fits)


def pair_parameters(backend, run: RoomRun, precision=FP32) -> np.ndarray:
    """[source][mic][band][6] = EDT, T20, T30 (s), C80 (dB), D50, Ts (s) of
    every pair, from one IR plan on the device."""
    plan = backend.plan(run.grid, [[(s, 1.0)] for s in run.sources], run.signal, run.receivers, [],
                        precision=precision, ir=True)
    try:
        plan.run()
        return plan.band_params(bands=run.bands, integrate=True, lundeby=True)
    finally:
        plan.close()


def band_means(pairs: np.ndarray) -> dict:
    """Per band means over all pairs of T20, EDT, D50 and C80, skipping
    undefined values (bras_wave.rs:88-91)."""
    flat = pairs.reshape(-1, pairs.shape[-2], pairs.shape[-1])

    def mean(k):
        out = []
        for b in range(flat.shape[1]):
            x = flat[:, b, k]
            x = x[np.isfinite(x)]
            out.append(float(x.sum() / max(len(x), 1)))
        return out

    return {"T20": mean(T20), "EDT": mean(EDT), "D50": mean(D50), "C80": mean(C80)}
