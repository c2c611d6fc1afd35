"""Absorption spectra and boundary admittance fits (wavey-materials).

Python face of libwavey_host.so's material functions:
  Spectrum          wavey-materials/src/spectrum.rs:7-44
  Material          wavey-materials/src/material.rs:6-77 (absorption only)
  AdmittanceFit     wavey-materials/src/impedance_fit.rs:34-70
  fit_admittance    wavey-materials/src/impedance_fit.rs:158-235
  fit_surfaces      wavey-solver/src/fdtd.rs:213-222
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native as N


@dataclass(frozen=True)
class Spectrum:
    """A scalar, or a table interpolated over log-frequency and held outside."""

    value: float = 0.0
    freqs_hz: tuple = ()
    values: tuple = ()

    @staticmethod
    def bands(freqs_hz, values) -> "Spectrum":
        if len(freqs_hz) != len(values):
            raise ValueError("band table needs matching frequency and value lists")
        return Spectrum(0.0, tuple(float(f) for f in freqs_hz), tuple(float(v) for v in values))

    def _c(self):
        if not self.freqs_hz:
            return N.WhSpectrum(0, float(self.value), None, None), ()
        f = np.ascontiguousarray(self.freqs_hz, dtype=np.float64)
        v = np.ascontiguousarray(self.values, dtype=np.float64)
        return N.WhSpectrum(len(f), 0.0, N.ptr(f, C.c_double), N.ptr(v, C.c_double)), (f, v)

    def eval(self, f: float) -> float:
        s, keep = self._c()
        return N.host().wh_spectrum_eval(C.byref(s), float(f))


@dataclass(frozen=True)
class Material:
    id: str
    absorption: Spectrum
    name: str = ""

    def absorption_at(self, f: float) -> float:
        return min(max(self.absorption.eval(f), 0.0), 1.0)


@dataclass(frozen=True)
class Branch:
    r: float
    m: float
    k: float


@dataclass(frozen=True)
class AdmittanceFit:
    beta0: float
    branches: tuple = ()
    band: tuple = (0.0, 0.0)
    rms_error: float = 0.0
    max_error: float = 0.0

    def _c(self) -> N.WhFit:
        f = N.WhFit()
        f.beta0 = self.beta0
        f.n_branches = len(self.branches)
        for i, b in enumerate(self.branches):
            f.r[i], f.m[i], f.k[i] = b.r, b.m, b.k
        f.band_lo, f.band_hi = self.band
        f.rms_error, f.max_error = self.rms_error, self.max_error
        return f

    @staticmethod
    def _from_c(f: N.WhFit) -> "AdmittanceFit":
        br = tuple(Branch(f.r[i], f.m[i], f.k[i]) for i in range(f.n_branches))
        return AdmittanceFit(f.beta0, br, (f.band_lo, f.band_hi), f.rms_error, f.max_error)

    def admittance(self, f: float) -> complex:
        out = (C.c_double * 2)()
        c = self._c()
        N.host().wh_fit_admittance_at(C.byref(c), float(f), out)
        return complex(out[0], out[1])

    def impedance(self, f: float) -> complex:
        y = self.admittance(f)
        return complex(1e9, 0.0) if abs(y) < 1e-9 else 1.0 / y

    def absorption(self, f: float) -> float:
        c = self._c()
        return N.host().wh_fit_absorption(C.byref(c), float(f))

    def is_rigid(self) -> bool:
        return self.beta0 < 1e-12 and not self.branches


def fit_real_impedance(alpha: float) -> float:
    return N.host().wh_fit_real_impedance(float(alpha))


def fit_admittance(material: Material, band: tuple, max_branches: int = 2) -> AdmittanceFit:
    s, keep = material.absorption._c()
    out = N.WhFit()
    st = N.host().wh_fit_admittance(C.byref(s), float(band[0]), float(band[1]), int(max_branches), C.byref(out))
    if st != 0:
        raise ValueError(f"fit_admittance failed ({st})")
    return AdmittanceFit._from_c(out)


def fit_surfaces(materials: list, band: tuple) -> list:
    """One fit per surface; a material id is fitted once (fdtd.rs:213-222)."""
    cache: dict = {}
    out = []
    for m in materials:
        if m.id not in cache:
            cache[m.id] = fit_admittance(m, band, 2)
        out.append(cache[m.id])
    return out


def scalar_material(alpha: float) -> Material:
    """A frequency-independent absorber, as the reference's test fixture
    `material(alpha)` (wavey-solver/tests/common/mod.rs:13-25)."""
    return Material(id=f"a{alpha!r}", absorption=Spectrum(float(alpha)), name="test")
