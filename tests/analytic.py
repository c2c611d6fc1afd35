"""The reference's analytic known-answer tests for the FDTD path
(core/wavey-solver/tests/fdtd.rs), written once against a runner

    run(grid, taps, signal, receivers, freqs) -> spectra [n_recv, nf]

so that they pin the oracle (tests/test_oracle_pins.py) and check the CUDA
path (tests/test_gpu_analytic.py) with the same thresholds.
"""
from __future__ import annotations

import math

import numpy as np

from conftest import C_AIR
from wavey_gb300.fdtd import (COURANT, BoxRoom, FdtdGrid, FdtdSettings, component_weights, fit_first_order,
                              source_components, source_signal, speaker_rotation, to_transfer)
from wavey_gb300.materials import fit_surfaces, scalar_material

c = C_AIR


def direct_sound_is_calibrated(run):
    """fdtd.rs:13-47: free-field level within 0.1 dB of 1/r and phase lag
    within 0.3 deg of the scheme's axial dispersion."""
    room = BoxRoom(12.0, 10.0, 8.0)
    f_max = 600.0
    g = FdtdGrid.build(room, fit_surfaces([scalar_material(0.2)] * 6, (20.0, f_max)), c, f_max, 10.0)
    src = g.nearest_air((6.0, 5.0, 4.0))
    rcv = g.nearest_air((7.5, 5.0, 4.0))
    r = float(np.linalg.norm(g.pos(rcv) - g.pos(src)))
    steps = int(0.016 / g.dt)
    sig = source_signal(f_max, g.dt, steps)
    freqs = np.array([150.0, 250.0, 350.0, 450.0])
    spec = run(g, [(src, 1.0)], sig, [rcv], freqs)
    t = to_transfer(spec, sig, g, freqs, c, 1.0, np.ones(4))
    out = []
    for fi, f in enumerate(freqs):
        k = 2 * math.pi * f / c
        want = np.exp(-1j * k * r) / r
        db = 20 * math.log10(abs(t[0, fi]) / abs(want))
        deg = math.degrees(np.angle(t[0, fi] / want))
        predicted = -FdtdSettings.phase_error_deg_per_m(f, c, g.dx) * r
        assert abs(db) < 0.1, f"{f} Hz: {db} dB"
        assert abs(deg - predicted) < 0.3, f"{f} Hz: {deg} deg vs {predicted} deg"
        out.append((f, db, deg, predicted))
    return out


def _peak_modes(freqs, mag, modes, sep=0.03, window=0.015):
    """Strongest response within +-window of each mode with no other mode
    within sep (fdtd.rs:77-88, 127-143)."""
    res = []
    for m in modes:
        if any(abs(o / m - 1) > 1e-9 and abs(o / m - 1) < sep for o in modes):
            continue
        sel = np.flatnonzero(np.abs(freqs / m - 1) < window)
        k = sel[np.argmax(mag[sel])]
        res.append((m, freqs[k], freqs[k] / m - 1))
    return res


def rigid_box_eigenfrequencies(run):
    """fdtd.rs:49-90: modes 45-115 Hz of a rigid 3 x 2.5 x 2 m box within 0.5 %."""
    lx, ly, lz = 3.0, 2.5, 2.0
    room = BoxRoom(lx, ly, lz)
    f_max = c
    g = FdtdGrid.build(room, fit_surfaces([scalar_material(0.0)] * 6, (20.0, f_max)), c, f_max, 10.0)
    assert abs(g.dx - 0.1) < 1e-12
    src = g.nearest_air((0.05, 0.05, 0.05))
    rcv = g.nearest_air((lx - 0.05, ly - 0.05, lz - 0.05))
    steps = int(2.0 / g.dt)
    sig = source_signal(400.0, g.dt, steps)
    freqs = 40.0 + np.arange(1000) * 0.08
    mag = np.abs(run(g, [(src, 1.0)], sig, [rcv], freqs)[0])
    modes = [c / 2 * math.sqrt((a / lx) ** 2 + (b / ly) ** 2 + (d / lz) ** 2)
             for a in range(4) for b in range(4) for d in range(4)]
    modes = [m for m in modes if 45.0 < m < 115.0]
    found = _peak_modes(freqs, mag, modes)
    assert len(found) >= 4
    for m, f, e in found:
        assert abs(e) < 0.005, f"mode {m:.2f} Hz -> {f:.2f} Hz"
    return found


def rigid_cube_modes_to_800_hz(run):
    """fdtd.rs:92-145: 1 m rigid cube on 15 points per wavelength at 800 Hz,
    every isolated analytic mode 100-800 Hz within 0.6 %."""
    room = BoxRoom(1.0, 1.0, 1.0)
    n = math.ceil(1.0 / (c / (800.0 * 15.0)))
    f_max = c * n / 15.0
    g = FdtdGrid.build(room, fit_surfaces([scalar_material(0.0)] * 6, (20.0, f_max)), c, f_max, 15.0)
    src = g.nearest_air((0.2, 0.2, 0.2))
    rcv = g.nearest_air((0.9, 0.9, 0.9))
    steps = int(4.0 / g.dt)
    sig = source_signal(1600.0, g.dt, steps)
    freqs = 90.0 + np.arange(7400) * 0.1
    mag = np.abs(run(g, [(src, 1.0)], sig, [rcv], freqs)[0])
    modes = []
    for a in range(6):
        for b in range(a + 1):
            for d in range(b + 1):
                m = c / 2 * math.sqrt(a * a + b * b + d * d)
                if 100.0 <= m <= 800.0:
                    modes.append(m)
    found = _peak_modes(freqs, mag, modes)
    assert len(found) >= 5
    worst = max(abs(e) for _, _, e in found)
    assert worst < 0.006, f"worst mode shift {worst * 100:.2f} %"
    return worst


def tube_reflection_matches_fitted_impedance(run, library):
    """fdtd.rs:256-321: a plane wave in a rigid tube reflects off a fitted
    end wall with |R_meas - (zeta - 1)/(zeta + 1)| < 0.03."""
    f_max, ppw = 500.0, 15.0
    dx = c / (f_max * ppw)
    cells = lambda v: round(v / dx) * dx  # noqa: E731
    length, w = cells(30.0), cells(0.3)
    worst_all = {}
    for mid in ["audience-standing", "mineral-wool-50", "carpet-heavy"]:
        room = BoxRoom(length, w, w)
        mats = [scalar_material(0.0)] * 6
        mats[5] = library[mid]  # the wall at x = 0 (normal +x)
        fits = fit_surfaces(mats, (20.0, f_max))
        g = FdtdGrid.build(room, fits, c, f_max, ppw)
        src = g.nearest_air((15.0, w / 2, w / 2))
        rcv = g.nearest_air((2.0, w / 2, w / 2))
        xr = g.pos(rcv)[0]
        steps = int(0.075 / g.dt)
        sig = source_signal(f_max, g.dt, steps)
        freqs = 40.0 + np.arange(15) * 22.0
        spec_all = run(g, [(src, 1.0)], sig, [rcv], freqs)[0]
        long_room = BoxRoom(length * 2 + cells(15.0), w, w)
        gl = FdtdGrid.build(long_room, fit_surfaces([scalar_material(0.0)] * 6, (20.0, f_max)), c, f_max, ppw)
        shift = cells(30.0)
        src_l = gl.nearest_air((15.0 + shift, w / 2, w / 2))
        rcv_l = gl.nearest_air((xr + shift, w / 2, w / 2))
        spec_inc = run(gl, [(src_l, 1.0)], sig, [rcv_l], freqs)[0]
        worst = 0.0
        for fi, f in enumerate(freqs):
            wf = 2 * math.pi * f
            k_num = 2.0 / g.dx * math.asin(math.sin(wf * g.dt / 2.0) / COURANT)
            r_meas = (spec_all[fi] - spec_inc[fi]) / spec_inc[fi] * np.exp(1j * k_num * 2.0 * xr)
            z = fits[5].impedance(f)
            r_true = (z - 1) / (z + 1)
            worst = max(worst, abs(r_meas - r_true))
        assert worst < 0.03, f"{mid}: worst |dR| {worst}"
        worst_all[mid] = worst
    return worst_all


def branch_boundaries_are_stable(run_ir, library, steps=200_000):
    """fdtd.rs:323-350: strongly absorbing multi-branch walls over 200 k steps
    only lose energy: the spectrum's contributions by thirds of the run
    shrink more than tenfold each.  The thirds are the partial sums of the
    recorded time series (identical to the reference's three runs)."""
    room = BoxRoom(3.0, 2.4, 2.1)
    ids = ["mineral-wool-100", "audience-standing", "carpet-heavy", "curtain-heavy", "gypsum-board", "wood-panel"]
    fits = fit_surfaces([library[ids[i % 6]] for i in range(6)], (20.0, 300.0))
    g = FdtdGrid.build(room, fits, c, 300.0, 12.0)
    assert any(g.bstart[b + 1] - g.bstart[b] >= 3 for b in range(g.n_boundary))
    src = g.nearest_air((0.7, 0.6, 0.5))
    rcv = g.nearest_air((2.3, 1.7, 1.6))
    sig = source_signal(300.0, g.dt, steps)
    ir = run_ir(g, [(src, 1.0)], sig, [rcv])[0]
    assert np.all(np.isfinite(ir))
    n = np.arange(steps, dtype=np.float64)
    out = {}
    for f in [1.0, 80.0, 200.0]:
        x = f * g.dt * n
        terms = ir * np.exp(-2j * math.pi * (x - np.trunc(x)))
        a = terms[: steps // 3].sum()
        b = terms[: 2 * steps // 3].sum()
        cc = terms.sum()
        first, mid, last = abs(a), abs(b - a), abs(cc - b)
        assert mid < 0.1 * first and last < 0.1 * mid, f"{f} Hz: {first:.2e} {mid:.2e} {last:.2e}"
        out[f] = (first, mid, last)
    return out


def cardioid(_f, d):
    return complex(0.5 + 0.5 * d[0], 0.0)


def directional_source_reproduces_directivity(run_batch):
    """fdtd.rs:446-518 (the cardioid case): monopole + dipoles weighted by the
    first-order fit reproduce the fitted directivity (with the dipoles'
    near-field term) within 0.05 in free field."""
    room = BoxRoom(14.0, 12.0, 10.0)
    f_max = 500.0
    g = FdtdGrid.build(room, fit_surfaces([scalar_material(0.2)] * 6, (20.0, f_max)), c, f_max, 12.0)
    centre = np.array([7.0, 6.0, 5.0])
    src = g.nearest_air(centre)
    comps = source_components(g, src, 1)
    r = 1.6
    angles = [0.0, 60.0, 90.0, 135.0, 180.0, 270.0]
    rx = [g.nearest_air(centre + r * np.array([math.cos(math.radians(a)), math.sin(math.radians(a)), 0.0]))
          for a in angles]
    rx.append(g.nearest_air(centre + np.array([0.0, 0.0, r])))
    steps = int(0.018 / g.dt)
    sig = source_signal(f_max, g.dt, steps)
    freqs = np.array([120.0, 200.0, 300.0])
    spec = run_batch(g, comps, sig, rx, freqs)  # [4, n_rx, nf]
    tr = [to_transfer(spec[ci], sig, g, freqs, c, 1.0, np.ones(3)) for ci in range(len(comps))]
    rot = speaker_rotation(90.0, 0.0, 0.0)
    worst = 0.0
    for fi, f in enumerate(freqs):
        a0, a, _res = fit_first_order(cardioid, rot, f)
        w = component_weights(a0, a, 2 * math.pi * f / c, g.dx)
        for ri, cell in enumerate(rx):
            total = sum(w[ci] * tr[ci][ri, fi] for ci in range(len(comps)))
            measured = total / tr[0][ri, fi]
            d = g.pos(cell) - g.pos(src)
            dist = float(np.linalg.norm(d))
            dr = d / dist
            k = 2 * math.pi * f / c
            near = 1.0 + 1.0 / (1j * k * dist)
            fit = a0 + (a[0] * dr[0] + a[1] * dr[1] + a[2] * dr[2]) * near
            worst = max(worst, abs(measured - fit))
    assert worst < 0.05, f"cardioid: {worst}"
    return worst


def spherical_reflection(zeta: complex, cos: float, k: float, r: float) -> complex:
    """Reflection factor of a point source off a locally reacting plane of
    normalised impedance zeta (Weyl-van der Pol; reflection.rs:71-82), in
    the solver's e^{jwt} convention: Q = R + (1 - R) F(w) with
    F(w) = 1 + j sqrt(pi) w wofz(w) and the numerical distance
    w = (1 + j)/2 sqrt(k r) (cos + 1/zeta), written in the literature's
    e^{-iwt} convention (conjugated impedance, conjugated result).  wofz is
    the Faddeeva function w(z) = e^{-z^2} erfc(-iz) (scipy.special)."""
    from scipy.special import wofz

    cos = min(max(cos, 0.0), 1.0)
    beta = 1.0 / np.conj(zeta)
    rp = (cos - beta) / (cos + beta)
    w = complex(0.5, 0.5) * math.sqrt(k * r) * (cos + beta)
    f = 1.0 + 1j * math.sqrt(math.pi) * w * wofz(w)
    return complex(np.conj(rp + (1.0 - rp) * f))


def plane_reflection(zeta: complex, cos: float) -> complex:
    """Plane-wave reflection factor (reflection.rs:84-88)."""
    zc = zeta * max(cos, 1e-6)
    return (zc - 1.0) / (zc + 1.0)


def oblique_reflection_matches_spherical_wave_theory(run):
    """fdtd.rs:519-591: a source and receivers 1.2 m above an impedance
    floor (alpha 0.3; every other surface rigid), incidence 30-75 deg,
    gated before any other reflection.  The floor-reflected part is
    isolated with a second run over a rigid floor:
    Q = (p_imp - p_dir) / (p_rigid - p_dir), the direct sound along a grid
    axis known analytically (with the scheme's dispersion).  Q must match
    the point-source reflection off a locally reacting plane for the fitted
    impedance within |dQ| < 0.05."""
    room = BoxRoom(20.0, 14.0, 8.0)
    f_max = 600.0
    floor = 0  # BoxRoom surface order: floor first
    freqs = np.array([200.0, 300.0, 450.0])

    def build(alpha):
        mats = [scalar_material(0.0)] * room.n_surfaces
        mats[floor] = scalar_material(alpha)
        fits = fit_surfaces(mats, (20.0, f_max))
        return FdtdGrid.build(room, fits, c, f_max, 10.0), fits

    g_imp, fits = build(0.3)
    g_rig, _ = build(0.0)
    src = g_imp.nearest_air((8.0, 7.0, 1.2))
    sp = g_imp.pos(src)
    h = sp[2]  # the floor is at z = 0
    angles = [30.0, 45.0, 60.0, 70.0, 75.0]
    rx = [g_imp.nearest_air(sp + np.array([2.0 * h * math.tan(math.radians(a)), 0.0, 0.0])) for a in angles]
    steps = int(12.0 / c / g_imp.dt)
    sig = source_signal(f_max, g_imp.dt, steps)
    h0 = np.ones(len(freqs))
    p_imp = to_transfer(run(g_imp, [(src, 1.0)], sig, rx, freqs), sig, g_imp, freqs, c, 1.0, h0)
    p_rig = to_transfer(run(g_rig, [(src, 1.0)], sig, rx, freqs), sig, g_rig, freqs, c, 1.0, h0)
    worst, rows = 0.0, []
    for ri, cell in enumerate(rx):
        d = float(np.linalg.norm(g_imp.pos(cell) - sp))
        r2 = math.sqrt(d * d + 4.0 * h * h)
        cos = 2.0 * h / r2
        for fi, f in enumerate(freqs):
            k = 2.0 * math.pi * f / c
            lag = math.radians(FdtdSettings.phase_error_deg_per_m(f, c, g_imp.dx)) * d
            direct = np.exp(-1j * (k * d + lag)) / d
            q = (p_imp[ri, fi] - direct) / (p_rig[ri, fi] - direct)
            zeta = fits[floor].impedance(f)
            qs = spherical_reflection(zeta, cos, k, r2)
            err = abs(q - qs)
            worst = max(worst, err)
            rows.append((math.degrees(math.acos(cos)), f, abs(q), abs(qs), abs(plane_reflection(zeta, cos)), err))
    assert worst < 0.05, f"worst |dQ| {worst}: {rows}"
    return rows
