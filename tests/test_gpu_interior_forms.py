"""The two forms of the interior update give identical results.

Standalone FP32 and FP16-storage plans use the TMA-fed z-march
(interior_tma) beside a special-cell kernel; WAVEY_INTERIOR=regq selects the
fused step kernel's register-queue z-march instead.  Both evaluate the same
formula in the same order from the same stored values, so every receiver
sample must agree bit for bit -- for 1, 2 and 4 lanes per cell (a tile row
of 128, 64 and 32 cells) and for FP16 storage with its slab scales.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from scenes import branch_room, directional_components, spread_source
from wavey_gb300.backend import FP16_STORAGE, FP32

pytestmark = pytest.mark.gpu


def _both(backend, *args, **kw):
    tma = backend.run_batch(*args, ir=True, **kw)
    os.environ["WAVEY_INTERIOR"] = "regq"
    try:
        regq = backend.run_batch(*args, ir=True, **kw)
    finally:
        del os.environ["WAVEY_INTERIOR"]
    return tma, regq


@pytest.mark.parametrize("precision", [FP32, FP16_STORAGE], ids=["fp32", "fp16"])
@pytest.mark.parametrize("lanes", [1, 2, 4])
def test_tma_and_fused_interior_agree(backend, library, precision, lanes):
    g, taps, sig, rcv, freqs = branch_room(library, 0.15)
    comps = directional_components(g, (1.6, 1.3, 1.1))
    sources = (comps + [taps])[:lanes]
    (s1, ir1), (s2, ir2) = _both(backend, g, sources, sig, rcv, freqs, precision=precision)
    assert np.array_equal(ir1, ir2)
    assert np.array_equal(s1, s2)


def test_fp16_plan_uses_tma(backend):
    g, taps, sig, rcv, freqs = spread_source()
    plan = backend.plan(g, [taps], sig[:300], rcv, freqs, precision=FP16_STORAGE)
    assert plan.info()["interior_kernel"] == 1
    plan.close()


@pytest.mark.parametrize("precision", [FP32, FP16_STORAGE], ids=["fp32", "fp16"])
@pytest.mark.parametrize("cfg", range(7))
def test_every_tma_shape_agrees(backend, library, precision, cfg):
    """Every tile shape of the TMA kernel (8, 16 or 32 rows with their ring
    depths), with z-runs of 1 plane (a CTA per plane), 3 planes and 64
    planes (longer than the grid: one run per tile column), gives the
    register-queue kernel's results bit for bit."""
    g, taps, sig, rcv, freqs = branch_room(library, 0.1)
    comps = directional_components(g, (1.6, 1.3, 1.1))
    sources = comps + [taps]
    os.environ["WAVEY_INTERIOR"] = "regq"
    try:
        ref = backend.run_batch(g, sources, sig, rcv, freqs, precision=precision, ir=True)
    finally:
        del os.environ["WAVEY_INTERIOR"]
    for zt in (1, 3, 64):
        os.environ["WAVEY_TMA_CFG"], os.environ["WAVEY_TMA_ZT"] = str(cfg), str(zt)
        try:
            plan = backend.plan(g, sources, sig, rcv, freqs, precision=precision, ir=True)
            info = plan.info()
            assert (info["tma_depth"], info["tma_zt"]) == (cfg, zt)
            plan.run()
            spec, ir = plan.read()
            plan.close()
        finally:
            del os.environ["WAVEY_TMA_CFG"], os.environ["WAVEY_TMA_ZT"]
        assert np.array_equal(ir, ref[1]), (cfg, zt)
        assert np.array_equal(spec, ref[0]), (cfg, zt)


@pytest.mark.parametrize("precision", [FP32, FP16_STORAGE], ids=["fp32", "fp16"])
@pytest.mark.parametrize("cfg", [0, 4, 6])
def test_march_direction_does_not_change_results(backend, library, precision, cfg):
    """The interior kernel marches z upwards on even steps and downwards on
    odd ones; WAVEY_ZALT=0 keeps every step upwards.  Both give identical
    receiver series, with z-runs of 1, 3 (the last run ragged) and 64 planes,
    over an odd number of steps."""
    g, taps, sig, rcv, freqs = branch_room(library, 0.1)
    comps = directional_components(g, (1.6, 1.3, 1.1))
    sources = comps + [taps]
    sig = sig[:301]
    for zt in (1, 3, 64):
        out = []
        for zalt in ("0", "1"):
            os.environ.update(WAVEY_TMA_CFG=str(cfg), WAVEY_TMA_ZT=str(zt), WAVEY_ZALT=zalt)
            try:
                out.append(backend.run_batch(g, sources, sig, rcv, freqs, precision=precision, ir=True))
            finally:
                for k in ("WAVEY_TMA_CFG", "WAVEY_TMA_ZT", "WAVEY_ZALT"):
                    del os.environ[k]
        assert np.array_equal(out[0][1], out[1][1]), zt
        assert np.array_equal(out[0][0], out[1][0]), zt


@pytest.mark.parametrize("precision", [FP32, FP16_STORAGE], ids=["fp32", "fp16"])
def test_fused_kernel_z_run_does_not_change_results(backend, library, precision):
    """The fused step kernel (WAVEY_INTERIOR=regq; FP64 plans and multi-room
    runs use it too) splits z into runs of WAVEY_FUSED_ZT planes per CTA:
    runs of 1, 5 and 64 planes give the default's (16) results bit for bit."""
    g, taps, sig, rcv, freqs = branch_room(library, 0.1)
    sources = directional_components(g, (1.6, 1.3, 1.1)) + [taps]
    sig = sig[:300]
    out = []
    for zt in ("16", "1", "5", "64"):
        os.environ.update(WAVEY_INTERIOR="regq", WAVEY_FUSED_ZT=zt)
        try:
            out.append(backend.run_batch(g, sources, sig, rcv, freqs, precision=precision, ir=True))
        finally:
            for k in ("WAVEY_INTERIOR", "WAVEY_FUSED_ZT"):
                del os.environ[k]
    for got in out[1:]:
        assert np.array_equal(got[1], out[0][1])
        assert np.array_equal(got[0], out[0][0])


@pytest.mark.parametrize("lanes", [1, 2, 4])
def test_programmatic_launch_does_not_change_results(backend, library, lanes):
    """Where one wave of interior CTAs and a special-cell block fit on every
    SM, each step's interior kernel is a programmatic dependent of the
    previous step (its CTAs may start early and wait in the kernel);
    WAVEY_PDL=0 launches it after the previous step ends.  Same results."""
    g, taps, sig, rcv, freqs = branch_room(library, 0.1)
    comps = directional_components(g, (1.6, 1.3, 1.1))
    sources = (comps + [taps])[:lanes]
    sig = sig[:401]
    out = []
    for pdl in ("1", "0"):
        os.environ.update(WAVEY_PDL=pdl, WAVEY_TMA_ZT="64")
        try:
            plan = backend.plan(g, sources, sig, rcv, freqs, ir=True)
        finally:
            for k in ("WAVEY_PDL", "WAVEY_TMA_ZT"):
                del os.environ[k]
        try:
            assert plan.info()["programmatic"] == int(pdl)
            plan.run()
            out.append(plan.read())
        finally:
            plan.close()
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][0], out[1][0])


@pytest.mark.parametrize("lanes", [1, 2, 4])
@pytest.mark.parametrize("cfg", range(7))
def test_special_cells_inside_the_march_agree(backend, library, lanes, cfg):
    """The fused form (WAVEY_BRANCH=9: every interior CTA also updates the
    special cells of its tile from the staged planes) gives the register-
    queue kernel's results bit for bit, for every tile shape, z-runs of 1, 3
    and 64 planes, and 1, 2 or 4 lanes per cell: rigid faces, boundary nodes
    with branch states, and merged source taps."""
    g, taps, sig, rcv, freqs = branch_room(library, 0.1)
    comps = directional_components(g, (1.6, 1.3, 1.1))
    sources = (comps + [taps])[:lanes] if lanes < 4 else comps + [taps]
    os.environ["WAVEY_INTERIOR"] = "regq"
    try:
        ref = backend.run_batch(g, sources, sig, rcv, freqs, precision=FP32, ir=True)
    finally:
        del os.environ["WAVEY_INTERIOR"]
    for zt in (1, 3, 64):
        os.environ.update(WAVEY_TMA_CFG=str(cfg), WAVEY_TMA_ZT=str(zt), WAVEY_BRANCH="9")
        try:
            plan = backend.plan(g, sources, sig, rcv, freqs, precision=FP32, ir=True)
            info = plan.info()
            assert (info["tma_depth"], info["tma_zt"], info["branch"]) == (cfg, zt, 9)
            plan.run()
            spec, ir = plan.read()
            plan.close()
        finally:
            for k in ("WAVEY_TMA_CFG", "WAVEY_TMA_ZT", "WAVEY_BRANCH"):
                del os.environ[k]
        assert np.array_equal(ir, ref[1]), (cfg, zt)
        assert np.array_equal(spec, ref[0]), (cfg, zt)


def test_fused_form_on_the_pillar_room(backend):
    """The fused form on a room with pillars and a spread source (taps on
    several cells of one tile), against the concurrent-branch form."""
    from scenes import pillar_room

    g, taps, sig, rcv, freqs = pillar_room(0.2)
    ref = backend.run_batch(g, [taps, taps], sig, rcv, freqs, precision=FP32, ir=True)
    os.environ["WAVEY_BRANCH"] = "9"
    try:
        got = backend.run_batch(g, [taps, taps], sig, rcv, freqs, precision=FP32, ir=True)
    finally:
        del os.environ["WAVEY_BRANCH"]
    assert np.array_equal(got[1], ref[1])
    assert np.array_equal(got[0], ref[0])


@pytest.mark.parametrize("cfg", range(7, 14))
def test_fp32_shapes_with_capped_registers_agree(backend, library, cfg):
    """FP32 shapes 7-13 (the shapes of 0-6 compiled for three resident CTAs
    per SM) give the register-queue kernel's results bit for bit."""
    g, taps, sig, rcv, freqs = branch_room(library, 0.1)
    sources = directional_components(g, (1.6, 1.3, 1.1)) + [taps]
    os.environ["WAVEY_INTERIOR"] = "regq"
    try:
        ref = backend.run_batch(g, sources, sig, rcv, freqs, precision=FP32, ir=True)
    finally:
        del os.environ["WAVEY_INTERIOR"]
    for zt in (1, 3, 64):
        os.environ["WAVEY_TMA_CFG"], os.environ["WAVEY_TMA_ZT"] = str(cfg), str(zt)
        try:
            plan = backend.plan(g, sources, sig, rcv, freqs, precision=FP32, ir=True)
            assert (plan.info()["tma_depth"], plan.info()["tma_zt"]) == (cfg, zt)
            plan.run()
            spec, ir = plan.read()
            plan.close()
        finally:
            del os.environ["WAVEY_TMA_CFG"], os.environ["WAVEY_TMA_ZT"]
        assert np.array_equal(ir, ref[1]), (cfg, zt)
        assert np.array_equal(spec, ref[0]), (cfg, zt)
