"""The FP16-storage interior update evaluated in the centre plane's scale
(interior_tma.cuh) equals the update in the fields' own scale bit for bit.

The kernel adds the z neighbours and the old value into plane z's scale
through power-of-two ratios of the slab scales and multiplies by the scale
once at the store; the oracle (oracle/fp16_oracle.c) scales every value as it
reads it.  Both are emulated here in numpy float32 arithmetic (IEEE, one
rounding per operation, no contraction) over random FP16 values -- normals,
subnormals, zeros of both signs -- and random slab exponents over the range
the slab scales take (2^-60 .. 2^20), and the stored FP16 bits and the slab
maxima must agree exactly.  The mixed-precision add of the kernel
(add.rn.f32.f16) is float32(h) + c, rounded once."""
from __future__ import annotations

import numpy as np

F = np.float32
L2 = F(0.5773502691896257 ** 2)


def _halves(rng, n):
    bits = rng.integers(0, 1 << 16, n, dtype=np.uint32).astype(np.uint16)
    # keep finite values (the fields never hold inf or NaN): clear exponent 31
    bits = np.where((bits & 0x7C00) == 0x7C00, bits & 0x83FF, bits)
    return bits.view(np.float16).astype(F)


def _scale(e):
    return np.ldexp(F(1.0), e).astype(F)


def test_rescaled_update_matches_the_oracle_order():
    rng = np.random.default_rng(11)
    n = 1_000_000
    xm, xp, ym, yp, c, zm, zp, q = (_halves(rng, n) for _ in range(8))
    # slab exponents: planes z-1, z, z+1 of level n within a few binades of
    # each other, level n-1 and n+1 near them, all clamped at 2^-60
    ec = rng.integers(-60, 21, n)
    em = np.clip(ec + rng.integers(-12, 13, n), -60, 20)
    ep = np.clip(ec + rng.integers(-12, 13, n), -60, 20)
    eo = np.clip(ec + rng.integers(-4, 5, n), -60, 20)
    en = np.clip(ec + rng.integers(-4, 5, n), -60, 20)
    sm, sc, sp, so, sn = (_scale(e) for e in (em, ec, ep, eo, en))
    sinv = _scale(-en)

    with np.errstate(over="ignore", invalid="ignore"):
        # the oracle's order: every value scaled as it is read
        cv = c * sc
        a = ((xm + xp) + ym) + yp
        s = (a * sc + zm * sm) + zp * sp
        old = q * so
        nx = (F(2) * cv - old) + L2 * (s - F(6) * cv)
        h_ref = (nx * sinv).astype(np.float16)

        # the kernel's order: plane z's scale, ratios, one scaling at the store
        r_cm, r_mp, r_pk, r_ok = sc / sm, sm / sp, sp / sc, so / sc
        s2 = ((a * r_cm + zm) * r_mp + zp) * r_pk
        old2 = q * r_ok
        nx2 = (F(2) * c - old2) + L2 * (s2 - F(6) * c)
        h_new = (nx2 * (sc * sinv)).astype(np.float16)

    assert np.array_equal(h_ref.view(np.uint16), h_new.view(np.uint16))
    # the slab maximum, taken in plane z's scale and scaled back
    assert np.array_equal(np.abs(nx).view(np.uint32), (np.abs(nx2) * sc).view(np.uint32))


def test_unwritten_levels_give_zero():
    """At the first steps the scales of a level not yet written are zero
    (over zero fields): the ratios the kernel takes for them (1 for level n,
    0 for level n-1) keep the update at zero."""
    z = np.zeros(4, F)
    for sc, so in ((F(0), F(0)), (F(2.0 ** -20), F(0))):
        r = F(1) if sc == 0 else F(1)  # level-n ratios: all scales of the level are zero or none
        r_ok = F(0) if so == 0 else so / sc
        s2 = ((z * r + z) * r + z) * r
        nx2 = (F(2) * z - z * r_ok) + L2 * (s2 - F(6) * z)
        assert np.array_equal((nx2 * (sc * F(1))).astype(np.float16).view(np.uint16), np.zeros(4, np.uint16))
