"""The oracle's restatement of FP16 field storage (oracle/fp16_oracle.c):
its own properties on the CPU -- close to the FP32 oracle, lanes of one
chunk independent, the rounding to FP16 exact on known values.  The CUDA
path is compared with it bit for bit in tests/test_gpu_fp16_oracle.py."""
from __future__ import annotations

import numpy as np

from oracle import fdtd as ofd
from scenes import branch_room, directional_components, spread_source


def test_fp16_oracle_is_close_to_the_fp32_oracle(library):
    g, taps, sig, rcv, freqs = branch_room(library, 0.05)
    comps = directional_components(g, (1.6, 1.3, 1.1))
    srcs = comps + [taps]
    ir16 = ofd.run_f16(g, srcs, sig, rcv)
    for s, src in enumerate(srcs):
        _, ir32 = ofd.run(g, src, sig, rcv, freqs, "f32", ir=True)
        assert np.abs(ir16[s] - ir32).max() <= 0.016 * np.abs(ir32).max()


def test_fp16_oracle_lanes_are_independent_of_their_neighbours():
    g, taps, sig, rcv, freqs = spread_source()
    one = ofd.run_f16(g, [taps, taps], sig[:200], rcv)
    assert np.array_equal(one[0], one[1])
    # A zero-weight lane leaves its chunk's scales alone.
    zero = [(c, 0.0) for c, _ in taps]
    two = ofd.run_f16(g, [taps, zero], sig[:200], rcv)
    assert np.array_equal(two[0], one[0]) and not np.any(two[1])


def test_fp16_oracle_stored_values_are_fp16_values():
    """Time series are FP16 values times powers of two: every sample of a
    single-source run, divided by a power of two, is exactly an FP16 value."""
    g, taps, sig, rcv, freqs = spread_source()
    ir = ofd.run_f16(g, [taps], sig[:120], rcv)[0]
    v = ir[ir != 0.0]
    m, e = np.frexp(v)  # v = m * 2^e, 0.5 <= |m| < 1
    # An FP16 normal has 11 significant bits: m * 2^11 is an integer.
    assert np.array_equal(m * 2048.0, np.round(m * 2048.0))
    assert np.array_equal(np.float16(m).astype(np.float64), m)
