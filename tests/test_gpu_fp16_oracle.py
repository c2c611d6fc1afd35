"""FP16 field storage on the GPU is bit-identical to the oracle's
restatement of it (oracle/fp16_oracle.c): receiver time series of 1, 2, 3
(one padded 4-lane chunk), 4 and 5 (two chunks) right-hand sides, through
the TMA interior kernel and through the fused register-queue step."""
from __future__ import annotations

import os

import numpy as np
import pytest

from oracle import fdtd as ofd
from scenes import branch_room, directional_components
from wavey_gb300.backend import FP16_STORAGE

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("lanes", [1, 2, 3, 4, 5])
def test_fp16_storage_matches_its_restatement(backend, library, lanes):
    g, taps, sig, rcv, freqs = branch_room(library, 0.05)
    comps = directional_components(g, (1.6, 1.3, 1.1))
    srcs = (comps + [taps])[:lanes]
    ref = ofd.run_f16(g, srcs, sig, rcv)
    _, ir = backend.run_batch(g, srcs, sig, rcv, freqs, precision=FP16_STORAGE, ir=True)
    assert np.array_equal(ir, ref)
    os.environ["WAVEY_INTERIOR"] = "regq"
    try:
        _, ir2 = backend.run_batch(g, srcs, sig, rcv, freqs, precision=FP16_STORAGE, ir=True)
    finally:
        del os.environ["WAVEY_INTERIOR"]
    assert np.array_equal(ir2, ref)
