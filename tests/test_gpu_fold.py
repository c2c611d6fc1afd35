"""The receiver fold's two kernels agree bit for bit: FP32 plans whose chunk
twiddles fit in shared memory (up to 96 frequencies) fold with
dft_chunk_tiled, longer frequency lists with dft_chunk.  Each spectrum bin
is an independent sum over the same steps in the same order, so the bins
two plans share must be identical -- with one, two and four sources per
chunk, two chunks, and a step count that ends in a partial chunk."""
from __future__ import annotations

import numpy as np
import pytest

from scenes import branch_room, directional_components

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n_sources", [1, 2, 4, 8])
def test_tiled_and_plain_folds_agree(backend, library, n_sources):
    g, taps, sig, rcv, freqs = branch_room(library, 0.06)
    comps = directional_components(g, (1.6, 1.3, 1.1)) + directional_components(g, (3.0, 2.2, 1.8))
    sources = comps[:n_sources]
    sig = sig[:300]
    short = 30.0 + 7.0 * np.arange(62)                            # tiled (62 bins)
    long_ = np.concatenate([short, 500.0 + 3.0 * np.arange(60)])  # 122 bins: plain
    a = backend.run_batch(g, sources, sig, rcv, short)
    b = backend.run_batch(g, sources, sig, rcv, long_)
    assert np.array_equal(a, b[:, :, :62])
