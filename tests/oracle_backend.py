"""The oracle behind the backend interface that the wave stage calls
(run_batch, run_rooms): lets the host-side orchestration be checked on the
CPU against the FP64 restatement of run_cpu.  Test infrastructure only."""
from __future__ import annotations

import numpy as np

from oracle import fdtd as ofd


class OracleBackend:
    def __init__(self):
        self.calls = []  # (kind, number of right-hand sides) per call

    def run_batch(self, grid, sources, signal, receivers, freqs, precision=None, cancel=None, progress=None):
        self.calls.append(("batch", len(sources)))
        return np.stack([ofd.run(grid, taps, signal, receivers, freqs, "f64") for taps in sources])

    def run_fdtd(self, grid, source, signal, receivers, freqs, cancel=None, progress=None):
        self.calls.append(("single", 1))
        return ofd.run(grid, source, signal, receivers, freqs, "f64")

    def run_rooms(self, jobs, precision=None, cancel=None, progress=None):
        self.calls.append(("rooms", len(jobs)))
        return [np.stack([ofd.run(j.grid, taps, j.signal, j.receivers, j.freqs, "f64") for taps in j.sources])
                for j in jobs]
