"""The CUDA backend: the Python face of libwavey_cuda.so.

`CudaBackend.run_fdtd` keeps the contract of the reference's
`Gpu::run_fdtd` (wavey-solver/src/gpu_fdtd.rs:45-54) and of the CPU twin
`fdtd::run_cpu` (fdtd.rs:616-626):

    run_fdtd(grid, source_taps, signal, receivers, freqs, cancel, progress)
        -> spectra [n_recv, nf] complex, or None when cancelled

Limit and device failures raise `WaveyError` (the reference's Err(String)).
There is no CPU fallback.  `run_batch` advances several right-hand sides
(speakers x directional components) in one launch per step; `Plan` keeps a
run resident on the device for repeated timing.
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from . import _native as N

FP32 = N.WAVEY_FP32
FP64 = N.WAVEY_FP64
FP16_STORAGE = N.WAVEY_FP16_STORAGE


class WaveyError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{msg} (status {code})")
        self.code = code


def _grid_struct(g):
    """WaveyGrid over the arrays of an FdtdGrid (or anything with the same
    attributes: n, dx, dt, flags, bidx, bstart, slots)."""
    flags = np.ascontiguousarray(g.flags, dtype=np.uint8)
    bidx = np.ascontiguousarray(g.bidx, dtype=np.uint32)
    bstart = np.ascontiguousarray(g.bstart, dtype=np.uint32)
    slots = np.ascontiguousarray(g.slots, dtype=np.float64).reshape(-1)
    nb = len(bstart) - 1
    s = N.WaveyGrid(g.n[0], g.n[1], g.n[2], g.dx, g.dt, N.ptr(flags, C.c_uint8), N.ptr(bidx, C.c_uint32), nb,
                    N.ptr(bstart, C.c_uint32), N.ptr(slots, C.c_double))
    return s, (flags, bidx, bstart, slots)


def _sources_struct(sources):
    keep = []
    arr = (N.WaveySource * len(sources))()
    for i, taps in enumerate(sources):
        t = (N.WaveyTap * max(len(taps), 1))(*[N.WaveyTap(int(c), float(w)) for c, w in taps])
        keep.append(t)
        arr[i].taps = C.cast(t, C.POINTER(N.WaveyTap))
        arr[i].n_taps = len(taps)
    return arr, keep


def _signals(signal, n_sources: int, steps: int):
    s = np.asarray(signal, dtype=np.float64)
    if s.ndim == 1:
        return np.ascontiguousarray(s), 0
    if s.shape[0] != n_sources or s.shape[1] < steps:
        raise ValueError("signals must be [n_sources, steps]")
    s = np.ascontiguousarray(s)
    return s, s.shape[1]


def _callbacks(cancel, progress):
    flag = None
    if cancel is not None:
        flag = cancel if isinstance(cancel, CancelFlag) else None
        if flag is None:
            raise TypeError("cancel must be a CancelFlag")
    cb = N.PROGRESS_FN(lambda f, _u: progress(f)) if progress is not None else N.PROGRESS_FN()
    return (C.cast(C.byref(flag._v), C.POINTER(C.c_int32)) if flag else None), cb


class CancelFlag:
    """The reference's `&AtomicBool`: set() from any thread cancels a run at
    its next 128-step boundary."""

    def __init__(self):
        self._v = C.c_int32(0)

    def set(self):
        self._v.value = 1

    def clear(self):
        self._v.value = 0

    def is_set(self) -> bool:
        return bool(self._v.value)


class CudaBackend:
    """One device context (libwavey_cuda's wavey_cuda_ctx)."""

    def __init__(self, device: int = 0):
        self._lib = N.cuda()
        h = C.c_void_p()
        st = self._lib.wavey_cuda_create(int(device), C.byref(h))
        if st != 0:
            raise WaveyError(st, f"no usable CUDA device {device}")
        self._h = h
        self._lock = threading.Lock()

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.wavey_cuda_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def _check(self, st: int):
        if st < 0:
            raise WaveyError(st, self._lib.wavey_cuda_last_error(self._h).decode())
        return st

    def device_info(self):
        name = C.create_string_buffer(256)
        sms = C.c_int()
        self._lib.wavey_cuda_device_info(self._h, name, 256, C.byref(sms))
        return name.value.decode(), sms.value

    # ---------------------------------------------------------------- runs
    def run_fdtd(self, grid, source, signal, receivers, freqs, cancel=None, progress=None, ir: bool = False):
        """Gpu::run_fdtd: spectra [n_recv, nf] (and the time series
        [n_recv, steps] when ir=True), or None when cancelled."""
        res = self.run_batch(grid, [source], signal, receivers, freqs, FP32, cancel, progress, ir)
        if res is None:
            return None
        if ir:
            return res[0][0], res[1][0]
        return res[0]

    def run_batch(self, grid, sources, signal, receivers, freqs, precision=FP32, cancel=None, progress=None,
                  ir: bool = False):
        """S right-hand sides: spectra [S, n_recv, nf] (and ir [S, n_recv,
        steps]), or None when cancelled.  signal is one shared signal or
        [S, steps]."""
        g, keep_g = _grid_struct(grid)
        srcs, keep_s = _sources_struct(sources)
        steps = (np.asarray(signal).shape[-1])
        sig, stride = _signals(signal, len(sources), steps)
        rx = np.ascontiguousarray(receivers, dtype=np.uint64)
        fr = np.ascontiguousarray(freqs, dtype=np.float64)
        S, R, F = len(sources), len(rx), len(fr)
        out = np.zeros((S, R, F), dtype=np.complex128)
        irbuf = np.zeros((S, R, steps), dtype=np.float64) if ir else None
        cflag, cb = _callbacks(cancel, progress)
        with self._lock:
            st = self._lib.wavey_cuda_fdtd_run_batch(
                self._h, C.byref(g), srcs, S, N.ptr(sig, C.c_double), stride, steps, N.ptr(rx, C.c_uint64), R,
                N.ptr(fr, C.c_double), F, int(precision), N.ptr(out.view(np.float64), C.c_double),
                N.ptr(irbuf, C.c_double), cflag, cb, None)
            self._check(st)
        if st == N.WAVEY_CANCELLED:
            return None
        return (out, irbuf) if ir else out

    def build_grid(self, room, fits, c: float, dx: float, solids=()):
        """FdtdGrid.build_dx on the device (wavey_cuda_grid_build, or
        wavey_cuda_grid_build_mesh for a MeshRoom with optional rigid boxes
        `solids`): the same arrays as the host builder, returned as an
        FdtdGrid."""
        from .fdtd import FdtdGrid

        if len(fits) != room.n_surfaces:
            raise ValueError(f"{len(fits)} fits for {room.n_surfaces} surfaces")
        arr = (N.WhFit * len(fits))(*[f._c() for f in fits])
        dg, sh = C.c_void_p(), N.WaveyGridShape()
        if hasattr(room, "triangles"):  # MeshRoom
            pos, srf = room.triangles()
            pos = np.ascontiguousarray(pos, dtype=np.float64)
            srf = np.ascontiguousarray(srf, dtype=np.uint32)
            sol = np.ascontiguousarray(np.asarray(solids, dtype=np.float64).reshape(-1, 6))
            with self._lock:
                self._check(self._lib.wavey_cuda_grid_build_mesh(
                    self._h, N.ptr(pos, C.c_double), N.ptr(srf, C.c_uint32), len(srf),
                    N.ptr(sol, C.c_double) if len(sol) else None, len(sol), arr, len(fits), float(c), float(dx),
                    C.byref(dg), C.byref(sh)))
        else:
            r, keep = room._c()
            with self._lock:
                self._check(self._lib.wavey_cuda_grid_build(self._h, C.byref(r), arr, len(fits), float(c), float(dx),
                                                            C.byref(dg), C.byref(sh)))
        try:
            out = C.c_void_p()
            st = N.host().wh_grid_alloc(sh.n, sh.origin, sh.dx, sh.dt, sh.air_cells, sh.n_boundary, sh.n_slots,
                                        C.byref(out))
            if st != 0:
                raise WaveyError(st, "host grid allocation failed")
            p = [C.POINTER(C.c_uint8)(), C.POINTER(C.c_uint32)(), C.POINTER(C.c_uint32)(), C.POINTER(C.c_uint32)(),
                 C.POINTER(C.c_double)()]
            N.host().wh_grid_arrays(out, *[C.byref(q) for q in p])
            grid = FdtdGrid(out.value)  # owns the host arrays from here
            with self._lock:
                self._check(self._lib.wavey_cuda_grid_read(dg, *p))
            return grid
        finally:
            self._lib.wavey_cuda_grid_free(dg)

    def plan(self, grid, sources, signal, receivers, freqs, precision=FP32, ir: bool = False) -> "Plan":
        return Plan(self, grid, sources, signal, receivers, freqs, precision, ir)

    def run_rooms(self, jobs, precision=FP32, cancel=None, progress=None, ir: bool = False):
        """Several rooms in one launch per step.  jobs: list of RoomJob.
        Returns per room spectra [S, n_recv, nf] (and time series), or None
        when cancelled."""
        packed = _pack_jobs(jobs, ir)
        cflag, cb = _callbacks(cancel, progress)
        with self._lock:
            st = self._check(self._lib.wavey_cuda_fdtd_run_rooms(self._h, packed.arr, len(jobs), int(precision),
                                                                   cflag, cb, None))
        if st == N.WAVEY_CANCELLED:
            return None
        return [(o, i) if ir else o for o, i in zip(packed.outs, packed.irs)]

    def rooms_plan(self, jobs, precision=FP32, ir: bool = False) -> "RoomsPlan":
        return RoomsPlan(self, jobs, precision, ir)


class RoomJob:
    """One room of a multi-room run: the arguments of run_batch."""

    def __init__(self, grid, sources, signal, receivers, freqs):
        self.grid, self.sources, self.signal, self.receivers, self.freqs = grid, sources, signal, receivers, freqs


class _Packed:
    pass


def _pack_jobs(jobs, ir):
    pk = _Packed()
    pk.keep, pk.outs, pk.irs = [], [], []
    pk.arr = (N.WaveyRoomJob * len(jobs))()
    for r, j in enumerate(jobs):
        g, kg = _grid_struct(j.grid)
        srcs, ks = _sources_struct(j.sources)
        steps = np.asarray(j.signal).shape[-1]
        sig, stride = _signals(j.signal, len(j.sources), steps)
        rx = np.ascontiguousarray(j.receivers, dtype=np.uint64)
        fr = np.ascontiguousarray(j.freqs, dtype=np.float64)
        out = np.zeros((len(j.sources), len(rx), len(fr)), dtype=np.complex128)
        irb = np.zeros((len(j.sources), len(rx), steps)) if ir else None
        pk.keep += [g, kg, srcs, ks, sig, rx, fr]
        pk.outs.append(out)
        pk.irs.append(irb)
        a = pk.arr[r]
        a.grid = C.pointer(g)
        a.sources = C.cast(srcs, C.POINTER(N.WaveySource))
        a.n_sources = len(j.sources)
        a.signals = N.ptr(sig, C.c_double)
        a.signal_stride = stride
        a.steps = steps
        a.receivers = N.ptr(rx, C.c_uint64)
        a.n_recv = len(rx)
        a.freqs = N.ptr(fr, C.c_double)
        a.nf = len(fr)
        a.out = N.ptr(out.view(np.float64), C.c_double)
        a.ir_out = N.ptr(irb, C.c_double)
    return pk


class RoomsPlan:
    """A multi-room run kept on the device (wavey_cuda_rooms_*)."""

    def __init__(self, backend: CudaBackend, jobs, precision, ir):
        self._b = backend
        self._packed = _pack_jobs(jobs, ir)
        self.ir = ir
        h = C.c_void_p()
        with backend._lock:
            backend._check(backend._lib.wavey_cuda_rooms_create(backend._h, self._packed.arr, len(jobs), int(precision),
                                                                int(ir), C.byref(h)))
        self._h = h
        self.n = len(jobs)

    def run(self, cancel=None, progress=None, stats: bool = False):
        cflag, cb = _callbacks(cancel, progress)
        s = N.WaveyRunStats()
        with self._b._lock:
            st = self._b._check(self._b._lib.wavey_cuda_rooms_run(self._h, cflag, cb, None,
                                                                  C.byref(s) if stats else None))
        if st == N.WAVEY_CANCELLED:
            return None
        if stats:
            return {"total_ms": s.total_ms, "step_ms": s.step_ms, "step_launches": s.step_launches, "chunks": s.chunks}
        return True

    def read(self, room: int):
        out, irb = self._packed.outs[room], self._packed.irs[room]
        with self._b._lock:
            self._b._check(self._b._lib.wavey_cuda_rooms_read(self._h, room, N.ptr(out.view(np.float64), C.c_double),
                                                              N.ptr(irb, C.c_double)))
        return (out.copy(), irb.copy()) if self.ir else out.copy()

    def info(self, room: int = 0) -> dict:
        i = N.WaveyPlanInfo()
        self._b._lib.wavey_cuda_rooms_info(self._h, room, C.byref(i))
        return {k: getattr(i, k) for k, _ in N.WaveyPlanInfo._fields_}

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._b._lib.wavey_cuda_rooms_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Plan:
    """A run kept on the device: inputs uploaded once, run() repeatable."""

    def __init__(self, backend: CudaBackend, grid, sources, signal, receivers, freqs, precision, ir):
        self._b = backend
        g, keep_g = _grid_struct(grid)
        srcs, keep_s = _sources_struct(sources)
        steps = np.asarray(signal).shape[-1]
        sig, stride = _signals(signal, len(sources), steps)
        rx = np.ascontiguousarray(receivers, dtype=np.uint64)
        fr = np.ascontiguousarray(freqs, dtype=np.float64)
        self.shape = (len(sources), len(rx), len(fr))
        self.steps = steps
        self.ir = ir
        h = C.c_void_p()
        with backend._lock:
            backend._check(backend._lib.wavey_cuda_plan_create(
                backend._h, C.byref(g), srcs, len(sources), N.ptr(sig, C.c_double), stride, steps,
                N.ptr(rx, C.c_uint64), len(rx), N.ptr(fr, C.c_double), len(fr), int(precision), int(ir),
                C.byref(h)))
        self._h = h

    def run(self, cancel=None, progress=None, stats: bool = False):
        cflag, cb = _callbacks(cancel, progress)
        s = N.WaveyRunStats()
        with self._b._lock:
            st = self._b._check(self._b._lib.wavey_cuda_plan_run(self._h, cflag, cb, None,
                                                                 C.byref(s) if stats else None))
        if st == N.WAVEY_CANCELLED:
            return None
        if stats:
            return {"total_ms": s.total_ms, "step_ms": s.step_ms, "step_launches": s.step_launches,
                    "chunks": s.chunks}
        return True

    def read(self):
        out = np.zeros(self.shape, dtype=np.complex128)
        irbuf = np.zeros((self.shape[0], self.shape[1], self.steps)) if self.ir else None
        with self._b._lock:
            self._b._check(self._b._lib.wavey_cuda_plan_read(self._h, N.ptr(out.view(np.float64), C.c_double),
                                                             N.ptr(irbuf, C.c_double)))
        return (out, irbuf) if self.ir else out

    def autotune(self) -> dict:
        """Times every candidate shape of the interior kernel, then every
        launch form of the special-cell branch, on this plan's grid and keeps
        the fastest (wavey_cuda_plan_autotune).  Candidates are
        (cfg, zt, branch, step_us)."""
        r = N.WaveyTuneResult()
        with self._b._lock:
            self._b._check(self._b._lib.wavey_cuda_plan_autotune(self._h, C.byref(r)))
        return {"cfg": r.cfg, "zt": r.zt, "rows": r.rows, "p_planes": r.p_planes, "q_planes": r.q_planes,
                "branch": r.branch, "step_us": r.step_us,
                "candidates": [(r.cand_cfg[i], r.cand_zt[i], r.cand_branch[i], r.cand_step_us[i])
                               for i in range(r.candidates)]}

    def transfers(self, lane_speaker, factors, n_mics: int, plane_points=()) -> np.ndarray:
        """Per-speaker transfer functions combined on the device
        (wavey_cuda_plan_transfers): complex64 in the results.bin transfer
        layout, mics [mic][speaker][f] then per plane [speaker][point][f],
        flattened.  lane_speaker: speaker of each right-hand side (-1: left
        out); factors: complex [sources][nf]."""
        ls = np.ascontiguousarray(lane_speaker, dtype=np.int32)
        fac = np.ascontiguousarray(np.asarray(factors, dtype=np.complex128))
        pp = np.ascontiguousarray(plane_points, dtype=np.int64)
        S = max(int(ls.max()) + 1, 0) if ls.size else 0
        info = self.info()
        out = np.zeros(int(info["receivers"]) * int(info["freqs"]) * S, dtype=np.complex64)
        lay = N.WaveyTransferLayout(S, N.ptr(ls, C.c_int32), N.ptr(fac.view(np.float64), C.c_double), int(n_mics),
                                    len(pp), N.ptr(pp, C.c_int64) if len(pp) else None)
        with self._b._lock:
            self._b._check(self._b._lib.wavey_cuda_plan_transfers(self._h, C.byref(lay),
                                                                  N.ptr(out.view(np.float32), C.c_float),
                                                                  2 * out.size))
        return out

    def band_params(self, bands=(63.0, 125.0, 250.0, 500.0, 1000.0, 2000.0, 4000.0, 8000.0), integrate: bool = True,
                    lundeby: bool = False) -> np.ndarray:
        """ISO 3382-1 parameters of every receiver's time series, computed on
        the device (wavey_cuda_plan_band_params; IR plans only):
        [source][receiver][band][6] = edt, t20, t30, c80, d50, ts."""
        b = np.ascontiguousarray(bands, dtype=np.float64)
        info = self.info()
        out = np.zeros((int(info["sources"]), int(info["receivers"]), len(b), 6))
        flags = (N.WAVEY_IR_INTEGRATE if integrate else 0) | (N.WAVEY_IR_LUNDEBY if lundeby else 0)
        with self._b._lock:
            self._b._check(self._b._lib.wavey_cuda_plan_band_params(self._h, N.ptr(b, C.c_double), len(b), flags,
                                                                    N.ptr(out, C.c_double), out.size))
        return out

    def info(self) -> dict:
        i = N.WaveyPlanInfo()
        self._b._lib.wavey_cuda_plan_info(self._h, C.byref(i))
        return {k: getattr(i, k) for k, _ in N.WaveyPlanInfo._fields_}

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._b._lib.wavey_cuda_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
