"""Benchmark of the FDTD wave-solver hot path on one GB300 (or N, source-sharded).

Workload (default): room_pillars -- a 20 x 15 x 8 m room with four pillars
at a 500 Hz crossover (294 x 221 x 119 cells, 7.4 M air), five fitted
frequency-dependent materials, one cardioid source (monopole + 3 dipoles =
4 right-hand sides), 64 receivers plus a 1.2 m cut plane (4844 receivers),
62 frequency bins, 1.0 s (8661 steps).  Seeded synthetic inputs.

One bench step = one full run of that workload: all 8661 time steps of all 4
right-hand sides, batched in one launch per time step, FP32.  The fields
(2 x 135 MB per source chunk) are larger than L2 for the batched run.

  value     air-cell updates per second over all right-hand sides, inputs
            resident on the device (plan_run, CUDA events on the stream the
            kernels run on), in G/s
  e2e       the same metric through the C-ABI call wavey_cuda_fdtd_run_batch
            with host buffers: packing, upload, run and read-back inside
  roofline  one time step (the TMA-fed interior kernel and, beside it, the
            special-cell/receiver kernel): 12 B per air-cell update per
            source (read p, read and write the older buffer) / the mean step
            span measured with CUDA events around each chunk's step launches
  plain     the same four right-hand sides run one at a time (S = 1 kernel)
  rooms_batch      the multi-room configuration (room_small's room with 32
            speakers plus four shoeboxes in one launch per step) against every
            right-hand side run alone
  reference_grid   the same room on the grid the reference's `--fdtd 500`
            builds by default (15 points per wavelength at 707 Hz, 72 M
            cells), a bounded prefix of its steps, untuned
  fp16_storage     FP16 field storage, autotuned, its error against FP64

Multi-GPU (--gpus N under torchrun): room_pillars is source-sharded -- rank r
runs speaker r's four right-hand sides on its own copy of the grid, with no
exchange on the data path; other workloads run as replicas.

Other workloads: room_hall (the 376 M-cell hall, 64 right-hand sides, a bounded prefix of its steps),
rooms_batch (room_small's room with 32 speakers plus four shoeboxes in one launch per step, against every
right-hand side run alone) and
room_pillars_32spk (the mixed-precision configuration: the pillar room with 32 seeded speakers = 71
right-hand sides; with --precision fp16 --ir-accuracy it reports the FP16-storage throughput and the error
of every mic impulse response and octave-band level against an FP64 GPU run of the same grid).

--impl reference times the reference's CPU algorithm (the oracle's C
restatement of fdtd::run_cpu, FP64, OpenMP over z-slabs as the reference's
rayon loop) on the host cores, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "FDTD Gcell-updates/s/source & HBM GB/s: batched vs plain, ≤0.1 dB vs FP64"
UNIT = "Gcell-updates/s"
BYTES_PER_UPDATE = 12  # FP32: read p^n, read p^(n-1), write p^(n+1)


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int = 0):
        self.device = self.smi_id(device)
        self.proc = None
        self.path = Path(tempfile.gettempdir()) / f"wavey_clocks_{os.getpid()}.csv"

    @staticmethod
    def smi_id(device: int) -> str:
        """nvidia-smi's id of the CUDA device: its PCI bus id.  nvidia-smi
        numbers GPUs in its own order and ignores CUDA_VISIBLE_DEVICES, so the
        CUDA ordinal could name another GPU of the machine."""
        try:
            import torch

            pr = torch.cuda.get_device_properties(device)
            return f"{pr.pci_domain_id:08X}:{pr.pci_bus_id:02X}:{pr.pci_device_id:02X}.0"
        except Exception:
            return str(device)

    def __enter__(self):
        self.f = None
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            if self.f is not None:
                self.f.close()
            self.path.unlink(missing_ok=True)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        text = self.path.read_text()
        self.path.unlink(missing_ok=True)
        for line in text.splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------- setup
def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if os.environ.get("WAVEY_BENCH_GLOO") is None else "gloo"
        if backend == "nccl":
            import torch

            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group(backend=backend)
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(v: float, world: int) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(workload: str, precision: str = "fp32"):
    """DRAM bytes per launch of the step kernel from the committed ncu summary."""
    f = ROOT / "profiles" / (f"fdtd_step_{workload}.md" if precision == "fp32" else f"fdtd_step_{workload}_{precision}.md")
    if not f.exists():
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", f.read_text())
    return float(m.group(1)) if m else None


def make_scene(workload: str, rank: int, args=None):
    from wavey_gb300 import workloads as W

    if workload == "room_pillars":
        # Source-sharded over ranks: rank r runs speaker r's four right-hand
        # sides on its own copy of the grid (rank 0 alone: room_pillars).
        world = int(os.environ.get("WORLD_SIZE", "1"))
        return W.room_pillars_shard(rank, world) if world > 1 else W.room_pillars(seed=2)
    if workload == "room_small":
        return W.room_small(seed=1)
    if workload == "room_pillars_32spk":
        # The mixed-precision configuration: room_pillars' room with 32 seeded
        # speakers (monopoles and cardioids), run with --precision fp16.
        return W.room_pillars_speakers(32)
    if workload == "room_hall":
        # 376 M cells: a full 2 s run is 34,641 steps; the throughput of a step
        # does not change along the run, so a bounded prefix is timed.
        sc = W.room_hall(speakers=args.hall_speakers if args else 16)
        steps = args.hall_steps if args else 384
        sc.signal = sc.signal[:steps]
        sc.notes["steps_timed"] = f"first {steps} of {W.math.ceil(2.0 / sc.grid.dt)} steps"
        return sc
    raise SystemExit(f"unknown workload {workload}")


# ------------------------------------------------------------ CPU baseline
def cpu_sample(scene, sample_steps: int, threads: int = 0):
    """Times the oracle (the reference's CPU loop) on the first sample_steps
    steps of one right-hand side with every receiver and frequency.  The time
    is the step loop's alone: the fields are allocated and first touched
    before the oracle starts its clock."""
    from oracle import fdtd as ofd

    sig = scene.signal[:sample_steps]
    ofd.run(scene.grid, scene.sources[0], sig, scene.receivers, scene.freqs, "f64", threads=threads)
    dt = ofd.last_loop_seconds()
    updates = scene.grid.air * sample_steps
    return updates / dt / 1e9, dt, ofd.max_threads() if threads == 0 else threads


def run_reference(args, rank, world):
    if rank != 0:
        return
    from oracle import build as obuild

    obuild.build()
    scene = make_scene(args.workload, 0, args)
    sample = args.sample_steps
    for _ in range(args.warmup):
        cpu_sample(scene, sample)
    vals, secs = [], []
    cores = 1
    for _ in range(args.steps):
        v, dt, cores = cpu_sample(scene, sample)
        vals.append(v)
        secs.append(dt)
    value = float(np.mean(vals))
    desc = (f"{args.workload}: 1 of {len(scene.sources)} right-hand sides, first {sample} of {scene.steps} steps, "
            f"all {len(scene.receivers)} receivers x {len(scene.freqs)} bins, FP64, step loop timed alone "
            f"(fields allocated and first touched before the clock starts)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(secs)), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "sample": desc},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "notes": "the reference is Rust + wgpu and cannot be built here (no cargo/rustc); its CPU loop "
                 "fdtd::run_cpu is timed through the oracle's C restatement on the host cores",
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------ many rooms
def rooms_leg(b, warmup: int, runs: int, plain: bool = True, clocks=None):
    """The multi-room configuration: room_small's room with 32 speakers plus
    four shoeboxes, every room with its own right-hand sides, signals and
    receivers, advanced together in one launch per time step
    (wavey_cuda_rooms_*), and (plain) every right-hand side run alone in a
    standalone plan of its own.  Returns the numbers and the timed seconds."""
    from wavey_gb300 import workloads as W
    from wavey_gb300.backend import FP32, RoomJob

    scenes = W.rooms_batch()
    jobs = [RoomJob(sc.grid, sc.sources, sc.signal, sc.receivers, sc.freqs) for sc in scenes]
    updates = sum(sc.grid.air * sc.steps * len(sc.sources) for sc in scenes)
    rhs = sum(len(sc.sources) for sc in scenes)
    p = b.rooms_plan(jobs)
    for _ in range(warmup):
        p.run()
    total_ms = 0.0
    for _ in range(runs):
        total_ms += p.run(stats=True)["total_ms"]
    info = p.info(0)
    steps = max(sc.steps for sc in scenes)
    launches = info["graph_kernels"] * (steps // 128) + (steps % 128 + 2 if steps % 128 else 0)
    p.close()
    t_plain = 0.0
    if plain:
        for sc in scenes:
            for src in sc.sources:
                q = b.plan(sc.grid, [src], sc.signal, sc.receivers, sc.freqs, FP32)
                q.run()
                t_plain += q.run(stats=True)["total_ms"] / 1e3
                q.close()
    value = updates * runs / (total_ms / 1e3) / 1e9
    plain_v = updates / t_plain / 1e9 if t_plain else None
    return {
        "value": value, "unit": UNIT, "per_source": value / rhs,
        "rooms": len(scenes), "right_hand_sides": rhs, "grids": [list(sc.grid.n) for sc in scenes],
        "time_steps": steps,
        "plain": plain_v, "batched_over_plain": None if plain_v is None else value / plain_v,
        "launches_per_run": int(launches),
        "note": "small grids (not HBM-bound); batched = all rooms in one launch per step, plain = each "
                "right-hand side in its own plan",
    }, total_ms / 1e3


def run_rooms(args, rank, world):
    """The multi-room configuration on its own (workload rooms_batch)."""
    from wavey_gb300 import _build

    _build.build()
    import torch

    from wavey_gb300.backend import CudaBackend

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    b = CudaBackend(dev)
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(dev) as clocks:
        leg, secs = rooms_leg(b, args.warmup, args.steps, plain=not args.no_plain)
    torch.cuda.synchronize()
    barrier(world)
    elapsed = max_over_ranks(secs, world)
    value = leg["value"] * secs * world / elapsed
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "rooms_batch", "rooms": leg["rooms"], "right_hand_sides": leg["right_hand_sides"],
                       "grids": leg["grids"], "time_steps": leg["time_steps"],
                       "l2": "small grids (not HBM-bound); no flush",
                       "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
            "per_source": value / leg["right_hand_sides"],
            "plain": {"value": leg["plain"],
                      "batched_over_plain": None if leg["plain"] is None else value / world / leg["plain"]},
            "roofline": None,
            "e2e": None,
            "cpu_baseline": None,
            "gpu_launches": int(leg["launches_per_run"] * args.steps),
            "clocks": clocks.summary(),
        }
        print(json.dumps(line), flush=True)
    b.close()


def reference_grid_leg(b, steps_timed: int):
    """room_pillars on the grid `wavey simulate --fdtd 500` builds by default
    (15 points per wavelength at f_c sqrt 2, ~72 M cells), FP32, untuned
    default shape, a bounded prefix of its 1.0 s run timed: the step's
    throughput does not change along the run."""
    from wavey_gb300 import workloads as W
    from wavey_gb300.backend import FP32

    sc = W.room_pillars(seed=2, reference_grid=True)
    full = sc.steps
    sig = sc.signal[:steps_timed]
    g = sc.grid
    p = b.plan(g, sc.sources, sig, sc.receivers, sc.freqs, FP32)
    p.run()
    st = p.run(stats=True)
    info = p.info()
    p.close()
    S = len(sc.sources)
    value = g.air * steps_timed * S / (st["total_ms"] / 1e3) / 1e9
    step_s = st["step_ms"] / 1e3 / st["step_launches"]
    peak, kind = peaks()
    achieved = BYTES_PER_UPDATE * g.air * S / step_s / 1e9
    return {"value": value, "unit": UNIT, "per_source": value / S, "grid": list(g.n), "air_cells": g.air,
            "ppw": 15.0, "grid_fmax_hz": sc.notes["grid_fmax"], "right_hand_sides": S,
            "steps_timed": f"first {steps_timed} of {full} steps", "step_us": step_s * 1e6,
            "roofline_frac": achieved / peak, "peak_kind": peak_kind_label(kind), "tma_zt": info["tma_zt"],
            "tma_depth": info["tma_depth"], "branch": info["branch"], "autotuned": False}


def peak_kind_label(kind: str) -> str:
    return "of measured" if kind == "measured" else "of fallback"


# ------------------------------------------------------------------ our arm
def run_ours(args, rank, world):
    from wavey_gb300 import _build

    _build.build()
    import torch

    from wavey_gb300.backend import FP32, FP64, CudaBackend
    from wavey_gb300 import workloads as W
    from wavey_gb300.fdtd import to_transfer

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    scene = make_scene(args.workload, rank, args)
    g = scene.grid
    if args.workload == "room_hall":
        # Memory check before allocating: fields, ring and spectra of the batch.
        free, _total = torch.cuda.mem_get_info()
        S_pad = -(-len(scene.sources) // 4) * 4
        need = 2 * (-(-g.n[0] // 32) * 32) * g.n[1] * g.n[2] * S_pad * 4 * 1.15
        if need > free:
            raise SystemExit(f"room_hall needs about {need / 1e9:.0f} GB of device memory, {free / 1e9:.0f} GB free")
        args.no_plain = args.no_e2e_big = True
        args.no_accuracy = args.no_cpu = args.no_autotune = True
        args.grid_build = True
    S = len(scene.sources)
    b = CudaBackend(dev)
    grid_build = None
    if getattr(args, "grid_build", False):
        # The grid build on the host (wh_grid_build, OpenMP) and on the device
        # (wavey_cuda_grid_build, arrays read back), identical arrays.
        from wavey_gb300.fdtd import FdtdGrid

        t0 = time.perf_counter()
        FdtdGrid.build_dx(scene.room, scene.fits, W.C_AIR, g.dx)
        t1 = time.perf_counter()
        gd = b.build_grid(scene.room, scene.fits, W.C_AIR, g.dx)
        t2 = time.perf_counter()
        same = bool(np.array_equal(gd.flags, g.flags) and np.array_equal(gd.slots, g.slots)
                    and np.array_equal(gd.bidx, g.bidx))
        del gd
        grid_build = {"cells": g.cells, "host_s": t1 - t0, "device_s": t2 - t1, "identical": same,
                      "host_threads": os.cpu_count()}
        log(f"[rank {rank}] grid build: host {t1 - t0:.2f} s, device {t2 - t1:.2f} s, identical {same}")
    name, sms = b.device_info()
    log(f"[rank {rank}] {name} ({sms} SMs): {scene.name} grid {g.n}, air {g.air}, {scene.steps} steps, S={S}, "
        f"{len(scene.receivers)} receivers x {len(scene.freqs)} bins")
    from wavey_gb300.backend import FP16_STORAGE

    main_precision = FP16_STORAGE if args.precision == "fp16" else FP32
    bytes_per_update = 6 if args.precision == "fp16" else BYTES_PER_UPDATE
    if args.precision == "fp16":
        args.no_fp16 = True  # the main leg is the FP16 one
    plan = b.plan(g, scene.sources, scene.signal, scene.receivers, scene.freqs, main_precision)
    tuned = plan.autotune() if not args.no_autotune else None
    if tuned:
        log(f"[rank {rank}] autotuned: rows {tuned['rows']}, rings {tuned['p_planes']}/{tuned['q_planes']}, "
            f"z-run {tuned['zt']}: {tuned['step_us']:.1f} us/step")
    info = plan.info()
    log(f"[rank {rank}] plan: {info}")
    for _ in range(args.warmup):
        plan.run()
    updates_per_run = g.air * scene.steps * S

    barrier(world)
    torch.cuda.synchronize()
    step_ms = 0.0
    launches = 0
    total_ms = 0.0
    chunks = 0
    with ClockSampler(dev) as clocks:
        for _ in range(args.steps):
            st = plan.run(stats=True)
            total_ms += st["total_ms"]
            step_ms += st["step_ms"]
            launches += st["step_launches"]
            chunks = st["chunks"]
    torch.cuda.synchronize()
    barrier(world)
    elapsed = max_over_ranks(total_ms / 1e3, world)
    value = updates_per_run * args.steps * world / elapsed / 1e9
    spec32 = plan.read()
    plan.close()  # frees its device memory before the other legs allocate theirs

    # Roofline of the fused step kernel.
    peak, peak_kind = peaks()
    launch_s = step_ms / 1e3 / launches
    alg_bytes = bytes_per_update * g.air * S
    achieved = alg_bytes / launch_s / 1e9
    traffic = profiled_traffic(args.workload, args.precision)

    # Plain: the same right-hand sides one at a time with the S = 1 kernel.
    plain = None
    if not args.no_plain:
        t_plain = 0.0
        for src in scene.sources:
            p1 = b.plan(g, [src], scene.signal, scene.receivers, scene.freqs, main_precision)
            p1.run()
            t_plain += p1.run(stats=True)["total_ms"] / 1e3
            p1.close()
        plain = updates_per_run / t_plain / 1e9

    # End to end through the C-ABI with host buffers.
    e2e_times = []
    for _ in range(0 if getattr(args, "no_e2e_big", False) else args.e2e_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.run_batch(g, scene.sources, scene.signal, scene.receivers, scene.freqs, main_precision)
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(float(np.median(e2e_times)), world) if e2e_times else None
    e2e = updates_per_run * world / e2e_s / 1e9 if e2e_s else None

    # Accuracy: FP32 against an FP64 GPU run of the same grid, as octave-band
    # levels of the directional source's combined transfer function.
    acc = None
    if not args.no_accuracy:
        p64 = b.plan(g, scene.sources, scene.signal, scene.receivers, scene.freqs, FP64)
        p64.run()
        spec64 = p64.read()
        p64.close()
        h0 = np.ones(len(scene.freqs), complex)
        t32 = np.stack([to_transfer(spec32[s], scene.signal, g, scene.freqs, W.C_AIR, 1.0, h0) for s in range(S)])
        t64 = np.stack([to_transfer(spec64[s], scene.signal, g, scene.freqs, W.C_AIR, 1.0, h0) for s in range(S)])
        if scene.weights:
            w = np.array(scene.weights)  # [nf, S]
            t32 = np.einsum("fs,srf->rf", w, t32)
            t64 = np.einsum("fs,srf->rf", w, t64)
        cent = [c for c in W.OCTAVES if c <= scene.crossover]
        l32 = W.octave_levels(t32, scene.freqs, cent)
        l64 = W.octave_levels(t64, scene.freqs, cent)
        acc = {"octave_band_max_abs_db": float(np.abs(l32 - l64).max()),
               "octave_bands_hz": cent,
               "spectra_worst_rel": float(np.abs(spec32 - spec64).max() / np.abs(spec64).max()),
               "reference": "FP64 GPU run of the same grid (WAVEY_FP64)"}

    # The receiver DFT with FP64 twiddles and FP64 chunk sums (the plan option
    # WAVEY_DFT_FP64=1), on the same shape: its cost and its effect.
    dft64 = None
    if not args.no_dft64 and main_precision == FP32 and world == 1:
        env = {"WAVEY_DFT_FP64": "1", "WAVEY_TMA_CFG": str(info["tma_depth"]), "WAVEY_TMA_ZT": str(info["tma_zt"]),
               "WAVEY_BRANCH": str(info["branch"])}
        saved = {k: os.environ.get(k) for k in env}
        os.environ.update(env)
        try:
            pd = b.plan(g, scene.sources, scene.signal, scene.receivers, scene.freqs, FP32)
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
        pd.run()
        rd = [pd.run(stats=True) for _ in range(2)]
        assert pd.info()["dft_fp64"] == 1
        specd = pd.read()
        pd.close()
        vd = updates_per_run / (sum(r["total_ms"] for r in rd) / len(rd) / 1e3) / 1e9
        dft64 = {"value": vd, "unit": UNIT, "cost_vs_fp32_sums": value / vd - 1.0,
                 "spectra_rel_change": float(np.abs(specd - spec32).max() / np.abs(spec32).max())}
        if acc is not None:
            dft64["spectra_worst_rel_vs_fp64"] = float(np.abs(specd - spec64).max() / np.abs(spec64).max())

    # Receiver impulse responses against an FP64 GPU run of the same grid
    # (the mixed-precision configuration): every right-hand side at every mic,
    # IR mode, and octave-band levels of the mics' spectra.
    ir_acc = None
    if args.ir_accuracy:
        mics = scene.receivers[:scene.notes.get("mics", len(scene.receivers))]
        out = {}
        for prec in (main_precision, FP64):
            pi = b.plan(g, scene.sources, scene.signal, mics, scene.freqs, prec, ir=True)
            pi.run()
            out[prec] = pi.read()
            pi.close()
        (spec_m, ir_m), (spec_d, ir_d) = out[main_precision], out[FP64]
        ir_peak = np.abs(ir_d).max(axis=-1)                   # [S][mics]
        rel = np.abs(ir_m - ir_d).max(axis=-1) / np.where(ir_peak > 0, ir_peak, 1.0)
        h0 = np.ones(len(scene.freqs), complex)
        tm = np.stack([to_transfer(spec_m[s], scene.signal, g, scene.freqs, W.C_AIR, 1.0, h0) for s in range(S)])
        td = np.stack([to_transfer(spec_d[s], scene.signal, g, scene.freqs, W.C_AIR, 1.0, h0) for s in range(S)])
        cent = [c for c in W.OCTAVES if c <= scene.crossover]

        def band_err(a, b):
            d = np.abs(W.octave_levels(a, scene.freqs, cent) - W.octave_levels(b, scene.freqs, cent))
            return {"worst": float(d.max()), "p99": float(np.quantile(d, 0.99)), "median": float(np.median(d)),
                    "per_band_worst": [float(x) for x in d.reshape(-1, len(cent)).max(axis=0)]}

        ir_acc = {"precision": args.precision, "reference": "FP64 GPU run of the same grid (WAVEY_FP64)",
                  "impulse_responses": int(rel.size), "mics": len(mics), "right_hand_sides": S,
                  "ir_max_abs_err_over_peak": {"worst": float(rel.max()), "p99": float(np.quantile(rel, 0.99)),
                                               "median": float(np.median(rel))},
                  "octave_bands_hz": cent,
                  "octave_band_abs_db_per_rhs": band_err(tm, td)}
        if scene.notes.get("speaker_rhs"):
            # Each speaker's transfer function: its right-hand sides combined
            # with its component weights (a monopole's is its one RHS).
            def speakers(t):
                return np.stack([np.einsum("fc,crf->rf", np.array(w), t[a:a + n])
                                 for (a, n), w in zip(scene.notes["speaker_rhs"], scene.notes["speaker_weights"])])
            ir_acc["speakers"] = len(scene.notes["speaker_rhs"])
            ir_acc["octave_band_abs_db_per_speaker"] = band_err(speakers(tm), speakers(td))
        log(f"[rank {rank}] IR accuracy vs FP64: {ir_acc}")

    # FP16 field storage: throughput and its error against the FP64 run.
    fp16 = None
    if not args.no_fp16:
        from wavey_gb300.backend import FP16_STORAGE

        p16 = b.plan(g, scene.sources, scene.signal, scene.receivers, scene.freqs, FP16_STORAGE)
        tuned16 = p16.autotune() if not args.no_autotune else None
        p16.run()
        runs16 = [p16.run(stats=True) for _ in range(2)]
        info16 = p16.info()
        spec16 = p16.read()
        p16.close()
        ms16 = sum(r["total_ms"] for r in runs16) / len(runs16)
        step16 = sum(r["step_ms"] for r in runs16) / sum(r["step_launches"] for r in runs16)
        fp16 = {"value": updates_per_run / (ms16 / 1e3) / 1e9, "unit": UNIT,
                "bytes_per_update": 6,
                "step_us": 1e3 * step16,
                "runs_timed": len(runs16),
                "kernel": ("interior_tma<__half> (TMA-fed z-march over FP16 planes) || fdtd_step_half special/record"
                           if info16["interior_kernel"] else "fdtd_step_half (fused, register-queue z-march)"),
                "autotuned": None if not tuned16 else {k: tuned16[k] for k in ("rows", "p_planes", "q_planes", "zt",
                                                                             "branch")}}
        if acc is not None:
            h0 = np.ones(len(scene.freqs), complex)
            t16 = np.stack([to_transfer(spec16[s], scene.signal, g, scene.freqs, W.C_AIR, 1.0, h0) for s in range(S)])
            t64b = np.stack([to_transfer(spec64[s], scene.signal, g, scene.freqs, W.C_AIR, 1.0, h0) for s in range(S)])
            if scene.weights:
                t16 = np.einsum("fs,srf->rf", np.array(scene.weights), t16)
                t64b = np.einsum("fs,srf->rf", np.array(scene.weights), t64b)
            cent = [c for c in W.OCTAVES if c <= scene.crossover]
            d = np.abs(W.octave_levels(t16, scene.freqs, cent) - W.octave_levels(t64b, scene.freqs, cent))
            fp16["octave_band_max_abs_db"] = float(d.max())
            fp16["octave_band_p99_abs_db"] = float(np.quantile(d, 0.99))
            fp16["spectra_worst_rel"] = float(np.abs(spec16 - spec64).max() / np.abs(spec64).max())

    # CPU baseline (rank 0 at N = 1): the oracle on a bounded sample.
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle import build as obuild

        obuild.build()
        v, dt, cores = cpu_sample(scene, args.sample_steps)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"1 right-hand side, first {args.sample_steps} steps, all receivers and bins, FP64, "
                         f"{dt:.1f} s of step loop (fields allocated and first touched before the clock starts)"}

    # Config 3 (many rooms in one launch per step) and the reference's own
    # default --fdtd grid of this room, as extra keys of the same line.
    rooms = refgrid = None
    if world == 1 and args.workload == "room_pillars":
        if not args.no_rooms:
            rooms, _ = rooms_leg(b, warmup=1, runs=2, plain=not args.no_plain)
        if not args.no_refgrid:
            refgrid = reference_grid_leg(b, args.refgrid_steps)

    kernels_per_run = info["graph_kernels"] * (scene.steps // 128) + (scene.steps % 128 + 2 if scene.steps % 128 else 0)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if args.precision == "fp32" else "f32 arithmetic, f16 field storage", "data": "synthetic",
            "config": {"workload": scene.name, "grid": list(g.n), "air_cells": g.air, "time_steps": scene.steps,
                       "right_hand_sides": S, "receivers": len(scene.receivers), "freq_bins": len(scene.freqs),
                       "batched": True,
                       "l2": "fields 2x%.0f MB > L2 (no flush needed)" % (
                           info["padded_nx"] * g.n[1] * g.n[2] * info["lanes"] * info["chunks"] * 4 / 1e6),
                       "parallelism": (f"source-sharded x{world}: rank r runs speaker r's right-hand sides, "
                                       f"no data-path exchange" if world > 1 and args.workload == "room_pillars"
                                       else f"replicas x{world}" if world > 1 else "1 GPU"),
                       "autotuned": None if not tuned else {k: tuned[k] for k in ("rows", "p_planes", "q_planes", "zt",
                                                                                  "branch", "step_us")}},
            "per_source": value / S,
            "plain": {"value": plain, "per_source": None if plain is None else plain / S,
                      "batched_over_plain": None if plain is None else value / world / plain},
            "hbm_gbs": achieved,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": ("step = interior_tma || fdtd_step special/record branch" if info["interior_kernel"]
                                    else "fdtd_step<float,4> (fused)"),
                         "bytes_per_launch": alg_bytes, "mean_launch_us": launch_s * 1e6},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": info["h2d_bytes"],
                    "d2h_bytes_per_step": info["d2h_bytes"], "seconds": e2e_s},
            "accuracy": acc,
            "ir_accuracy": ir_acc,
            "fp16_storage": fp16,
            "dft_fp64": dft64,
            "rooms_batch": rooms,
            "reference_grid": refgrid,
            "grid_build": grid_build,
            "cpu_baseline": cpu,
            "gpu_launches": int(kernels_per_run * args.steps),
            "clocks": clocks.summary(),
        }
        print(json.dumps(line), flush=True)
    plan.close()
    b.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="room_pillars")
    ap.add_argument("--sample-steps", type=int, default=300)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp16", action="store_true")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp16"],
                    help="field storage of the main timed leg (fp16: FP16 storage, FP32 arithmetic)")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-rooms", action="store_true", help="leave out the multi-room key (rooms_batch)")
    ap.add_argument("--no-dft64", action="store_true", help="leave out the FP64-accumulation key (dft_fp64)")
    ap.add_argument("--no-refgrid", action="store_true", help="leave out the reference-default-grid key")
    ap.add_argument("--refgrid-steps", type=int, default=384)
    ap.add_argument("--hall-steps", type=int, default=384)
    ap.add_argument("--hall-speakers", type=int, default=16)
    ap.add_argument("--ir-accuracy", action="store_true",
                    help="impulse responses of every right-hand side at the mics and their octave-band levels "
                         "against an FP64 GPU run (IR mode)")
    args = ap.parse_args()
    if args.warmup < 3:
        log("warm-up raised to 3 (timing rule)")
        args.warmup = 3
    rank, world = dist_init()
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "rooms_batch":
        run_rooms(args, rank, world)
    else:
        run_ours(args, rank, world)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
