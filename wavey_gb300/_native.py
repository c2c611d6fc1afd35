"""ctypes bindings of libwavey_cuda.so and libwavey_host.so.

The structs mirror include/wavey_cuda.h and include/wavey_host.h field by
field.  Loading fails loudly when a library is missing: there is no Python
or CPU fallback for the CUDA path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB = Path(__file__).resolve().parent / "_lib"

c_double_p = C.POINTER(C.c_double)
c_int64_p = C.POINTER(C.c_int64)
c_uint32_p = C.POINTER(C.c_uint32)
c_uint8_p = C.POINTER(C.c_uint8)
c_uint64_p = C.POINTER(C.c_uint64)

WAVEY_OK = 0
WAVEY_CANCELLED = 1
WAVEY_E_INVALID = -1
WAVEY_E_LIMIT = -2
WAVEY_E_CUDA = -3
WAVEY_E_NOMEM = -4
WAVEY_E_DEVICE = -5

WAVEY_FP32 = 0
WAVEY_FP64 = 1
WAVEY_FP16_STORAGE = 2

# include/wavey_cuda.h: frequency limit of wavey_cuda_receiver_dft_noalloc
WAVEY_NOALLOC_MAX_FREQS = 2048

WH_MAX_BRANCHES = 4
WH_FIT_DIRECTIONS = 400


# ----------------------------------------------------------------- host lib
class WhSpectrum(C.Structure):
    _fields_ = [("n", C.c_int32), ("value", C.c_double), ("freqs_hz", c_double_p), ("values", c_double_p)]


class WhFit(C.Structure):
    _fields_ = [
        ("beta0", C.c_double),
        ("n_branches", C.c_int32),
        ("r", C.c_double * WH_MAX_BRANCHES),
        ("m", C.c_double * WH_MAX_BRANCHES),
        ("k", C.c_double * WH_MAX_BRANCHES),
        ("band_lo", C.c_double),
        ("band_hi", C.c_double),
        ("rms_error", C.c_double),
        ("max_error", C.c_double),
    ]


class WhRoom(C.Structure):
    _fields_ = [
        ("x0", C.c_double), ("y0", C.c_double), ("x1", C.c_double), ("y1", C.c_double),
        ("height", C.c_double),
        ("n_pillars", C.c_int32), ("pillars", c_double_p),
        ("n_blocks", C.c_int32), ("blocks", c_double_p),
        ("n_solids", C.c_int32), ("solids", c_double_p),
    ]


class WhGridView(C.Structure):
    _fields_ = [
        ("nx", C.c_int64), ("ny", C.c_int64), ("nz", C.c_int64),
        ("origin", C.c_double * 3),
        ("dx", C.c_double), ("dt", C.c_double),
        ("flags", c_uint8_p), ("bidx", c_uint32_p),
        ("n_boundary", C.c_int64),
        ("bcell", c_uint32_p), ("bstart", c_uint32_p), ("slots", c_double_p),
        ("n_slots", C.c_int64), ("air_cells", C.c_int64),
    ]


# ----------------------------------------------------------------- cuda lib
class WaveyGrid(C.Structure):
    _fields_ = [
        ("nx", C.c_int64), ("ny", C.c_int64), ("nz", C.c_int64),
        ("dx", C.c_double), ("dt", C.c_double),
        ("flags", c_uint8_p), ("bidx", c_uint32_p),
        ("n_boundary", C.c_int64),
        ("bstart", c_uint32_p), ("slots", c_double_p),
    ]


class WaveyTap(C.Structure):
    _fields_ = [("cell", C.c_int64), ("w", C.c_double)]


class WaveySource(C.Structure):
    _fields_ = [("taps", C.POINTER(WaveyTap)), ("n_taps", C.c_size_t)]


class WaveyRoomJob(C.Structure):
    _fields_ = [
        ("grid", C.POINTER(WaveyGrid)), ("sources", C.POINTER(WaveySource)), ("n_sources", C.c_size_t),
        ("signals", c_double_p), ("signal_stride", C.c_size_t), ("steps", C.c_size_t),
        ("receivers", c_uint64_p), ("n_recv", C.c_size_t), ("freqs", c_double_p), ("nf", C.c_size_t),
        ("out", c_double_p), ("ir_out", c_double_p),
    ]


class WaveyRunStats(C.Structure):
    _fields_ = [("total_ms", C.c_double), ("step_ms", C.c_double), ("step_launches", C.c_int64), ("chunks", C.c_int64)]


class WaveyPlanInfo(C.Structure):
    _fields_ = [
        ("cells", C.c_int64), ("air_cells", C.c_int64), ("interior_cells", C.c_int64),
        ("special_cells", C.c_int64), ("boundary_slots", C.c_int64),
        ("sources", C.c_int64), ("lanes", C.c_int64), ("chunks", C.c_int64),
        ("receivers", C.c_int64), ("freqs", C.c_int64), ("steps", C.c_int64),
        ("device_bytes", C.c_int64), ("padded_nx", C.c_int64), ("precision", C.c_int32),
        ("h2d_bytes", C.c_int64), ("d2h_bytes", C.c_int64), ("graph_kernels", C.c_int64),
        ("interior_kernel", C.c_int32), ("tma_zt", C.c_int32), ("tma_depth", C.c_int32), ("branch", C.c_int32),
        ("dft_fp64", C.c_int32), ("two_step", C.c_int32), ("two_step_rows", C.c_int32), ("two_step_zt", C.c_int32),
        ("programmatic", C.c_int32),
    ]


WAVEY_TUNE_MAX = 512
WAVEY_IR_INTEGRATE = 1
WAVEY_IR_LUNDEBY = 2


class WaveyTuneResult(C.Structure):
    _fields_ = [
        ("cfg", C.c_int32), ("zt", C.c_int32), ("rows", C.c_int32), ("p_planes", C.c_int32), ("q_planes", C.c_int32),
        ("branch", C.c_int32), ("step_us", C.c_double), ("candidates", C.c_int32),
        ("cand_cfg", C.c_int32 * WAVEY_TUNE_MAX), ("cand_zt", C.c_int32 * WAVEY_TUNE_MAX),
        ("cand_branch", C.c_int32 * WAVEY_TUNE_MAX), ("cand_step_us", C.c_double * WAVEY_TUNE_MAX),
    ]


class WaveyTransferLayout(C.Structure):
    _fields_ = [
        ("n_speakers", C.c_int32), ("lane_speaker", C.POINTER(C.c_int32)), ("factor", C.POINTER(C.c_double)),
        ("n_mics", C.c_int64), ("n_planes", C.c_int32), ("plane_points", C.POINTER(C.c_int64)),
    ]


class WaveyGridShape(C.Structure):
    _fields_ = [("n", C.c_int64 * 3), ("origin", C.c_double * 3), ("dx", C.c_double), ("dt", C.c_double),
                ("air_cells", C.c_int64), ("n_boundary", C.c_int64), ("n_slots", C.c_int64)]


PROGRESS_FN = C.CFUNCTYPE(None, C.c_double, C.c_void_p)

_host = None
_cuda = None


def _load(name: str) -> C.CDLL:
    path = _LIB / name
    if not path.exists():
        raise RuntimeError(
            f"{path} is missing: build the native libraries first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    return C.CDLL(str(path))


def host() -> C.CDLL:
    global _host
    if _host is not None:
        return _host
    L = _load("libwavey_host.so")
    sig = {
        "wh_spectrum_eval": (C.c_double, [C.POINTER(WhSpectrum), C.c_double]),
        "wh_fit_real_impedance": (C.c_double, [C.c_double]),
        "wh_fit_absorption": (C.c_double, [C.POINTER(WhFit), C.c_double]),
        "wh_fit_admittance_at": (None, [C.POINTER(WhFit), C.c_double, c_double_p]),
        "wh_fit_admittance": (C.c_int, [C.POINTER(WhSpectrum), C.c_double, C.c_double, C.c_int32, C.POINTER(WhFit)]),
        "wh_room_surface_count": (C.c_int32, [C.POINTER(WhRoom)]),
        "wh_room_contains": (C.c_int, [C.POINTER(WhRoom), c_double_p]),
        "wh_grid_build": (C.c_int, [C.POINTER(WhRoom), C.POINTER(WhFit), C.c_int32, C.c_double, C.c_double,
                                    C.POINTER(C.c_void_p)]),
        "wh_grid_spacing": (C.c_double, [C.POINTER(WhRoom), C.c_double, C.c_double, C.c_double]),
        "wh_mesh_room_build": (C.c_int, [c_double_p, C.c_int64, c_uint32_p, c_int64_p, C.POINTER(C.c_int32),
                                         C.c_int64, C.POINTER(C.c_void_p)]),
        "wh_mesh_room_free": (None, [C.c_void_p]),
        "wh_mesh_room_surface_count": (C.c_int32, [C.c_void_p]),
        "wh_mesh_room_triangle_count": (C.c_int64, [C.c_void_p]),
        "wh_mesh_room_surface": (None, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                        c_double_p, c_double_p, c_double_p]),
        "wh_mesh_room_triangles": (None, [C.c_void_p, c_double_p, c_uint32_p]),
        "wh_mesh_room_bounds": (None, [C.c_void_p, c_double_p, c_double_p]),
        "wh_mesh_room_contains": (C.c_int, [C.c_void_p, c_double_p]),
        "wh_mesh_room_volume": (C.c_double, [C.c_void_p]),
        "wh_grid_build_mesh": (C.c_int, [C.c_void_p, c_double_p, C.c_int32, C.POINTER(WhFit), C.c_int32,
                                         C.c_double, C.c_double, C.POINTER(C.c_void_p)]),
        "wh_grid_view_of": (None, [C.c_void_p, C.POINTER(WhGridView)]),
        "wh_grid_free": (None, [C.c_void_p]),
        "wh_grid_alloc": (C.c_int, [c_int64_p, c_double_p, C.c_double, C.c_double, C.c_int64, C.c_int64, C.c_int64,
                                    C.POINTER(C.c_void_p)]),
        "wh_grid_arrays": (None, [C.c_void_p, C.POINTER(C.POINTER(C.c_uint8)), C.POINTER(C.POINTER(C.c_uint32)),
                                  C.POINTER(C.POINTER(C.c_uint32)), C.POINTER(C.POINTER(C.c_uint32)),
                                  C.POINTER(C.POINTER(C.c_double))]),
        "wh_nearest_air": (C.c_int64, [C.c_void_p, c_double_p]),
        "wh_taps_at": (C.c_int32, [C.c_void_p, c_double_p, c_int64_p, c_double_p]),
        "wh_source_components": (C.c_int32, [C.c_void_p, C.c_int64, C.c_int32, c_int64_p, c_double_p,
                                             C.POINTER(C.c_int32)]),
        "wh_baffle_point": (None, [C.c_void_p, c_double_p, c_double_p, c_double_p]),
        "wh_air_along": (C.c_int64, [C.c_void_p, c_double_p, c_double_p]),
        "wh_source_signal": (None, [C.c_double, C.c_double, C.c_int64, c_double_p]),
        "wh_frequency_grid": (C.c_int32, [C.c_double, C.c_double, C.c_int32, c_double_p, C.c_int32]),
        "wh_crossover_weight": (C.c_double, [C.c_double, C.c_double]),
        "wh_phase_error_deg_per_m": (C.c_double, [C.c_double, C.c_double, C.c_double]),
        "wh_auto_duration": (C.c_double, [c_double_p, C.c_int32]),
        "wh_to_transfer": (None, [c_double_p, C.c_int64, c_double_p, C.c_int64, C.c_double, C.c_double, c_double_p,
                                  C.c_int64, C.c_double, C.c_double, c_double_p, c_double_p]),
        "wh_blend": (None, [c_double_p, c_double_p, C.c_double, c_double_p]),
        "wh_fit_directions": (None, [c_double_p]),
        "wh_fit_first_order": (None, [c_double_p, c_double_p, c_double_p, c_double_p, c_double_p]),
        "wh_component_weights": (None, [c_double_p, c_double_p, C.c_double, C.c_double, c_double_p]),
        "wh_speaker_rotation": (None, [C.c_double, C.c_double, C.c_double, c_double_p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _host = L
    return L


def cuda() -> C.CDLL:
    global _cuda
    if _cuda is not None:
        return _cuda
    L = _load("libwavey_cuda.so")
    vp = C.c_void_p
    cancel_p = C.POINTER(C.c_int32)
    sig = {
        "wavey_cuda_create": (C.c_int, [C.c_int, C.POINTER(vp)]),
        "wavey_cuda_destroy": (None, [vp]),
        "wavey_cuda_last_error": (C.c_char_p, [vp]),
        "wavey_cuda_device_info": (C.c_int, [vp, C.c_char_p, C.c_size_t, C.POINTER(C.c_int)]),
        "wavey_cuda_fdtd_run": (C.c_int, [vp, C.POINTER(WaveyGrid), C.POINTER(WaveyTap), C.c_size_t, c_double_p,
                                          C.c_size_t, c_uint64_p, C.c_size_t, c_double_p, C.c_size_t, c_double_p,
                                          c_double_p, cancel_p, PROGRESS_FN, vp]),
        "wavey_cuda_fdtd_run_batch": (C.c_int, [vp, C.POINTER(WaveyGrid), C.POINTER(WaveySource), C.c_size_t,
                                                c_double_p, C.c_size_t, C.c_size_t, c_uint64_p, C.c_size_t,
                                                c_double_p, C.c_size_t, C.c_int32, c_double_p, c_double_p, cancel_p,
                                                PROGRESS_FN, vp]),
        "wavey_cuda_plan_create": (C.c_int, [vp, C.POINTER(WaveyGrid), C.POINTER(WaveySource), C.c_size_t,
                                             c_double_p, C.c_size_t, C.c_size_t, c_uint64_p, C.c_size_t, c_double_p,
                                             C.c_size_t, C.c_int32, C.c_int32, C.POINTER(vp)]),
        "wavey_cuda_plan_run": (C.c_int, [vp, cancel_p, PROGRESS_FN, vp, C.POINTER(WaveyRunStats)]),
        "wavey_cuda_plan_read": (C.c_int, [vp, c_double_p, c_double_p]),
        "wavey_cuda_plan_info": (C.c_int, [vp, C.POINTER(WaveyPlanInfo)]),
        "wavey_cuda_plan_destroy": (None, [vp]),
        "wavey_cuda_plan_autotune": (C.c_int, [vp, C.POINTER(WaveyTuneResult)]),
        "wavey_cuda_plan_transfers": (C.c_int, [vp, C.POINTER(WaveyTransferLayout), C.POINTER(C.c_float),
                                                C.c_size_t]),
        "wavey_cuda_plan_band_params": (C.c_int, [vp, c_double_p, C.c_int32, C.c_int32, c_double_p, C.c_size_t]),
        "wavey_cuda_grid_build": (C.c_int, [vp, C.POINTER(WhRoom), C.POINTER(WhFit), C.c_int32, C.c_double, C.c_double,
                                            C.POINTER(vp), C.POINTER(WaveyGridShape)]),
        "wavey_cuda_grid_build_mesh": (C.c_int, [vp, c_double_p, c_uint32_p, C.c_int64, c_double_p, C.c_int32,
                                                 C.POINTER(WhFit), C.c_int32, C.c_double, C.c_double,
                                                 C.POINTER(C.c_void_p), C.POINTER(WaveyGridShape)]),
        "wavey_cuda_grid_read": (C.c_int, [vp, C.POINTER(C.c_uint8), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                           C.POINTER(C.c_uint32), c_double_p]),
        "wavey_cuda_grid_free": (None, [vp]),
        "wavey_cuda_fdtd_run_rooms": (C.c_int, [vp, C.POINTER(WaveyRoomJob), C.c_size_t, C.c_int32, cancel_p,
                                                PROGRESS_FN, vp]),
        "wavey_cuda_rooms_create": (C.c_int, [vp, C.POINTER(WaveyRoomJob), C.c_size_t, C.c_int32, C.c_int32,
                                              C.POINTER(vp)]),
        "wavey_cuda_rooms_run": (C.c_int, [vp, cancel_p, PROGRESS_FN, vp, C.POINTER(WaveyRunStats)]),
        "wavey_cuda_rooms_read": (C.c_int, [vp, C.c_size_t, c_double_p, c_double_p]),
        "wavey_cuda_rooms_info": (C.c_int, [vp, C.c_size_t, C.POINTER(WaveyPlanInfo)]),
        "wavey_cuda_rooms_destroy": (None, [vp]),
        "wavey_cuda_receiver_dft_noalloc": (C.c_int, [C.c_int, C.POINTER(C.c_float), C.c_int64, C.c_int64, c_double_p,
                                                      C.c_int64, C.c_double, c_double_p, vp, C.c_char_p, C.c_size_t]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _cuda = L
    return L


def ptr(a, ctype):
    """Pointer to a contiguous numpy array's data (None for None)."""
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))
