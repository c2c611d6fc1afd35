/*
 * wavey_cuda.h -- C-ABI of libwavey_cuda.so, the GB300 (sm_103a) backend of
 * Wavey's FDTD wave solver.
 *
 * It replaces the wgpu backend `Gpu::run_fdtd` (core/wavey-solver/src/
 * gpu_fdtd.rs:45-277, shaders core/wavey-solver/src/fdtd.wgsl:44-135) behind
 * the same contract as its CPU twin `fdtd::run_cpu` (core/wavey-solver/src/
 * fdtd.rs:616-626) and the `GridRunner` type (fdtd.rs:884-885):
 *
 *     (grid, source taps, signal, receiver cells, freqs) -> spectra
 *
 * with spectra receiver-major, [receiver][freq] complex.  The scheme, grid
 * and Courant conventions are the reference's: p^n is recorded before the
 * update, the update overwrites the older buffer in place, taps are added
 * after the update, lambda = 1/sqrt(3).
 *
 * Status codes are those of wavey_status.h: WAVEY_OK, WAVEY_CANCELLED (the
 * reference's Ok(None)), or a negative code (the reference's Err(String));
 * the message is available from wavey_cuda_last_error().  There is no CPU
 * fallback: a missing or failing device is an error.
 *
 * Threading: a context serialises its calls with a mutex; use one context
 * per thread for concurrent runs.  All host buffers are borrowed for the
 * duration of a call and never retained.
 */
#ifndef WAVEY_CUDA_H
#define WAVEY_CUDA_H

#include <stddef.h>
#include <stdint.h>

#include "wavey_host.h"

#include "wavey_status.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct wavey_cuda_ctx wavey_cuda_ctx;
typedef struct wavey_cuda_plan wavey_cuda_plan;

/* The voxelised room, `FdtdGrid` (fdtd.rs:196-209) with its boundary nodes
 * flattened to CSR exactly as the reference packs them for the GPU
 * (gpu_fdtd.rs:82-88), but in FP64. */
typedef struct {
    int64_t nx, ny, nz;        /* cells per axis, x fastest: (z*ny + y)*nx + x */
    double dx, dt;             /* spacing (m) and time step (s) */
    const uint8_t *flags;      /* [cells] bit 6 air, bits 0-5 air neighbour -x,+x,-y,+y,-z,+z */
    const uint32_t *bidx;      /* [cells] boundary node index or 0xFFFFFFFF */
    int64_t n_boundary;
    const uint32_t *bstart;    /* [n_boundary + 1] slot range of each boundary node */
    const double *slots;       /* [bstart[n_boundary]][4] = inv_d, cv, k, w */
} wavey_grid;

/* A source tap (usize, f64). */
typedef struct {
    int64_t cell;
    double w;
} wavey_tap;

/* One right-hand side of a batched run: a source component's taps. */
typedef struct {
    const wavey_tap *taps;
    size_t n_taps;
} wavey_source;

/* Storage precision of the fields. */
#define WAVEY_FP32 0          /* FP32 throughout, the reference GPU's arithmetic order */
#define WAVEY_FP64 1          /* FP64 throughout, the reference CPU's order: the GPU oracle */
#define WAVEY_FP16_STORAGE 2  /* fields stored in FP16 with a power-of-two scale per z slab; FP32 updates,
                                 FP32 branch states, FP64 spectra */

/* Per-run timing, filled when a stats pointer is given (the run then waits
 * for each 128-step chunk to read its events). */
typedef struct {
    double total_ms;          /* whole run on the device stream */
    double step_ms;           /* summed span of the fused step launches */
    int64_t step_launches;
    int64_t chunks;
} wavey_run_stats;

typedef struct {
    int64_t cells, air_cells, interior_cells, special_cells, boundary_slots;
    int64_t sources, lanes, chunks;       /* lanes per cell in a chunk: 1, 2 or 4 */
    int64_t receivers, freqs, steps;
    int64_t device_bytes;                 /* device memory held by the plan */
    int64_t padded_nx;
    int32_t precision;
    int64_t h2d_bytes;                    /* host-to-device bytes of plan_create */
    int64_t d2h_bytes;                    /* device-to-host bytes of plan_read */
    int64_t graph_kernels;                /* kernels per replay of the 128-step graph */
    int32_t interior_kernel;              /* 1: TMA-fed z-march beside the special-cell kernel; 0: fused step kernel */
    int32_t tma_zt;                       /* z planes per CTA of the TMA kernel */
    int32_t tma_depth;                    /* shape of the TMA kernel, rows/p ring/old ring: 0: 8/6/4, 1: 8/8/4,
                                             2: 16/6/4, 3: 16/8/4, 4: 16/5/3, 5: 32/5/3, 6: 32/4/2; FP32
                                             plans also 7-13: the same shapes with registers capped for
                                             three resident CTAs per SM (-1: no TMA kernel) */
    int32_t branch;                       /* form of the special-cell branch beside it (see wavey_tune_result) */
    int32_t dft_fp64;                     /* 1: receiver DFT with FP64 twiddles and FP64 sums over each 128-step
                                             chunk (FP64 plans, and FP32 / FP16 plans created with
                                             WAVEY_DFT_FP64=1 in the environment); 0: FP32 chunk sums added
                                             into the FP64 spectra */
    int32_t two_step;                     /* 1: two steps per pass over the fields (FP32, four sources per chunk,
                                             created with WAVEY_TBLOCK=1): interior_tb2 beside the special-cell
                                             kernel, then the shell and special cells of the second step */
    int32_t two_step_rows, two_step_zt;   /* its output rows per tile and z-run */
    int32_t programmatic;                 /* 1: each step's interior kernel is a programmatic dependent of the
                                             previous step (FP32 plans where one interior wave and a special-cell
                                             block fit on every SM together; WAVEY_PDL=0 turns it off) */
} wavey_plan_info;

int wavey_cuda_create(int device, wavey_cuda_ctx **out);
void wavey_cuda_destroy(wavey_cuda_ctx *ctx);
const char *wavey_cuda_last_error(const wavey_cuda_ctx *ctx);
/* Name and SM count of the context's device. */
int wavey_cuda_device_info(wavey_cuda_ctx *ctx, char *name, size_t name_cap, int *sm_count);

/* Gpu::run_fdtd (gpu_fdtd.rs:45-54): one source, FP32.  out is
 * [n_recv][nf][2] (re, im); ir_out (nullable) receives the time series
 * [n_recv][steps] that `run_cpu_ir` (fdtd.rs:630-641) records.  cancel
 * (nullable) is polled and progress (nullable) called once per 128 steps. */
int wavey_cuda_fdtd_run(wavey_cuda_ctx *ctx, const wavey_grid *grid, const wavey_tap *taps, size_t n_taps,
                        const double *signal, size_t steps, const uint64_t *receivers, size_t n_recv,
                        const double *freqs, size_t nf, double *out, double *ir_out, const volatile int32_t *cancel,
                        void (*progress)(double, void *), void *user);

/* S right-hand sides on one grid in one launch per step (source-interleaved
 * fields).  signals is [S][signal_stride] with signal_stride >= steps, or a
 * single signal shared by every source when signal_stride == 0.  out is
 * [S][n_recv][nf][2]; ir_out (nullable) is [S][n_recv][steps]. */
int wavey_cuda_fdtd_run_batch(wavey_cuda_ctx *ctx, const wavey_grid *grid, const wavey_source *sources,
                              size_t n_sources, const double *signals, size_t signal_stride, size_t steps,
                              const uint64_t *receivers, size_t n_recv, const double *freqs, size_t nf,
                              int32_t precision, double *out, double *ir_out, const volatile int32_t *cancel,
                              void (*progress)(double, void *), void *user);

/* Device-resident form of wavey_cuda_fdtd_run_batch: plan_create uploads
 * and packs the inputs, plan_run runs (repeatable; each run starts from rest),
 * plan_read copies the last run's results to the host. */
int wavey_cuda_plan_create(wavey_cuda_ctx *ctx, const wavey_grid *grid, const wavey_source *sources, size_t n_sources,
                           const double *signals, size_t signal_stride, size_t steps, const uint64_t *receivers,
                           size_t n_recv, const double *freqs, size_t nf, int32_t precision, int32_t want_ir,
                           wavey_cuda_plan **out);
int wavey_cuda_plan_run(wavey_cuda_plan *plan, const volatile int32_t *cancel, void (*progress)(double, void *),
                        void *user, wavey_run_stats *stats);
int wavey_cuda_plan_read(wavey_cuda_plan *plan, double *out, double *ir_out);
int wavey_cuda_plan_info(const wavey_cuda_plan *plan, wavey_plan_info *info);

/* Per-speaker transfer functions straight from a plan's device spectra, in
 * the transfer section of results.bin (result.rs:444-456): complex64, mics
 * first as [mic][speaker][f], then each plane as [speaker][point][f] -- the
 * plan's receivers must be the mics followed by the planes' inside points
 * in plane order (run.rs:380-392).  Speaker s's transfer is the sum over its
 * right-hand sides of factor[lane][f] x spectrum[lane][r][f] (the factor
 * carries the component weight, to_transfer's scale and the cabinet
 * calibration, run.rs:631-660), summed in FP64 on the device; only the
 * complex64 result crosses to the host.  Replaces reading every right-hand
 * side's FP64 spectra and combining them on the host (Gpu::run_fdtd's
 * Spectra, then to_transfer per component); no counterpart call in the
 * reference. */
typedef struct {
    int32_t n_speakers;
    const int32_t *lane_speaker;  /* [plan sources]: speaker of each right-hand side, -1 to leave it out */
    const double *factor;         /* [plan sources][nf][2] complex factor per right-hand side and frequency */
    int64_t n_mics;               /* receivers [0, n_mics) are mics */
    int32_t n_planes;
    const int64_t *plane_points;  /* [n_planes] inside points per plane, after the mics, in order */
} wavey_transfer_layout;
int wavey_cuda_plan_transfers(wavey_cuda_plan *plan, const wavey_transfer_layout *layout, float *out,
                              size_t out_floats);

/* ISO 3382-1 band parameters of a plan's receiver time series, computed on
 * the device (core/wavey-solver/src/analysis.rs), for IR-mode plans
 * (want_ir): per right-hand side, receiver and band -- octave band-pass
 * (six biquads forward and backward, analysis.rs:143-183) of the series
 * from the broadband onset (analysis.rs:185-189), Schroeder integration,
 * EDT, T20, T30, C80, D50 and centre time (analysis.rs:266-325).  Only these
 * numbers cross to the host, not the series.  Replaces reading the series
 * (run_cpu_ir) and calling octave_filter / band_params per receiver and band
 * on the host (bras_wave.rs:46-58); no counterpart call in the reference.
 * flags: WAVEY_IR_INTEGRATE analyses the running sum of the series (the
 * response to the source pulse's integral, bras_wave.rs:46-52);
 * WAVEY_IR_LUNDEBY truncates and compensates the noise tail
 * (energy_params, analysis.rs:291-294) instead of integrating all of it
 * (noise_free_params).  out: [source][receiver][band][6] = edt, t20, t30 (s),
 * c80 (dB), d50, ts (s); NaN where undefined.  1 to 64 bands, each below
 * fs / 2 = 1 / (2 dt). */
#define WAVEY_IR_INTEGRATE 1
#define WAVEY_IR_LUNDEBY 2
int wavey_cuda_plan_band_params(wavey_cuda_plan *plan, const double *bands_hz, int32_t n_bands, int32_t flags,
                                double *out, size_t out_doubles);

/* FdtdGrid::build_dx (fdtd.rs:289-378) on the device: the same
 * classification, neighbour flags, face lookup and boundary slots as
 * wh_grid_build, computed per cell on the GPU (boundary nodes numbered in
 * cell order by a scan), for rooms whose host build takes seconds (the
 * 376 M-cell hall).  The arrays are identical to wh_grid_build's.  Two
 * steps: wavey_cuda_grid_build leaves the grid on the device and reports its
 * shape; wavey_cuda_grid_read copies it into host arrays of that shape (e.g.
 * those of wh_grid_alloc / wh_grid_arrays).  No counterpart in the
 * reference, whose grid build is CPU-only. */
typedef struct wavey_device_grid wavey_device_grid;
typedef struct {
    int64_t n[3];
    double origin[3];
    double dx, dt;
    int64_t air_cells, n_boundary, n_slots;
} wavey_grid_shape;
int wavey_cuda_grid_build(wavey_cuda_ctx *ctx, const wh_room *room, const wh_fit *fits, int32_t n_fits, double c,
                          double dx, wavey_device_grid **out, wavey_grid_shape *shape);
/* The same for a room imported as a mesh (FdtdGrid::build_dx's mesh branch:
 * column_fill, fdtd.rs:385-422, one thread per grid column, and the closest
 * triangle behind each missing face): positions [n_tri][3][3] and
 * tri_surface [n_tri] as wh_mesh_room_triangles gives them, optional rigid
 * boxes solids [n_solids][6], one fit per surface.  Identical to
 * wh_grid_build_mesh.  WAVEY_E_LIMIT if a grid column crosses the mesh more
 * than 128 times. */
int wavey_cuda_grid_build_mesh(wavey_cuda_ctx *ctx, const double *positions, const uint32_t *tri_surface,
                               int64_t n_tri, const double *solids, int32_t n_solids, const wh_fit *fits, int32_t n_fits,
                               double c, double dx, wavey_device_grid **out, wavey_grid_shape *shape);
int wavey_cuda_grid_read(wavey_device_grid *grid, uint8_t *flags, uint32_t *bidx, uint32_t *bcell, uint32_t *bstart,
                         double *slots);
void wavey_cuda_grid_free(wavey_device_grid *grid);

/* Autotuner of a plan's step kernels (FP32 plans of at least 256 steps).
 * Stage 1 times every shape of the interior kernel -- tile rows (8, 16 or 32)
 * with ring depths, and z planes per CTA (8, 16, 32 and the runs that cut
 * the planes into one to eight equal z-tiles) -- each with special-cell forms
 * 3 and 8 (below) beside it; stage 2 times, with that shape,
 * every form of the special-cell update: forms 0-8 run it in a concurrent
 * kernel, with its register cap (branch / 3: 1, 3 or 4 blocks per SM) and
 * launch priority (branch % 3: equal, special cells first, interior first);
 * form 9 (FP32 plans) has every interior CTA update the special cells of its
 * own tile from the planes it stages, with only the receiver samples on the
 * concurrent kernel.  If form 9 wins, stage 3 times every interior shape
 * again with it.  Each candidate runs three 128-step chunks of the plan's own
 * grid (the last two timed; two chunks, one timed, for plans of under 384
 * steps); stage 4 times the four fastest again over up
 * to four chunks each (plans of at least 640 steps), and the plan keeps the
 * fastest of those.  result->step_us is the winner's last timing.
 * result (nullable) lists the candidates' first step times (every candidate: at
 * most 14 shapes x 11 z-runs x 2 families, 9 other forms and the fused
 * form's 154 shapes, 471 in all).  Neither stage changes any arithmetic.
 * Other plans are left as they are. */
#define WAVEY_TUNE_MAX 512
typedef struct {
    int32_t cfg, zt, rows, p_planes, q_planes, branch;
    double step_us;
    int32_t candidates;
    int32_t cand_cfg[WAVEY_TUNE_MAX], cand_zt[WAVEY_TUNE_MAX], cand_branch[WAVEY_TUNE_MAX];
    double cand_step_us[WAVEY_TUNE_MAX];
} wavey_tune_result;
int wavey_cuda_plan_autotune(wavey_cuda_plan *plan, wavey_tune_result *result);
void wavey_cuda_plan_destroy(wavey_cuda_plan *plan);

/* Several rooms in one launch per time step: the rooms' step blocks are laid
 * end to end in one grid (a work-tile table; each block finds its room), so
 * rooms of uneven sizes, each with its own right-hand sides, signals,
 * receivers and step count, fill the GPU together.  It replaces running
 * `GridRunner` once per room (fdtd.rs:884-885; e.g. the per-cabinet
 * calibration pairs of fdtd.rs:941-942).  FP32 or FP64. */
typedef struct wavey_cuda_rooms wavey_cuda_rooms;
typedef struct {
    const wavey_grid *grid;
    const wavey_source *sources;
    size_t n_sources;
    const double *signals;     /* as wavey_cuda_fdtd_run_batch */
    size_t signal_stride;
    size_t steps;
    const uint64_t *receivers;
    size_t n_recv;
    const double *freqs;
    size_t nf;
    double *out;               /* [S][n_recv][nf][2], written by wavey_cuda_fdtd_run_rooms */
    double *ir_out;            /* nullable [S][n_recv][steps] */
} wavey_room_job;

int wavey_cuda_fdtd_run_rooms(wavey_cuda_ctx *ctx, const wavey_room_job *jobs, size_t n_jobs, int32_t precision,
                              const volatile int32_t *cancel, void (*progress)(double, void *), void *user);
int wavey_cuda_rooms_create(wavey_cuda_ctx *ctx, const wavey_room_job *jobs, size_t n_jobs, int32_t precision,
                            int32_t want_ir, wavey_cuda_rooms **out);
int wavey_cuda_rooms_run(wavey_cuda_rooms *rooms, const volatile int32_t *cancel, void (*progress)(double, void *),
                         void *user, wavey_run_stats *stats);
int wavey_cuda_rooms_read(wavey_cuda_rooms *rooms, size_t room, double *out, double *ir_out);
int wavey_cuda_rooms_info(const wavey_cuda_rooms *rooms, size_t room, wavey_plan_info *info);
void wavey_cuda_rooms_destroy(wavey_cuda_rooms *rooms);

/* Receiver spectra from receiver time series, allocating no device memory.
 * No counterpart in the reference: it exists for callers that cannot
 * allocate device memory when they need the spectra, such as a real-time
 * audio thread (cudaMalloc/cudaFree can stall the device) or a host whose
 * own pool allocator owns all device memory.
 *
 * series (device, [n_recv][steps] FP32) holds p^n per receiver, freqs
 * (device, [nf]) the bins, out (device, [n_recv][nf][2] FP64) receives
 * sum_n p^n exp(-j 2 pi frac(f dt n)), the running DFT of fdtd.rs:673-683,
 * computed as the FDTD runs compute it (FP32 sums over 128-step chunks added
 * into FP64).  stream may be NULL (the default stream).  At most
 * WAVEY_NOALLOC_MAX_FREQS frequencies (WAVEY_E_LIMIT beyond).  err (nullable)
 * receives a message on failure.
 *
 * Scratch is one fixed 2 MiB array inside the library (every GPU that loads
 * the library holds it until exit).  The first call on a device looks up
 * that array's device address, so make it before any stream capture; after
 * a device reset (cudaDeviceReset) the next call looks it up again, so make
 * that call before any capture too.  All calls share the array.  A call
 * queues all of its kernels under one process-wide lock, so calls from
 * several host threads on one stream do not interleave; calls on different
 * streams whose kernels overlap on the GPU race and must be serialised by
 * the caller. */
#define WAVEY_NOALLOC_MAX_FREQS 2048
int wavey_cuda_receiver_dft_noalloc(int device, const float *series, int64_t n_recv, int64_t steps, const double *freqs,
                                    int64_t nf, double dt, double *out, void *stream, char *err, size_t err_cap);

#ifdef __cplusplus
}
#endif
#endif
