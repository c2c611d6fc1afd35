// wavey_cuda.cu -- libwavey_cuda.so: the C-ABI backend that replaces
// `Gpu::run_fdtd` (core/wavey-solver/src/gpu_fdtd.rs:45-277).
//
// Host side of a run:
//   1. validate the grid, taps and receivers (the reference's limit checks,
//      gpu_fdtd.rs:56-66, become error codes; indices are checked here so no
//      kernel ever sees an out-of-range cell);
//   2. pack: the interior mask and the compacted special-cell list on the
//      padded device layout, slot constants, merged taps (gpu_fdtd.rs:67-75),
//      signals and receivers, in the run's precision;
//   3. capture one 128-step chunk (128 fused step launches, the chunk's
//      twiddles and DFT, the optional time-series copy, and the step-counter
//      advance) into a CUDA graph, and replay it steps/128 times; the
//      remaining steps are launched directly;
//   4. read the FP64 spectra (and time series) back.
// The reference's blocking poll per 128-step submit (gpu_fdtd.rs:254-259)
// becomes an event wait only when a cancel flag, a progress callback or
// statistics are requested.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <memory>
#include <string>
#include <thread>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "../../include/wavey_cuda.h"
#include "fdtd_half.cuh"
#include "fdtd_kernels.cuh"
#include "interior_tma.cuh"
#include "ir_analysis.cuh"
#include "tblock.cuh"
#include "grid_build.cuh"

namespace {

constexpr double COURANT = 0.5773502691896257;  // fdtd.rs:138
constexpr uint64_t MAX_CELLS = 600000000ull;      // fdtd.rs:140
constexpr uint32_t NO_BOUNDARY = 0xFFFFFFFFu;
constexpr uint8_t AIR = 64;
constexpr int ZT = 16;  // z planes marched by one interior CTA of the fused step kernel (default)

// cuTensorMapEncodeTiled, fetched from the driver once (no link-time
// dependency on libcuda).
using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_tiled() {
    static EncodeTiled fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
        cudaGetLastError();
    });
    return fn;
}

// Interior kernel variant of FP32 runs: the TMA-fed z-march (default) or the
// register-queue z-march inside the fused step kernel.
bool tma_selected() {
    const char *v = getenv("WAVEY_INTERIOR");
    return !(v && strcmp(v, "regq") == 0);
}

int env_int(const char *name, int dflt, int lo, int hi) {
    const char *v = getenv(name);
    if (!v) return dflt;
    int x = atoi(v);
    return x < lo ? lo : (x > hi ? hi : x);
}

// Threads of the host-side loops (grid packing, conversions, reordering the
// spectra): every hardware thread, or WAVEY_HOST_THREADS.  Set per loop, so
// an OpenMP default inherited from the process (often 1) does not serialise
// them.
int host_threads() {
    static const int n = env_int("WAVEY_HOST_THREADS", std::max(1, (int)std::thread::hardware_concurrency()), 1, 256);
    return n;
}

}  // namespace

struct wavey_cuda_ctx {
    int device = 0;
    int sm_count = 0;
    int max_persist_l2 = 0;     // bytes of L2 that may be set aside for persisting accesses
    int64_t regs_per_sm = 0, smem_per_sm = 0, smem_reserved = 0, threads_per_sm = 0;
    int max_window = 0;         // largest access-policy window
    size_t l2_bytes = 0;        // L2 size
    size_t persist_set = 0;     // persisting set-aside now in force
    const void *persist_owner = nullptr;  // the plan whose set-aside and lines are in force
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;  // the special-cell branch of a TMA step
    cudaStream_t folds = nullptr; // the previous chunk's receiver fold, beside a chunk's steps
    std::mutex mu;
    std::string err;
    char name[256] = {0};

    int fail(int code, const char *fmt, ...) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        err = buf;
        return code;
    }
    int cuda(cudaError_t e, const char *what) {
        if (e == cudaSuccess) return WAVEY_OK;
        return fail(e == cudaErrorMemoryAllocation ? WAVEY_E_NOMEM : WAVEY_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
    }
};

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

struct wavey_cuda_plan {
    wavey_cuda_ctx *ctx = nullptr;
    int precision = WAVEY_FP32;
    int V = 1;
    int chunks = 1;
    int n_sources = 0;
    int lanes_total = 0;
    int64_t nx = 0, ny = 0, nz = 0, nxp = 0, cells = 0, cells_p = 0;
    int64_t air = 0, interior = 0, n_special = 0, n_slots = 0;
    int64_t steps = 0, n_recv = 0, nf = 0;
    bool want_ir = false;
    double dt = 0.0;
    std::vector<DevBuf> bufs;
    // device pointers
    void *field[2] = {nullptr, nullptr};
    uint32_t *mask = nullptr, *recv = nullptr;
    uint4 *sp = nullptr;
    void *slots = nullptr, *su = nullptr, *sg = nullptr, *tapw = nullptr, *sig = nullptr, *ring = nullptr, *tw = nullptr,
         *ir = nullptr;
    double *acc = nullptr, *freqs = nullptr;
    long long *base = nullptr;
    int64_t sig_stride = 0;
    size_t field_bytes = 0, state_bytes = 0, acc_bytes = 0, ir_bytes = 0;
    size_t elem = 4;        // bytes of the arithmetic type (slots, states, ring, spectra inputs)
    size_t field_elem = 4;  // bytes of a stored field value (2 in FP16 storage)
    unsigned int *amax = nullptr;  // FP16 storage: slab maxima ring
    float2 *scale = nullptr;       // FP16 storage: slab scale ring
    int fp16_shift = 14;           // FP16 storage: the slab bound maps just below 2^shift
    float *wmax = nullptr;         // FP16 storage: sum |tap weight| per source
    // launch geometry
    int tiles_x = 0, tiles_y = 0, tiles_z = 0;
    int zt = ZT;  // z planes per interior CTA of the fused step kernel
    int interior_blocks = 0, special_blocks = 0, record_blocks = 0;
    cudaGraphExec_t graph = nullptr;
    int64_t graph_kernels = 0;  // kernel launches per replay of the chunk graph
    // TMA interior path (FP32)
    bool tma = false;
    CUtensorMap tm_p[2], tm_q[2];  // per parity: p^n of field[parity], old of field[parity^1]
    int tma_tiles_x = 0, tma_tiles_y = 0, tma_tiles_z = 0, tma_zt = 32, tma_blocks = 0;
    int tma_cfg = 0;      // shape of the TMA kernel, an index into TMA_CFGS
    bool zalt = true;     // alternate the interior's z-march direction from step to step
    // Two receiver rings used by alternate chunks: each chunk's graph folds
    // the previous chunk's ring on the fold stream beside its own steps.
    bool fold_overlap = false;
    int64_t ring_stride = 0;  // elements between the two rings
    cudaEvent_t ev_ffork = nullptr, ev_fjoin = nullptr;
    bool pdl = false;     // interior launched as a programmatic dependent of the previous step (FP32)
    bool pdl_wanted = false;
    // Two steps per pass (FP32, four sources per chunk): two more field
    // buffers for p^(n+1) and p^(n+2), the deep-cell mask, the shell list and
    // the pass's tensor maps (per pair parity) and geometry.
    bool tb2 = false;
    void *field2[2] = {nullptr, nullptr};
    uint32_t *deep = nullptr, *shell = nullptr;
    int64_t n_shell = 0;
    CUtensorMap tb_p[2], tb_q[2];
    int tb_cfg = 0, tb_rows = 0, tb_zt = 0, tb_tiles_x = 0, tb_tiles_y = 0, tb_tiles_z = 0, tb_blocks = 0;
    int branch = 0;             // special-cell form: branch < 9: a concurrent kernel with register cap
                                // (branch / 3) and priority (branch % 3); BRANCH_FUSED: inside the interior CTAs
    std::vector<uint4> sp_host;   // special records in cell order (host copy, for the tile orders)
    // The special cells' records, slot constants and branch states in one
    // block, kept resident in L2 across steps by a persisting access-policy
    // window on the special-cell kernel (the field streams would otherwise
    // evict them every step).
    bool dft64 = false;  // FP32 / FP16 plans: receiver DFT with FP64 twiddles and chunk sums
    void *l2_block = nullptr;
    size_t l2_block_bytes = 0;
    cudaAccessPolicyWindow l2_window = {};
    size_t l2_setaside = 0;   // persisting set-aside this plan asks for
    uint4 *sp_tile[3] = {nullptr, nullptr, nullptr};     // per tile height 8, 16, 32: records by (tile, plane)
    uint32_t *sp_off[3] = {nullptr, nullptr, nullptr};   // and the first record of each (tile, plane)
    int prio_lo = 0, prio_hi = 0;
    int *err = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t ev_a = nullptr, ev_b = nullptr, ev_t0 = nullptr, ev_t1 = nullptr;
    cudaEvent_t inflight[4] = {nullptr, nullptr, nullptr, nullptr};
    bool ran = false;
    int64_t device_bytes = 0;
    int64_t h2d_bytes = 0;  // bytes uploaded by plan_create

    ~wavey_cuda_plan() {
        if (graph) cudaGraphExecDestroy(graph);
        // Lines of the freed special block would keep their persisting state.
        if (ctx && ctx->persist_owner == this) {
            cudaCtxResetPersistingL2Cache();
            ctx->persist_owner = nullptr;
        }
        for (cudaEvent_t e : {ev_a, ev_b, ev_t0, ev_t1, inflight[0], inflight[1], inflight[2], inflight[3], ev_fork, ev_join,
                              ev_ffork, ev_fjoin})
            if (e) cudaEventDestroy(e);
        for (DevBuf &b : bufs)
            if (b.p) cudaFree(b.p);
    }
};

// Several rooms advanced together: their plans (buffers and packing), one
// shared step counter, the device table of RoomStep entries and one graph per
// 128-step chunk whose step launches cover every room's blocks.
// A grid built on the device (wavey_cuda_grid_build).
struct wavey_device_grid {
    wavey_cuda_ctx *ctx = nullptr;
    wavey_grid_shape shape{};
    uint8_t *flags = nullptr;
    uint32_t *bidx = nullptr, *bcell = nullptr, *bstart = nullptr;
    double *slots = nullptr;
};

struct wavey_cuda_rooms {
    wavey_cuda_ctx *ctx = nullptr;
    int precision = WAVEY_FP32;
    std::vector<wavey_cuda_plan *> plans;
    long long *base = nullptr;
    void *table = nullptr;
    int total_blocks = 0;
    int64_t max_steps = 0;
    cudaGraphExec_t graph = nullptr;
    int64_t graph_kernels = 0;
    cudaEvent_t ev_a = nullptr, ev_b = nullptr, ev_t0 = nullptr, ev_t1 = nullptr;
    bool ran = false;

    ~wavey_cuda_rooms() {
        if (graph) cudaGraphExecDestroy(graph);
        for (cudaEvent_t e : {ev_a, ev_b, ev_t0, ev_t1})
            if (e) cudaEventDestroy(e);
        if (base) cudaFree(base);
        if (table) cudaFree(table);
        for (wavey_cuda_plan *p : plans) delete p;
    }
};

namespace {

template <class T>
int alloc(wavey_cuda_plan *pl, T **out, size_t bytes) {
    void *p = nullptr;
    size_t b = std::max<size_t>(bytes, 16);
    cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return pl->ctx->fail(WAVEY_E_NOMEM, "device allocation of %zu bytes failed: %s", b, cudaGetErrorString(e));
    }
    pl->bufs.push_back({p, b});
    pl->device_bytes += (int64_t)b;
    *out = reinterpret_cast<T *>(p);
    return WAVEY_OK;
}

template <class T>
int upload(wavey_cuda_plan *pl, T **out, const void *host, size_t bytes) {
    int st = alloc(pl, out, bytes);
    if (st) return st;
    pl->h2d_bytes += (int64_t)bytes;
    if (bytes) return pl->ctx->cuda(cudaMemcpyAsync(*out, host, bytes, cudaMemcpyHostToDevice, pl->ctx->stream), "upload");
    return WAVEY_OK;
}

inline int64_t round_up(int64_t v, int64_t m) { return (v + m - 1) / m * m; }

int validate_grid(wavey_cuda_ctx *ctx, const wavey_grid *g) {
    if (!g) return ctx->fail(WAVEY_E_INVALID, "grid is null");
    if (g->nx < 3 || g->ny < 3 || g->nz < 3) return ctx->fail(WAVEY_E_INVALID, "grid must be at least 3 cells per axis");
    const uint64_t cells = (uint64_t)g->nx * (uint64_t)g->ny * (uint64_t)g->nz;
    if (cells > MAX_CELLS)
        return ctx->fail(WAVEY_E_LIMIT, "the wave solver grid would have %.0f M cells; lower the crossover frequency",
                         cells / 1e6);
    if (!g->flags || !g->bidx) return ctx->fail(WAVEY_E_INVALID, "grid flags/bidx are null");
    if (!(g->dt > 0.0) || !(g->dx > 0.0)) return ctx->fail(WAVEY_E_INVALID, "grid dx/dt must be positive");
    if (g->n_boundary < 0 || (g->n_boundary > 0 && (!g->bstart || !g->slots)))
        return ctx->fail(WAVEY_E_INVALID, "grid boundary arrays are null");
    if (g->n_boundary >= (1ll << 31)) return ctx->fail(WAVEY_E_LIMIT, "too many boundary nodes");
    if (g->n_boundary > 0) {
        if (g->bstart[0] != 0) return ctx->fail(WAVEY_E_INVALID, "bstart[0] must be 0");
        for (int64_t b = 0; b < g->n_boundary; b++) {
            if (g->bstart[b + 1] < g->bstart[b]) return ctx->fail(WAVEY_E_INVALID, "bstart is not ascending at %lld", (long long)b);
            if (g->bstart[b + 1] - g->bstart[b] > wk::META_SLOT_MASK)
                return ctx->fail(WAVEY_E_LIMIT, "boundary node %lld has more than %u slots", (long long)b, wk::META_SLOT_MASK);
        }
    }
    return WAVEY_OK;
}

template <class T>
void fill_args(wavey_cuda_plan *pl, wk::StepArgs<T> &a, int parity) {
    a.cur = reinterpret_cast<const T *>(pl->field[parity]);
    a.nxt = reinterpret_cast<T *>(pl->field[parity ^ 1]);
    a.out = a.nxt;
    a.interior = pl->mask;
    a.sp = pl->sp;
    a.slots = reinterpret_cast<const T *>(pl->slots);
    a.su = reinterpret_cast<T *>(pl->su);
    a.sg = reinterpret_cast<T *>(pl->sg);
    a.tapw = reinterpret_cast<const T *>(pl->tapw);
    a.sig = reinterpret_cast<const T *>(pl->sig);
    a.recv = pl->recv;
    a.ring = reinterpret_cast<T *>(pl->ring);
    a.ring_stride = pl->ring_stride;
    a.base = pl->base;
    a.cells_p = pl->cells_p;
    a.sig_stride = pl->sig_stride;
    a.nxp = (int)pl->nxp;
    a.ny = (int)pl->ny;
    a.nz = (int)pl->nz;
    a.nxw = (int)(pl->nxp / 32);
    a.n_special = (int)pl->n_special;
    a.n_slots = (int)pl->n_slots;
    a.n_recv = (int)pl->n_recv;
    a.chunks = pl->chunks;
    a.lanes_total = pl->lanes_total;
    a.tiles_x = pl->tiles_x;
    a.tiles_y = pl->tiles_y;
    a.tiles_z = pl->tiles_z;
    a.zt = pl->zt;
    a.interior_blocks = pl->interior_blocks;
    a.special_blocks = pl->special_blocks;
    a.record_blocks = pl->record_blocks;
    a.l2 = (T)(COURANT * COURANT);
    a.lam = (T)COURANT;
    a.half_dt = (T)0.5 * (T)pl->dt;
}

template <class T, int V, bool RUST>
void launch_step(wavey_cuda_plan *pl, int t, int parity) {
    wk::StepArgs<T> a;
    fill_args<T>(pl, a, parity);
    const int blocks = pl->interior_blocks + pl->special_blocks + pl->record_blocks;
    if (blocks > 0) wk::fdtd_step<T, V, RUST><<<blocks, wk::BLOCK, 0, pl->ctx->stream>>>(a, t);
}

// Shapes of the TMA interior kernel: rows per tile, ring depths and the
// register policy of FP32 kernels (the launch bounds' minimum resident CTAs:
// 1 lets ptxas take up to 90 registers in the 16-row shapes, two CTAs per SM
// with room for a special-cell block beside them; 3 caps them for three CTAs
// per SM and more bytes in flight).  Shapes 7-13 are 0-6 with the second
// policy; FP16 and fused (SPEC) kernels have one policy, shapes 0-6.
struct TmaCfg {
    int rows, np, nq, lb;
};
constexpr TmaCfg TMA_CFGS[] = {{8, 6, 4, 1},  {8, 8, 4, 1},  {16, 6, 4, 1}, {16, 8, 4, 1}, {16, 5, 3, 1},
                               {32, 5, 3, 1}, {32, 4, 2, 1}, {8, 6, 4, 3},  {8, 8, 4, 3},  {16, 6, 4, 3},
                               {16, 8, 4, 3}, {16, 5, 3, 3}, {32, 5, 3, 3}, {32, 4, 2, 3}};
constexpr int TMA_NCFG = 14;
constexpr int TMA_NCFG_ONE_POLICY = 7;
// Special-cell form in which the interior CTAs update the special cells of
// their tiles (FP32 plans); forms 0-8 run them in a concurrent kernel.
constexpr int BRANCH_FUSED = 9;

// Index of a tile height (8, 16 or 32 rows) in the plan's tile-ordered special lists.
inline int tile_slot(int rows) { return rows == 8 ? 0 : rows == 16 ? 1 : 2; }

// One instantiation of the TMA kernel: its entry and dynamic shared memory.
struct TmaKernel {
    const void *fn;
    uint32_t smem;
};

template <class E, int V, int R, int NP, int NQ, bool SPEC, int LB>
TmaKernel tma_kernel_of() {
    return {(const void *)wk::interior_tma<E, V, R, NP, NQ, SPEC, LB>, wk::tma_smem_of<E, R, NP, NQ, SPEC>()};
}

// The kernel of shape cfg (TMA_CFGS).  FP16 and fused kernels have one
// register policy: their shapes 7-13 are shapes 0-6.
template <class E, int V, bool SPEC>
TmaKernel tma_kernel(int cfg) {
    constexpr bool two_policies = sizeof(E) == 4 && !SPEC;
    constexpr int L1 = sizeof(E) == 2 ? 0 : 1;
    if constexpr (two_policies) {
        switch (cfg) {
            case 7: return tma_kernel_of<E, V, 8, 6, 4, SPEC, 3>();
            case 8: return tma_kernel_of<E, V, 8, 8, 4, SPEC, 3>();
            case 9: return tma_kernel_of<E, V, 16, 6, 4, SPEC, 3>();
            case 10: return tma_kernel_of<E, V, 16, 8, 4, SPEC, 3>();
            case 11: return tma_kernel_of<E, V, 16, 5, 3, SPEC, 3>();
            case 12: return tma_kernel_of<E, V, 32, 5, 3, SPEC, 3>();
            case 13: return tma_kernel_of<E, V, 32, 4, 2, SPEC, 3>();
            default: break;
        }
    }
    switch (cfg % TMA_NCFG_ONE_POLICY) {
        case 1: return tma_kernel_of<E, V, 8, 8, 4, SPEC, L1>();
        case 2: return tma_kernel_of<E, V, 16, 6, 4, SPEC, L1>();
        case 3: return tma_kernel_of<E, V, 16, 8, 4, SPEC, L1>();
        case 4: return tma_kernel_of<E, V, 16, 5, 3, SPEC, L1>();
        case 5: return tma_kernel_of<E, V, 32, 5, 3, SPEC, L1>();
        case 6: return tma_kernel_of<E, V, 32, 4, 2, SPEC, L1>();
        default: return tma_kernel_of<E, V, 8, 6, 4, SPEC, L1>();
    }
}

// pdl: launched as a programmatic dependent of the stream's previous work
// (its CTAs may be scheduled while the previous step drains; the kernel
// waits for it before touching the fields).
template <class E, int V, bool SPEC>
void launch_tma_cfg(int cfg, int blocks, cudaStream_t s, int prio, const CUtensorMap &p, const CUtensorMap &q,
                    const wk::TmaArgs<E> &ta, const wk::SpecTile &sp, bool pdl = false) {
    const TmaKernel k = tma_kernel<E, V, SPEC>(cfg);
    cudaLaunchConfig_t lc = {};
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributePriority;
    attr[0].val.priority = prio;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    lc.gridDim = dim3(blocks);
    lc.blockDim = dim3(256);
    lc.dynamicSmemBytes = k.smem;
    lc.stream = s;
    lc.attrs = attr;
    lc.numAttrs = pdl ? 2 : 1;
    void *args[] = {const_cast<CUtensorMap *>(&p), const_cast<CUtensorMap *>(&q), const_cast<wk::TmaArgs<E> *>(&ta),
                    const_cast<wk::SpecTile *>(&sp)};
    cudaLaunchKernelExC(&lc, k.fn, args);
}

template <class E, int V>
cudaError_t tma_attrs() {
    for (int cfg = 0; cfg < TMA_NCFG; cfg++) {
        const TmaKernel k = tma_kernel<E, V, false>(cfg);
        cudaError_t e = cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem);
        if (e != cudaSuccess) return e;
        if constexpr (sizeof(E) == 4) {
            const TmaKernel f = tma_kernel<E, V, true>(cfg);
            e = cudaFuncSetAttribute(f.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)f.smem);
            if (e != cudaSuccess) return e;
        }
    }
    return cudaSuccess;
}

// The TMA kernel's arguments for one step (FP16 fields are unused in FP32).
template <class E>
wk::TmaArgs<E> tma_args(const wavey_cuda_plan *pl, int t, int parity) {
    wk::TmaArgs<E> ta;
    ta.interior = pl->mask;
    ta.nxt = reinterpret_cast<E *>(pl->field[parity ^ 1]);
    ta.error = pl->err;
    ta.cells_p = pl->cells_p;
    ta.nxp = (int)pl->nxp;
    ta.ny = (int)pl->ny;
    ta.nz = (int)pl->nz;
    ta.nxw = (int)(pl->nxp / 32);
    ta.tiles_x = pl->tma_tiles_x;
    ta.tiles_y = pl->tma_tiles_y;
    ta.tiles_z = pl->tma_tiles_z;
    ta.zt = pl->tma_zt;
    ta.rev = pl->zalt ? (parity & 1) : 0;
    ta.l2 = (float)(COURANT * COURANT);
    ta.base = pl->base;
    ta.t = t;
    ta.chunks = pl->chunks;
    ta.scale = pl->scale;
    ta.amax = pl->amax;
    return ta;
}

template <int V>
void launch_step_tma(wavey_cuda_plan *pl, int t, int parity) {
    cudaStream_t s = pl->ctx->stream, side = pl->ctx->side;
    const bool fused = pl->branch == BRANCH_FUSED;
    const bool branch = (fused ? 0 : pl->special_blocks) + pl->record_blocks > 0;
    wk::SpecTile sp = {};
    if (fused) {
        const int slot = tile_slot(TMA_CFGS[pl->tma_cfg].rows);
        sp.rec = pl->sp_tile[slot];
        sp.off = pl->sp_off[slot];
        fill_args<float>(pl, sp.a, parity);
    }
    if (branch) {
        // Special cells and receiver samples on a concurrent branch (the fused
        // kernel's special and record roles): they read only p^n and write
        // cells the interior kernel does not touch.
        cudaEventRecord(pl->ev_fork, s);
        cudaStreamWaitEvent(side, pl->ev_fork, 0);
        wk::StepArgs<float> a;
        fill_args<float>(pl, a, parity);
        a.interior_blocks = 0;
        cudaLaunchConfig_t lc = {};
        cudaLaunchAttribute attr[2];
        attr[0].id = cudaLaunchAttributePriority;
        attr[0].val.priority = pl->branch % 3 == 1 ? pl->prio_hi : pl->prio_lo;
        attr[1].id = cudaLaunchAttributeAccessPolicyWindow;
        attr[1].val.accessPolicyWindow = pl->l2_window;
        lc.blockDim = dim3(wk::BLOCK);
        lc.stream = side;
        lc.attrs = attr;
        lc.numAttrs = pl->l2_window.num_bytes ? 2 : 1;
        if (fused) a.special_blocks = 0;  // receivers only: the special cells run inside the interior CTAs
        lc.gridDim = dim3(a.special_blocks + pl->record_blocks);
        switch (fused ? 0 : pl->branch / 3) {
            case 1: cudaLaunchKernelEx(&lc, wk::special_branch<V, 3>, a, t); break;
            case 2: cudaLaunchKernelEx(&lc, wk::special_branch<V, 4>, a, t); break;
            default: cudaLaunchKernelEx(&lc, wk::special_branch<V, 1>, a, t); break;
        }
    }
    if (pl->tma_blocks > 0 && fused)
        launch_tma_cfg<float, V, true>(pl->tma_cfg, pl->tma_blocks, s, pl->prio_lo, pl->tm_p[parity], pl->tm_q[parity],
                                       tma_args<float>(pl, t, parity), sp);
    else if (pl->tma_blocks > 0)
        launch_tma_cfg<float, V, false>(pl->tma_cfg, pl->tma_blocks, s, pl->branch % 3 == 2 ? pl->prio_hi : pl->prio_lo,
                                        pl->tm_p[parity], pl->tm_q[parity], tma_args<float>(pl, t, parity), sp,
                                        pl->pdl && t > 0);
    if (branch) {
        cudaEventRecord(pl->ev_join, side);
        cudaStreamWaitEvent(s, pl->ev_join, 0);
    }
}

// Shapes of the two-step kernel: the largest p^(n+1) region (output rows +
// 2) its shared memory holds and its ring depths.
struct TbCfg {
    int r2max, np, nq;
};
constexpr TbCfg TB_CFGS[] = {{24, 6, 4}, {16, 5, 2}};
constexpr int TB_NCFG = 2;

template <int R2MAX, int NP, int NQ>
TmaKernel tb_kernel_of() {
    return {(const void *)wk::interior_tb2<R2MAX, NP, NQ>, wk::tb_smem_of<R2MAX, NP, NQ>()};
}
TmaKernel tb_kernel(int cfg) { return cfg == 1 ? tb_kernel_of<16, 5, 2>() : tb_kernel_of<24, 6, 4>(); }

// Buffers of a two-step pass with pair parity pp (steps t, t+1 of a chunk,
// pp = t / 2 % 2): p^n, p^(n-1) in, p^(n+1), p^(n+2) out.  Pair parity 1
// writes its levels back into field[1] and field[0], so every chunk, and the
// single steps after the last full chunk, start from p^n in field[0].
struct TbBufs {
    float *cur, *old, *out1, *out2;
};
TbBufs tb_bufs(const wavey_cuda_plan *pl, int pp) {
    auto f = [](void *p) { return static_cast<float *>(p); };
    if (pp == 0) return {f(pl->field[0]), f(pl->field[1]), f(pl->field2[0]), f(pl->field2[1])};
    return {f(pl->field2[1]), f(pl->field2[0]), f(pl->field[1]), f(pl->field[0])};
}

// Two steps (t, t+1) in one pass over the fields: step t's special cells and
// receivers beside interior_tb2 (both levels of the interior), then
// tb2_second (step t+1's shell and special cells, its receivers).
void launch_pair_tb2(wavey_cuda_plan *pl, int t, int pp) {
    wavey_cuda_ctx *ctx = pl->ctx;
    cudaStream_t s = ctx->stream, side = ctx->side;
    const TbBufs fb = tb_bufs(pl, pp);
    wk::StepArgs<float> a;
    fill_args<float>(pl, a, 0);
    a.interior_blocks = 0;
    a.cur = fb.cur;
    a.nxt = fb.old;
    a.out = fb.out1;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributePriority;
    attr[0].val.priority = pl->branch % 3 == 1 ? pl->prio_hi : pl->prio_lo;
    attr[1].id = cudaLaunchAttributeAccessPolicyWindow;
    attr[1].val.accessPolicyWindow = pl->l2_window;
    const int nattr = pl->l2_window.num_bytes ? 2 : 1;
    const int branch_blocks = a.special_blocks + pl->record_blocks;
    if (branch_blocks > 0) {
        cudaEventRecord(pl->ev_fork, s);
        cudaStreamWaitEvent(side, pl->ev_fork, 0);
        cudaLaunchConfig_t lc = {};
        lc.blockDim = dim3(wk::BLOCK);
        lc.gridDim = dim3(branch_blocks);
        lc.stream = side;
        lc.attrs = attr;
        lc.numAttrs = nattr;
        switch (pl->branch / 3) {
            case 1: cudaLaunchKernelEx(&lc, wk::special_branch<4, 3>, a, t); break;
            case 2: cudaLaunchKernelEx(&lc, wk::special_branch<4, 4>, a, t); break;
            default: cudaLaunchKernelEx(&lc, wk::special_branch<4, 1>, a, t); break;
        }
    }
    if (pl->tb_blocks > 0) {
        wk::Tb2Args ta;
        ta.interior = pl->mask;
        ta.deep = pl->deep;
        ta.out1 = fb.out1;
        ta.out2 = fb.out2;
        ta.error = pl->err;
        ta.cells_p = pl->cells_p;
        ta.nxp = (int)pl->nxp;
        ta.ny = (int)pl->ny;
        ta.nz = (int)pl->nz;
        ta.nxw = (int)(pl->nxp / 32);
        ta.tiles_x = pl->tb_tiles_x;
        ta.tiles_y = pl->tb_tiles_y;
        ta.tiles_z = pl->tb_tiles_z;
        ta.zt = pl->tb_zt;
        ta.rows = pl->tb_rows;
        ta.l2 = (float)(COURANT * COURANT);
        const TmaKernel k = tb_kernel(pl->tb_cfg);
        cudaLaunchConfig_t lc = {};
        cudaLaunchAttribute pa[1];
        pa[0].id = cudaLaunchAttributePriority;
        pa[0].val.priority = pl->branch % 3 == 2 ? pl->prio_hi : pl->prio_lo;
        lc.gridDim = dim3(pl->tb_blocks);
        lc.blockDim = dim3(256);
        lc.dynamicSmemBytes = k.smem;
        lc.stream = s;
        lc.attrs = pa;
        lc.numAttrs = 1;
        void *args[] = {&pl->tb_p[pp], &pl->tb_q[pp], &ta};
        cudaLaunchKernelExC(&lc, k.fn, args);
    }
    if (branch_blocks > 0) {
        cudaEventRecord(pl->ev_join, side);
        cudaStreamWaitEvent(s, pl->ev_join, 0);
    }
    wk::Tb2Second sb;
    sb.a = a;
    sb.a.cur = fb.out1;
    sb.a.nxt = fb.cur;  // p^n is the older level of step t+1
    sb.a.out = fb.out2;
    sb.shell = pl->shell;
    sb.n_shell = (int)pl->n_shell;
    sb.shell_blocks = (int)((pl->n_shell * pl->chunks + wk::BLOCK - 1) / wk::BLOCK);
    const int blocks = sb.shell_blocks + a.special_blocks + pl->record_blocks;
    if (blocks > 0) {
        cudaLaunchConfig_t lc = {};
        lc.blockDim = dim3(wk::BLOCK);
        lc.gridDim = dim3(blocks);
        lc.stream = s;
        lc.attrs = attr + 1;
        lc.numAttrs = nattr - 1;
        switch (pl->branch / 3) {
            case 1: cudaLaunchKernelEx(&lc, wk::tb2_second<3>, sb, t + 1); break;
            case 2: cudaLaunchKernelEx(&lc, wk::tb2_second<4>, sb, t + 1); break;
            default: cudaLaunchKernelEx(&lc, wk::tb2_second<1>, sb, t + 1); break;
        }
    }
}

wk::HalfArgs half_args(const wavey_cuda_plan *pl, int parity) {
    wk::HalfArgs a;
    a.cur = reinterpret_cast<const __half *>(pl->field[parity]);
    a.nxt = reinterpret_cast<__half *>(pl->field[parity ^ 1]);
    a.interior = pl->mask;
    a.sp = pl->sp;
    a.slots = reinterpret_cast<const float *>(pl->slots);
    a.su = reinterpret_cast<float *>(pl->su);
    a.sg = reinterpret_cast<float *>(pl->sg);
    a.tapw = reinterpret_cast<const float *>(pl->tapw);
    a.sig = reinterpret_cast<const float *>(pl->sig);
    a.wmax = pl->wmax;
    a.recv = pl->recv;
    a.ring = reinterpret_cast<float *>(pl->ring);
    a.ring_stride = pl->ring_stride;
    a.base = pl->base;
    a.amax = pl->amax;
    a.scale = pl->scale;
    a.error = pl->err;
    a.cells_p = pl->cells_p;
    a.sig_stride = pl->sig_stride;
    a.nxp = (int)pl->nxp;
    a.ny = (int)pl->ny;
    a.nz = (int)pl->nz;
    a.nxw = (int)(pl->nxp / 32);
    a.n_special = (int)pl->n_special;
    a.n_slots = (int)pl->n_slots;
    a.n_recv = (int)pl->n_recv;
    a.chunks = pl->chunks;
    a.lanes_total = pl->lanes_total;
    a.tiles_x = pl->tiles_x;
    a.tiles_y = pl->tiles_y;
    a.tiles_z = pl->tiles_z;
    a.zt = pl->zt;
    a.interior_blocks = pl->interior_blocks;
    a.special_blocks = pl->special_blocks;
    a.record_blocks = pl->record_blocks;
    a.l2 = (float)(COURANT * COURANT);
    a.lam = (float)COURANT;
    a.half_dt = 0.5f * (float)pl->dt;
    a.shift = pl->fp16_shift;
    return a;
}

template <int V>
void launch_step_half(wavey_cuda_plan *pl, int t, int parity) {
    const wk::HalfArgs a = half_args(pl, parity);
    const int prep = (int)((pl->chunks * pl->nz + wk::BLOCK - 1) / wk::BLOCK);
    wk::half_prepare<V><<<prep, wk::BLOCK, 0, pl->ctx->stream>>>(a, t);
    const int blocks = pl->interior_blocks + pl->special_blocks + pl->record_blocks;
    if (blocks > 0) wk::fdtd_step_half<V><<<blocks, wk::BLOCK, 0, pl->ctx->stream>>>(a, t);
}

// FP16 storage with the TMA interior kernel: half_prepare fixes the scales of
// level n+1, then the special-cell and receiver roles of fdtd_step_half run
// beside the TMA kernel, as in the FP32 step.
template <int V>
void launch_step_half_tma(wavey_cuda_plan *pl, int t, int parity) {
    cudaStream_t s = pl->ctx->stream, side = pl->ctx->side;
    wk::HalfArgs a = half_args(pl, parity);
    const int prep = (int)((pl->chunks * pl->nz + wk::BLOCK - 1) / wk::BLOCK);
    wk::half_prepare<V><<<prep, wk::BLOCK, 0, s>>>(a, t);
    a.interior_blocks = 0;
    const int blocks = pl->special_blocks + pl->record_blocks;
    if (blocks > 0) {
        cudaEventRecord(pl->ev_fork, s);
        cudaStreamWaitEvent(side, pl->ev_fork, 0);
        cudaLaunchConfig_t lc = {};
        cudaLaunchAttribute attr[2];
        attr[0].id = cudaLaunchAttributePriority;
        attr[0].val.priority = pl->branch % 3 == 1 ? pl->prio_hi : pl->prio_lo;
        attr[1].id = cudaLaunchAttributeAccessPolicyWindow;
        attr[1].val.accessPolicyWindow = pl->l2_window;
        lc.blockDim = dim3(wk::BLOCK);
        lc.gridDim = dim3(blocks);
        lc.stream = side;
        lc.attrs = attr;
        lc.numAttrs = pl->l2_window.num_bytes ? 2 : 1;
        switch (pl->branch / 3) {
            case 1: cudaLaunchKernelEx(&lc, wk::special_branch_half<V, 3>, a, t); break;
            case 2: cudaLaunchKernelEx(&lc, wk::special_branch_half<V, 4>, a, t); break;
            default: cudaLaunchKernelEx(&lc, wk::special_branch_half<V, 1>, a, t); break;
        }
    }
    if (pl->tma_blocks > 0)
        launch_tma_cfg<__half, V, false>(pl->tma_cfg, pl->tma_blocks, s, pl->branch % 3 == 2 ? pl->prio_hi : pl->prio_lo,
                                         pl->tm_p[parity], pl->tm_q[parity], tma_args<__half>(pl, t, parity),
                                         wk::SpecTile{});
    if (blocks > 0) {
        cudaEventRecord(pl->ev_join, side);
        cudaStreamWaitEvent(s, pl->ev_join, 0);
    }
}

void step(wavey_cuda_plan *pl, int t, int parity) {
    if (pl->tma && pl->precision == WAVEY_FP16_STORAGE) {
        switch (pl->V) {
            case 1: launch_step_half_tma<1>(pl, t, parity); break;
            case 2: launch_step_half_tma<2>(pl, t, parity); break;
            default: launch_step_half_tma<4>(pl, t, parity); break;
        }
        return;
    }
    if (pl->tma) {
        switch (pl->V) {
            case 1: launch_step_tma<1>(pl, t, parity); break;
            case 2: launch_step_tma<2>(pl, t, parity); break;
            default: launch_step_tma<4>(pl, t, parity); break;
        }
        return;
    }
    if (pl->precision == WAVEY_FP16_STORAGE) {
        switch (pl->V) {
            case 1: launch_step_half<1>(pl, t, parity); break;
            case 2: launch_step_half<2>(pl, t, parity); break;
            default: launch_step_half<4>(pl, t, parity); break;
        }
        return;
    }
    if (pl->precision == WAVEY_FP64) {
        switch (pl->V) {
            case 1: launch_step<double, 1, true>(pl, t, parity); break;
            case 2: launch_step<double, 2, true>(pl, t, parity); break;
            default: launch_step<double, 4, true>(pl, t, parity); break;
        }
    } else {
        switch (pl->V) {
            case 1: launch_step<float, 1, false>(pl, t, parity); break;
            case 2: launch_step<float, 2, false>(pl, t, parity); break;
            default: launch_step<float, 4, false>(pl, t, parity); break;
        }
    }
}

// A: the type of the twiddles and of the chunk sums (T, or FP64 for FP32
// samples in a plan with FP64 receiver accumulation).
template <class T, int V, class A = T>
void launch_fold(wavey_cuda_plan *pl, int count, int lag, cudaStream_t s) {
    const int tw_threads = count * (int)pl->nf;
    if (tw_threads > 0)
        wk::twiddle_chunk<A><<<(tw_threads + 255) / 256, 256, 0, s>>>(pl->freqs, (int)pl->nf, pl->dt, pl->base, count,
                                                                       (long long)pl->steps, reinterpret_cast<A *>(pl->tw), lag);
    const long long total = (long long)pl->chunks * pl->n_recv * pl->nf;
    const size_t tiled_smem = (size_t)wk::RING * wk::dft_nfp((int)pl->nf) * sizeof(float2);
    bool tiled = false;
    if constexpr (std::is_same<T, float>::value && std::is_same<A, float>::value) {
        if (total > 0 && tiled_smem <= (size_t)wk::DFT_SMEM_MAX) {
            const long long threads = (long long)pl->chunks * (wk::dft_nfp((int)pl->nf) / wk::DFT_FB) * pl->n_recv;
            wk::dft_chunk_tiled<V><<<(unsigned)((threads + wk::BLOCK - 1) / wk::BLOCK), wk::BLOCK, tiled_smem, s>>>(
                reinterpret_cast<const float *>(pl->ring), reinterpret_cast<const float *>(pl->tw), pl->acc,
                (int)pl->n_recv, (int)pl->nf, pl->chunks, count, pl->base, (long long)pl->steps, lag, pl->ring_stride);
            tiled = true;
        }
    }
    if (!tiled && total > 0)
        wk::dft_chunk<T, V, A><<<(unsigned)((total + wk::BLOCK - 1) / wk::BLOCK), wk::BLOCK, 0, s>>>(
            reinterpret_cast<const T *>(pl->ring), reinterpret_cast<const A *>(pl->tw), pl->acc, (int)pl->n_recv, (int)pl->nf,
            pl->chunks, count, pl->base, (long long)pl->steps, lag, pl->ring_stride);
    if (pl->want_ir) {
        const long long n = (long long)pl->chunks * V * pl->n_recv * count;
        if (n > 0)
            wk::ir_chunk<T, V><<<(unsigned)((n + wk::BLOCK - 1) / wk::BLOCK), wk::BLOCK, 0, s>>>(
                reinterpret_cast<const T *>(pl->ring), reinterpret_cast<T *>(pl->ir), (int)pl->n_recv, pl->chunks,
                pl->n_sources, (long long)pl->steps, pl->base, count, lag, pl->ring_stride);
    }
}

// The receiver fold of the chunk that starts at step *base - lag (lag 0: the
// chunk just run; RING: the one before it), on stream s (default: the plan's).
void fold(wavey_cuda_plan *pl, int count, int lag = 0, cudaStream_t s = nullptr) {
    if (!s) s = pl->ctx->stream;
    if (pl->precision == WAVEY_FP64) {  // FP32 and FP16 storage fold in FP32
        switch (pl->V) {
            case 1: launch_fold<double, 1>(pl, count, lag, s); break;
            case 2: launch_fold<double, 2>(pl, count, lag, s); break;
            default: launch_fold<double, 4>(pl, count, lag, s); break;
        }
    } else if (pl->dft64) {  // FP32 samples, FP64 twiddles and chunk sums
        switch (pl->V) {
            case 1: launch_fold<float, 1, double>(pl, count, lag, s); break;
            case 2: launch_fold<float, 2, double>(pl, count, lag, s); break;
            default: launch_fold<float, 4, double>(pl, count, lag, s); break;
        }
    } else {
        switch (pl->V) {
            case 1: launch_fold<float, 1>(pl, count, lag, s); break;
            case 2: launch_fold<float, 2>(pl, count, lag, s); break;
            default: launch_fold<float, 4>(pl, count, lag, s); break;
        }
    }
}

int build_graph(wavey_cuda_plan *pl) {
    wavey_cuda_ctx *ctx = pl->ctx;
    cudaStream_t s = ctx->stream;
    cudaGraph_t g = nullptr;
    int st = ctx->cuda(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
    if (st) return st;
    cudaEventRecordWithFlags(pl->ev_a, s, cudaEventRecordExternal);
    if (pl->fold_overlap) {
        // The previous chunk's fold beside this chunk's steps (nothing in
        // the first chunk); the two use different rings.
        cudaEventRecord(pl->ev_ffork, s);
        cudaStreamWaitEvent(ctx->folds, pl->ev_ffork, 0);
        fold(pl, wk::RING, wk::RING, ctx->folds);
        cudaEventRecord(pl->ev_fjoin, ctx->folds);
    }
    if (pl->tb2)
        for (int t = 0; t < wk::RING; t += 2) launch_pair_tb2(pl, t, (t >> 1) & 1);
    else
        for (int t = 0; t < wk::RING; t++) step(pl, t, t & 1);
    cudaEventRecordWithFlags(pl->ev_b, s, cudaEventRecordExternal);
    if (pl->fold_overlap)
        cudaStreamWaitEvent(s, pl->ev_fjoin, 0);
    else
        fold(pl, wk::RING);
    wk::advance_base<<<1, 1, 0, s>>>(pl->base, wk::RING);
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (e != cudaSuccess) return ctx->cuda(e, "end capture");
    size_t nodes = 0;
    cudaGraphGetNodes(g, nullptr, &nodes);
    pl->graph_kernels = 0;
    {
        std::vector<cudaGraphNode_t> list(nodes);
        cudaGraphGetNodes(g, list.data(), &nodes);
        for (cudaGraphNode_t n : list) {
            cudaGraphNodeType ty;
            if (cudaGraphNodeGetType(n, &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel) pl->graph_kernels++;
        }
    }
    // Node priorities (the branch's launch attribute) count only with this flag.
    e = cudaGraphInstantiateWithFlags(&pl->graph, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    return ctx->cuda(e, "graph instantiate");
}

template <class T>
std::vector<T> convert(const double *src, size_t n) {
    std::vector<T> v(n);
#pragma omp parallel for schedule(static) num_threads(host_threads()) if (n >= (1u << 16))
    for (int64_t i = 0; i < (int64_t)n; i++) v[(size_t)i] = (T)src[i];
    return v;
}

template <class T>
int upload_typed(wavey_cuda_plan *pl, void **out, const std::vector<double> &src) {
    std::vector<T> v = convert<T>(src.data(), src.size());
    T *d = nullptr;
    int st = upload(pl, &d, v.data(), v.size() * sizeof(T));
    *out = d;
    if (st) return st;
    // The staging vector dies here: wait for the copy.
    return pl->ctx->cuda(cudaStreamSynchronize(pl->ctx->stream), "upload sync");
}

// Converts n values at src to T into an existing device buffer and waits
// for the copy.
template <class T>
int upload_into(wavey_cuda_plan *pl, void *dst, const double *src, size_t n) {
    std::vector<T> v = convert<T>(src, n);
    pl->h2d_bytes += (int64_t)(v.size() * sizeof(T));
    if (v.empty()) return WAVEY_OK;
    int st = pl->ctx->cuda(cudaMemcpyAsync(dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, pl->ctx->stream),
                           "upload");
    if (st) return st;
    return pl->ctx->cuda(cudaStreamSynchronize(pl->ctx->stream), "upload sync");
}

// The persisting L2 window over the plan's special block (records, slot
// constants, branch states), for blocks that fit whole in a set-aside of at
// most half of L2 (the field streams keep the other half for their halo
// reuse).  A block that does not fit gets no window: persisting a part of
// it was measured slower than none (72 M-cell grid: 786 vs 614 us per step).
// WAVEY_L2_PERSIST=0 leaves L2 alone.
void set_l2_window(wavey_cuda_plan *pl) {
    wavey_cuda_ctx *ctx = pl->ctx;
    pl->l2_window = {};
    pl->l2_setaside = 0;
    if (!env_int("WAVEY_L2_PERSIST", 1, 0, 1) || ctx->max_persist_l2 <= 0 || ctx->max_window <= 0 || !pl->l2_block_bytes)
        return;
    const size_t cap = std::min({(size_t)ctx->max_persist_l2, ctx->l2_bytes / 2, (size_t)ctx->max_window});
    if (pl->l2_block_bytes > cap) return;
    pl->l2_setaside = pl->l2_block_bytes;
    pl->l2_window.base_ptr = pl->l2_block;
    pl->l2_window.num_bytes = pl->l2_block_bytes;
    pl->l2_window.hitRatio = 1.0f;
    pl->l2_window.hitProp = cudaAccessPropertyPersisting;
    pl->l2_window.missProp = cudaAccessPropertyStreaming;
}

// Before a plan runs: the context's persisting set-aside becomes this
// plan's (a per-context limit, released with the context), and lines left
// persisting by another plan go back to normal.  A plan without a window
// gives the whole L2 back to normal lines.
void apply_l2(wavey_cuda_plan *pl) {
    wavey_cuda_ctx *ctx = pl->ctx;
    if (ctx->persist_owner == pl) return;
    if (ctx->persist_set) cudaCtxResetPersistingL2Cache();
    if (ctx->persist_set != pl->l2_setaside) {
        if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, pl->l2_setaside) == cudaSuccess) {
            ctx->persist_set = pl->l2_setaside;
        } else {
            cudaGetLastError();
            pl->l2_window = {};  // launch without the window
        }
    }
    ctx->persist_owner = pl;
}

// The special list ordered by (tile, plane) for tiles of `rows` rows, as the
// fused form reads it (wk::SpecTile): a stable counting sort of the records
// (in cell order) by the key (tile row, tile column, z), and the first record
// of every key.  Built once per tile height.
int tile_specials(wavey_cuda_plan *pl, int rows) {
    const int slot = tile_slot(rows);
    if (pl->sp_tile[slot]) return WAVEY_OK;
    const int64_t cells_row = wk::TMA_ROW_FLOATS / pl->V;
    const int64_t tiles_x = (pl->nx + cells_row - 1) / cells_row, tiles_y = (pl->ny - 2 + rows - 1) / rows;
    const int64_t keys = tiles_x * tiles_y * pl->nz;
    const int64_t nxy = pl->nxp * pl->ny;
    if (keys >= (int64_t)UINT32_MAX) return pl->ctx->fail(WAVEY_E_LIMIT, "too many tiles for the special-cell order");
    std::vector<uint32_t> off((size_t)keys + 1, 0u), key(pl->sp_host.size());
    for (size_t i = 0; i < pl->sp_host.size(); i++) {
        const int64_t cell = pl->sp_host[i].x;
        const int64_t z = cell / nxy, y = (cell % nxy) / pl->nxp, x = cell % pl->nxp;
        key[i] = (uint32_t)((((y - 1) / rows) * tiles_x + x / cells_row) * pl->nz + z);
        off[key[i] + 1]++;
    }
    for (int64_t k = 0; k < keys; k++) off[k + 1] += off[k];
    std::vector<uint32_t> pos(off.begin(), off.end() - 1);
    std::vector<uint4> rec(pl->sp_host.size());
    for (size_t i = 0; i < pl->sp_host.size(); i++) rec[pos[key[i]]++] = pl->sp_host[i];
    int st = upload(pl, &pl->sp_tile[slot], rec.data(), rec.size() * sizeof(uint4));
    if (!st) st = upload(pl, &pl->sp_off[slot], off.data(), off.size() * sizeof(uint32_t));
    // The staging vectors die here: wait for the copies.
    if (!st) st = pl->ctx->cuda(cudaStreamSynchronize(pl->ctx->stream), "upload sync");
    return st;
}

bool pdl_safe(const wavey_cuda_plan *pl);

// Shape of the TMA interior kernel: tile rows and ring depths (TMA_CFGS[cfg])
// and the z planes each CTA marches (zt).  Encodes the tensor maps, whose
// boxes depend on the tile rows, and sizes the grid.
int tma_shape(wavey_cuda_plan *pl, int cfg, int zt) {
    wavey_cuda_ctx *ctx = pl->ctx;
    EncodeTiled enc = encode_tiled();
    if (!enc) return ctx->fail(WAVEY_E_CUDA, "the driver lacks cuTensorMapEncodeTiled");
    const int64_t V = pl->V, nx = pl->nx, ny = pl->ny, nz = pl->nz;
    const bool half = pl->precision == WAVEY_FP16_STORAGE;
    const int64_t es = half ? 2 : 4;
    const CUtensorMapDataType dt = half ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    const cuuint64_t dims[4] = {(cuuint64_t)(nx * V), (cuuint64_t)ny, (cuuint64_t)nz, (cuuint64_t)pl->chunks};
    const cuuint64_t strides[3] = {(cuuint64_t)(pl->nxp * V * es), (cuuint64_t)(pl->nxp * ny * V * es),
                                   (cuuint64_t)(pl->cells_p * V * es)};
    const int rows = TMA_CFGS[cfg].rows;
    const int prow = half ? wk::tma_p_row<__half>() : wk::tma_p_row<float>();
    const cuuint32_t box_p[4] = {(cuuint32_t)prow, (cuuint32_t)(rows + 2), 1, 1};
    const cuuint32_t box_q[4] = {(cuuint32_t)wk::TMA_ROW_FLOATS, (cuuint32_t)rows, 1, 1};
    const cuuint32_t unit[4] = {1, 1, 1, 1};
    for (int k = 0; k < 2; k++) {
        CUresult r1 = enc(&pl->tm_p[k], dt, 4, pl->field[k], dims, strides, box_p, unit, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        CUresult r2 = enc(&pl->tm_q[k], dt, 4, pl->field[k ^ 1], dims, strides, box_q, unit, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r1 != CUDA_SUCCESS || r2 != CUDA_SUCCESS)
            return ctx->fail(WAVEY_E_CUDA, "tensor map encoding failed (%d, %d)", (int)r1, (int)r2);
    }
    // The FP16 kernel stages a z-run's scales in shared memory, the fused form
    // its special-cell offsets: their z-runs have at most TMA_MAX_ZT planes.
    if (half || pl->branch == BRANCH_FUSED) zt = std::min(zt, wk::TMA_MAX_ZT);
    if (pl->branch == BRANCH_FUSED) {
        const int st = tile_specials(pl, rows);
        if (st) return st;
    }
    pl->tma_cfg = cfg;
    pl->tma_zt = zt;
    pl->tma_tiles_x = (int)((nx + (wk::TMA_ROW_FLOATS / V) - 1) / (wk::TMA_ROW_FLOATS / V));
    pl->tma_tiles_y = (int)((ny - 2 + rows - 1) / rows);
    pl->tma_tiles_z = (int)((nz - 2 + zt - 1) / zt);
    const int64_t tb = (int64_t)pl->tma_tiles_x * pl->tma_tiles_y * pl->tma_tiles_z * pl->chunks;
    if (tb >= (1ll << 31)) return ctx->fail(WAVEY_E_LIMIT, "launch grid too large");
    pl->tma_blocks = (int)tb;
    pl->pdl = pl->pdl_wanted && pdl_safe(pl);
    return WAVEY_OK;
}

// Shape of the two-step pass: kernel shape cfg (TB_CFGS), output rows per
// tile and z-run.  Encodes its tensor maps (p^n with a two-cell ring, p^(n-1)
// with a one-cell ring, per pair parity) and sizes the grid.
int tb_shape(wavey_cuda_plan *pl, int cfg, int rows, int zt) {
    wavey_cuda_ctx *ctx = pl->ctx;
    EncodeTiled enc = encode_tiled();
    if (!enc) return ctx->fail(WAVEY_E_CUDA, "the driver lacks cuTensorMapEncodeTiled");
    rows = std::max(1, std::min(rows, TB_CFGS[cfg].r2max - 2));
    zt = std::max(1, zt);
    const int64_t nx = pl->nx, ny = pl->ny, nz = pl->nz;
    const cuuint64_t dims[4] = {(cuuint64_t)(nx * 4), (cuuint64_t)ny, (cuuint64_t)nz, (cuuint64_t)pl->chunks};
    const cuuint64_t strides[3] = {(cuuint64_t)(pl->nxp * 4 * 4), (cuuint64_t)(pl->nxp * ny * 4 * 4),
                                   (cuuint64_t)(pl->cells_p * 4 * 4)};
    const cuuint32_t box_p[4] = {(cuuint32_t)wk::TB_PROW, (cuuint32_t)(rows + 4), 1, 1};
    const cuuint32_t box_q[4] = {(cuuint32_t)wk::TMA_ROW_FLOATS, (cuuint32_t)(rows + 2), 1, 1};
    const cuuint32_t unit[4] = {1, 1, 1, 1};
    for (int pp = 0; pp < 2; pp++) {
        const TbBufs fb = tb_bufs(pl, pp);
        CUresult r1 = enc(&pl->tb_p[pp], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, fb.cur, dims, strides, box_p, unit,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        CUresult r2 = enc(&pl->tb_q[pp], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, fb.old, dims, strides, box_q, unit,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r1 != CUDA_SUCCESS || r2 != CUDA_SUCCESS)
            return ctx->fail(WAVEY_E_CUDA, "tensor map encoding failed (%d, %d)", (int)r1, (int)r2);
    }
    pl->tb_cfg = cfg;
    pl->tb_rows = rows;
    pl->tb_zt = zt;
    pl->tb_tiles_x = (int)((nx - 2 + wk::TB_CELLS - 1) / wk::TB_CELLS);
    pl->tb_tiles_y = (int)((ny - 2 + rows - 1) / rows);
    pl->tb_tiles_z = (int)((nz - 2 + zt - 1) / zt);
    const int64_t tb = (int64_t)pl->tb_tiles_x * pl->tb_tiles_y * pl->tb_tiles_z * pl->chunks;
    if (tb >= (1ll << 31)) return ctx->fail(WAVEY_E_LIMIT, "launch grid too large");
    pl->tb_blocks = (int)tb;
    return WAVEY_OK;
}

// Two steps per pass: the deep-cell mask (interior cells whose six
// neighbours are interior cells) and the shell list (the other interior
// cells) from the interior mask, the two extra field buffers, and a shape:
// the output rows that best fill whole waves of resident CTAs (one z-run per
// column where a layer fills a wave), unless WAVEY_TB_CFG / WAVEY_TB_ROWS /
// WAVEY_TB_ZT say otherwise.
int tb_setup(wavey_cuda_plan *pl, const std::vector<uint32_t> &mask) {
    wavey_cuda_ctx *ctx = pl->ctx;
    const int64_t nx = pl->nx, ny = pl->ny, nz = pl->nz, nxw = pl->nxp / 32;
    auto bit = [&](int64_t z, int64_t y, int64_t x) { return (mask[(size_t)((z * ny + y) * nxw + x / 32)] >> (x % 32)) & 1u; };
    std::vector<uint32_t> deep(mask.size(), 0u), shell;
    for (int64_t z = 1; z < nz - 1; z++)
        for (int64_t y = 1; y < ny - 1; y++)
            for (int64_t x = 1; x < nx - 1; x++) {
                if (!bit(z, y, x)) continue;
                if (bit(z, y, x - 1) && bit(z, y, x + 1) && bit(z, y - 1, x) && bit(z, y + 1, x) && bit(z - 1, y, x) &&
                    bit(z + 1, y, x))
                    deep[(size_t)((z * ny + y) * nxw + x / 32)] |= 1u << (x % 32);
                else
                    shell.push_back((uint32_t)((z * ny + y) * pl->nxp + x));
            }
    int st;
    for (int k = 0; k < 2; k++)
        if ((st = alloc(pl, &pl->field2[k], pl->field_bytes))) return st;
    if ((st = upload(pl, &pl->deep, deep.data(), deep.size() * 4))) return st;
    if ((st = upload(pl, &pl->shell, shell.data(), shell.size() * 4))) return st;
    pl->n_shell = (int64_t)shell.size();
    if ((st = ctx->cuda(cudaStreamSynchronize(ctx->stream), "upload sync"))) return st;
    for (int cfg = 0; cfg < TB_NCFG; cfg++) {
        const TmaKernel k = tb_kernel(cfg);
        if ((st = ctx->cuda(cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem),
                            "shared memory attribute")))
            return st;
    }
    const int cfg = env_int("WAVEY_TB_CFG", 0, 0, TB_NCFG - 1);
    int occ = 0;
    const TmaKernel k = tb_kernel(cfg);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k.fn, 256, k.smem) != cudaSuccess) cudaGetLastError();
    const int64_t slots = std::max<int64_t>(1, (int64_t)occ * ctx->sm_count);
    const int64_t tiles_x = (nx - 2 + wk::TB_CELLS - 1) / wk::TB_CELLS;
    int best_rows = TB_CFGS[cfg].r2max - 2, best_tz = 1;
    double best = -1.0;
    for (int rows = TB_CFGS[cfg].r2max - 2; rows >= 6; rows--) {
        const int64_t layer = tiles_x * ((ny - 2 + rows - 1) / rows) * pl->chunks;
        const int64_t tz = std::max<int64_t>(1, std::min<int64_t>(slots / layer, nz - 2));
        const int64_t ctas = layer * tz, waves = (ctas + slots - 1) / slots;
        const double score = (double)ctas / (double)(waves * slots) * rows / (rows + 2.0);
        if (score > best + 1e-9) {
            best = score;
            best_rows = rows;
            best_tz = (int)tz;
        }
    }
    const int rows = env_int("WAVEY_TB_ROWS", best_rows, 1, TB_CFGS[cfg].r2max - 2);
    const int zt = env_int("WAVEY_TB_ZT", (int)((nz - 2 + best_tz - 1) / best_tz), 1, 1 << 20);
    if ((st = tb_shape(pl, cfg, rows, zt))) return st;
    pl->tb2 = true;
    return WAVEY_OK;
}

// Whether the FP32 interior may be launched as a programmatic dependent of
// the previous step: the special cells in their own kernel, the interior
// grid within one wave, and room on every SM for one block of the
// special-cell kernel beside the interior CTAs that fit there -- so that
// next-step CTAs, waiting on an SM for this step to end, can never keep the
// special-cell kernel they wait for from running.
template <int V>
bool pdl_safe_v(const wavey_cuda_plan *pl) {
    const wavey_cuda_ctx *ctx = pl->ctx;
    const TmaKernel k = tma_kernel<float, V, false>(pl->tma_cfg);
    const void *sfn = pl->branch / 3 == 1 ? (const void *)wk::special_branch<V, 3>
                      : pl->branch / 3 == 2 ? (const void *)wk::special_branch<V, 4>
                                            : (const void *)wk::special_branch<V, 1>;
    cudaFuncAttributes fi, fs;
    int occ = 0;
    if (cudaFuncGetAttributes(&fi, k.fn) != cudaSuccess || cudaFuncGetAttributes(&fs, sfn) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k.fn, 256, k.smem) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    auto regs = [](int per_thread, int threads) { return (int64_t)((per_thread + 7) / 8 * 8) * threads; };
    const int64_t r = occ * regs(fi.numRegs, 256) + regs(fs.numRegs, wk::BLOCK);
    const int64_t sm = occ * ((int64_t)k.smem + fi.sharedSizeBytes + ctx->smem_reserved) + fs.sharedSizeBytes + ctx->smem_reserved;
    const int64_t th = occ * 256 + wk::BLOCK;
    return occ > 0 && pl->tma_blocks <= (int64_t)occ * ctx->sm_count && r <= ctx->regs_per_sm && sm <= ctx->smem_per_sm &&
           th <= ctx->threads_per_sm;
}

bool pdl_safe(const wavey_cuda_plan *pl) {
    if (pl->precision != WAVEY_FP32 || pl->branch == BRANCH_FUSED || !pl->tma) return false;
    return pl->V == 4 ? pdl_safe_v<4>(pl) : pl->V == 2 ? pdl_safe_v<2>(pl) : pdl_safe_v<1>(pl);
}

// Resident CTAs per SM of one shape of the TMA interior kernel.
template <class E, int V, bool SPEC>
int tma_occupancy(int cfg) {
    int occ = 0;
    const TmaKernel k = tma_kernel<E, V, SPEC>(cfg);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k.fn, 256, k.smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return occ;
}

template <class E>
int tma_occupancy_v(int V, int cfg) {
    return V == 4 ? tma_occupancy<E, 4, false>(cfg) : V == 2 ? tma_occupancy<E, 2, false>(cfg) : tma_occupancy<E, 1, false>(cfg);
}

int tma_occupancy_fused(int V, int cfg) {
    return V == 4 ? tma_occupancy<float, 4, true>(cfg) : V == 2 ? tma_occupancy<float, 2, true>(cfg)
                                                               : tma_occupancy<float, 1, true>(cfg);
}

// Shapes a plan may take: 14 for FP32 plans with a concurrent special-cell
// kernel, 7 for FP16 and fused plans.
int tma_ncfg(const wavey_cuda_plan *pl) {
    return pl->precision == WAVEY_FP32 && pl->branch != BRANCH_FUSED ? TMA_NCFG : TMA_NCFG_ONE_POLICY;
}

// The z-run that makes the grid of one shape just fill w waves of resident
// CTAs (every CTA of a launch does about the same work, so a partly filled
// last wave idles SMs); 0 if none lies in 4..64 planes.
int wave_zt(const wavey_cuda_plan *pl, int cfg, int w) {
    const int occ = pl->precision == WAVEY_FP16_STORAGE ? tma_occupancy_v<__half>(pl->V, cfg)
                    : pl->branch == BRANCH_FUSED            ? tma_occupancy_fused(pl->V, cfg)
                                                            : tma_occupancy_v<float>(pl->V, cfg);
    const int64_t planes = pl->nz - 2, rows = TMA_CFGS[cfg].rows, cells_row = wk::TMA_ROW_FLOATS / pl->V;
    const int64_t layer = ((pl->nx + cells_row - 1) / cells_row) * ((pl->ny - 2 + rows - 1) / rows) * pl->chunks;
    const int64_t slots = (int64_t)occ * pl->ctx->sm_count;
    if (slots <= 0 || layer <= 0) return 0;
    const int64_t runs = w * slots / layer;  // z-runs per column that fit w waves
    if (runs < 1) return 0;
    const int zt = (int)((planes + runs - 1) / runs);
    return zt >= 4 && zt <= 64 ? zt : 0;
}

// Candidate z-runs: 8, 16 and 32 planes, and the runs that cut the interior
// planes into 1 to 8 equal z-tiles (a partial wave of interior CTAs can beat
// a full one: the special-cell kernel then has room beside them).
std::vector<int> tune_zts(const wavey_cuda_plan *pl) {
    const bool capped = pl->precision == WAVEY_FP16_STORAGE || pl->branch == BRANCH_FUSED;
    const int planes = (int)pl->nz - 2;
    std::vector<int> zts;
    auto add = [&](int zt) {
        if (capped) zt = std::min(zt, wk::TMA_MAX_ZT);
        if (zt >= 1 && std::find(zts.begin(), zts.end(), zt) == zts.end()) zts.push_back(zt);
    };
    for (int zt : {8, 16, 32}) add(zt);
    for (int k = 1; k <= 8; k++) add((planes + k - 1) / k);
    return zts;
}

// standalone: a plan that runs by itself (TMA interior path where it
// applies, its own chunk graph).  Plans inside a rooms plan are not
// standalone: the rooms plan launches their fused step blocks together.
int plan_create(wavey_cuda_ctx *ctx, const wavey_grid *grid, const wavey_source *sources, size_t n_sources,
                const double *signals, size_t signal_stride, size_t steps, const uint64_t *receivers, size_t n_recv,
                const double *freqs, size_t nf, int32_t precision, int32_t want_ir, wavey_cuda_plan **out,
                bool standalone = true) {
    if (!out) return ctx->fail(WAVEY_E_INVALID, "out is null");
    *out = nullptr;
    int st = validate_grid(ctx, grid);
    if (st) return st;
    if (precision != WAVEY_FP32 && precision != WAVEY_FP64 && precision != WAVEY_FP16_STORAGE)
        return ctx->fail(WAVEY_E_INVALID, "unknown precision %d", precision);
    if (n_sources == 0 || !sources) return ctx->fail(WAVEY_E_INVALID, "no sources");
    if (n_sources > 4096) return ctx->fail(WAVEY_E_LIMIT, "at most 4096 sources per run");
    if (steps > 0 && !signals) return ctx->fail(WAVEY_E_INVALID, "signals are null");
    if (signal_stride != 0 && signal_stride < steps) return ctx->fail(WAVEY_E_INVALID, "signal_stride is shorter than steps");
    if (steps >= (1ull << 40)) return ctx->fail(WAVEY_E_LIMIT, "too many steps");
    if (n_recv > 0 && !receivers) return ctx->fail(WAVEY_E_INVALID, "receivers are null");
    if (nf > 0 && !freqs) return ctx->fail(WAVEY_E_INVALID, "freqs are null");
    if (n_recv > (1u << 26) || nf > (1u << 20)) return ctx->fail(WAVEY_E_LIMIT, "too many receivers or frequencies");

    const int64_t nx = grid->nx, ny = grid->ny, nz = grid->nz;
    const int64_t cells = nx * ny * nz;
    wavey_cuda_plan *pl = new (std::nothrow) wavey_cuda_plan();
    if (!pl) return ctx->fail(WAVEY_E_NOMEM, "host allocation failed");
    pl->ctx = ctx;
    pl->precision = precision;
    pl->elem = precision == WAVEY_FP64 ? 8 : 4;
    pl->field_elem = precision == WAVEY_FP64 ? 8 : (precision == WAVEY_FP16_STORAGE ? 2 : 4);
    pl->n_sources = (int)n_sources;
    pl->V = n_sources >= 4 ? 4 : (n_sources == 1 ? 1 : (n_sources == 2 ? 2 : 4));
    pl->chunks = (int)((n_sources + pl->V - 1) / pl->V);
    pl->lanes_total = pl->chunks * pl->V;
    pl->nx = nx;
    pl->ny = ny;
    pl->nz = nz;
    pl->nxp = round_up(nx, 32);
    pl->cells = cells;
    pl->cells_p = pl->nxp * ny * nz;
    pl->steps = (int64_t)steps;
    pl->n_recv = (int64_t)n_recv;
    pl->nf = (int64_t)nf;
    pl->want_ir = want_ir != 0;
    pl->dt = grid->dt;
    auto bail = [&](int code) {
        delete pl;
        return code;
    };
    const uint8_t *flags = grid->flags;
    const uint32_t *bidx = grid->bidx;
    const int64_t nb = grid->n_boundary;
    const int64_t nslots = nb > 0 ? (int64_t)grid->bstart[nb] : 0;
    pl->n_slots = nslots;

    // Taps: merged per cell in FP64 per source (gpu_fdtd.rs:67-75), then one
    // row per distinct cell across all sources.
    std::unordered_map<int64_t, int64_t> tap_row;
    std::vector<int64_t> tap_cells;
    std::vector<double> tapw;  // [rows][lanes_total]
    for (size_t s = 0; s < n_sources; s++) {
        const wavey_source &src = sources[s];
        if (src.n_taps > 0 && !src.taps) return bail(ctx->fail(WAVEY_E_INVALID, "source %zu: taps are null", s));
        for (size_t t = 0; t < src.n_taps; t++) {
            const int64_t c = src.taps[t].cell;
            if (c < 0 || c >= cells) return bail(ctx->fail(WAVEY_E_INVALID, "source %zu: tap cell %lld out of range", s, (long long)c));
            if (!(flags[c] & AIR))
                return bail(ctx->fail(WAVEY_E_INVALID, "source %zu: tap cell %lld is not air", s, (long long)c));
            auto it = tap_row.find(c);
            int64_t row;
            if (it == tap_row.end()) {
                row = (int64_t)tap_cells.size();
                tap_row.emplace(c, row);
                tap_cells.push_back(c);
                tapw.resize(tapw.size() + pl->lanes_total, 0.0);
            } else {
                row = it->second;
            }
            tapw[row * pl->lanes_total + s] += src.taps[t].w;
        }
    }
    if (tap_cells.size() >= (size_t)NO_BOUNDARY) return bail(ctx->fail(WAVEY_E_LIMIT, "too many taps"));
    for (size_t r = 0; r < n_recv; r++)
        if (receivers[r] >= (uint64_t)cells)
            return bail(ctx->fail(WAVEY_E_INVALID, "receiver %zu: cell %llu out of range", r, (unsigned long long)receivers[r]));

    // Border cells must be solid: the reference pads every grid with one
    // solid layer (fdtd.rs:292-299), and the kernels rely on it to keep every
    // neighbour in range.  Boundary indices must point into the slot table.
    std::vector<uint32_t> mask((size_t)(pl->cells_p / 32), 0u);
    const int64_t nxw = pl->nxp / 32;
    struct Special {
        uint32_t cell, meta, slot0;
    };
    std::vector<std::vector<Special>> sp(nz);
    std::vector<int64_t> air_z(nz, 0), int_z(nz, 0);
    std::vector<int> bad_z(nz, 0);
    // One plane per iteration; counts and mask words are built in locals and
    // stored once (per plane, per 32 cells), so threads share no cache line
    // cell by cell.
#pragma omp parallel for schedule(dynamic, 1) num_threads(host_threads())
    for (int64_t z = 0; z < nz; z++) {
        int64_t n_air = 0, n_int = 0;
        int bad = 0;
        for (int64_t y = 0; y < ny; y++) {
            const uint8_t *frow = flags + (z * ny + y) * nx;
            const uint32_t *brow = bidx + (z * ny + y) * nx;
            uint32_t *mrow = mask.data() + (size_t)((z * ny + y) * nxw);
            for (int64_t x0 = 0; x0 < nx; x0 += 32) {
                uint32_t word = 0;
                const int64_t x1 = std::min<int64_t>(x0 + 32, nx);
                for (int64_t x = x0; x < x1; x++) {
                    const uint8_t f = frow[x];
                    if (!(f & AIR)) continue;
                    if (x == 0 || y == 0 || z == 0 || x == nx - 1 || y == ny - 1 || z == nz - 1) {
                        bad = 1;
                        continue;
                    }
                    const uint32_t b = brow[x];
                    if (b != NO_BOUNDARY && (int64_t)b >= nb) {
                        bad = 2;
                        continue;
                    }
                    n_air++;
                    if (f == (AIR | 63) && b == NO_BOUNDARY) {
                        word |= 1u << (x - x0);
                        n_int++;
                    } else {
                        const uint32_t ns = b == NO_BOUNDARY ? 0 : grid->bstart[b + 1] - grid->bstart[b];
                        sp[z].push_back({(uint32_t)((z * ny + y) * pl->nxp + x), (uint32_t)(f & 63) | (ns << wk::META_SLOT_SHIFT),
                                         b == NO_BOUNDARY ? 0u : grid->bstart[b]});
                    }
                }
                mrow[x0 / 32] = word;
            }
        }
        air_z[z] = n_air;
        int_z[z] = n_int;
        bad_z[z] = bad;
    }
    for (int64_t z = 0; z < nz; z++) {
        if (bad_z[z] == 1)
            return bail(ctx->fail(WAVEY_E_INVALID,
                                  "air cell on the grid border (plane z=%lld): the grid needs a solid padding layer",
                                  (long long)z));
        if (bad_z[z] == 2) return bail(ctx->fail(WAVEY_E_INVALID, "boundary index out of range in plane z=%lld", (long long)z));
    }
    if (pl->cells_p >= (int64_t)NO_BOUNDARY) return bail(ctx->fail(WAVEY_E_LIMIT, "padded grid exceeds 2^32 cells"));
    // Tap cells leave the interior mask and join the special list, which
    // stays sorted by cell.
    std::vector<uint32_t> tap_p(tap_cells.size());
    for (size_t r = 0; r < tap_cells.size(); r++) {
        const int64_t c = tap_cells[r];
        const int64_t x = c % nx, y = (c / nx) % ny, z = c / (nx * ny);
        tap_p[r] = (uint32_t)((z * ny + y) * pl->nxp + x);
        uint32_t &w = mask[(size_t)((z * ny + y) * nxw + x / 32)];
        if (w & (1u << (x % 32))) {
            w &= ~(1u << (x % 32));
            int_z[z]--;
            sp[z].push_back({tap_p[r], 63u, 0u});
            std::sort(sp[z].begin(), sp[z].end(), [](const Special &a, const Special &b) { return a.cell < b.cell; });
        }
    }
    std::vector<uint32_t> cell_l, meta_l, slot0_l, tap_l;
    for (int64_t z = 0; z < nz; z++) {
        for (const Special &q : sp[z]) {
            cell_l.push_back(q.cell);
            meta_l.push_back(q.meta);
            slot0_l.push_back(q.slot0);
        }
        std::vector<Special>().swap(sp[z]);
    }
    tap_l.assign(cell_l.size(), wk::NO_TAP);
    for (size_t r = 0; r < tap_p.size(); r++) {
        auto it = std::lower_bound(cell_l.begin(), cell_l.end(), tap_p[r]);
        tap_l[(size_t)(it - cell_l.begin())] = (uint32_t)r;
    }
    for (int64_t z = 0; z < nz; z++) {
        pl->air += air_z[z];
        pl->interior += int_z[z];
    }
    pl->n_special = (int64_t)cell_l.size();
    if ((int64_t)pl->n_special * pl->chunks >= (1ll << 40)) return bail(ctx->fail(WAVEY_E_LIMIT, "too many special cells"));

    // Launch geometry.
    pl->tiles_x = (int)(pl->nxp / 32);
    pl->tiles_y = (int)((ny - 2 + wk::TILE_Y - 1) / wk::TILE_Y);
    pl->zt = env_int("WAVEY_FUSED_ZT", ZT, 1, 4096);
    pl->tiles_z = (int)((nz - 2 + pl->zt - 1) / pl->zt);
    const int64_t ib = (int64_t)pl->tiles_x * pl->tiles_y * pl->tiles_z * pl->chunks;
    const int64_t sb = (pl->n_special * pl->chunks + wk::BLOCK - 1) / wk::BLOCK;
    const int64_t rb = (pl->n_recv * pl->chunks + wk::BLOCK - 1) / wk::BLOCK;
    if (ib + sb + rb >= (1ll << 31)) return bail(ctx->fail(WAVEY_E_LIMIT, "launch grid too large"));
    pl->interior_blocks = (int)ib;
    pl->special_blocks = (int)sb;
    pl->record_blocks = (int)rb;

    // Device buffers.
    const size_t E = pl->elem;
    pl->field_bytes = (size_t)pl->cells_p * pl->V * pl->chunks * pl->field_elem;
    for (int k = 0; k < 2; k++)
        if ((st = alloc(pl, &pl->field[k], pl->field_bytes))) return bail(st);
    if ((st = upload(pl, &pl->mask, mask.data(), mask.size() * 4))) return bail(st);
    pl->sp_host.resize(cell_l.size());
    for (size_t i = 0; i < pl->sp_host.size(); i++) pl->sp_host[i] = make_uint4(cell_l[i], meta_l[i], slot0_l[i], tap_l[i]);
    // One block: records | slot constants | branch states u | g, each part
    // 256-byte aligned.
    const size_t sp_bytes = round_up((int64_t)(pl->sp_host.size() * sizeof(uint4)), 256);
    const size_t slot_bytes = round_up((int64_t)(nslots * 4 * E), 256);
    pl->state_bytes = (size_t)pl->chunks * nslots * pl->V * E;
    const size_t st_bytes = round_up((int64_t)pl->state_bytes, 256);
    pl->l2_block_bytes = sp_bytes + slot_bytes + 2 * st_bytes;
    if ((st = alloc(pl, &pl->l2_block, pl->l2_block_bytes))) return bail(st);
    {
        unsigned char *blk = static_cast<unsigned char *>(pl->l2_block);
        pl->sp = reinterpret_cast<uint4 *>(blk);
        pl->slots = blk + sp_bytes;
        pl->su = blk + sp_bytes + slot_bytes;
        pl->sg = blk + sp_bytes + slot_bytes + st_bytes;
    }
    if (!pl->sp_host.empty() &&
        (st = ctx->cuda(cudaMemcpyAsync(pl->sp, pl->sp_host.data(), pl->sp_host.size() * sizeof(uint4),
                                        cudaMemcpyHostToDevice, ctx->stream), "upload")))
        return bail(st);
    pl->h2d_bytes += (int64_t)(pl->sp_host.size() * sizeof(uint4));
    std::vector<double> sig_v;
    if (signal_stride == 0) {
        sig_v.assign(signals, signals + steps);
        pl->sig_stride = 0;
    } else {
        sig_v.resize((size_t)pl->lanes_total * steps, 0.0);
        for (size_t s = 0; s < n_sources; s++)
            std::copy(signals + s * signal_stride, signals + s * signal_stride + steps, sig_v.begin() + s * steps);
        pl->sig_stride = (int64_t)steps;
    }
    std::vector<uint32_t> recv_p(n_recv);
    for (size_t r = 0; r < n_recv; r++) {
        const int64_t c = (int64_t)receivers[r];
        const int64_t x = c % nx, y = (c / nx) % ny, z = c / (nx * ny);
        recv_p[r] = (uint32_t)((z * ny + y) * pl->nxp + x);
    }
    if (precision == WAVEY_FP64) {
        if ((st = upload_into<double>(pl, pl->slots, grid->slots, grid->slots ? 4 * nslots : 0))) return bail(st);
        if ((st = upload_typed<double>(pl, &pl->tapw, tapw))) return bail(st);
        if ((st = upload_typed<double>(pl, &pl->sig, sig_v))) return bail(st);
    } else {
        if ((st = upload_into<float>(pl, pl->slots, grid->slots, grid->slots ? 4 * nslots : 0))) return bail(st);
        if ((st = upload_typed<float>(pl, &pl->tapw, tapw))) return bail(st);
        if ((st = upload_typed<float>(pl, &pl->sig, sig_v))) return bail(st);
    }
    set_l2_window(pl);
    if (precision == WAVEY_FP16_STORAGE) {
        std::vector<float> wm((size_t)pl->lanes_total, 0.0f);
        for (size_t s2 = 0; s2 < n_sources; s2++) {
            double acc = 0.0;
            for (size_t t2 = 0; t2 < sources[s2].n_taps; t2++) acc += std::fabs(sources[s2].taps[t2].w);
            wm[s2] = (float)(acc * (1.0 + 1e-6));
        }
        if ((st = upload(pl, &pl->wmax, wm.data(), wm.size() * 4))) return bail(st);
        if ((st = alloc(pl, &pl->amax, (size_t)wk::AMAX_RING * pl->chunks * nz * sizeof(unsigned int)))) return bail(st);
        if ((st = alloc(pl, &pl->scale, (size_t)wk::SCALE_RING * pl->chunks * nz * sizeof(float2)))) return bail(st);
        pl->fp16_shift = env_int("WAVEY_FP16_SHIFT", 14, 8, 15);
        if ((st = ctx->cuda(cudaStreamSynchronize(ctx->stream), "upload sync"))) return bail(st);
    }
    if ((st = upload(pl, &pl->recv, recv_p.data(), recv_p.size() * 4))) return bail(st);
    if ((st = upload(pl, &pl->freqs, freqs, nf * sizeof(double)))) return bail(st);
    // Standalone plans that run 128-step graphs get two rings (each chunk folds
    // the previous one beside its own steps).
    pl->fold_overlap = standalone && steps >= (size_t)wk::RING && env_int("WAVEY_FOLD_OVERLAP", 1, 0, 1) != 0;
    const int64_t ring_elems = (int64_t)pl->chunks * wk::RING * (int64_t)n_recv * pl->V;
    pl->ring_stride = pl->fold_overlap ? ring_elems : 0;
    if ((st = alloc(pl, &pl->ring, (size_t)ring_elems * (pl->fold_overlap ? 2 : 1) * E))) return bail(st);
    pl->dft64 = precision != WAVEY_FP64 && env_int("WAVEY_DFT_FP64", 0, 0, 1);
    if ((st = alloc(pl, &pl->tw, (size_t)wk::RING * nf * 2 * (pl->dft64 ? sizeof(double) : E)))) return bail(st);
    pl->acc_bytes = (size_t)pl->chunks * n_recv * nf * pl->V * 2 * sizeof(double);
    if ((st = alloc(pl, &pl->acc, pl->acc_bytes))) return bail(st);
    if ((st = alloc(pl, &pl->base, sizeof(long long)))) return bail(st);
    if (pl->want_ir) {
        pl->ir_bytes = (size_t)n_sources * n_recv * steps * E;
        if ((st = alloc(pl, &pl->ir, pl->ir_bytes))) return bail(st);
    }
    for (cudaEvent_t *e : {&pl->ev_a, &pl->ev_b, &pl->ev_t0, &pl->ev_t1, &pl->inflight[0], &pl->inflight[1], &pl->inflight[2],
                           &pl->inflight[3]})
        if ((st = ctx->cuda(cudaEventCreate(e), "event create"))) return bail(st);
    for (cudaEvent_t *e : {&pl->ev_fork, &pl->ev_join, &pl->ev_ffork, &pl->ev_fjoin})
        if ((st = ctx->cuda(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "event create"))) return bail(st);
    if ((st = alloc(pl, &pl->err, sizeof(int)))) return bail(st);
    if (standalone && (precision == WAVEY_FP32 || precision == WAVEY_FP16_STORAGE) && tma_selected()) {
        // Untuned default: 16-row tiles with 5/3-plane rings (FP32) or 32-row
        // tiles with 4/2-plane rings (FP16), the z-run that fills one wave of
        // resident CTAs, and beside it the special-cell kernel -- FP32: capped
        // at four blocks per SM with the interior first, so that one of its
        // blocks fits on every SM beside two interior CTAs; FP16: three blocks
        // per SM with the interior first -- the forms measured fastest on the
        // pillar room.
        cudaError_t e = precision == WAVEY_FP16_STORAGE ? tma_attrs<__half, 1>() : tma_attrs<float, 1>();
        if (e == cudaSuccess) e = precision == WAVEY_FP16_STORAGE ? tma_attrs<__half, 2>() : tma_attrs<float, 2>();
        if (e == cudaSuccess) e = precision == WAVEY_FP16_STORAGE ? tma_attrs<__half, 4>() : tma_attrs<float, 4>();
        if ((st = ctx->cuda(e, "shared memory attribute"))) return bail(st);
        cudaDeviceGetStreamPriorityRange(&pl->prio_lo, &pl->prio_hi);
        // FP32: where one z-layer of 16-row interior tiles (all chunks) fills
        // less than two waves of two CTAs per SM, the interior runs in a
        // partial wave with a special-cell block beside its CTAs (shape 4,
        // form 8); where it spans many waves (the 376 M-cell hall), the
        // three-CTA register policy and equal priority keep more bytes in
        // flight (shape 11, form 3).
        bool many_waves = false;
        if (precision == WAVEY_FP32) {
            const int64_t cells_row = wk::TMA_ROW_FLOATS / pl->V;
            const int64_t layer = ((nx + cells_row - 1) / cells_row) * ((ny - 2 + 15) / 16) * pl->chunks;
            many_waves = layer >= 2 * 2 * (int64_t)ctx->sm_count;
        }
        pl->branch = env_int("WAVEY_BRANCH", precision == WAVEY_FP32 ? (many_waves ? 3 : 8) : 5, 0,
                             precision == WAVEY_FP32 ? BRANCH_FUSED : BRANCH_FUSED - 1);
        const int cfg = env_int("WAVEY_TMA_CFG", precision == WAVEY_FP16_STORAGE ? 6 : (many_waves ? 11 : 4), 0,
                                tma_ncfg(pl) - 1);
        const int zw = wave_zt(pl, cfg, 1);
        const int zt1 = zw ? std::max(8, zw) : 16;
        if ((st = tma_shape(pl, cfg, env_int("WAVEY_TMA_ZT", zt1, 1, 4096)))) return bail(st);
        pl->zalt = env_int("WAVEY_ZALT", 1, 0, 1) != 0;
        pl->tma = true;
        pl->pdl_wanted = env_int("WAVEY_PDL", 1, 0, 1) != 0;
        pl->pdl = pl->pdl_wanted && pdl_safe(pl);
        if (precision == WAVEY_FP32 && pl->V == 4 && env_int("WAVEY_TBLOCK", 0, 0, 1))
            if ((st = tb_setup(pl, mask))) return bail(st);
    }
    if ((st = ctx->cuda(cudaStreamSynchronize(ctx->stream), "upload sync"))) return bail(st);
    if (standalone && steps >= (size_t)wk::RING)
        if ((st = build_graph(pl))) return bail(st);
    *out = pl;
    return WAVEY_OK;
}

// Clears a plan's fields, branch states, spectra, step counter, error word
// and scale tables: every run starts from rest.
int plan_reset(wavey_cuda_plan *pl) {
    wavey_cuda_ctx *ctx = pl->ctx;
    cudaStream_t s = ctx->stream;
    int st;
    apply_l2(pl);
    for (int k = 0; k < 2; k++)
        if ((st = ctx->cuda(cudaMemsetAsync(pl->field[k], 0, pl->field_bytes, s), "memset"))) return st;
    for (int k = 0; k < 2; k++)
        if (pl->field2[k] && (st = ctx->cuda(cudaMemsetAsync(pl->field2[k], 0, pl->field_bytes, s), "memset"))) return st;
    if (pl->state_bytes) {
        if ((st = ctx->cuda(cudaMemsetAsync(pl->su, 0, pl->state_bytes, s), "memset"))) return st;
        if ((st = ctx->cuda(cudaMemsetAsync(pl->sg, 0, pl->state_bytes, s), "memset"))) return st;
    }
    if ((st = ctx->cuda(cudaMemsetAsync(pl->acc, 0, pl->acc_bytes, s), "memset"))) return st;
    if ((st = ctx->cuda(cudaMemsetAsync(pl->base, 0, sizeof(long long), s), "memset"))) return st;
    if ((st = ctx->cuda(cudaMemsetAsync(pl->err, 0, sizeof(int), s), "memset"))) return st;
    if (pl->amax) {
        // Levels 0 and -1 are all zeros: any scale reads them back as zeros.
        if ((st = ctx->cuda(cudaMemsetAsync(pl->amax, 0, (size_t)wk::AMAX_RING * pl->chunks * pl->nz * sizeof(unsigned int), s),
                            "memset")))
            return st;
        if ((st = ctx->cuda(cudaMemsetAsync(pl->scale, 0, (size_t)wk::SCALE_RING * pl->chunks * pl->nz * sizeof(float2), s),
                            "memset")))
            return st;
    }
    return WAVEY_OK;
}

int plan_run(wavey_cuda_plan *pl, const volatile int32_t *cancel, void (*progress)(double, void *), void *user,
             wavey_run_stats *stats) {
    wavey_cuda_ctx *ctx = pl->ctx;
    cudaStream_t s = ctx->stream;
    int st;
    cudaEventRecord(pl->ev_t0, s);
    if ((st = plan_reset(pl))) return st;
    const bool watch = cancel || progress || stats;
    const int64_t full = pl->steps / wk::RING;
    const int rem = (int)(pl->steps % wk::RING);
    double step_ms = 0.0;
    int64_t launches = 0;
    for (int64_t c = 0; c < full; c++) {
        if (cancel && *cancel) {
            cudaStreamSynchronize(s);
            return WAVEY_CANCELLED;
        }
        if ((st = ctx->cuda(cudaGraphLaunch(pl->graph, s), "graph launch"))) return st;
        launches += wk::RING;
        if (stats) {
            if ((st = ctx->cuda(cudaEventSynchronize(pl->ev_b), "chunk wait"))) return st;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, pl->ev_a, pl->ev_b);
            step_ms += ms;
        } else if (watch) {
            // At most two chunks in flight, so cancel and progress keep up.
            cudaEventRecord(pl->inflight[c & 3], s);
            if (c >= 1 && (st = ctx->cuda(cudaEventSynchronize(pl->inflight[(c - 1) & 3]), "chunk wait"))) return st;
        }
        if (progress) progress((double)((c + 1) * wk::RING) / (double)pl->steps, user);
    }
    // The last full chunk's fold (the graphs fold each chunk in the next one).
    if (pl->fold_overlap && full > 0) fold(pl, wk::RING, wk::RING);
    if (rem > 0) {
        if (cancel && *cancel) {
            cudaStreamSynchronize(s);
            return WAVEY_CANCELLED;
        }
        cudaEventRecord(pl->ev_a, s);
        for (int t = 0; t < rem; t++) step(pl, t, t & 1);
        cudaEventRecord(pl->ev_b, s);
        fold(pl, rem);
        launches += rem;
        if ((st = ctx->cuda(cudaGetLastError(), "step launch"))) return st;
        if (stats) {
            if ((st = ctx->cuda(cudaEventSynchronize(pl->ev_b), "chunk wait"))) return st;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, pl->ev_a, pl->ev_b);
            step_ms += ms;
        }
    }
    cudaEventRecord(pl->ev_t1, s);
    if ((st = ctx->cuda(cudaStreamSynchronize(s), "run"))) return st;
    if ((st = ctx->cuda(cudaGetLastError(), "run"))) return st;
    int err_word = 0;
    if ((st = ctx->cuda(cudaMemcpy(&err_word, pl->err, sizeof(int), cudaMemcpyDeviceToHost), "error word"))) return st;
    if (err_word == wk::ERR_FP16_RANGE)
        return ctx->fail(WAVEY_E_DEVICE, "a field value left the FP16 range of its slab scale");
    if (err_word) return ctx->fail(WAVEY_E_DEVICE, "a kernel reported error %d (a bounded wait ran out)", err_word);
    if (progress) progress(1.0, user);
    if (stats) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, pl->ev_t0, pl->ev_t1);
        stats->total_ms = ms;
        stats->step_ms = step_ms;
        stats->step_launches = launches;
        stats->chunks = full + (rem > 0);
    }
    pl->ran = true;
    return WAVEY_OK;
}

int plan_transfers(wavey_cuda_plan *pl, const wavey_transfer_layout *L, float *out, size_t out_floats) {
    wavey_cuda_ctx *ctx = pl->ctx;
    if (!L || !out) return ctx->fail(WAVEY_E_INVALID, "layout or out is null");
    if (!pl->ran) return ctx->fail(WAVEY_E_INVALID, "the plan has not run");
    const int S = L->n_speakers;
    const int64_t R = pl->n_recv, F = pl->nf;
    if (S <= 0 || !L->lane_speaker || !L->factor) return ctx->fail(WAVEY_E_INVALID, "no speakers or factors");
    if (L->n_mics < 0 || L->n_planes < 0 || (L->n_planes > 0 && !L->plane_points))
        return ctx->fail(WAVEY_E_INVALID, "bad receiver layout");
    std::vector<long long> first(1, (long long)L->n_mics);
    for (int p = 0; p < L->n_planes; p++) {
        if (L->plane_points[p] < 0) return ctx->fail(WAVEY_E_INVALID, "negative plane size");
        first.push_back(first.back() + L->plane_points[p]);
    }
    if (first.back() != R) return ctx->fail(WAVEY_E_INVALID, "mics and plane points (%lld) are not the plan's %lld receivers",
                                            (long long)first.back(), (long long)R);
    if (L->n_planes == 0) first.push_back(R);  // one empty plane keeps the kernel's search simple
    if (out_floats != (size_t)(2 * R * F * S)) return ctx->fail(WAVEY_E_INVALID, "out holds %zu floats, not %lld", out_floats,
                                                               (long long)(2 * R * F * S));
    std::vector<int> start(S + 1, 0), lanes;
    for (int s = 0; s < S; s++) {
        for (int l = 0; l < pl->n_sources; l++) {
            const int32_t k = L->lane_speaker[l];
            if (k < -1 || k >= S) return ctx->fail(WAVEY_E_INVALID, "lane %d names speaker %d of %d", l, k, S);
            if (k == s) lanes.push_back(l);
        }
        start[s + 1] = (int)lanes.size();
    }
    if (lanes.empty()) lanes.push_back(0);
    cudaStream_t st0 = ctx->stream;
    void *d_start = nullptr, *d_lanes = nullptr, *d_fac = nullptr, *d_first = nullptr, *d_out = nullptr;
    const size_t fac_bytes = (size_t)pl->n_sources * F * 2 * sizeof(double), out_bytes = out_floats * sizeof(float);
    auto release = [&]() {
        for (void *q : {d_start, d_lanes, d_fac, d_first, d_out})
            if (q) cudaFree(q);
    };
    int st;
    if ((st = ctx->cuda(cudaMalloc(&d_start, start.size() * sizeof(int)), "alloc")) ||
        (st = ctx->cuda(cudaMalloc(&d_lanes, lanes.size() * sizeof(int)), "alloc")) ||
        (st = ctx->cuda(cudaMalloc(&d_fac, fac_bytes), "alloc")) ||
        (st = ctx->cuda(cudaMalloc(&d_first, first.size() * sizeof(long long)), "alloc")) ||
        (st = ctx->cuda(cudaMalloc(&d_out, out_bytes), "alloc"))) {
        release();
        return st;
    }
    cudaMemcpyAsync(d_start, start.data(), start.size() * sizeof(int), cudaMemcpyHostToDevice, st0);
    cudaMemcpyAsync(d_lanes, lanes.data(), lanes.size() * sizeof(int), cudaMemcpyHostToDevice, st0);
    cudaMemcpyAsync(d_fac, L->factor, fac_bytes, cudaMemcpyHostToDevice, st0);
    cudaMemcpyAsync(d_first, first.data(), first.size() * sizeof(long long), cudaMemcpyHostToDevice, st0);
    const long long total = (long long)S * R * F;
    const int n_planes = std::max(L->n_planes, 1);
    if (total > 0)
        wk::speaker_transfers<<<(unsigned)((total + wk::BLOCK - 1) / wk::BLOCK), wk::BLOCK, 0, st0>>>(
            pl->acc, (int)R, (int)F, pl->V, (const int *)d_start, (const int *)d_lanes, (const double2 *)d_fac, S,
            (const long long *)d_first, n_planes, (float2 *)d_out);
    st = ctx->cuda(cudaGetLastError(), "transfers launch");
    if (!st) st = ctx->cuda(cudaMemcpyAsync(out, d_out, out_bytes, cudaMemcpyDeviceToHost, st0), "read transfers");
    if (!st) st = ctx->cuda(cudaStreamSynchronize(st0), "transfers");
    release();
    return st;
}

int plan_band_params(wavey_cuda_plan *pl, const double *bands, int32_t nb, int32_t flags, double *out,
                     size_t out_doubles) {
    wavey_cuda_ctx *ctx = pl->ctx;
    if (!bands || !out) return ctx->fail(WAVEY_E_INVALID, "bands or out is null");
    if (!pl->ran) return ctx->fail(WAVEY_E_INVALID, "the plan has not run");
    if (!pl->want_ir) return ctx->fail(WAVEY_E_INVALID, "the plan records no time series");
    if (nb < 1 || nb > 64) return ctx->fail(WAVEY_E_INVALID, "1 to 64 bands");
    if (flags & ~(wk::IR_INTEGRATE | wk::IR_LUNDEBY)) return ctx->fail(WAVEY_E_INVALID, "unknown flags %d", flags);
    const double fs = 1.0 / pl->dt;
    for (int b = 0; b < nb; b++)
        if (!(bands[b] > 0.0 && bands[b] < 0.5 * fs)) return ctx->fail(WAVEY_E_INVALID, "band %g Hz is not below fs / 2", bands[b]);
    const long long series = (long long)pl->n_sources * pl->n_recv, steps = (long long)pl->steps;
    if (out_doubles != (size_t)(series * nb * 6)) return ctx->fail(WAVEY_E_INVALID, "out holds %zu doubles, not %lld",
                                                                   out_doubles, series * nb * 6);
    if (series == 0 || steps == 0) return WAVEY_OK;
    // Scratch of one launch: a band-passed series per thread; launches take
    // whole series, as many as 2 GiB (or half the free memory) holds.
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const size_t budget = std::min<size_t>((size_t)2 << 30, free_b / 2);
    const long long per_series = (long long)nb * steps * (long long)sizeof(double);
    const long long batch = std::max(1LL, std::min(series, (long long)(budget / (size_t)per_series)));
    cudaStream_t st0 = ctx->stream;
    void *d_onset = nullptr, *d_bands = nullptr, *d_out = nullptr, *d_scratch = nullptr;
    auto release = [&]() {
        for (void *q : {d_onset, d_bands, d_out, d_scratch})
            if (q) cudaFree(q);
    };
    int st;
    if ((st = ctx->cuda(cudaMalloc(&d_onset, series * sizeof(long long)), "alloc")) ||
        (st = ctx->cuda(cudaMalloc(&d_bands, nb * sizeof(double)), "alloc")) ||
        (st = ctx->cuda(cudaMalloc(&d_out, out_doubles * sizeof(double)), "alloc")) ||
        (st = ctx->cuda(cudaMalloc(&d_scratch, (size_t)(batch * per_series)), "alloc scratch"))) {
        release();
        return st;
    }
    cudaMemcpyAsync(d_bands, bands, nb * sizeof(double), cudaMemcpyHostToDevice, st0);
    const unsigned ob = (unsigned)((series + 127) / 128);
    if (pl->precision == WAVEY_FP64)
        wk::ir_onsets<double><<<ob, 128, 0, st0>>>((const double *)pl->ir, steps, series, flags, (long long *)d_onset);
    else
        wk::ir_onsets<float><<<ob, 128, 0, st0>>>((const float *)pl->ir, steps, series, flags, (long long *)d_onset);
    for (long long first = 0; first < series && !st; first += batch) {
        const long long n = std::min(batch, series - first);
        const unsigned blocks = (unsigned)((n * nb + 127) / 128);
        if (pl->precision == WAVEY_FP64)
            wk::ir_band_params<double><<<blocks, 128, 0, st0>>>((const double *)pl->ir, steps, (const long long *)d_onset,
                                                                first, n, (const double *)d_bands, nb, fs, flags,
                                                                (double *)d_scratch, (double *)d_out);
        else
            wk::ir_band_params<float><<<blocks, 128, 0, st0>>>((const float *)pl->ir, steps, (const long long *)d_onset,
                                                               first, n, (const double *)d_bands, nb, fs, flags,
                                                               (double *)d_scratch, (double *)d_out);
        st = ctx->cuda(cudaGetLastError(), "band parameters launch");
    }
    if (!st) st = ctx->cuda(cudaMemcpyAsync(out, d_out, out_doubles * sizeof(double), cudaMemcpyDeviceToHost, st0),
                            "read band parameters");
    if (!st) st = ctx->cuda(cudaStreamSynchronize(st0), "band parameters");
    release();
    return st;
}

// ---------------------------------------------------------------- grid build
void free_device_grid(wavey_device_grid *g) {
    if (!g) return;
    for (void *q : {(void *)g->flags, (void *)g->bidx, (void *)g->bcell, (void *)g->bstart, (void *)g->slots})
        if (q) cudaFree(q);
    delete g;
}

// Surfaces in build_room order: floor, ceiling, walls y0, x1, y1, x0, then 4
// faces per pillar and 6 per block (the host builder's list).
std::vector<wk::GbRect> room_rects_of(const wh_room *r) {
    std::vector<wk::GbRect> s;
    auto add = [&](int axis, double c, double x0, double y0, double z0, double x1, double y1, double z1) {
        wk::GbRect q;
        q.axis = axis;
        q.c = c;
        q.lo[0] = x0, q.lo[1] = y0, q.lo[2] = z0;
        q.hi[0] = x1, q.hi[1] = y1, q.hi[2] = z1;
        s.push_back(q);
    };
    const double h = r->height;
    add(2, 0.0, r->x0, r->y0, 0, r->x1, r->y1, 0);
    add(2, h, r->x0, r->y0, 0, r->x1, r->y1, 0);
    add(1, r->y0, r->x0, 0, 0.0, r->x1, 0, h);
    add(0, r->x1, 0, r->y0, 0.0, 0, r->y1, h);
    add(1, r->y1, r->x0, 0, 0.0, r->x1, 0, h);
    add(0, r->x0, 0, r->y0, 0.0, 0, r->y1, h);
    for (int i = 0; i < r->n_pillars; i++) {
        const double *p = r->pillars + 4 * i;
        add(1, p[1], p[0], 0, 0.0, p[2], 0, h);
        add(0, p[0], 0, p[1], 0.0, 0, p[3], h);
        add(1, p[3], p[0], 0, 0.0, p[2], 0, h);
        add(0, p[2], 0, p[1], 0.0, 0, p[3], h);
    }
    for (int i = 0; i < r->n_blocks; i++) {
        const double *b = r->blocks + 6 * i;
        add(0, b[0], 0, b[1], b[2], 0, b[4], b[5]);
        add(0, b[3], 0, b[1], b[2], 0, b[4], b[5]);
        add(1, b[1], b[0], 0, b[2], b[3], 0, b[5]);
        add(1, b[4], b[0], 0, b[2], b[3], 0, b[5]);
        add(2, b[2], b[0], b[1], 0, b[3], b[4], 0);
        add(2, b[5], b[0], b[1], 0, b[3], b[4], 0);
    }
    return s;
}

// A room given as triangles (wh_mesh_room_triangles' output): positions
// [n_tri][3][3], wound to their surface's normal, and each one's surface.
struct MeshIn {
    const double *pos;
    const uint32_t *tri_surface;
    int64_t n_tri;
};

// Triangles binned across one axis, as the host builder bins them
// (mesh.cpp, AxisBins): cells of side max(4 dx, extent / 4096) over the
// padded bounds; a triangle goes to every cell its padded extent touches.
struct HostBins {
    wk::GbBins b{};
    std::vector<uint32_t> start, list;
};

HostBins bins_for_axis(const MeshIn &m, int axis, const double lo[3], const double hi[3], double dx) {
    HostBins hb;
    wk::GbBins &b = hb.b;
    b.u = (axis + 1) % 3;
    b.v = (axis + 2) % 3;
    double ext2 = 0.0;
    for (int a = 0; a < 3; a++) ext2 += (hi[a] - lo[a]) * (hi[a] - lo[a]);
    const double pad = 1e-6 * (1.0 + std::sqrt(ext2));
    b.u0 = lo[b.u] - 2.0 * pad;
    b.v0 = lo[b.v] - 2.0 * pad;
    const double eu = hi[b.u] - lo[b.u] + 4.0 * pad, ev = hi[b.v] - lo[b.v] + 4.0 * pad;
    b.h = std::max(4.0 * dx, std::max(eu, ev) / 4096.0);
    b.nu = std::max<long long>(1, (long long)std::ceil(eu / b.h));
    b.nv = std::max<long long>(1, (long long)std::ceil(ev / b.h));
    auto cu = [&](double a) { return std::min(b.nu - 1, std::max<long long>(0, (long long)std::floor((a - b.u0) / b.h))); };
    auto cv = [&](double a) { return std::min(b.nv - 1, std::max<long long>(0, (long long)std::floor((a - b.v0) / b.h))); };
    std::vector<std::vector<uint32_t>> cells((size_t)(b.nu * b.nv));
    for (int64_t t = 0; t < m.n_tri; t++) {
        double a0 = INFINITY, a1 = -INFINITY, c0 = INFINITY, c1 = -INFINITY;
        for (int k = 0; k < 3; k++) {
            const double *q = m.pos + 9 * t + 3 * k;
            a0 = std::min(a0, q[b.u]);
            a1 = std::max(a1, q[b.u]);
            c0 = std::min(c0, q[b.v]);
            c1 = std::max(c1, q[b.v]);
        }
        for (long long j = cv(c0 - pad); j <= cv(c1 + pad); j++)
            for (long long i = cu(a0 - pad); i <= cu(a1 + pad); i++) cells[(size_t)(j * b.nu + i)].push_back((uint32_t)t);
    }
    hb.start.assign(cells.size() + 1, 0u);
    for (size_t k = 0; k < cells.size(); k++) hb.start[k + 1] = hb.start[k] + (uint32_t)cells[k].size();
    hb.list.reserve(hb.start.back());
    for (const auto &c : cells) hb.list.insert(hb.list.end(), c.begin(), c.end());
    return hb;
}

int grid_build(wavey_cuda_ctx *ctx, const wh_room *room, const MeshIn *mesh, const double *mesh_solids,
               int32_t mesh_n_solids, const wh_fit *fits, int32_t n_fits, double c, double dx, wavey_device_grid **out,
               wavey_grid_shape *shape) {
    if (!out || !shape) return ctx->fail(WAVEY_E_INVALID, "out or shape is null");
    *out = nullptr;
    std::vector<wk::GbRect> rects;
    double lo[3], hi[3];
    std::vector<double> tri;
    HostBins bins[3];
    if (mesh) {
        if (!mesh->pos || !mesh->tri_surface || mesh->n_tri <= 0 || mesh->n_tri >= (1ll << 31) || !(dx > 0.0) ||
            !(c > 0.0) || mesh_n_solids < 0 || (mesh_n_solids > 0 && !mesh_solids) || !fits || n_fits <= 0)
            return ctx->fail(WAVEY_E_INVALID, "invalid mesh room or spacing");
        for (int a = 0; a < 3; a++) lo[a] = INFINITY, hi[a] = -INFINITY;
        tri.resize((size_t)mesh->n_tri * 9);
        for (int64_t t = 0; t < mesh->n_tri; t++) {
            if (mesh->tri_surface[t] >= (uint32_t)n_fits)
                return ctx->fail(WAVEY_E_INVALID, "triangle %lld: surface %u without a fit", (long long)t,
                                 mesh->tri_surface[t]);
            const double *v = mesh->pos + 9 * t;
            for (int k = 0; k < 3; k++)
                for (int a = 0; a < 3; a++) {
                    lo[a] = std::min(lo[a], v[3 * k + a]);
                    hi[a] = std::max(hi[a], v[3 * k + a]);
                }
            for (int a = 0; a < 3; a++) {
                tri[9 * t + a] = v[a];
                tri[9 * t + 3 + a] = v[3 + a] - v[a];
                tri[9 * t + 6 + a] = v[6 + a] - v[a];
            }
        }
        for (int a = 0; a < 3; a++) bins[a] = bins_for_axis(*mesh, a, lo, hi, dx);
    } else {
        if (!room || !(dx > 0.0) || !(c > 0.0) || !(room->height > 0.0) || room->x1 <= room->x0 || room->y1 <= room->y0)
            return ctx->fail(WAVEY_E_INVALID, "invalid room or spacing");
        if ((room->n_pillars > 0 && !room->pillars) || (room->n_blocks > 0 && !room->blocks) ||
            (room->n_solids > 0 && !room->solids) || room->n_pillars < 0 || room->n_blocks < 0 || room->n_solids < 0)
            return ctx->fail(WAVEY_E_INVALID, "invalid room lists");
        rects = room_rects_of(room);
        if ((int)rects.size() != n_fits || !fits)
            return ctx->fail(WAVEY_E_INVALID, "%d fits for %zu surfaces", n_fits, rects.size());
        lo[0] = room->x0, lo[1] = room->y0, lo[2] = 0.0;
        hi[0] = room->x1, hi[1] = room->y1, hi[2] = room->height;
    }
    const int n_pillars = mesh ? 0 : room->n_pillars, n_blocks = mesh ? 0 : room->n_blocks;
    const int n_solids = mesh ? mesh_n_solids : room->n_solids;
    const double *solids = mesh ? mesh_solids : room->solids;
    wavey_grid_shape sh{};
    sh.dx = dx;
    sh.dt = WAVEY_COURANT * dx / c;
    for (int a = 0; a < 3; a++) {
        sh.origin[a] = lo[a] - dx * 0.5;
        sh.n[a] = (int64_t)std::ceil((hi[a] - lo[a]) / dx) + 2;
    }
    const long long cells = (long long)sh.n[0] * sh.n[1] * sh.n[2];
    if ((unsigned long long)cells > WAVEY_MAX_CELLS) return ctx->fail(WAVEY_E_LIMIT, "%lld cells > MAX_CELLS", cells);
    cudaStream_t s = ctx->stream;
    wavey_device_grid *g = new (std::nothrow) wavey_device_grid();
    if (!g) return ctx->fail(WAVEY_E_NOMEM, "host allocation failed");
    g->ctx = ctx;
    std::vector<void *> tmp;
    auto dalloc = [&](void **p, size_t bytes, bool keep) -> int {
        int st = ctx->cuda(cudaMalloc(p, std::max<size_t>(bytes, 8)), "grid alloc");
        if (!st && !keep) tmp.push_back(*p);
        return st;
    };
    auto fail = [&](int st) {
        for (void *q : tmp) cudaFree(q);
        free_device_grid(g);
        return st;
    };
    const long long nscan = (cells + wk::SCAN_BLOCK - 1) / wk::SCAN_BLOCK;
    void *d_pill = nullptr, *d_blk = nullptr, *d_sol = nullptr, *d_rects = nullptr, *d_fits = nullptr, *d_solid = nullptr,
         *d_air = nullptr, *d_cnt = nullptr, *d_atot = nullptr, *d_ntot = nullptr, *d_stot = nullptr, *d_grand = nullptr,
         *d_node_at = nullptr, *d_slot_at = nullptr;
    void *d_tri = nullptr, *d_tsurf = nullptr, *d_inside = nullptr, *d_err = nullptr, *d_bstart[3] = {}, *d_blist[3] = {};
    int st;
    if (mesh) {
        if ((st = dalloc(&d_tri, sizeof(double) * tri.size(), false)) ||
            (st = dalloc(&d_tsurf, sizeof(uint32_t) * (size_t)mesh->n_tri, false)) ||
            (st = dalloc(&d_inside, (size_t)cells, false)) || (st = dalloc(&d_err, sizeof(int), false)))
            return fail(st);
        for (int a = 0; a < 3; a++)
            if ((st = dalloc(&d_bstart[a], 4 * bins[a].start.size(), false)) ||
                (st = dalloc(&d_blist[a], 4 * bins[a].list.size(), false)))
                return fail(st);
    }
    if ((st = dalloc(&d_pill, sizeof(double) * 4 * n_pillars, false)) ||
        (st = dalloc(&d_blk, sizeof(double) * 6 * n_blocks, false)) ||
        (st = dalloc(&d_sol, sizeof(double) * 6 * n_solids, false)) ||
        (st = dalloc(&d_rects, sizeof(wk::GbRect) * rects.size(), false)) ||
        (st = dalloc(&d_fits, sizeof(wh_fit) * n_fits, false)) || (st = dalloc(&d_solid, cells, false)) ||
        (st = dalloc(&d_air, cells, false)) || (st = dalloc(&d_cnt, 4 * (size_t)cells, false)) ||
        (st = dalloc(&d_atot, 8 * (size_t)nscan, false)) || (st = dalloc(&d_ntot, 8 * (size_t)nscan, false)) ||
        (st = dalloc(&d_stot, 8 * (size_t)nscan, false)) || (st = dalloc(&d_grand, 24, false)) ||
        (st = dalloc(&d_node_at, 4 * (size_t)cells, false)) || (st = dalloc(&d_slot_at, 8 * (size_t)cells, false)) ||
        (st = dalloc((void **)&g->flags, cells, true)) || (st = dalloc((void **)&g->bidx, 4 * (size_t)cells, true)))
        return fail(st);
    if (n_pillars) cudaMemcpyAsync(d_pill, room->pillars, sizeof(double) * 4 * n_pillars, cudaMemcpyHostToDevice, s);
    if (n_blocks) cudaMemcpyAsync(d_blk, room->blocks, sizeof(double) * 6 * n_blocks, cudaMemcpyHostToDevice, s);
    if (n_solids) cudaMemcpyAsync(d_sol, solids, sizeof(double) * 6 * n_solids, cudaMemcpyHostToDevice, s);
    if (!rects.empty()) cudaMemcpyAsync(d_rects, rects.data(), sizeof(wk::GbRect) * rects.size(), cudaMemcpyHostToDevice, s);
    if (mesh) {
        cudaMemcpyAsync(d_tri, tri.data(), sizeof(double) * tri.size(), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(d_tsurf, mesh->tri_surface, sizeof(uint32_t) * (size_t)mesh->n_tri, cudaMemcpyHostToDevice, s);
        for (int a = 0; a < 3; a++) {
            cudaMemcpyAsync(d_bstart[a], bins[a].start.data(), 4 * bins[a].start.size(), cudaMemcpyHostToDevice, s);
            if (!bins[a].list.empty())
                cudaMemcpyAsync(d_blist[a], bins[a].list.data(), 4 * bins[a].list.size(), cudaMemcpyHostToDevice, s);
        }
        cudaMemsetAsync(d_err, 0, sizeof(int), s);
    }
    cudaMemcpyAsync(d_fits, fits, sizeof(wh_fit) * n_fits, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(g->flags, 0, cells, s);
    cudaMemsetAsync(g->bidx, 0xFF, 4 * (size_t)cells, s);
    wk::GbRoom r{};
    if (!mesh) r.x0 = room->x0, r.y0 = room->y0, r.x1 = room->x1, r.y1 = room->y1, r.height = room->height;
    r.n_pillars = n_pillars, r.n_blocks = n_blocks, r.n_solids = n_solids;
    r.n_rects = (int)rects.size();
    r.mesh = mesh ? 1 : 0;
    if (mesh) {
        r.n_tri = mesh->n_tri;
        r.tri = (const double *)d_tri;
        r.tri_surface = (const uint32_t *)d_tsurf;
        for (int a = 0; a < 3; a++) {
            r.bins[a] = bins[a].b;
            r.bins[a].start = (const uint32_t *)d_bstart[a];
            r.bins[a].list = (const uint32_t *)d_blist[a];
        }
        r.inside = (const uint8_t *)d_inside;
    }
    r.pillars = (const double *)d_pill, r.blocks = (const double *)d_blk, r.solids = (const double *)d_sol;
    r.rects = (const wk::GbRect *)d_rects;
    r.fits = (const wh_fit *)d_fits;
    r.nx = sh.n[0], r.ny = sh.n[1], r.nz = sh.n[2];
    for (int a = 0; a < 3; a++) r.origin[a] = sh.origin[a];
    r.dx = sh.dx, r.dt = sh.dt;
    const unsigned blocks = (unsigned)((cells + 255) / 256);
    if (mesh) {
        const long long cols = (long long)sh.n[0] * sh.n[1];
        wk::grid_column_fill<<<(unsigned)((cols + 255) / 256), 256, 0, s>>>(r, (uint8_t *)d_inside, (int *)d_err);
        int err = 0;
        cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, s);
        if ((st = ctx->cuda(cudaStreamSynchronize(s), "column fill"))) return fail(st);
        if (err)
            return fail(ctx->fail(WAVEY_E_LIMIT, "a grid column crosses the mesh more than %d times",
                                  wk::GB_MAX_CROSSINGS));
    }
    wk::grid_classify<<<blocks, 256, 0, s>>>(r, (uint8_t *)d_solid, (uint8_t *)d_air);
    wk::grid_flags<<<blocks, 256, 0, s>>>(r, (const uint8_t *)d_air, g->flags);
    wk::grid_nodes<<<blocks, 256, 0, s>>>(r, (const uint8_t *)d_solid, g->flags, (uint32_t *)d_cnt, false, nullptr,
                                          nullptr, nullptr, nullptr, nullptr, nullptr);
    wk::scan_totals<<<(unsigned)nscan, wk::SCAN_BLOCK, 0, s>>>((const uint32_t *)d_cnt, g->flags, cells,
                                                               (unsigned long long *)d_ntot, (unsigned long long *)d_stot,
                                                               (unsigned long long *)d_atot);
    wk::scan_block_totals<<<1, wk::SCAN_BLOCK, 0, s>>>((unsigned long long *)d_ntot, (unsigned long long *)d_stot,
                                                       (const unsigned long long *)d_atot, nscan,
                                                       (unsigned long long *)d_grand);
    wk::scan_apply<<<(unsigned)nscan, wk::SCAN_BLOCK, 0, s>>>((const uint32_t *)d_cnt, cells,
                                                              (const unsigned long long *)d_ntot,
                                                              (const unsigned long long *)d_stot, (uint32_t *)d_node_at,
                                                              (unsigned long long *)d_slot_at);
    unsigned long long grand[3] = {0, 0, 0};
    cudaMemcpyAsync(grand, d_grand, 24, cudaMemcpyDeviceToHost, s);
    if ((st = ctx->cuda(cudaStreamSynchronize(s), "grid build"))) return fail(st);
    if (grand[0] >= (unsigned long long)WAVEY_NO_BOUNDARY) return fail(ctx->fail(WAVEY_E_LIMIT, "too many boundary nodes"));
    sh.air_cells = (int64_t)grand[2];
    sh.n_boundary = (int64_t)grand[0];
    sh.n_slots = (int64_t)grand[1];
    if ((st = dalloc((void **)&g->bcell, 4 * (size_t)sh.n_boundary, true)) ||
        (st = dalloc((void **)&g->bstart, 4 * ((size_t)sh.n_boundary + 1), true)) ||
        (st = dalloc((void **)&g->slots, 32 * (size_t)sh.n_slots, true)))
        return fail(st);
    wk::grid_nodes<<<blocks, 256, 0, s>>>(r, (const uint8_t *)d_solid, g->flags, (uint32_t *)d_cnt, true,
                                          (const uint32_t *)d_node_at, (const unsigned long long *)d_slot_at, g->bidx,
                                          g->bcell, g->bstart, g->slots);
    const uint32_t last = (uint32_t)sh.n_slots;
    cudaMemcpyAsync(g->bstart + sh.n_boundary, &last, 4, cudaMemcpyHostToDevice, s);
    if ((st = ctx->cuda(cudaStreamSynchronize(s), "grid build"))) return fail(st);
    for (void *q : tmp) cudaFree(q);
    g->shape = sh;
    *shape = sh;
    *out = g;
    return WAVEY_OK;
}

int grid_read(wavey_device_grid *g, uint8_t *flags, uint32_t *bidx, uint32_t *bcell, uint32_t *bstart, double *slots) {
    wavey_cuda_ctx *ctx = g->ctx;
    const wavey_grid_shape &sh = g->shape;
    const size_t cells = (size_t)sh.n[0] * sh.n[1] * sh.n[2];
    if (!flags || !bidx || !bstart || (sh.n_boundary && !bcell) || (sh.n_slots && !slots))
        return ctx->fail(WAVEY_E_INVALID, "null output array");
    int st;
    if ((st = ctx->cuda(cudaMemcpy(flags, g->flags, cells, cudaMemcpyDeviceToHost), "read flags")) ||
        (st = ctx->cuda(cudaMemcpy(bidx, g->bidx, 4 * cells, cudaMemcpyDeviceToHost), "read bidx")) ||
        (sh.n_boundary && (st = ctx->cuda(cudaMemcpy(bcell, g->bcell, 4 * (size_t)sh.n_boundary, cudaMemcpyDeviceToHost), "read bcell"))) ||
        (st = ctx->cuda(cudaMemcpy(bstart, g->bstart, 4 * ((size_t)sh.n_boundary + 1), cudaMemcpyDeviceToHost), "read bstart")) ||
        (sh.n_slots && (st = ctx->cuda(cudaMemcpy(slots, g->slots, 32 * (size_t)sh.n_slots, cudaMemcpyDeviceToHost), "read slots"))))
        return st;
    return WAVEY_OK;
}

int plan_read(wavey_cuda_plan *pl, double *out, double *ir_out) {
    wavey_cuda_ctx *ctx = pl->ctx;
    if (!pl->ran) return ctx->fail(WAVEY_E_INVALID, "the plan has not run");
    int st;
    if (out && pl->acc_bytes) {
        // Copied into a zero-filled vector (its pages are in place before
        // the copy), then reordered in one sequential pass over it: from
        // [chunk][receiver][f][lane] to [source][receiver][f].  (Threads
        // writing the caller's fresh pages contend on page faults.)
        std::vector<double> acc(pl->acc_bytes / sizeof(double));
        if ((st = ctx->cuda(cudaMemcpy(acc.data(), pl->acc, pl->acc_bytes, cudaMemcpyDeviceToHost), "read spectra"))) return st;
        const int64_t R = pl->n_recv, F = pl->nf, V = pl->V, S = pl->n_sources;
        const double *a = acc.data();
        for (int64_t c = 0; c < pl->chunks; c++)
            for (int64_t r = 0; r < R; r++)
                for (int64_t f = 0; f < F; f++)
                    for (int64_t l = 0; l < V; l++, a += 2) {
                        const int64_t s = c * V + l;
                        if (s >= S) continue;
                        double *o = out + ((s * R + r) * F + f) * 2;
                        o[0] = a[0];
                        o[1] = a[1];
                    }
    }
    if (ir_out) {
        if (!pl->want_ir) return ctx->fail(WAVEY_E_INVALID, "the plan records no time series");
        const size_t n = pl->ir_bytes / pl->elem;
        if (pl->precision == WAVEY_FP64) {
            if ((st = ctx->cuda(cudaMemcpy(ir_out, pl->ir, pl->ir_bytes, cudaMemcpyDeviceToHost), "read ir"))) return st;
        } else {
            std::unique_ptr<float[]> v(new (std::nothrow) float[n]);
            if (!v) return ctx->fail(WAVEY_E_NOMEM, "host allocation failed");
            if ((st = ctx->cuda(cudaMemcpy(v.get(), pl->ir, pl->ir_bytes, cudaMemcpyDeviceToHost), "read ir"))) return st;
            const float *src = v.get();
#pragma omp parallel for schedule(static) num_threads(host_threads()) if (n >= (1u << 16))
            for (int64_t i = 0; i < (int64_t)n; i++) ir_out[i] = (double)src[i];
        }
    }
    return WAVEY_OK;
}


// ----------------------------------------------------------------- rooms
template <class T, bool RUST>
int rooms_table(wavey_cuda_rooms *rm) {
    std::vector<wk::RoomStep<T>> table(rm->plans.size());
    rm->total_blocks = 0;
    for (size_t r = 0; r < rm->plans.size(); r++) {
        wavey_cuda_plan *pl = rm->plans[r];
        for (int parity = 0; parity < 2; parity++) {
            fill_args<T>(pl, table[r].a[parity], parity);
            table[r].a[parity].base = rm->base;
        }
        table[r].lanes = pl->V;
        table[r].blocks = pl->interior_blocks + pl->special_blocks + pl->record_blocks;
        table[r].steps = pl->steps;
        if ((int64_t)rm->total_blocks + table[r].blocks >= (1ll << 31)) return rm->ctx->fail(WAVEY_E_LIMIT, "launch grid too large");
        rm->total_blocks += table[r].blocks;
    }
    const size_t bytes = table.size() * sizeof(wk::RoomStep<T>);
    cudaError_t e = cudaMalloc(&rm->table, bytes);
    if (e != cudaSuccess) return rm->ctx->cuda(e, "rooms table");
    return rm->ctx->cuda(cudaMemcpy(rm->table, table.data(), bytes, cudaMemcpyHostToDevice), "rooms table");
}

void rooms_step(wavey_cuda_rooms *rm, int t) {
    if (rm->total_blocks == 0) return;
    cudaStream_t s = rm->ctx->stream;
    const int n = (int)rm->plans.size();
    if (rm->precision == WAVEY_FP64)
        wk::fdtd_step_rooms<double, true><<<rm->total_blocks, wk::BLOCK, 0, s>>>(
            reinterpret_cast<const wk::RoomStep<double> *>(rm->table), n, t, t & 1);
    else
        wk::fdtd_step_rooms<float, false><<<rm->total_blocks, wk::BLOCK, 0, s>>>(
            reinterpret_cast<const wk::RoomStep<float> *>(rm->table), n, t, t & 1);
}

int rooms_graph(wavey_cuda_rooms *rm) {
    wavey_cuda_ctx *ctx = rm->ctx;
    cudaStream_t s = ctx->stream;
    cudaGraph_t g = nullptr;
    int st = ctx->cuda(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
    if (st) return st;
    cudaEventRecordWithFlags(rm->ev_a, s, cudaEventRecordExternal);
    for (int t = 0; t < wk::RING; t++) rooms_step(rm, t);
    cudaEventRecordWithFlags(rm->ev_b, s, cudaEventRecordExternal);
    for (wavey_cuda_plan *pl : rm->plans) fold(pl, wk::RING);  // each stops at its own last step
    wk::advance_base<<<1, 1, 0, s>>>(rm->base, wk::RING);
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (e != cudaSuccess) return ctx->cuda(e, "end capture");
    size_t nodes = 0;
    cudaGraphGetNodes(g, nullptr, &nodes);
    std::vector<cudaGraphNode_t> list(nodes);
    cudaGraphGetNodes(g, list.data(), &nodes);
    rm->graph_kernels = 0;
    for (cudaGraphNode_t nd : list) {
        cudaGraphNodeType ty;
        if (cudaGraphNodeGetType(nd, &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel) rm->graph_kernels++;
    }
    e = cudaGraphInstantiateWithFlags(&rm->graph, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    return ctx->cuda(e, "graph instantiate");
}

int rooms_create(wavey_cuda_ctx *ctx, const wavey_room_job *jobs, size_t n_jobs, int32_t precision, int32_t want_ir,
                 wavey_cuda_rooms **out) {
    if (!out) return ctx->fail(WAVEY_E_INVALID, "out is null");
    *out = nullptr;
    if (!jobs || n_jobs == 0) return ctx->fail(WAVEY_E_INVALID, "no rooms");
    if (n_jobs > 1024) return ctx->fail(WAVEY_E_LIMIT, "at most 1024 rooms per launch");
    if (precision != WAVEY_FP32 && precision != WAVEY_FP64)
        return ctx->fail(WAVEY_E_INVALID, "rooms run in FP32 or FP64 (precision %d)", precision);
    wavey_cuda_rooms *rm = new (std::nothrow) wavey_cuda_rooms();
    if (!rm) return ctx->fail(WAVEY_E_NOMEM, "host allocation failed");
    rm->ctx = ctx;
    rm->precision = precision;
    auto bail = [&](int code) {
        delete rm;
        return code;
    };
    int st;
    for (size_t r = 0; r < n_jobs; r++) {
        const wavey_room_job &j = jobs[r];
        wavey_cuda_plan *pl = nullptr;
        st = plan_create(ctx, j.grid, j.sources, j.n_sources, j.signals, j.signal_stride, j.steps, j.receivers, j.n_recv,
                         j.freqs, j.nf, precision, want_ir, &pl, false);
        if (st) {
            std::string msg = ctx->err;
            ctx->fail(st, "room %zu: %s", r, msg.c_str());
            return bail(st);
        }
        rm->plans.push_back(pl);
        rm->max_steps = std::max<int64_t>(rm->max_steps, pl->steps);
    }
    cudaError_t e = cudaMalloc(&rm->base, sizeof(long long));
    if (e != cudaSuccess) return bail(ctx->cuda(e, "step counter"));
    for (wavey_cuda_plan *pl : rm->plans) pl->base = rm->base;
    st = precision == WAVEY_FP64 ? rooms_table<double, true>(rm) : rooms_table<float, false>(rm);
    if (st) return bail(st);
    for (cudaEvent_t *ev : {&rm->ev_a, &rm->ev_b, &rm->ev_t0, &rm->ev_t1})
        if ((st = ctx->cuda(cudaEventCreate(ev), "event create"))) return bail(st);
    if ((st = rooms_graph(rm))) return bail(st);
    *out = rm;
    return WAVEY_OK;
}

int rooms_run(wavey_cuda_rooms *rm, const volatile int32_t *cancel, void (*progress)(double, void *), void *user,
              wavey_run_stats *stats) {
    wavey_cuda_ctx *ctx = rm->ctx;
    cudaStream_t s = ctx->stream;
    int st;
    cudaEventRecord(rm->ev_t0, s);
    for (wavey_cuda_plan *pl : rm->plans)
        if ((st = plan_reset(pl))) return st;
    if ((st = ctx->cuda(cudaMemsetAsync(rm->base, 0, sizeof(long long), s), "memset"))) return st;
    const int64_t chunks = (rm->max_steps + wk::RING - 1) / wk::RING;
    double step_ms = 0.0;
    for (int64_t c = 0; c < chunks; c++) {
        if (cancel && *cancel) {
            cudaStreamSynchronize(s);
            return WAVEY_CANCELLED;
        }
        if ((st = ctx->cuda(cudaGraphLaunch(rm->graph, s), "graph launch"))) return st;
        if (stats || cancel || progress) {
            if ((st = ctx->cuda(cudaEventSynchronize(rm->ev_b), "chunk wait"))) return st;
            if (stats) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, rm->ev_a, rm->ev_b);
                step_ms += ms;
            }
        }
        if (progress) progress((double)std::min<int64_t>((c + 1) * wk::RING, rm->max_steps) / (double)rm->max_steps, user);
    }
    cudaEventRecord(rm->ev_t1, s);
    if ((st = ctx->cuda(cudaStreamSynchronize(s), "run"))) return st;
    for (size_t r = 0; r < rm->plans.size(); r++) {
        int err_word = 0;
        if ((st = ctx->cuda(cudaMemcpy(&err_word, rm->plans[r]->err, sizeof(int), cudaMemcpyDeviceToHost), "error word")))
            return st;
        if (err_word) return ctx->fail(WAVEY_E_DEVICE, "room %zu: a kernel reported error %d", r, err_word);
        rm->plans[r]->ran = true;
    }
    if (stats) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, rm->ev_t0, rm->ev_t1);
        stats->total_ms = ms;
        stats->step_ms = step_ms;
        stats->step_launches = chunks * wk::RING;
        stats->chunks = chunks;
    }
    rm->ran = true;
    return WAVEY_OK;
}


// The autotuner.  Stage 1: every candidate shape of the TMA interior kernel
// (tile rows and ring depths, z-run), each with two forms of the
// special-cell kernel beside it -- equal priority at three blocks per SM, and
// interior first at four blocks per SM, which fits beside a partial wave of
// interior CTAs -- runs two 128-step chunks of this plan's own grid; the
// fastest step span wins.  Stage 2: with that shape, every other form of the
// special-cell update.  Stage 4: the four fastest distinct candidates again,
// each over up to four timed chunks after a warm one, so that a one-chunk
// timing's noise does not pick between near-equal candidates.  The plan keeps
// the winner.  Needs a TMA plan with at least 256 steps.
int plan_autotune(wavey_cuda_plan *pl, wavey_tune_result *res) {
    wavey_cuda_ctx *ctx = pl->ctx;
    if (res) *res = wavey_tune_result{};
    if (!pl->tma || pl->steps < 2 * wk::RING || !pl->graph) return WAVEY_OK;
    int best_cfg = pl->tma_cfg, best_zt = pl->tma_zt, best_branch = pl->branch, n = 0, st;
    double best = 1e30;
    cudaStream_t s = ctx->stream;
    struct Cand {
        int cfg, zt, branch;
        double us;
    };
    std::vector<Cand> all;
    // Mean step span of chunks 2..reps+1 of the plan in shape (cfg, zt, branch).
    auto timed = [&](int cfg, int zt, int branch, int reps, double *us) -> int {
        pl->branch = branch;
        if ((st = tma_shape(pl, cfg, zt))) return st;
        cudaGraphExecDestroy(pl->graph);
        pl->graph = nullptr;
        if ((st = build_graph(pl))) return st;
        if ((st = plan_reset(pl))) return st;
        double sum = 0.0;
        for (int rep = 0; rep <= reps; rep++) {
            float ms = 0.f;
            if ((st = ctx->cuda(cudaGraphLaunch(pl->graph, s), "graph launch"))) return st;
            if ((st = ctx->cuda(cudaEventSynchronize(pl->ev_b), "tune wait"))) return st;
            cudaEventElapsedTime(&ms, pl->ev_a, pl->ev_b);
            if (rep > 0) sum += ms;  // the first chunk warms up
        }
        *us = 1e3 * sum / reps / wk::RING;
        return WAVEY_OK;
    };
    auto trial = [&](int cfg, int zt, int branch) -> int {
        double us = 0.0;
        if ((st = timed(cfg, zt, branch, pl->steps >= 3 * wk::RING ? 2 : 1, &us))) return st;
        all.push_back({cfg, zt, branch, us});
        if (res && n < WAVEY_TUNE_MAX) {
            res->cand_cfg[n] = cfg;
            res->cand_zt[n] = zt;
            res->cand_branch[n] = branch;
            res->cand_step_us[n] = us;
        }
        n++;
        if (us < best) {
            best = us;
            best_cfg = cfg;
            best_zt = zt;
            best_branch = branch;
        }
        return WAVEY_OK;
    };
    for (int family : {3, 8}) {
        pl->branch = family;
        const std::vector<int> zts = tune_zts(pl);
        for (int cfg = 0; cfg < tma_ncfg(pl); cfg++)
            for (int zt : zts)
                if ((st = trial(cfg, zt, family))) return st;
    }
    const int cfg1 = best_cfg, zt1 = best_zt, br1 = best_branch;
    const int forms = pl->precision == WAVEY_FP32 ? BRANCH_FUSED + 1 : BRANCH_FUSED;
    for (int branch = 0; branch < forms; branch++)
        if (branch != br1 && (st = trial(cfg1, zt1, branch))) return st;
    if (best_branch == BRANCH_FUSED) {
        // Stage 3: the fused form's own best shape (its CTAs carry the
        // special cells, so another tile height or z-run may win).
        pl->branch = BRANCH_FUSED;
        const std::vector<int> zts = tune_zts(pl);
        for (int cfg = 0; cfg < tma_ncfg(pl); cfg++)
            for (int zt : zts)
                if (!(cfg == cfg1 && zt == zt1) && (st = trial(cfg, zt, BRANCH_FUSED))) return st;
    }
    // Stage 4: confirm among the fastest four (chunks the plan's own steps
    // cover: its signals end there).
    const int reps = (int)std::min<int64_t>(4, pl->steps / wk::RING - 1);
    if (reps >= 2) {
        std::sort(all.begin(), all.end(), [](const Cand &a, const Cand &b) { return a.us < b.us; });
        double confirmed = 1e30;
        for (size_t i = 0; i < all.size() && i < 4; i++) {
            double us = 0.0;
            if ((st = timed(all[i].cfg, all[i].zt, all[i].branch, reps, &us))) return st;
            if (us < confirmed) {
                confirmed = us;
                best_cfg = all[i].cfg;
                best_zt = all[i].zt;
                best_branch = all[i].branch;
            }
        }
        best = confirmed;
    }
    pl->branch = best_branch;
    if ((st = tma_shape(pl, best_cfg, best_zt))) return st;
    cudaGraphExecDestroy(pl->graph);
    pl->graph = nullptr;
    if ((st = build_graph(pl))) return st;
    if ((st = ctx->cuda(cudaStreamSynchronize(s), "tune"))) return st;
    if (res) {
        res->cfg = best_cfg;
        res->zt = best_zt;
        res->branch = best_branch;
        res->rows = TMA_CFGS[best_cfg].rows;
        res->p_planes = TMA_CFGS[best_cfg].np;
        res->q_planes = TMA_CFGS[best_cfg].nq;
        res->step_us = best;
        res->candidates = std::min(n, WAVEY_TUNE_MAX);
    }
    return WAVEY_OK;
}

}  // namespace

extern "C" {

int wavey_cuda_create(int device, wavey_cuda_ctx **out) {
    if (!out) return WAVEY_E_INVALID;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return WAVEY_E_CUDA;
    }
    if (device < 0 || device >= n) return WAVEY_E_INVALID;
    wavey_cuda_ctx *ctx = new (std::nothrow) wavey_cuda_ctx();
    if (!ctx) return WAVEY_E_NOMEM;
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->folds, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete ctx;
        return WAVEY_E_CUDA;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) {
        ctx->sm_count = prop.multiProcessorCount;
        snprintf(ctx->name, sizeof ctx->name, "%s", prop.name);
        ctx->max_persist_l2 = prop.persistingL2CacheMaxSize;
        ctx->max_window = prop.accessPolicyMaxWindowSize;
        ctx->l2_bytes = (size_t)prop.l2CacheSize;
        ctx->regs_per_sm = prop.regsPerMultiprocessor;
        ctx->smem_per_sm = (int64_t)prop.sharedMemPerMultiprocessor;
        ctx->smem_reserved = (int64_t)prop.reservedSharedMemPerBlock;
        ctx->threads_per_sm = prop.maxThreadsPerMultiProcessor;
    }
    // The tiled receiver fold stages up to DFT_SMEM_MAX bytes of twiddles.
    for (const void *fn : {(const void *)wk::dft_chunk_tiled<1>, (const void *)wk::dft_chunk_tiled<2>,
                           (const void *)wk::dft_chunk_tiled<4>})
        if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, wk::DFT_SMEM_MAX) != cudaSuccess) {
            cudaGetLastError();
            wavey_cuda_destroy(ctx);
            return WAVEY_E_CUDA;
        }
    *out = ctx;
    return WAVEY_OK;
}

void wavey_cuda_destroy(wavey_cuda_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->folds) cudaStreamDestroy(ctx->folds);
    delete ctx;
}

const char *wavey_cuda_last_error(const wavey_cuda_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int wavey_cuda_device_info(wavey_cuda_ctx *ctx, char *name, size_t name_cap, int *sm_count) {
    if (!ctx) return WAVEY_E_INVALID;
    if (name && name_cap) snprintf(name, name_cap, "%s", ctx->name);
    if (sm_count) *sm_count = ctx->sm_count;
    return WAVEY_OK;
}

int wavey_cuda_plan_create(wavey_cuda_ctx *ctx, const wavey_grid *grid, const wavey_source *sources, size_t n_sources,
                           const double *signals, size_t signal_stride, size_t steps, const uint64_t *receivers,
                           size_t n_recv, const double *freqs, size_t nf, int32_t precision, int32_t want_ir,
                           wavey_cuda_plan **out) {
    if (!ctx) return WAVEY_E_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mu);
    cudaSetDevice(ctx->device);
    return plan_create(ctx, grid, sources, n_sources, signals, signal_stride, steps, receivers, n_recv, freqs, nf, precision,
                       want_ir, out);
}

int wavey_cuda_plan_run(wavey_cuda_plan *plan, const volatile int32_t *cancel, void (*progress)(double, void *), void *user,
                        wavey_run_stats *stats) {
    if (!plan) return WAVEY_E_INVALID;
    std::lock_guard<std::mutex> lock(plan->ctx->mu);
    cudaSetDevice(plan->ctx->device);
    return plan_run(plan, cancel, progress, user, stats);
}

int wavey_cuda_plan_read(wavey_cuda_plan *plan, double *out, double *ir_out) {
    if (!plan) return WAVEY_E_INVALID;
    std::lock_guard<std::mutex> lock(plan->ctx->mu);
    cudaSetDevice(plan->ctx->device);
    return plan_read(plan, out, ir_out);
}

int wavey_cuda_plan_autotune(wavey_cuda_plan *plan, wavey_tune_result *result) {
    if (!plan) return WAVEY_E_INVALID;
    std::lock_guard<std::mutex> lock(plan->ctx->mu);
    cudaSetDevice(plan->ctx->device);
    return plan_autotune(plan, result);
}

int wavey_cuda_plan_transfers(wavey_cuda_plan *plan, const wavey_transfer_layout *layout, float *out,
                              size_t out_floats) {
    if (!plan) return WAVEY_E_INVALID;
    std::lock_guard<std::mutex> lock(plan->ctx->mu);
    cudaSetDevice(plan->ctx->device);
    return plan_transfers(plan, layout, out, out_floats);
}

int wavey_cuda_plan_band_params(wavey_cuda_plan *plan, const double *bands_hz, int32_t n_bands, int32_t flags,
                                double *out, size_t out_doubles) {
    if (!plan) return WAVEY_E_INVALID;
    std::lock_guard<std::mutex> lock(plan->ctx->mu);
    cudaSetDevice(plan->ctx->device);
    return plan_band_params(plan, bands_hz, n_bands, flags, out, out_doubles);
}

int wavey_cuda_grid_build(wavey_cuda_ctx *ctx, const wh_room *room, const wh_fit *fits, int32_t n_fits, double c,
                          double dx, wavey_device_grid **out, wavey_grid_shape *shape) {
    if (!ctx) return WAVEY_E_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mu);
    cudaSetDevice(ctx->device);
    return grid_build(ctx, room, nullptr, nullptr, 0, fits, n_fits, c, dx, out, shape);
}

int wavey_cuda_grid_build_mesh(wavey_cuda_ctx *ctx, const double *positions, const uint32_t *tri_surface,
                               int64_t n_tri, const double *solids, int32_t n_solids, const wh_fit *fits, int32_t n_fits,
                               double c, double dx, wavey_device_grid **out, wavey_grid_shape *shape) {
    if (!ctx) return WAVEY_E_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mu);
    cudaSetDevice(ctx->device);
    const MeshIn m{positions, tri_surface, n_tri};
    return grid_build(ctx, nullptr, &m, solids, n_solids, fits, n_fits, c, dx, out, shape);
}

int wavey_cuda_grid_read(wavey_device_grid *grid, uint8_t *flags, uint32_t *bidx, uint32_t *bcell, uint32_t *bstart,
                         double *slots) {
    if (!grid) return WAVEY_E_INVALID;
    std::lock_guard<std::mutex> lock(grid->ctx->mu);
    cudaSetDevice(grid->ctx->device);
    return grid_read(grid, flags, bidx, bcell, bstart, slots);
}

void wavey_cuda_grid_free(wavey_device_grid *grid) {
    if (!grid) return;
    std::lock_guard<std::mutex> lock(grid->ctx->mu);
    cudaSetDevice(grid->ctx->device);
    free_device_grid(grid);
}

int wavey_cuda_plan_info(const wavey_cuda_plan *pl, wavey_plan_info *info) {
    if (!pl || !info) return WAVEY_E_INVALID;
    info->cells = pl->cells;
    info->air_cells = pl->air;
    info->interior_cells = pl->interior;
    info->special_cells = pl->n_special;
    info->boundary_slots = pl->n_slots;
    info->sources = pl->n_sources;
    info->lanes = pl->V;
    info->chunks = pl->chunks;
    info->receivers = pl->n_recv;
    info->freqs = pl->nf;
    info->steps = pl->steps;
    info->device_bytes = pl->device_bytes;
    info->padded_nx = pl->nxp;
    info->precision = pl->precision;
    info->h2d_bytes = pl->h2d_bytes;
    info->d2h_bytes = (int64_t)pl->acc_bytes + (int64_t)pl->ir_bytes;
    info->graph_kernels = pl->graph_kernels;
    info->interior_kernel = pl->tma ? 1 : 0;
    info->tma_zt = pl->tma ? pl->tma_zt : 0;
    info->tma_depth = pl->tma ? pl->tma_cfg : -1;
    info->branch = pl->tma ? pl->branch : -1;
    info->dft_fp64 = pl->precision == WAVEY_FP64 || pl->dft64 ? 1 : 0;
    info->two_step = pl->tb2 ? 1 : 0;
    info->two_step_rows = pl->tb2 ? pl->tb_rows : 0;
    info->two_step_zt = pl->tb2 ? pl->tb_zt : 0;
    info->programmatic = pl->pdl ? 1 : 0;
    return WAVEY_OK;
}

void wavey_cuda_plan_destroy(wavey_cuda_plan *plan) {
    if (!plan) return;
    wavey_cuda_ctx *ctx = plan->ctx;
    std::lock_guard<std::mutex> lock(ctx->mu);
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    delete plan;
}

int wavey_cuda_fdtd_run_batch(wavey_cuda_ctx *ctx, const wavey_grid *grid, const wavey_source *sources, size_t n_sources,
                              const double *signals, size_t signal_stride, size_t steps, const uint64_t *receivers,
                              size_t n_recv, const double *freqs, size_t nf, int32_t precision, double *out, double *ir_out,
                              const volatile int32_t *cancel, void (*progress)(double, void *), void *user) {
    if (!ctx) return WAVEY_E_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mu);
    cudaSetDevice(ctx->device);
    if (!out && n_recv * nf > 0) return ctx->fail(WAVEY_E_INVALID, "out is null");
    wavey_cuda_plan *pl = nullptr;
    int st = plan_create(ctx, grid, sources, n_sources, signals, signal_stride, steps, receivers, n_recv, freqs, nf,
                         precision, ir_out != nullptr, &pl);
    if (st) return st;
    st = plan_run(pl, cancel, progress, user, nullptr);
    if (st == WAVEY_OK) st = plan_read(pl, out, ir_out);
    cudaStreamSynchronize(ctx->stream);
    delete pl;
    return st;
}

int wavey_cuda_fdtd_run(wavey_cuda_ctx *ctx, const wavey_grid *grid, const wavey_tap *taps, size_t n_taps,
                        const double *signal, size_t steps, const uint64_t *receivers, size_t n_recv, const double *freqs,
                        size_t nf, double *out, double *ir_out, const volatile int32_t *cancel,
                        void (*progress)(double, void *), void *user) {
    wavey_source src{taps, n_taps};
    return wavey_cuda_fdtd_run_batch(ctx, grid, &src, 1, signal, 0, steps, receivers, n_recv, freqs, nf, WAVEY_FP32, out,
                                     ir_out, cancel, progress, user);
}

int wavey_cuda_rooms_create(wavey_cuda_ctx *ctx, const wavey_room_job *jobs, size_t n_jobs, int32_t precision,
                            int32_t want_ir, wavey_cuda_rooms **out) {
    if (!ctx) return WAVEY_E_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mu);
    cudaSetDevice(ctx->device);
    return rooms_create(ctx, jobs, n_jobs, precision, want_ir, out);
}

int wavey_cuda_rooms_run(wavey_cuda_rooms *rooms, const volatile int32_t *cancel, void (*progress)(double, void *),
                         void *user, wavey_run_stats *stats) {
    if (!rooms) return WAVEY_E_INVALID;
    std::lock_guard<std::mutex> lock(rooms->ctx->mu);
    cudaSetDevice(rooms->ctx->device);
    return rooms_run(rooms, cancel, progress, user, stats);
}

int wavey_cuda_rooms_read(wavey_cuda_rooms *rooms, size_t room, double *out, double *ir_out) {
    if (!rooms) return WAVEY_E_INVALID;
    std::lock_guard<std::mutex> lock(rooms->ctx->mu);
    cudaSetDevice(rooms->ctx->device);
    if (room >= rooms->plans.size()) return rooms->ctx->fail(WAVEY_E_INVALID, "room %zu out of range", room);
    return plan_read(rooms->plans[room], out, ir_out);
}

int wavey_cuda_rooms_info(const wavey_cuda_rooms *rooms, size_t room, wavey_plan_info *info) {
    if (!rooms || room >= rooms->plans.size()) return WAVEY_E_INVALID;
    int st = wavey_cuda_plan_info(rooms->plans[room], info);
    info->graph_kernels = rooms->graph_kernels;
    return st;
}

void wavey_cuda_rooms_destroy(wavey_cuda_rooms *rooms) {
    if (!rooms) return;
    wavey_cuda_ctx *ctx = rooms->ctx;
    std::lock_guard<std::mutex> lock(ctx->mu);
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    delete rooms;
}

int wavey_cuda_fdtd_run_rooms(wavey_cuda_ctx *ctx, const wavey_room_job *jobs, size_t n_jobs, int32_t precision,
                              const volatile int32_t *cancel, void (*progress)(double, void *), void *user) {
    if (!ctx) return WAVEY_E_INVALID;
    std::lock_guard<std::mutex> lock(ctx->mu);
    cudaSetDevice(ctx->device);
    bool want_ir = false;
    for (size_t r = 0; jobs && r < n_jobs; r++) want_ir = want_ir || jobs[r].ir_out;
    wavey_cuda_rooms *rm = nullptr;
    int st = rooms_create(ctx, jobs, n_jobs, precision, want_ir, &rm);
    if (st) return st;
    st = rooms_run(rm, cancel, progress, user, nullptr);
    for (size_t r = 0; st == WAVEY_OK && r < n_jobs; r++)
        if (jobs[r].out || jobs[r].ir_out) st = plan_read(rm->plans[r], jobs[r].out, jobs[r].ir_out);
    cudaStreamSynchronize(ctx->stream);
    delete rm;
    return st;
}

}  // extern "C"

