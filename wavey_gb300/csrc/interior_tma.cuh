// interior_tma.cuh -- the interior leapfrog update fed by TMA (FP32).
//
// A CTA owns a tile of R rows x 128 floats of one z-run (32 cells of a
// 4-source chunk, 64 cells of a 2-source chunk or 128 cells of one source)
// and marches z -- FP32 fields upwards on even steps and downwards on odd
// ones (TmaArgs::rev), so that a step begins on the planes the previous step
// touched last: on grids a few times the size of L2 those reads hit in L2.  One thread
// issues cp.async.bulk.tensor loads of whole planes several planes ahead
// into a ring in shared memory:
//
//   P ring (NP planes): p^n with a one-row halo in y and a 16-byte halo in x
//                       (box 136 floats x R+2 rows), so the x, y and z
//                       neighbours of every cell are read from shared memory;
//   Q ring (NQ planes): p^(n-1) of the tile (box 128 floats x R rows).
//
// Each plane's arrival is an mbarrier phase (arrive.expect_tx + complete_tx).
// Out-of-range boxes (the first x tile's left halo, rows past the grid)
// are filled with zeros by the TMA unit without touching memory, and the x
// extent of the tensor stops at the real row end, so the row padding is
// never read.  Writes of p^(n+1) go straight to global memory, masked to the
// interior cells; every other cell belongs to the special-cell kernel that
// runs beside this one.
//
// The arithmetic is interior_update's (rounded separately, shader order), so
// results are identical to the register-queue kernel's.
//
// The same kernel serves FP16 storage (E = __half): the rings then hold FP16
// planes (a row is still 128 elements, the x halo 8 elements = 16 bytes so
// every box starts on a 16-byte boundary), p^(n+1) is stored with the next
// level's scale, and every warp raises its slab maximum.  The update is that
// of fdtd_step_half's interior role (every value scaled by its slab's power
// of two, the same FP32 operations in the same order), evaluated in the
// centre plane's own scale with most neighbours entering through
// mixed-precision adds (see the row loop): the two give identical results.
//
// With SPEC (FP32 only) the CTA also updates the special cells of its tile:
// after the interior cells of plane z it takes the tile's special cells of
// that plane from a list ordered by (tile, plane) and runs the special-cell
// update on them -- rigid faces, boundary nodes with their branch states,
// source taps -- reading p^n and p^(n-1) from the rings it already holds
// (every neighbour of a tile cell lies in the staged planes and halos) and
// the slot constants and branch states from global memory.  The special work
// then rides on the interior's bytes in flight instead of a separate kernel
// whose dependent load chains run after the interior's.  The update is
// special_core's, so results do not change by a bit.
//
// Every wait on an mbarrier is bounded.  If one runs out, the kernel records
// the failure in the error word, waits (again bounded) for the copies it has
// issued, and returns; the host reports WAVEY_E_DEVICE.
#pragma once
#include <cuda.h>
#include <cstdint>

#include "fdtd_half.cuh"
#include "fdtd_kernels.cuh"

namespace wk {

constexpr int TMA_ROW_FLOATS = 128;         // elements per tile row (32 lanes x 4)
template <class E>
__host__ __device__ constexpr int tma_halo() { return 16 / (int)sizeof(E); }  // 16-byte halo on each side in x
template <class E>
__host__ __device__ constexpr int tma_p_row() { return TMA_ROW_FLOATS + 2 * tma_halo<E>(); }  // 136 or 144

constexpr uint32_t WAIT_LIMIT = 1u << 24;   // try_wait rounds before a wait is declared lost
constexpr int ERR_TMA_WAIT = 1;

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: true when the phase completed.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t i = 0; i < WAIT_LIMIT; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(dst),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
}

template <class E>
struct TmaArgs {
    const uint32_t *interior;  // [nz][ny][nxw]
    E *nxt;                    // p^(n-1) in, p^(n+1) out, [chunks][cells_p][V]
    int *error;                // error word
    long long cells_p;
    int nxp, ny, nz, nxw;
    int tiles_x, tiles_y, tiles_z, zt;
    int rev;                   // march z downwards (1) or upwards (0)
    float l2;
    // FP16 storage only: the step (*base + t), slab scales and maxima.
    const long long *base;
    int t, chunks;
    const float2 *scale;       // [SCALE_RING][chunks][nz]
    unsigned int *amax;        // [AMAX_RING][chunks][nz]
};

// Four consecutive elements of shared memory as floats (times the slab scale sc for FP16).
__device__ __forceinline__ void ld4(const float *p, float o[4], float) {
    const float4 v = *reinterpret_cast<const float4 *>(p);
    o[0] = v.x, o[1] = v.y, o[2] = v.z, o[3] = v.w;
}
__device__ __forceinline__ void ld4(const __half *p, float o[4], float sc) {
    const uint2 raw = *reinterpret_cast<const uint2 *>(p);
    const __half2 a = *reinterpret_cast<const __half2 *>(&raw.x), b = *reinterpret_cast<const __half2 *>(&raw.y);
    o[0] = __low2float(a) * sc;
    o[1] = __high2float(a) * sc;
    o[2] = __low2float(b) * sc;
    o[3] = __high2float(b) * sc;
}

// Four consecutive FP16 elements of shared memory as stored (bit patterns).
__device__ __forceinline__ void ld4h(const __half *p, uint16_t o[4]) {
    const uint2 raw = *reinterpret_cast<const uint2 *>(p);
    o[0] = (uint16_t)(raw.x & 0xffffu), o[1] = (uint16_t)(raw.x >> 16);
    o[2] = (uint16_t)(raw.y & 0xffffu), o[3] = (uint16_t)(raw.y >> 16);
}

// c + h for an FP16 h, rounded once to nearest (sm_100's mixed-precision
// add: h converts to FP32 exactly inside the add), so it equals
// radd(c, float(h)) bit for bit with one instruction instead of two.
__device__ __forceinline__ float radd_h(float c, uint16_t h) {
    float r;
    asm("add.rn.f32.f16 %0, %1, %2;" : "=f"(r) : "h"(h), "f"(c));
    return r;
}

// a / b for slab scales a and b: powers of two in FP32's normal range, or
// both zero (a level not yet written), whose ratio is taken as 1.  Exact, by
// subtracting the exponents in the bit patterns.
__device__ __forceinline__ float scale_ratio(float a, float b) {
    return __int_as_float(__float_as_int(a) - __float_as_int(b) + 0x3f800000);
}

// max(m, |x|) with NaN propagated (a NaN among the maxima must reach the
// range check).
__device__ __forceinline__ float max_abs_nan(float m, float x) {
    float r;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(m), "f"(fabsf(x)));
    return r;
}

// The same without the slab scale: FP16 values as stored, converted exactly.
__device__ __forceinline__ void ld4u(const float *p, float o[4]) { ld4(p, o, 1.0f); }
__device__ __forceinline__ void ld4u(const __half *p, float o[4]) {
    const uint2 raw = *reinterpret_cast<const uint2 *>(p);
    const __half2 a = *reinterpret_cast<const __half2 *>(&raw.x), b = *reinterpret_cast<const __half2 *>(&raw.y);
    o[0] = __low2float(a);
    o[1] = __high2float(a);
    o[2] = __low2float(b);
    o[3] = __high2float(b);
}

// Field access of the special-cell update from the staged planes (FP32): the
// cell's element in the p^n planes z, z - 1 and z + 1 and in the p^(n-1)
// plane, all in shared memory, and the global store of p^(n+1).
template <int V>
__device__ __forceinline__ Lanes<float, V> lds(const float *p) {
    Lanes<float, V> o;
    if constexpr (V == 4) {
        const float4 v = *reinterpret_cast<const float4 *>(p);
        o.v[0] = v.x, o.v[1] = v.y, o.v[2] = v.z, o.v[3] = v.w;
    } else if constexpr (V == 2) {
        const float2 v = *reinterpret_cast<const float2 *>(p);
        o.v[0] = v.x, o.v[1] = v.y;
    } else {
        o.v[0] = *p;
    }
    return o;
}

template <int V>
struct SmemField {
    static constexpr bool STREAM = true;
    const float *c, *zm, *zp, *q;  // the cell in p^n planes z, z-1, z+1 and in the p^(n-1) plane
    int prow;                      // elements per staged p row
    float *Q;                      // the chunk's p^(n-1) / p^(n+1) field in global memory
    __device__ __forceinline__ Lanes<float, V> p(long long, int) const { return lds<V>(c); }
    __device__ __forceinline__ Lanes<float, V> nb(long long, int d, long long) const {
        return lds<V>(d == 0 ? c - V : d == 1 ? c + V : d == 2 ? c - prow : d == 3 ? c + prow : d == 4 ? zm : zp);
    }
    __device__ __forceinline__ Lanes<float, V> old(long long) const { return lds<V>(q); }
    __device__ __forceinline__ void put(long long cell, const Lanes<float, V> &v) const { store<float, V>(Q + cell * V, v); }
};

// One right-hand side (lane l) of a special cell, from the staged planes:
// special_core's FP32 arithmetic (shader order) for a single lane.  A
// cell's V lanes run on V neighbouring threads, so each thread holds one
// lane's values: the constants and branch states of up to SLOT_REGS slots
// are loaded together, before the neighbour sums, in one round of memory
// latency.  Every lane computes the cell's s1 and denominator itself, with
// the same operations, so the lanes agree with the V-wide update bit for bit.
template <int V>
__device__ __forceinline__ void special_lane(const StepArgs<float> &a, const SmemField<V> &f, const uint4 rec, int c,
                                             int l, long long n) {
    const uint32_t m = rec.y;
    const long long j0 = rec.z;
    const uint32_t tap = rec.w;
    const int ns = (int)((m >> META_SLOT_SHIFT) & META_SLOT_MASK);
    float *SU = a.su + (long long)c * a.n_slots * V + l;
    float *SG = a.sg + (long long)c * a.n_slots * V + l;
    const float4 *K = reinterpret_cast<const float4 *>(a.slots);
    float4 k[SLOT_REGS];
    float u[SLOT_REGS], g[SLOT_REGS];
#pragma unroll
    for (int q = 0; q < SLOT_REGS; q++)
        if (q < ns) {
            k[q] = __ldg(K + j0 + q);
            u[q] = SU[(j0 + q) * V];
            g[q] = SG[(j0 + q) * V];
        }
    const float pc = f.c[l], pp = f.q[l];
    float sum = 0.0f, kk = 0.0f;
#pragma unroll
    for (int d = 0; d < 6; d++)
        if ((m >> d) & 1u) {
            const float *nb = d == 0 ? f.c - V : d == 1 ? f.c + V : d == 2 ? f.c - f.prow : d == 3 ? f.c + f.prow
                            : d == 4 ? f.zm : f.zp;
            sum = radd(sum, nb[l]);
            kk = radd(kk, 1.0f);
        }
    const float lap = rmul(a.l2, rsub(sum, rmul(kk, pc)));
    float next;
    if (ns == 0) {
        next = radd(rsub(rmul(2.0f, pc), pp), lap);
    } else {
        float s1 = 0.0f, s2 = 0.0f;
        for (int q = 0; q < ns; q++) {
            float4 kq;
            float uq, gq;
            if (q < SLOT_REGS) {
#pragma unroll
                for (int i = 0; i < SLOT_REGS; i++)
                    if (i == q) kq = k[i], uq = u[i], gq = g[i];
            } else {
                kq = __ldg(K + j0 + q);
                uq = SU[(j0 + q) * V];
                gq = SG[(j0 + q) * V];
            }
            // kq = (inv_d, cv, k, w)
            const float e = rmul(radd(radd(rsub(rmul(kq.y, uq), rmul(kq.z, gq)), rmul(0.5f, pc)), rmul(kq.w, pp)), kq.x);
            s2 = rsub(radd(s2, e), uq);
            s1 = radd(s1, rmul(rsub(0.5f, kq.w), kq.x));
        }
        const float den = radd(1.0f, rmul(a.lam, s1));
        next = rdiv(rsub(radd(rsub(rmul(2.0f, pc), pp), lap), rmul(a.lam, s2)), den);
        for (int q = 0; q < ns; q++) {
            float4 kq;
            float uq, gq;
            if (q < SLOT_REGS) {
#pragma unroll
                for (int i = 0; i < SLOT_REGS; i++)
                    if (i == q) kq = k[i], uq = u[i], gq = g[i];
            } else {
                kq = __ldg(K + j0 + q);
                uq = SU[(j0 + q) * V];
                gq = SG[(j0 + q) * V];
            }
            const float e = rmul(radd(radd(rsub(rmul(kq.y, uq), rmul(kq.z, gq)), rmul(0.5f, pc)), rmul(kq.w, pp)), kq.x);
            const float un = radd(rmul(rmul(rsub(0.5f, kq.w), kq.x), next), e);
            SG[(j0 + q) * V] = radd(gq, rmul(a.half_dt, radd(un, uq)));
            SU[(j0 + q) * V] = un;
        }
    }
    if (tap != NO_TAP) {
        const int s = c * V + l;
        next = radd(next, rmul(a.sig[(long long)s * a.sig_stride + n], a.tapw[(long long)tap * a.lanes_total + s]));
    }
    f.Q[(long long)rec.x * V + l] = next;
}

// The special cells of every tile, for the SPEC form: records (as in
// StepArgs::sp) ordered by (tile row ty, tile column tx, z, y, x); off[(ty *
// tiles_x + tx) * nz + z] is the first record of that tile and plane, and the
// next entry ends it.  a carries the update's slots, branch states, taps and
// signals.
struct SpecTile {
    const uint4 *rec;
    const uint32_t *off;
    StepArgs<float> a;
};

// V: sources per cell in a chunk (1, 2 or 4); a tile row holds 128 / V cells.
// R: rows per tile (8 or 16; 256 threads, R / 8 rows per thread).
// NP / NQ: planes in the two rings; NP - 3 p planes and NQ - 1 old planes are
// in flight while one plane is computed.
template <class E, int R>
__host__ __device__ constexpr uint32_t tma_p_bytes() { return tma_p_row<E>() * (R + 2) * sizeof(E); }
template <class E, int R>
__host__ __device__ constexpr uint32_t tma_p_stride() { return (tma_p_bytes<E, R>() + 127) / 128 * 128; }
template <class E, int R>
__host__ __device__ constexpr uint32_t tma_q_bytes() { return TMA_ROW_FLOATS * R * sizeof(E); }
// FP16: the slab scales of a CTA's z-run, staged in shared memory (z-runs of
// FP16 plans are at most TMA_MAX_ZT planes).
constexpr int TMA_MAX_ZT = 64;
constexpr int TMA_SCALE_STRIDE = TMA_MAX_ZT + 2;
// SPEC: the first special record of each plane of the z-run (z-runs of
// SPEC plans are at most TMA_MAX_ZT planes too).
template <class E, bool SPEC>
__host__ __device__ constexpr uint32_t tma_scale_bytes() {
    return sizeof(E) == 2 ? 4 * TMA_SCALE_STRIDE * 4 : SPEC ? TMA_SCALE_STRIDE * 4 : 0;
}
template <class E, int R, int NP, int NQ, bool SPEC = false>
__host__ __device__ constexpr uint32_t tma_smem_of() {
    return NP * tma_p_stride<E, R>() + NQ * tma_q_bytes<E, R>() + 256 + tma_scale_bytes<E, SPEC>() + 128;
}

// Registers (LB: the launch bounds' minimum resident CTAs per SM): FP32
// kernels come in two policies, LB = 1 (ptxas gives the 16-row shape 90
// registers: two CTAs per SM, with room on every SM for a block of the
// special-cell kernel beside them) and LB = 3 (three CTAs per SM, more bytes
// in flight where the interior dominates); the FP16 kernel, instruction-
// bound, uses LB = 0, the compiler's own choice; SPEC caps at three CTAs.
// ALT: the march direction follows TmaArgs::rev (FP32); FP16 kernels, whose
// time is instruction issue rather than HBM, always march upwards and keep
// the registers the choice would cost.
template <class E, int V, int R, int NP, int NQ, bool SPEC = false, int LB = 1, bool ALT = (sizeof(E) == 4)>
__global__ void __launch_bounds__(256, SPEC ? 3 : LB) interior_tma(const __grid_constant__ CUtensorMap tm_p,
                                                    const __grid_constant__ CUtensorMap tm_q, TmaArgs<E> a,
                                                    const __grid_constant__ SpecTile sp) {
    static_assert(!SPEC || sizeof(E) == 4, "special cells inside the march: FP32 fields only");
    constexpr bool HALF = sizeof(E) == 2;
    constexpr int RT = R / 8;                    // rows per thread
    constexpr int HALO = tma_halo<E>(), PROW = tma_p_row<E>();
    constexpr uint32_t PB = tma_p_bytes<E, R>(), PS = tma_p_stride<E, R>(), QB = tma_q_bytes<E, R>();
    constexpr int CELLS = TMA_ROW_FLOATS / V;    // cells per tile row
    constexpr uint32_t GROUP = (1u << (4 / V)) - 1u;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    E *Pbuf = reinterpret_cast<E *>(base);
    E *Qbuf = reinterpret_cast<E *>(base + NP * PS);
    uint64_t *bars = reinterpret_cast<uint64_t *>(base + NP * PS + NQ * QB);
    const uint32_t barP = smem_addr(bars), barQ = smem_addr(bars + NP);

    const int per_chunk = a.tiles_x * a.tiles_y * a.tiles_z;
    int b = blockIdx.x;
    const int c = b / per_chunk;
    b -= c * per_chunk;
    const int tz = b / (a.tiles_x * a.tiles_y);
    b -= tz * a.tiles_x * a.tiles_y;
    const int ty = b / a.tiles_x;
    const int tx = b - ty * a.tiles_x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int y0 = 1 + ty * R;
    const int zs = 1 + tz * a.zt;
    const int ze = min(zs + a.zt, a.nz - 1);
    const int Kq = ze - zs;      // output planes
    const int Kp = Kq + 2;       // p planes zs-1 .. ze
    const int cx = tx * TMA_ROW_FLOATS;
    // March direction.  Upwards the p planes arrive as zs-1, zs, .., ze and
    // the output planes as zs .. ze-1; downwards as ze, ze-1, .., zs-1 and
    // ze-1 .. zs.  Alternating it from step to step starts each step on the
    // planes the previous one touched last, which are still in L2.
    const bool rev = ALT && a.rev;
    const int dz = rev ? -1 : 1;
    const int zq0 = rev ? ze - 1 : zs;     // first output plane
    const int zp0 = zq0 - dz;              // first p plane

    // FP16: slab scales of the z-run -- p^n of planes zs-1..ze (2^E of level
    // n), p^(n-1) of planes zs..ze-1 (level n-1), the inverse scales of level
    // n+1 for the stores and their range limits -- staged once, so no plane
    // waits on them.
    float *ssc = reinterpret_cast<float *>(base + NP * PS + NQ * QB + 256);
    unsigned int *wmax = reinterpret_cast<unsigned int *>(bars + 16);  // FP16: [2][8] warp maxima of two planes
    if constexpr (HALF) {
        const long long n = *a.base + a.t;
        const float2 *s_now = a.scale + ((int)(n % SCALE_RING) * a.chunks + c) * a.nz;
        const float2 *s_old = a.scale + ((int)((n + SCALE_RING - 1) % SCALE_RING) * a.chunks + c) * a.nz;
        const float2 *s_new = a.scale + ((int)((n + 1) % SCALE_RING) * a.chunks + c) * a.nz;
        for (int i = threadIdx.x; i < Kp; i += 256) ssc[i] = s_now[zs - 1 + i].x;
        for (int i = threadIdx.x; i < Kq; i += 256) {
            ssc[TMA_SCALE_STRIDE + i] = s_old[zs + i].x;
            ssc[2 * TMA_SCALE_STRIDE + i] = s_new[zs + i].y;
            // Largest |p^(n+1)| the plane can store: 65504 * 2^E, as float bits
            // (at most FLT_MAX's, so that infinities and NaNs exceed it).
            ssc[3 * TMA_SCALE_STRIDE + i] =
                __uint_as_float(min(__float_as_uint(65504.0f * s_new[zs + i].x), 0x7f7fffffu));
        }
    }
    // SPEC: the first special record of planes zs..ze of this tile (the last
    // one ends plane ze - 1), staged once.
    uint32_t *soff = reinterpret_cast<uint32_t *>(base + NP * PS + NQ * QB + 256);
    if constexpr (SPEC) {
        const uint32_t *src = sp.off + ((long long)ty * a.tiles_x + tx) * a.nz + zs;
        for (int i = threadIdx.x; i <= Kq; i += 256) soff[i] = __ldg(src + i);
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < NP + NQ; i++) mbar_init(smem_addr(bars + i), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    // Launched as a programmatic dependent of the previous step, the CTA
    // may start before that step's kernels end: everything above reads
    // only data that no step writes; from here on the fields are touched.
    // (Without a programmatic dependency this returns at once.)
    asm volatile("griddepcontrol.wait;" ::: "memory");

    int np_issued = 0, nq_issued = 0;  // thread 0 is the only issuer
    auto issue_p = [&]() {
        const int k = np_issued++;
        const uint32_t bar = barP + 8 * (k % NP);
        mbar_expect_tx(bar, PB);
        tma_load_4d(smem_addr(Pbuf) + (k % NP) * PS, &tm_p, cx - HALO, y0 - 1, zp0 + dz * k, c, bar);
    };
    auto issue_q = [&]() {
        const int j = nq_issued++;
        const uint32_t bar = barQ + 8 * (j % NQ);
        mbar_expect_tx(bar, QB);
        tma_load_4d(smem_addr(Qbuf) + (j % NQ) * QB, &tm_q, cx, y0, zq0 + dz * j, c, bar);
    };
    if (threadIdx.x == 0) {
        while (np_issued < NP && np_issued < Kp) issue_p();
        while (nq_issued < NQ && nq_issued < Kq) issue_q();
    }

    const int x0 = tx * CELLS + lane * (4 / V);
    E *Q = a.nxt + (long long)c * a.cells_p * V;
    const long long nstep = SPEC ? *a.base + a.t : 0;  // SPEC: the step (signals are indexed by it)
    const long long mstep = (long long)dz * a.ny * a.nxw;  // mask words of the next plane in march order
    // FP16: the maxima slot of level n+1.
    unsigned int *amax_new = nullptr;
    if constexpr (HALF) amax_new = a.amax + ((long long)((*a.base + a.t + 1) % AMAX_RING) * a.chunks + c) * a.nz;
    // Rows of this thread: tile rows warp + 8 r (r < RT).  Interior-mask
    // words, four planes ahead, per row.
    bool rok[RT];
    const uint32_t *mrow[RT];
    uint32_t mw[RT][4];
#pragma unroll
    for (int r = 0; r < RT; r++) {
        const int y = y0 + warp + 8 * r;
        rok[r] = y < a.ny - 1 && x0 < a.nxp;
        mrow[r] = a.interior + ((long long)zq0 * a.ny + (rok[r] ? y : 1)) * a.nxw + (rok[r] ? (x0 >> 5) : 0);
#pragma unroll
        for (int d = 0; d < 4; d++) mw[r][d] = (rok[r] && d < Kq) ? __ldg(mrow[r] + d * mstep) : 0u;
    }
    const int g = HALO + lane * 4;  // this lane's four elements in a p row
    // Planes 0 and 1 of the p ring are waited for once; afterwards each plane
    // j waits only for p plane j + 2 and old plane j.
    bool ok = mbar_wait(barP, 0) && mbar_wait(barP + 8, 0);
    int bm = 0, bc = 1, bp = 2;      // buffers of p planes j, j+1, j+2 in march order
    uint32_t php = 0;                // parity of p plane j+2
    int bq = 0;
    uint32_t phq = 0;
    bool failed = false;
    for (int j = 0; j < Kq; j++) {
        if (j > 0 && threadIdx.x == 0) {
            if (np_issued < Kp) issue_p();
            if (nq_issued < Kq) issue_q();
        }
        // On its last plane the CTA lets the next step's CTAs be scheduled
        // (they wait above until this step has ended).
        if (j == Kq - 1) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
        const int z = zq0 + dz * j;
        const int iz = z - zs;       // the plane within the z-run
        float scm = 1.0f, scc = 1.0f, scp = 1.0f, sco = 1.0f, sinv = 1.0f, slim = 0.0f;
        // FP16: the update is evaluated in plane z's own scale (values
        // divided by scc); the ratios between the planes' scales, all powers
        // of two, carry the other terms into it.  A level not yet written has
        // zero scales (all of level n at once, at n = 0; level n-1 at n <= 1)
        // over zero fields.
        float r_cm = 1.0f, r_mp = 1.0f, r_pk = 1.0f, r_ok = 1.0f, ksinv = 1.0f;
        if constexpr (HALF) {
            scm = ssc[iz];
            scc = ssc[iz + 1];
            scp = ssc[iz + 2];
            sco = ssc[TMA_SCALE_STRIDE + iz];
            sinv = ssc[2 * TMA_SCALE_STRIDE + iz];
            slim = ssc[3 * TMA_SCALE_STRIDE + iz];
            r_cm = scale_ratio(scc, scm);
            r_mp = scale_ratio(scm, scp);
            r_pk = scale_ratio(scp, scc);
            r_ok = sco == 0.0f ? 0.0f : scale_ratio(sco, scc);
            ksinv = scc * sinv;
        }
        ok = ok && mbar_wait(barP + 8 * bp, php) && mbar_wait(barQ + 8 * bq, phq);
        uint32_t mb = 0;  // FP16: largest |p^(n+1)| stored, as float bits
        float mbf = 0.0f; // FP16: the same while the rows run, in plane z's scale
        if (ok) {
            const E *pc = Pbuf + bc * (PS / sizeof(E));
            const E *qo = Qbuf + bq * (QB / sizeof(E));
            // p^n of planes z - 1 and z + 1: behind and ahead in march order.
            const E *pm = Pbuf + (rev ? bp : bm) * (PS / sizeof(E));
            const E *pn = Pbuf + (rev ? bm : bp) * (PS / sizeof(E));
#pragma unroll
            for (int r = 0; r < RT; r++) {
                const uint32_t word = mw[r][0];
                mw[r][0] = mw[r][1];
                mw[r][1] = mw[r][2];
                mw[r][2] = mw[r][3];
                if (rok[r] && j + 4 < Kq) mw[r][3] = __ldg(mrow[r] + (long long)(j + 4) * mstep);
                const uint32_t bits = (word >> (x0 & 31)) & GROUP;
                if (!bits) continue;
                const int row = warp + 8 * r;
                const E *rc = pc + (row + 1) * PROW;
                // The plane's own values (x and y neighbours, centre) are read
                // without the slab scale: it is a power of two, so the first
                // three sums scaled once give the scaled sums bit for bit (FP16
                // values scaled stay far inside FP32's normal range).
                float vod[4], nx4[4];
                ld4(qo + row * TMA_ROW_FLOATS + lane * 4, vod, HALF ? r_ok : sco);
                if constexpr (HALF) {
                    // The x- neighbour and the centre are converted; the other
                    // neighbours enter the sum through mixed-precision adds,
                    // unscaled.  With A the plane's own four-neighbour sum,
                    // the sum is ((A sc_z + zm sc_m) + zp sc_p), evaluated in
                    // plane z's scale as ((A sc_z/sc_m + zm) sc_m/sc_p + zp)
                    // sc_p/sc_z, and the whole update with it (p^(n-1) as
                    // q sc_o/sc_z; the store multiplies by sc_z 2^-E of level
                    // n+1).  Every scaling is by a power of two in FP32's
                    // normal range, which commutes with rounding (FP16 values
                    // times scales of 2^-60 and more stay far above FP32's
                    // subnormals), so each rounded value is the original one
                    // scaled, and the stored result has the same bits.
                    float w[8];
                    uint16_t hxp[12], hym[4], hyp[4], hzm[4], hzp[4];
                    ld4u(rc + g - 4, w);
                    ld4u(rc + g, w + 4);
                    ld4h(rc + g - 4, hxp);
                    ld4h(rc + g, hxp + 4);
                    ld4h(rc + g + 4, hxp + 8);
                    ld4h(pc + row * PROW + g, hym);
                    ld4h(pc + (row + 2) * PROW + g, hyp);
                    ld4h(pm + (row + 1) * PROW + g, hzm);
                    ld4h(pn + (row + 1) * PROW + g, hzp);
                    const float r_cm = scale_ratio(scc, scm), r_mp = scale_ratio(scm, scp);
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        const float cv = w[4 + e];
                        float s = radd_h(w[4 + e - V], hxp[4 + e + V]);
                        s = radd_h(s, hym[e]);
                        s = radd_h(s, hyp[e]);
                        s = radd_h(rmul(s, r_cm), hzm[e]);
                        s = radd_h(rmul(s, r_mp), hzp[e]);
                        s = rmul(s, r_pk);
                        nx4[e] = radd(rsub(rmul(2.0f, cv), vod[e]), rmul(a.l2, rsub(s, rmul(6.0f, cv))));
                    }
                } else {
                    float zmv[4], zpv[4];
                    ld4(pm + (row + 1) * PROW + g, zmv, scm);
                    ld4(pn + (row + 1) * PROW + g, zpv, scp);
                    float w[12], vym[4], vyp[4];
                    ld4u(rc + g - 4, w);
                    ld4u(rc + g + 4, w + 8);
                    ld4u(rc + g, w + 4);
                    ld4u(pc + row * PROW + g, vym);
                    ld4u(pc + (row + 2) * PROW + g, vyp);
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        const float cv = w[4 + e];
                        float s = radd(w[4 + e - V], w[4 + e + V]);
                        s = radd(s, vym[e]);
                        s = radd(s, vyp[e]);
                        s = radd(s, zmv[e]);
                        s = radd(s, zpv[e]);
                        nx4[e] = radd(rsub(rmul(2.0f, cv), vod[e]), rmul(a.l2, rsub(s, rmul(6.0f, cv))));
                    }
                }
                E *dst = Q + (((long long)z * a.ny + (y0 + row)) * a.nxp + x0) * V;
                if constexpr (HALF) {
                    const __half2 h01 = __floats2half2_rn(nx4[0] * ksinv, nx4[1] * ksinv);
                    const __half2 h23 = __floats2half2_rn(nx4[2] * ksinv, nx4[3] * ksinv);
#pragma unroll
                    for (int e = 0; e < 4; e++)
                        if ((bits >> (e / V)) & 1u) mbf = max_abs_nan(mbf, nx4[e]);
                    if (bits == GROUP) {
                        uint2 raw;
                        raw.x = *reinterpret_cast<const unsigned int *>(&h01);
                        raw.y = *reinterpret_cast<const unsigned int *>(&h23);
                        *reinterpret_cast<uint2 *>(dst) = raw;
                    } else {
                        const __half hv[4] = {__low2half(h01), __high2half(h01), __low2half(h23), __high2half(h23)};
#pragma unroll
                        for (int e = 0; e < 4; e++)
                            if ((bits >> (e / V)) & 1u) dst[e] = hv[e];
                    }
                } else if (bits == GROUP) {
                    *reinterpret_cast<float4 *>(dst) = make_float4(nx4[0], nx4[1], nx4[2], nx4[3]);
                } else {
#pragma unroll
                    for (int q = 0; q < 4 / V; q++)
                        if ((bits >> q) & 1u)
#pragma unroll
                            for (int l = 0; l < V; l++) dst[q * V + l] = nx4[q * V + l];
                }
            }
            if constexpr (SPEC) {
                // The tile's special cells of plane z, from the same staged
                // planes: one thread per (cell, lane), a cell's lanes on
                // neighbouring threads.
                const uint32_t k0 = soff[iz], tasks = (soff[iz + 1] - k0) * V;
                for (uint32_t t = threadIdx.x; t < tasks; t += 256) {
                    const uint4 rec = __ldg(sp.rec + k0 + t / V);
                    const int l = (int)(t % V);
                    const uint32_t xg = rec.x % (uint32_t)a.nxp;
                    const int row = (int)((rec.x / (uint32_t)a.nxp) % (uint32_t)a.ny) - y0;
                    const int e0 = ((int)xg - tx * CELLS) * V;
                    const int at = (row + 1) * PROW + HALO + e0;
                    const SmemField<V> f{reinterpret_cast<const float *>(pc) + at,
                                         reinterpret_cast<const float *>(pm) + at,
                                         reinterpret_cast<const float *>(pn) + at,
                                         reinterpret_cast<const float *>(qo) + row * TMA_ROW_FLOATS + e0, PROW,
                                         reinterpret_cast<float *>(Q)};
                    special_lane<V>(sp.a, f, rec, c, l, nstep);
                }
            }
        }
        if constexpr (HALF) {
            // The row maxima were taken in plane z's scale: back to the
            // field's own (exact; NaN stays NaN, and its bits exceed any
            // finite limit's).
            mb = __float_as_uint(mbf * scc);
            // A value beyond the FP16 range of its slab scale is an error,
            // not a saturation.
            if (mb > __float_as_uint(slim) && *reinterpret_cast<volatile int *>(a.error) == 0)
                atomicExch(a.error, ERR_FP16_RANGE);
            mb = __reduce_max_sync(0xffffffffu, mb);
            if (lane == 0) wmax[(j & 1) * 8 + warp] = mb;
        }
        // One barrier per plane: everyone is done with this plane's buffers
        // (thread 0 refills them next), and a lost wait stops the whole CTA.
        if (__syncthreads_or(!ok)) {
            failed = true;
            if (threadIdx.x == 0) atomicExch(a.error, ERR_TMA_WAIT);
            break;
        }
        if constexpr (HALF) {
            // The CTA's maximum of the plane raises the slab maximum with one
            // reduction (RED): one per CTA and plane, not one per warp.
            if (threadIdx.x == 0) {
                unsigned int m = 0u;
                for (int w = 0; w < 8; w++) m = max(m, wmax[(j & 1) * 8 + w]);
                if (m > 0u) atomicMax(amax_new + z, m);
            }
        }
        bm = bc;
        bc = bp;
        if (++bp == NP) {
            bp = 0;
            php ^= 1u;
        }
        if (++bq == NQ) {
            bq = 0;
            phq ^= 1u;
        }
    }
    if (failed && threadIdx.x == 0) {
        // Let every copy this CTA issued land before its shared memory goes away:
        // the last plane issued into each buffer is its only phase that can be pending.
        for (int k = max(0, np_issued - NP); k < np_issued; k++) mbar_wait(barP + 8 * (k % NP), (k / NP) & 1);
        for (int j = max(0, nq_issued - NQ); j < nq_issued; j++) mbar_wait(barQ + 8 * (j % NQ), (j / NQ) & 1);
    }
}

}  // namespace wk
