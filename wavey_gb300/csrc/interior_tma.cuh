// interior_tma.cuh -- the interior leapfrog update fed by TMA (FP32).
//
// A CTA owns a tile of R rows x 128 floats of one z-run (32 cells of a
// 4-source chunk, 64 cells of a 2-source chunk or 128 cells of one source)
// and marches z.  One thread issues cp.async.bulk.tensor loads of whole
// planes several planes ahead into a ring in shared memory:
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
// Every wait on an mbarrier is bounded.  If one runs out, the kernel records
// the failure in the error word, waits (again bounded) for the copies it has
// issued, and returns; the host reports WAVEY_E_DEVICE.
#pragma once
#include <cuda.h>
#include <cstdint>

#include "fdtd_kernels.cuh"

namespace wk {

constexpr int TMA_ROW_FLOATS = 128;         // floats per tile row (32 lanes x 16 B)
constexpr int TMA_HALO_FLOATS = 4;          // 16-byte halo on each side in x
constexpr int TMA_P_ROW = TMA_ROW_FLOATS + 2 * TMA_HALO_FLOATS;  // 136

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

struct TmaArgs {
    const uint32_t *interior;  // [nz][ny][nxw]
    float *nxt;                // p^(n-1) in, p^(n+1) out, [chunks][cells_p][V]
    int *error;                // error word
    long long cells_p;
    int nxp, ny, nz, nxw;
    int tiles_x, tiles_y, tiles_z, zt;
    float l2;
};

// V: sources per cell in a chunk (1, 2 or 4); a tile row holds 128 / V cells.
// R: rows per tile (8 or 16; 256 threads, R / 8 rows per thread).
// NP / NQ: planes in the two rings; NP - 3 p planes and NQ - 1 old planes are
// in flight while one plane is computed.
template <int R>
__host__ __device__ constexpr uint32_t tma_p_bytes() { return TMA_P_ROW * (R + 2) * 4; }
template <int R>
__host__ __device__ constexpr uint32_t tma_p_stride() { return (tma_p_bytes<R>() + 127) / 128 * 128; }
template <int R>
__host__ __device__ constexpr uint32_t tma_q_bytes() { return TMA_ROW_FLOATS * R * 4; }
template <int R, int NP, int NQ>
__host__ __device__ constexpr uint32_t tma_smem_of() { return NP * tma_p_stride<R>() + NQ * tma_q_bytes<R>() + 256 + 128; }

template <int V, int R, int NP, int NQ>
__global__ void __launch_bounds__(256) interior_tma(const __grid_constant__ CUtensorMap tm_p,
                                                    const __grid_constant__ CUtensorMap tm_q, TmaArgs a) {
    constexpr int RT = R / 8;                    // rows per thread
    constexpr uint32_t PB = tma_p_bytes<R>(), PS = tma_p_stride<R>(), QB = tma_q_bytes<R>();
    constexpr int CELLS = TMA_ROW_FLOATS / V;    // cells per tile row
    constexpr uint32_t GROUP = (1u << (4 / V)) - 1u;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    float *Pbuf = reinterpret_cast<float *>(base);
    float *Qbuf = reinterpret_cast<float *>(base + NP * PS);
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

    if (threadIdx.x == 0) {
        for (int i = 0; i < NP + NQ; i++) mbar_init(smem_addr(bars + i), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();

    int np_issued = 0, nq_issued = 0;  // thread 0 is the only issuer
    auto issue_p = [&]() {
        const int k = np_issued++;
        const uint32_t bar = barP + 8 * (k % NP);
        mbar_expect_tx(bar, PB);
        tma_load_4d(smem_addr(Pbuf) + (k % NP) * PS, &tm_p, cx - TMA_HALO_FLOATS, y0 - 1, zs - 1 + k, c, bar);
    };
    auto issue_q = [&]() {
        const int j = nq_issued++;
        const uint32_t bar = barQ + 8 * (j % NQ);
        mbar_expect_tx(bar, QB);
        tma_load_4d(smem_addr(Qbuf) + (j % NQ) * QB, &tm_q, cx, y0, zs + j, c, bar);
    };
    if (threadIdx.x == 0) {
        while (np_issued < NP && np_issued < Kp) issue_p();
        while (nq_issued < NQ && nq_issued < Kq) issue_q();
    }

    const int x0 = tx * CELLS + lane * (4 / V);
    float *Q = a.nxt + (long long)c * a.cells_p * V;
    const long long mstep = (long long)a.ny * a.nxw;
    // Interior-mask words, four planes ahead, per row of this thread.
    bool rok[RT];
    const uint32_t *mrow[RT];
    uint32_t mw[RT][4];
#pragma unroll
    for (int r = 0; r < RT; r++) {
        const int y = y0 + warp + 8 * r;
        rok[r] = y < a.ny - 1 && x0 < a.nxp;
        mrow[r] = a.interior + ((long long)zs * a.ny + (rok[r] ? y : 1)) * a.nxw + (rok[r] ? (x0 >> 5) : 0);
#pragma unroll
        for (int d = 0; d < 4; d++) mw[r][d] = (rok[r] && d < Kq) ? __ldg(mrow[r] + d * mstep) : 0u;
    }
    // Planes 0 and 1 of the p ring are waited for once; afterwards each plane
    // j waits only for p plane j + 2 and old plane j.
    bool ok = mbar_wait(barP, 0) && mbar_wait(barP + 8, 0);
    int bm = 0, bc = 1, bp = 2;      // buffers of p planes j, j+1, j+2
    uint32_t php = 0;                // parity of p plane j+2
    int bq = 0;
    uint32_t phq = 0;
    bool failed = false;
    for (int j = 0; j < Kq; j++) {
        if (j > 0 && threadIdx.x == 0) {
            if (np_issued < Kp) issue_p();
            if (nq_issued < Kq) issue_q();
        }
        ok = ok && mbar_wait(barP + 8 * bp, php) && mbar_wait(barQ + 8 * bq, phq);
        const int z = zs + j;
        if (ok) {
            const float *pm = Pbuf + bm * (PS / 4);
            const float *pc = Pbuf + bc * (PS / 4);
            const float *pn = Pbuf + bp * (PS / 4);
            const float *qo = Qbuf + bq * (QB / 4);
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
                const int g = TMA_HALO_FLOATS + lane * 4;
                const float *rc = pc + (row + 1) * TMA_P_ROW;
                const float4 cl = *reinterpret_cast<const float4 *>(rc + g - 4);
                const float4 cc = *reinterpret_cast<const float4 *>(rc + g);
                const float4 cr = *reinterpret_cast<const float4 *>(rc + g + 4);
                const float4 ym = *reinterpret_cast<const float4 *>(pc + row * TMA_P_ROW + g);
                const float4 yp = *reinterpret_cast<const float4 *>(pc + (row + 2) * TMA_P_ROW + g);
                const float4 zm = *reinterpret_cast<const float4 *>(pm + (row + 1) * TMA_P_ROW + g);
                const float4 zp = *reinterpret_cast<const float4 *>(pn + (row + 1) * TMA_P_ROW + g);
                const float4 od = *reinterpret_cast<const float4 *>(qo + row * TMA_ROW_FLOATS + lane * 4);
                const float w[12] = {cl.x, cl.y, cl.z, cl.w, cc.x, cc.y, cc.z, cc.w, cr.x, cr.y, cr.z, cr.w};
                const float vym[4] = {ym.x, ym.y, ym.z, ym.w}, vyp[4] = {yp.x, yp.y, yp.z, yp.w};
                const float vzm[4] = {zm.x, zm.y, zm.z, zm.w}, vzp[4] = {zp.x, zp.y, zp.z, zp.w};
                const float vod[4] = {od.x, od.y, od.z, od.w};
                float nx4[4];
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const float cv = w[4 + e];
                    float s = radd(w[4 + e - V], w[4 + e + V]);
                    s = radd(s, vym[e]);
                    s = radd(s, vyp[e]);
                    s = radd(s, vzm[e]);
                    s = radd(s, vzp[e]);
                    nx4[e] = radd(rsub(rmul(2.0f, cv), vod[e]), rmul(a.l2, rsub(s, rmul(6.0f, cv))));
                }
                float *dst = Q + (((long long)z * a.ny + (y0 + row)) * a.nxp + x0) * V;
                if (bits == GROUP) {
                    *reinterpret_cast<float4 *>(dst) = make_float4(nx4[0], nx4[1], nx4[2], nx4[3]);
                } else {
#pragma unroll
                    for (int q = 0; q < 4 / V; q++)
                        if ((bits >> q) & 1u)
#pragma unroll
                            for (int l = 0; l < V; l++) dst[q * V + l] = nx4[q * V + l];
                }
            }
        }
        // One barrier per plane: everyone is done with this plane's buffers
        // (thread 0 refills them next), and a lost wait stops the whole CTA.
        if (__syncthreads_or(!ok)) {
            failed = true;
            if (threadIdx.x == 0) atomicExch(a.error, ERR_TMA_WAIT);
            break;
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
