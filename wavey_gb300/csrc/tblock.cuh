// tblock.cuh -- two time steps per pass over the fields (FP32, chunks of four
// right-hand sides).
//
// interior_tb2 reads p^n and p^(n-1) once and writes p^(n+1) and p^(n+2).  A
// CTA owns an output tile of TB_CELLS (30) cells x `rows` rows of one z-run
// and marches z, computing for each plane w
//
//   step n+1 on the tile and a one-cell ring around it (32 cells, the lanes
//            of a warp row, x rows + 2), from p^n staged by TMA with a
//            two-cell ring and p^(n-1) with a one-cell ring, into a ring of
//            four planes in shared memory; the tile's own interior cells also
//            go to HBM as p^(n+1);
//   step n+2 two planes behind (plane w - 2), at the tile's deep cells --
//            interior cells whose six neighbours are interior cells, so that
//            every p^(n+1) it reads was computed in the first part -- from
//            that ring and p^n, to HBM as p^(n+2).
//
// Both levels go to two other buffers, since neighbouring CTAs still read p^n
// and p^(n-1) as halo.  Beside it special_branch advances the special cells to
// n+1 into the p^(n+1) buffer; afterwards tb2_second advances the shell
// (interior cells with a special neighbour) and the special cells to n+2.
// Every update is the one-step kernels' arithmetic on the same values, so the
// results are identical to two single steps.
//
// Waits on mbarriers are bounded as in interior_tma.
#pragma once
#include "interior_tma.cuh"

namespace wk {

constexpr int TB_CELLS = 30;     // output cells per tile row (V = 4); with the ring, 32 = a warp row
constexpr int TB_PROW = 136;     // floats per staged p^n row: 34 cells (a two-cell ring) x 4 sources
constexpr int TB_N1 = 4;         // planes of p^(n+1) kept in shared memory

struct Tb2Args {
    const uint32_t *interior;  // [nz][ny][nxw] interior cells (one-step mask)
    const uint32_t *deep;      // [nz][ny][nxw] interior cells whose six neighbours are interior cells
    float *out1;               // p^(n+1) [chunks][cells_p][4]
    float *out2;               // p^(n+2)
    int *error;
    long long cells_p;
    int nxp, ny, nz, nxw;
    int tiles_x, tiles_y, tiles_z, zt;
    int rows;                  // output rows per tile; the p^(n+1) region has rows + 2
    float l2;
};

template <int R2MAX>
__host__ __device__ constexpr uint32_t tb_p_stride() { return (TB_PROW * (R2MAX + 2) * 4 + 127) / 128 * 128; }
template <int R2MAX>
__host__ __device__ constexpr uint32_t tb_q_stride() { return TMA_ROW_FLOATS * R2MAX * 4; }
template <int R2MAX, int NP, int NQ>
__host__ __device__ constexpr uint32_t tb_smem_of() {
    return NP * tb_p_stride<R2MAX>() + NQ * tb_q_stride<R2MAX>() + TB_N1 * tb_q_stride<R2MAX>() + 256 + 128;
}

// Bit x of row (z, y) of a one-bit-per-cell mask; 0 outside the rows and the padded row.
__device__ __forceinline__ uint32_t tb_bit(const uint32_t *m, const Tb2Args &a, int z, int y, int x) {
    if (y >= a.ny || x >= a.nxp) return 0u;
    return (__ldg(m + ((long long)z * a.ny + y) * a.nxw + (x >> 5)) >> (x & 31)) & 1u;
}

// The interior update of four sources from shared memory: centre c, x
// neighbours c -/+ 4 floats, y neighbours c -/+ row, z neighbours at the same
// place in planes zm / zp, old value at o.  interior_update's operations and
// order.
__device__ __forceinline__ float4 tb_update(const float *c, int row, const float *zm, const float *zp, const float *o,
                                            float l2) {
    const float4 cv = *reinterpret_cast<const float4 *>(c);
    const float4 xm = *reinterpret_cast<const float4 *>(c - 4), xp = *reinterpret_cast<const float4 *>(c + 4);
    const float4 ym = *reinterpret_cast<const float4 *>(c - row), yp = *reinterpret_cast<const float4 *>(c + row);
    const float4 a = *reinterpret_cast<const float4 *>(zm), b = *reinterpret_cast<const float4 *>(zp);
    const float4 od = *reinterpret_cast<const float4 *>(o);
    auto one = [&](float cc, float x0, float x1, float y0, float y1, float z0, float z1, float oo) {
        float s = radd(x0, x1);
        s = radd(s, y0);
        s = radd(s, y1);
        s = radd(s, z0);
        s = radd(s, z1);
        return radd(rsub(rmul(2.0f, cc), oo), rmul(l2, rsub(s, rmul(6.0f, cc))));
    };
    return make_float4(one(cv.x, xm.x, xp.x, ym.x, yp.x, a.x, b.x, od.x), one(cv.y, xm.y, xp.y, ym.y, yp.y, a.y, b.y, od.y),
                       one(cv.z, xm.z, xp.z, ym.z, yp.z, a.z, b.z, od.z), one(cv.w, xm.w, xp.w, ym.w, yp.w, a.w, b.w, od.w));
}

// R2MAX: the largest p^(n+1) region (rows + 2) the shared memory is laid out
// for; NP / NQ: planes in the p^n and p^(n-1) rings (NP - 4 and NQ - 1 in
// flight while a plane is computed).  One CTA per SM: 256 threads, warp w
// takes region rows w, w + 8, ...
template <int R2MAX, int NP, int NQ>
__global__ void __launch_bounds__(256, 1) interior_tb2(const __grid_constant__ CUtensorMap tm_p,
                                                       const __grid_constant__ CUtensorMap tm_q, Tb2Args a) {
    static_assert(NP >= 5 && NQ >= 2, "rings too shallow");
    constexpr int RT = (R2MAX + 7) / 8;
    constexpr uint32_t PS = tb_p_stride<R2MAX>(), QS = tb_q_stride<R2MAX>();
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    float *Pbuf = reinterpret_cast<float *>(base);
    float *Qbuf = reinterpret_cast<float *>(base + NP * PS);
    float *Nbuf = reinterpret_cast<float *>(base + NP * PS + NQ * QS);
    uint64_t *bars = reinterpret_cast<uint64_t *>(base + NP * PS + (NQ + TB_N1) * QS);
    const uint32_t barP = smem_addr(bars), barQ = smem_addr(bars + NP);

    const int R2 = a.rows + 2;
    const uint32_t PB = TB_PROW * (R2 + 2) * 4, QB = TMA_ROW_FLOATS * R2 * 4;
    const int per_chunk = a.tiles_x * a.tiles_y * a.tiles_z;
    int b = blockIdx.x;
    const int c = b / per_chunk;
    b -= c * per_chunk;
    const int tz = b / (a.tiles_x * a.tiles_y);
    b -= tz * a.tiles_x * a.tiles_y;
    const int ty = b / a.tiles_x;
    const int tx = b - ty * a.tiles_x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int xr = tx * TB_CELLS;   // first region cell; the tile is xr+1 .. xr+30
    const int yr = ty * a.rows;     // first region row; the tile is yr+1 .. yr+rows
    const int zs = 1 + tz * a.zt;
    const int ze = min(zs + a.zt, a.nz - 1);
    const int Kq = ze - zs;         // output planes
    const int Kn = Kq + 2;          // p^(n+1) planes zs-1 .. ze
    const int Kp = Kq + 4;          // p^n planes zs-2 .. ze+1

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
        tma_load_4d(smem_addr(Pbuf) + (k % NP) * PS, &tm_p, (xr - 1) * 4, yr - 1, zs - 2 + k, c, bar);
    };
    auto issue_q = [&]() {
        const int j = nq_issued++;
        const uint32_t bar = barQ + 8 * (j % NQ);
        mbar_expect_tx(bar, QB);
        tma_load_4d(smem_addr(Qbuf) + (j % NQ) * QS, &tm_q, xr * 4, yr, zs - 1 + j, c, bar);
    };
    if (threadIdx.x == 0) {
        while (np_issued < NP && np_issued < Kp) issue_p();
        while (nq_issued < NQ && nq_issued < Kn) issue_q();
    }

    const int x = xr + lane;
    const bool out_lane = lane >= 1 && lane <= TB_CELLS;
    float *O1 = a.out1 + (long long)c * a.cells_p * 4;
    float *O2 = a.out2 + (long long)c * a.cells_p * 4;
    // Mask bits of this thread's rows, one plane ahead: interior cells for
    // the first part, deep cells for the second.
    uint32_t mi[RT], md[RT];
#pragma unroll
    for (int j = 0; j < RT; j++) {
        const int r = warp + 8 * j;
        mi[j] = r < R2 ? tb_bit(a.interior, a, zs - 1, yr + r, x) : 0u;
        md[j] = 0u;
    }
    bool ok = mbar_wait(barP, 0) && mbar_wait(barP + 8, 0);
    bool failed = false;
    for (int i = 0; i <= Kq + 2; i++) {
        // p^n plane k is read in iterations k-2 .. k+1 and p^(n-1) plane j in
        // iteration j: at the start of iteration i, p^n plane i-2 and
        // p^(n-1) plane i-1 are free.
        if (threadIdx.x == 0) {
            if (i >= 2 && np_issued < Kp) issue_p();
            if (i >= 1 && nq_issued < Kn) issue_q();
        }
        const bool first = i < Kn;   // step n+1 at plane w
        const bool second = i >= 3;  // step n+2 at plane z
        const int w = zs - 1 + i, z = zs - 3 + i;
        uint32_t bi[RT], bd[RT];
#pragma unroll
        for (int j = 0; j < RT; j++) {
            bi[j] = mi[j];
            bd[j] = md[j];
            const int r = warp + 8 * j;
            mi[j] = (r < R2 && i + 1 < Kn) ? tb_bit(a.interior, a, w + 1, yr + r, x) : 0u;
            md[j] = (r >= 1 && r <= R2 - 2 && out_lane && i + 1 >= 3) ? tb_bit(a.deep, a, z + 1, yr + r, x) : 0u;
        }
        if (first) {
            const int k = i + 2;
            ok = ok && mbar_wait(barP + 8 * (k % NP), (k / NP) & 1) && mbar_wait(barQ + 8 * (i % NQ), (i / NQ) & 1);
        }
        if (ok && first) {
            const float *pm = Pbuf + (i % NP) * (PS / 4), *pc = Pbuf + ((i + 1) % NP) * (PS / 4),
                        *pp = Pbuf + ((i + 2) % NP) * (PS / 4);
            const float *qo = Qbuf + (i % NQ) * (QS / 4);
            float *n1 = Nbuf + (i % TB_N1) * (QS / 4);
            const bool keep = w >= zs && w < ze && out_lane;  // a plane and lane of the tile itself
#pragma unroll
            for (int j = 0; j < RT; j++) {
                const int r = warp + 8 * j;
                if (!bi[j]) continue;
                const int o = (r + 1) * TB_PROW + (lane + 1) * 4;
                const float4 v = tb_update(pc + o, TB_PROW, pm + o, pp + o, qo + r * TMA_ROW_FLOATS + lane * 4, a.l2);
                *reinterpret_cast<float4 *>(n1 + r * TMA_ROW_FLOATS + lane * 4) = v;
                if (keep && r >= 1 && r <= R2 - 2)
                    *reinterpret_cast<float4 *>(O1 + (((long long)w * a.ny + yr + r) * a.nxp + x) * 4) = v;
            }
        }
        if (ok && second) {
            // p^(n+1) of planes z-1, z, z+1 (computed in iterations i-3 ..
            // i-1) and p^n of plane z (ring plane i-1).
            const float *a0 = Nbuf + ((i - 3) % TB_N1) * (QS / 4), *a1 = Nbuf + ((i - 2) % TB_N1) * (QS / 4),
                        *a2 = Nbuf + ((i - 1) % TB_N1) * (QS / 4);
            const float *pz = Pbuf + ((i - 1) % NP) * (PS / 4);
#pragma unroll
            for (int j = 0; j < RT; j++) {
                const int r = warp + 8 * j;
                if (!bd[j]) continue;
                const int o = r * TMA_ROW_FLOATS + lane * 4;
                const float4 v =
                    tb_update(a1 + o, TMA_ROW_FLOATS, a0 + o, a2 + o, pz + (r + 1) * TB_PROW + (lane + 1) * 4, a.l2);
                *reinterpret_cast<float4 *>(O2 + (((long long)z * a.ny + yr + r) * a.nxp + x) * 4) = v;
            }
        }
        // One barrier per plane: the p^(n+1) plane just written is complete
        // for the next iterations, the buffers freed here can be refilled,
        // and a lost wait stops the whole CTA.
        if (__syncthreads_or(!ok)) {
            failed = true;
            if (threadIdx.x == 0) atomicExch(a.error, ERR_TMA_WAIT);
            break;
        }
    }
    if (failed && threadIdx.x == 0) {
        for (int k = max(0, np_issued - NP); k < np_issued; k++) mbar_wait(barP + 8 * (k % NP), (k / NP) & 1);
        for (int j = max(0, nq_issued - NQ); j < nq_issued; j++) mbar_wait(barQ + 8 * (j % NQ), (j / NQ) & 1);
    }
}

// The second kernel of a two-step pass: the shell cells' step n+2 (the
// interior update from p^(n+1), written by interior_tb2 and special_branch),
// then the special cells' step n+2 and the receiver samples of step n+1 --
// special_branch's roles on the arguments a (cur = p^(n+1), nxt = p^n, out =
// p^(n+2)).
struct Tb2Second {
    StepArgs<float> a;
    const uint32_t *shell;  // [n_shell] padded cells, ascending
    int n_shell, shell_blocks;
};

template <int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) tb2_second(const __grid_constant__ Tb2Second s, int t) {
    constexpr int SR = MINB >= 4 ? 0 : MINB == 3 ? 2 : SLOT_REGS;
    const StepArgs<float> &a = s.a;
    int b = blockIdx.x;
    if (b < s.shell_blocks) {
        const long long k = (long long)b * BLOCK + threadIdx.x;
        if (k >= (long long)s.n_shell * a.chunks) return;
        const int c = (int)(k / s.n_shell);
        const long long i = __ldg(s.shell + (k - (long long)c * s.n_shell));
        const long long nxy = (long long)a.nxp * a.ny;
        const float *P = a.cur + (long long)c * a.cells_p * 4;
        const float *Q = a.nxt + (long long)c * a.cells_p * 4;
        const Lanes<float, 4> zc = load<float, 4, false>(P + i * 4), xm = load<float, 4, false>(P + (i - 1) * 4),
                              xp = load<float, 4, false>(P + (i + 1) * 4), ym = load<float, 4, false>(P + (i - a.nxp) * 4),
                              yp = load<float, 4, false>(P + (i + a.nxp) * 4), zm = load<float, 4, false>(P + (i - nxy) * 4),
                              zp = load<float, 4, false>(P + (i + nxy) * 4), old = load<float, 4, false>(Q + i * 4);
        store<float, 4>(a.out + (long long)c * a.cells_p * 4 + i * 4,
                        interior_update<float, 4>(zc, old, xm, xp, ym, yp, zm, zp, a.l2));
        return;
    }
    b -= s.shell_blocks;
    if (b < a.special_blocks) {
        const long long k = (long long)b * BLOCK + threadIdx.x;
        if (k >= (long long)a.n_special * a.chunks) return;
        special_cell<float, 4, false, SR>(a, k, *a.base + t);
        return;
    }
    b -= a.special_blocks;
    const long long k = (long long)b * BLOCK + threadIdx.x;
    if (k >= (long long)a.n_recv * a.chunks) return;
    record_one<float, 4>(a, k, t);
}

}  // namespace wk
