// fdtd_half.cuh -- the time step with FP16 field storage.
//
// p^n and p^(n-1) are stored as FP16 with a power-of-two scale per z slab,
// per source chunk and per time level: a cell of slab z at time level k holds
// half(p * 2^-E) and reads back as float(h) * 2^E, with E = E^k[z].  Updates
// are computed in FP32 (the FP32 path's formulas and order), branch states
// stay FP32, receiver samples go to the FP32 ring and FP64 spectra.
//
// Before the step that writes level n+1, half_prepare fixes its slab scales
// from the slab maxima of the two previous levels over slabs z-1..z+1:
//
//     M = 8 * max(amax^n[z-1..z+1], amax^(n-1)[z-1..z+1]) + injection bound
//     E^(n+1)[z] = max(e - shift, E_FLOOR) with M < 2^e (shift 14 by default).
//
// The factor 8 bounds the growth of one leapfrog step of pressure alone over
// a cell's neighbourhood (|p+| <= 2|p| + |p-| + 12 l2 |p|max); boundary nodes
// can exceed it, because their branch states hold energy the pressure maxima
// do not see, so M maps to 2^14, leaving 4 times headroom below 65504.  FP16
// is floating point: power-of-two scaling does not change its rounding, so
// the mapping only trades headroom against the subnormal range (values below
// 2^-28 of M lose bits).  A value outside the FP16 range anyway sets the
// error word (the host reports WAVEY_E_DEVICE) instead of saturating.  Scales (2^E and 2^-E) live in a ring of three levels, slab
// maxima in a ring of three levels; half_prepare also clears the maxima slot
// the step is about to accumulate.
#pragma once
#include <cuda_fp16.h>

#include "fdtd_kernels.cuh"

namespace wk {

constexpr int AMAX_RING = 3;
constexpr int SCALE_RING = 3;
constexpr int E_FLOOR = -60;  // lowest slab exponent: slabs that hold only zeros or near-zeros
constexpr int ERR_FP16_RANGE = 2;

struct HalfArgs {
    const __half *cur;         // p^n     [chunks][cells_p][V]
    __half *nxt;               // p^(n-1) in, p^(n+1) out
    const uint32_t *interior;
    const uint4 *sp;           // [n_special] {cell, meta, first slot, tap row}
    const float *slots;        // [n_slots][4]
    float *su, *sg;            // [chunks][n_slots][V]
    const float *tapw;         // [n_tap_rows][lanes_total]
    const float *sig;          // [lanes_total][sig_stride]
    const float *wmax;         // [lanes_total] sum of |tap weight| per source
    const uint32_t *recv;
    float *ring;               // [chunks][RING][n_recv][V]
    const long long *base;
    unsigned int *amax;        // [AMAX_RING][chunks][nz] slab maxima as float bits
    float2 *scale;             // [SCALE_RING][chunks][nz] (2^E, 2^-E) of a time level
    int *error;
    long long cells_p, sig_stride;
    int nxp, ny, nz, nxw;
    int n_special, n_slots, n_recv, chunks, lanes_total;
    int tiles_x, tiles_y, tiles_z, zt;
    int interior_blocks, special_blocks, record_blocks;
    float l2, lam, half_dt;
    int shift;  // the bound M maps just below 2^shift
};

__device__ __forceinline__ float slab_max(const HalfArgs &a, long long level, int c, int z) {
    if (level < 0) return 0.0f;
    return __uint_as_float(a.amax[((int)(level % AMAX_RING) * a.chunks + c) * a.nz + z]);
}

// Largest |tap weight x signal| that the step producing level k injects into chunk c.
template <int V>
__device__ __forceinline__ float inject_bound(const HalfArgs &a, long long k, int c) {
    if (k < 1) return 0.0f;
    float m = 0.0f;
#pragma unroll
    for (int l = 0; l < V; l++) {
        const int s = c * V + l;
        m = fmaxf(m, fabsf(a.sig[(long long)s * a.sig_stride + (k - 1)]) * a.wmax[s]);
    }
    return m;
}

// E^k[z] of chunk c from the maxima of levels k-1 and k-2.
template <int V>
__device__ __forceinline__ int slab_exponent(const HalfArgs &a, long long k, int c, int z) {
    float m = 0.0f;
    const int z0 = max(z - 1, 0), z1 = min(z + 1, a.nz - 1);
    for (int zz = z0; zz <= z1; zz++) m = fmaxf(m, fmaxf(slab_max(a, k - 1, c, zz), slab_max(a, k - 2, c, zz)));
    m = 8.0f * m + inject_bound<V>(a, k, c);
    if (m == 0.0f) return E_FLOOR;
    int e;
    frexpf(m, &e);
    // Slabs ahead of a wave front can hold FP32 subnormals; their exponent is
    // clamped to the floor (they read back as the zeros they nearly are), which
    // also keeps 2^E and 2^-E inside the normal FP32 range that pow2 builds.
    return max(e - a.shift, E_FLOOR);
}

// 2^e for -126 <= e <= 127 (slab exponents stay in [E_FLOOR, 127 - 10]).
__device__ __forceinline__ float pow2(int e) { return __int_as_float((127 + e) << 23); }

// (2^E, 2^-E) of level k, slab z, chunk c.
__device__ __forceinline__ float2 slab_scale(const HalfArgs &a, long long k, int c, int z) {
    return a.scale[((int)(k % SCALE_RING) * a.chunks + c) * a.nz + z];
}

// Before step n: the scales of level n+1, and a cleared maxima slot for it.
template <int V>
__global__ void __launch_bounds__(BLOCK) half_prepare(HalfArgs a, int t) {
    const long long n = *a.base + t;
    float2 *out = a.scale + (long long)((n + 1) % SCALE_RING) * a.chunks * a.nz;
    unsigned int *slot = a.amax + (long long)((n + 1) % AMAX_RING) * a.chunks * a.nz;
    for (int i = blockIdx.x * BLOCK + threadIdx.x; i < a.chunks * a.nz; i += gridDim.x * BLOCK) {
        const int c = i / a.nz, z = i - c * a.nz;
        const int e = slab_exponent<V>(a, n + 1, c, z);
        out[i] = make_float2(pow2(e), pow2(-e));
    }
    // The slot of level n+1 held level n-2, which nothing reads any more; the
    // maxima of levels n and n-1 read above are in the other two slots.
    for (int i = blockIdx.x * BLOCK + threadIdx.x; i < a.chunks * a.nz; i += gridDim.x * BLOCK) slot[i] = 0u;
}

// Loads FP16 values times the slab scale sc (a power of two: exact).
template <int V>
__device__ __forceinline__ Lanes<float, V> load_h(const __half *p, float sc) {
    Lanes<float, V> o;
    if constexpr (V == 4) {
        const uint2 raw = *reinterpret_cast<const uint2 *>(p);
        const __half2 a = *reinterpret_cast<const __half2 *>(&raw.x), b = *reinterpret_cast<const __half2 *>(&raw.y);
        o.v[0] = __low2float(a) * sc;
        o.v[1] = __high2float(a) * sc;
        o.v[2] = __low2float(b) * sc;
        o.v[3] = __high2float(b) * sc;
    } else if constexpr (V == 2) {
        const __half2 a = *reinterpret_cast<const __half2 *>(p);
        o.v[0] = __low2float(a) * sc;
        o.v[1] = __high2float(a) * sc;
    } else {
        o.v[0] = __half2float(*p) * sc;
    }
    return o;
}

// Stores v * inv (inv = 2^-E, exact) as FP16 rounded to nearest; returns
// max |v| and flags values FP16 cannot hold.  (Unbiased stochastic rounding
// was tried: it lowers the spectra's worst error a little but raises the
// octave-band level error, its noise floor adding energy to quiet bands.)
template <int V>
__device__ __forceinline__ float store_h(__half *p, const Lanes<float, V> &v, float inv, int *error) {
    float m = 0.0f;
    __half h[V];
#pragma unroll
    for (int l = 0; l < V; l++) {
        const float s = v.v[l] * inv;
        if (!(fabsf(s) <= 65504.0f) && *reinterpret_cast<volatile int *>(error) == 0) atomicExch(error, ERR_FP16_RANGE);
        h[l] = __float2half_rn(s);
        m = fmaxf(m, fabsf(v.v[l]));
    }
    if constexpr (V == 4) {
        uint2 raw;
        __half2 a = __halves2half2(h[0], h[1]), b = __halves2half2(h[2], h[3]);
        raw.x = *reinterpret_cast<unsigned int *>(&a);
        raw.y = *reinterpret_cast<unsigned int *>(&b);
        *reinterpret_cast<uint2 *>(p) = raw;
    } else if constexpr (V == 2) {
        *reinterpret_cast<__half2 *>(p) = __halves2half2(h[0], h[1]);
    } else {
        *p = h[0];
    }
    return m;
}

// Raises the slab maximum, skipping the atomic when it cannot change it.
__device__ __forceinline__ void raise_max(unsigned int *slot, float m) {
    if (m > __uint_as_float(*reinterpret_cast<volatile unsigned int *>(slot))) atomicMax(slot, __float_as_uint(m));
}

__device__ __forceinline__ float warp_max(float m) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    return m;
}

template <int V>
__global__ void __launch_bounds__(BLOCK) fdtd_step_half(HalfArgs a, int t) {
    const long long n = *a.base + t;
    const long long nxy = (long long)a.nxp * a.ny;
    int b = blockIdx.x;
    unsigned int *amax_new = a.amax + (long long)((n + 1) % AMAX_RING) * a.chunks * a.nz;
    if (b < a.interior_blocks) {
        const int per_chunk = a.tiles_x * a.tiles_y * a.tiles_z;
        const int c = b / per_chunk;
        int r = b - c * per_chunk;
        const int tz = r / (a.tiles_x * a.tiles_y);
        r -= tz * a.tiles_x * a.tiles_y;
        const int ty = r / a.tiles_x;
        const int tx = r - ty * a.tiles_x;
        const int lane = threadIdx.x & 31;
        const int y = 1 + ty * TILE_Y + (threadIdx.x >> 5);
        const bool row_ok = y < a.ny - 1;
        const int x = tx * 32 + lane;
        const int zs = 1 + tz * a.zt;
        const int ze = min(zs + a.zt, a.nz - 1);
        const __half *P = a.cur + (long long)c * a.cells_p * V;
        __half *Q = a.nxt + (long long)c * a.cells_p * V;
        long long i = ((long long)zs * a.ny + (row_ok ? y : 1)) * a.nxp + x;
        const uint32_t *mrow = a.interior + ((long long)zs * a.ny + (row_ok ? y : 1)) * a.nxw + tx;
        const long long mstep = (long long)a.ny * a.nxw;
        const float2 *s_now = a.scale + ((int)(n % SCALE_RING) * a.chunks + c) * a.nz;
        const float2 *s_old = a.scale + ((int)((n + SCALE_RING - 1) % SCALE_RING) * a.chunks + c) * a.nz;
        const float2 *s_new = a.scale + ((int)((n + 1) % SCALE_RING) * a.chunks + c) * a.nz;
        float szm = s_now[zs - 1].x, szc = s_now[zs].x;
        Lanes<float, V> zm = load_h<V>(P + (i - nxy) * V, szm), zc = load_h<V>(P + i * V, szc);
        for (int z = zs; z < ze; ++z, i += nxy, mrow += mstep) {
            const float szp = s_now[z + 1].x;
            const Lanes<float, V> zp = load_h<V>(P + (i + nxy) * V, szp);
            const uint32_t word = row_ok ? __ldg(mrow) : 0u;
            float m = 0.0f;
            if ((word >> lane) & 1u) {
                const Lanes<float, V> xm = load_h<V>(P + (i - 1) * V, szc);
                const Lanes<float, V> xp = load_h<V>(P + (i + 1) * V, szc);
                const Lanes<float, V> ym = load_h<V>(P + (i - a.nxp) * V, szc);
                const Lanes<float, V> yp = load_h<V>(P + (i + a.nxp) * V, szc);
                const Lanes<float, V> old = load_h<V>(Q + i * V, s_old[z].x);
                const Lanes<float, V> nx = interior_update<float, V>(zc, old, xm, xp, ym, yp, zm, zp, a.l2);
                m = store_h<V>(Q + i * V, nx, s_new[z].y, a.error);
            }
            m = warp_max(m);
            if (lane == 0 && m > 0.0f) raise_max(amax_new + c * a.nz + z, m);
            zm = zc;
            zc = zp;
            szm = szc;
            szc = szp;
        }
        return;
    }
    b -= a.interior_blocks;
    if (b < a.special_blocks) {
        long long k = (long long)b * BLOCK + threadIdx.x;
        if (k >= (long long)a.n_special * a.chunks) return;
        const int c = (int)(k / a.n_special);
        k -= (long long)c * a.n_special;
        const uint4 rec = __ldg(a.sp + k);
        const long long cell = rec.x;
        const uint32_t m = rec.y;
        const int z = (int)(cell / nxy);
        const __half *P = a.cur + (long long)c * a.cells_p * V;
        __half *Q = a.nxt + (long long)c * a.cells_p * V;
        const float sc = slab_scale(a, n, c, z).x;
        const Lanes<float, V> pc = load_h<V>(P + cell * V, sc);
        const Lanes<float, V> pp = load_h<V>(Q + cell * V, slab_scale(a, n + SCALE_RING - 1, c, z).x);
        const long long offs[6] = {-1, 1, -(long long)a.nxp, (long long)a.nxp, -nxy, nxy};
        Lanes<float, V> sum;
#pragma unroll
        for (int l = 0; l < V; l++) sum.v[l] = 0.0f;
        float kk = 0.0f;
#pragma unroll
        for (int d = 0; d < 6; d++) {
            if ((m >> d) & 1u) {
                const float sd = d < 4 ? sc : slab_scale(a, n, c, z + (d == 4 ? -1 : 1)).x;
                const Lanes<float, V> nb = load_h<V>(P + (cell + offs[d]) * V, sd);
#pragma unroll
                for (int l = 0; l < V; l++) sum.v[l] = radd(sum.v[l], nb.v[l]);
                kk = radd(kk, 1.0f);
            }
        }
        Lanes<float, V> lap, next;
#pragma unroll
        for (int l = 0; l < V; l++) lap.v[l] = rmul(a.l2, rsub(sum.v[l], rmul(kk, pc.v[l])));
        const int ns = (int)((m >> META_SLOT_SHIFT) & META_SLOT_MASK);
        if (ns == 0) {
#pragma unroll
            for (int l = 0; l < V; l++) next.v[l] = radd(rsub(rmul(2.0f, pc.v[l]), pp.v[l]), lap.v[l]);
        } else {
            const long long j0 = rec.z;
            float *SU = a.su + (long long)c * a.n_slots * V;
            float *SG = a.sg + (long long)c * a.n_slots * V;
            float s1 = 0.0f;
            Lanes<float, V> s2;
#pragma unroll
            for (int l = 0; l < V; l++) s2.v[l] = 0.0f;
            for (int q = 0; q < ns; q++) {
                const long long j = j0 + q;
                const float4 sl = __ldg(reinterpret_cast<const float4 *>(a.slots) + j);
                const Lanes<float, V> u = load<float, V, false>(SU + j * V);
                const Lanes<float, V> g = load<float, V, false>(SG + j * V);
#pragma unroll
                for (int l = 0; l < V; l++) {
                    const float e = rmul(radd(radd(rsub(rmul(sl.y, u.v[l]), rmul(sl.z, g.v[l])), rmul(0.5f, pc.v[l])),
                                              rmul(sl.w, pp.v[l])),
                                         sl.x);
                    s2.v[l] = rsub(radd(s2.v[l], e), u.v[l]);
                }
                s1 = radd(s1, rmul(rsub(0.5f, sl.w), sl.x));
            }
            const float den = radd(1.0f, rmul(a.lam, s1));
#pragma unroll
            for (int l = 0; l < V; l++)
                next.v[l] = rdiv(rsub(radd(rsub(rmul(2.0f, pc.v[l]), pp.v[l]), lap.v[l]), rmul(a.lam, s2.v[l])), den);
            for (int q = 0; q < ns; q++) {
                const long long j = j0 + q;
                const float4 sl = __ldg(reinterpret_cast<const float4 *>(a.slots) + j);
                Lanes<float, V> u = load<float, V, false>(SU + j * V);
                Lanes<float, V> g = load<float, V, false>(SG + j * V);
#pragma unroll
                for (int l = 0; l < V; l++) {
                    const float e = rmul(radd(radd(rsub(rmul(sl.y, u.v[l]), rmul(sl.z, g.v[l])), rmul(0.5f, pc.v[l])),
                                              rmul(sl.w, pp.v[l])),
                                         sl.x);
                    const float un = radd(rmul(rmul(rsub(0.5f, sl.w), sl.x), next.v[l]), e);
                    g.v[l] = radd(g.v[l], rmul(a.half_dt, radd(un, u.v[l])));
                    u.v[l] = un;
                }
                store<float, V>(SU + j * V, u);
                store<float, V>(SG + j * V, g);
            }
        }
        const uint32_t tap = rec.w;
        if (tap != NO_TAP) {
#pragma unroll
            for (int l = 0; l < V; l++) {
                const int s = c * V + l;
                next.v[l] = radd(next.v[l], rmul(a.sig[(long long)s * a.sig_stride + n], a.tapw[(long long)tap * a.lanes_total + s]));
            }
        }
        const float mx = store_h<V>(Q + cell * V, next, slab_scale(a, n + 1, c, z).y, a.error);
        if (mx > 0.0f) raise_max(amax_new + c * a.nz + z, mx);
        return;
    }
    b -= a.special_blocks;
    const long long k = (long long)b * BLOCK + threadIdx.x;
    if (k >= (long long)a.n_recv * a.chunks) return;
    const int c = (int)(k / a.n_recv);
    const long long r = k - (long long)c * a.n_recv;
    const long long cell = a.recv[r];
    const __half *P = a.cur + (long long)c * a.cells_p * V;
    const Lanes<float, V> v = load_h<V>(P + cell * V, slab_scale(a, n, c, (int)(cell / nxy)).x);
    store<float, V>(a.ring + (((long long)c * RING + t) * a.n_recv + r) * V, v);
}

}  // namespace wk
