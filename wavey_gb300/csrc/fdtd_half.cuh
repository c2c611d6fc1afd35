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
    float *ring;               // [chunks][RING][n_recv][V], or two rings ring_stride apart (StepArgs::ring)
    long long ring_stride;
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

__device__ __forceinline__ float warp_max(float m) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    return m;
}

// Field access of the special-cell update with FP16 storage: values are
// scaled by their slab's power of two on load (level n for p, the planes
// below and above for the z neighbours, level n-1 for p^(n-1)) and by the
// inverse of level n+1's on store, which also raises the slab maximum.
template <int V>
struct HalfField {
    static constexpr bool STREAM = false;
    const __half *P;
    __half *Q;
    float sm, sc, sp, so, inv;
    int *error;
    mutable float mx;  // max |p^(n+1)| stored, for the slab maximum
    __device__ __forceinline__ Lanes<float, V> p(long long cell, int dz) const {
        return load_h<V>(P + cell * V, dz < 0 ? sm : (dz > 0 ? sp : sc));
    }
    __device__ __forceinline__ Lanes<float, V> nb(long long cell, int d, long long off) const {
        return p(cell + off, d == 4 ? -1 : (d == 5 ? 1 : 0));
    }
    __device__ __forceinline__ Lanes<float, V> old(long long cell) const { return load_h<V>(Q + cell * V, so); }
    __device__ __forceinline__ void put(long long cell, const Lanes<float, V> &v) const {
        mx = store_h<V>(Q + cell * V, v, inv, error);
    }
};

// Special cell k (over all chunks) at step n with FP16 storage.  Special
// cells lie strictly inside the grid, so slabs z - 1 and z + 1 exist.
template <int V, int SR>
__device__ __forceinline__ void special_half(const HalfArgs &a, long long k, long long n, unsigned alive) {
    const int c = (int)(k / a.n_special);
    k -= (long long)c * a.n_special;
    const uint4 rec = __ldg(a.sp + k);
    const int z = (int)((long long)rec.x / ((long long)a.nxp * a.ny));
    HalfField<V> f;
    f.P = a.cur + (long long)c * a.cells_p * V;
    f.Q = a.nxt + (long long)c * a.cells_p * V;
    f.sm = slab_scale(a, n, c, z - 1).x;
    f.sc = slab_scale(a, n, c, z).x;
    f.sp = slab_scale(a, n, c, z + 1).x;
    f.so = slab_scale(a, n + SCALE_RING - 1, c, z).x;
    f.inv = slab_scale(a, n + 1, c, z).y;
    f.error = a.error;
    f.mx = 0.0f;
    special_core<float, V, false, SR>(a, f, rec, c, n);
    // Raise the slab maximum.  Special cells are sorted by cell, so a full
    // warp mostly shares one slab and chunk: it combines first and issues one
    // reduction without return (RED); otherwise every lane issues its own.
    // alive: the lanes of this warp that hold a special cell.
    unsigned int *slot = a.amax + ((long long)((n + 1) % AMAX_RING) * a.chunks + c) * a.nz + z;
    __syncwarp(alive);
    const int key = c * a.nz + z;
    if (alive == 0xffffffffu && __all_sync(alive, key == __shfl_sync(alive, key, 0))) {
        const float m = warp_max(f.mx);
        if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(slot, __float_as_uint(m));
    } else if (f.mx > 0.0f) {
        atomicMax(slot, __float_as_uint(f.mx));
    }
}

// Receiver k (over all chunks) into ring slot t: p^n in FP32.
template <int V>
__device__ __forceinline__ void record_half(const HalfArgs &a, long long k, int t, long long n) {
    const int c = (int)(k / a.n_recv);
    const long long r = k - (long long)c * a.n_recv;
    const long long cell = a.recv[r];
    const __half *P = a.cur + (long long)c * a.cells_p * V;
    const Lanes<float, V> v = load_h<V>(P + cell * V, slab_scale(a, n, c, (int)(cell / ((long long)a.nxp * a.ny))).x);
    float *ring = a.ring + ((*a.base / RING) & 1) * a.ring_stride;
    store<float, V>(ring + (((long long)c * RING + t) * a.n_recv + r) * V, v);
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
            if (lane == 0 && m > 0.0f) atomicMax(amax_new + c * a.nz + z, __float_as_uint(m));  // RED
            zm = zc;
            zc = zp;
            szm = szc;
            szc = szp;
        }
        return;
    }
    b -= a.interior_blocks;
    if (b < a.special_blocks) {
        const long long k = (long long)b * BLOCK + threadIdx.x;
        const bool live = k < (long long)a.n_special * a.chunks;
        const unsigned alive = __ballot_sync(0xffffffffu, live);
        if (!live) return;
        special_half<V, 0>(a, k, n, alive);  // lean: shares the kernel with the interior role
        return;
    }
    b -= a.special_blocks;
    const long long k = (long long)b * BLOCK + threadIdx.x;
    if (k >= (long long)a.n_recv * a.chunks) return;
    record_half<V>(a, k, t, n);
}

// The special and record roles alone (interior_blocks == 0), for the branch
// beside the TMA interior kernel; MINB caps the registers as in
// special_branch.
template <int V, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) special_branch_half(HalfArgs a, int t) {
    constexpr int SR = MINB >= 4 ? (V == 4 ? 0 : 1) : MINB == 3 ? 2 : SLOT_REGS;
    const long long n = *a.base + t;
    int b = blockIdx.x;
    if (b < a.special_blocks) {
        const long long k = (long long)b * BLOCK + threadIdx.x;
        const bool live = k < (long long)a.n_special * a.chunks;
        const unsigned alive = __ballot_sync(0xffffffffu, live);
        if (!live) return;
        special_half<V, SR>(a, k, n, alive);
        return;
    }
    b -= a.special_blocks;
    const long long k = (long long)b * BLOCK + threadIdx.x;
    if (k >= (long long)a.n_recv * a.chunks) return;
    record_half<V>(a, k, t, n);
}

}  // namespace wk
