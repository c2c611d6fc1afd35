// fdtd_kernels.cuh -- the FDTD time step on sm_103a.
//
// One fused launch per time step.  Its CTAs take one of three roles, all of
// which read only p^n and write disjoint cells of the older buffer, so they
// need no ordering among themselves:
//
//   interior  the leapfrog update of plain air cells (six air neighbours, no
//             boundary slot, no source tap), selected by a one-bit-per-cell
//             mask.  A warp owns 32 consecutive x cells of one row and marches
//             a run of z planes, keeping p(z-1), p(z), p(z+1) in registers.
//             Reference: fdtd.rs:697-708 (CPU), fdtd.wgsl:50-62 (GPU).
//   special   every other air cell, from a compacted list sorted by cell:
//             cells with rigid faces (K < 6 air neighbours, fdtd.wgsl:64-81),
//             boundary nodes with admittance slots solved jointly with their
//             branch states (boundary_update, fdtd.rs:580-598, fdtd.wgsl:
//             83-104), and source taps, whose injection (fdtd.rs:718-720,
//             fdtd.wgsl:110-119) is fused as the last operation of the update.
//   record    copies p^n at every receiver into a ring buffer of RING steps
//             (the samples of fdtd.rs:674-683, taken before the update).
//
// Every 128 steps a twiddle kernel and a DFT kernel fold the ring into the
// FP64 receiver spectra; see dft_chunk below.  Standalone plans keep two
// rings, used by alternate chunks, and fold each chunk while the next one
// runs.
//
// Fields are source-interleaved: a chunk of V right-hand sides (V = 1, 2 or
// 4) stores the V values of a cell contiguously, so one 128-bit access
// carries four sources in FP32.  Rows are padded to a multiple of 32 cells
// (128 bytes per lane), so every warp row access is aligned and a warp's
// interior mask is one 32-bit word.
//
// Arithmetic: every product, sum and quotient is rounded separately, in the
// order of the reference (WGSL order for FP32, the CPU's Rust order for
// FP64), so that receiver time series match a restatement of the reference
// bit for bit.  The stencil is memory-bound, so the lost FMA contraction
// costs nothing.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace wk {

constexpr int RING = 128;          // steps per chunk; even, so buffer parity repeats per chunk
constexpr int BLOCK = 256;         // threads per CTA, every role
constexpr int TILE_Y = BLOCK / 32; // rows per interior CTA
constexpr uint32_t NO_TAP = 0xFFFFFFFFu;
constexpr int META_SLOT_SHIFT = 6;
constexpr uint32_t META_SLOT_MASK = 31u;

// ------------------------------------------------------------ rounded ops
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float rdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double rdiv(double a, double b) { return __ddiv_rn(a, b); }

// -------------------------------------------------------- lane vectors
template <class T, int V>
struct Lanes {
    T v[V];
};

// Loads of the current field go through the read-only path (p^n is never
// written during a step); the older buffer is read and written.
template <class T, int V, bool RO>
__device__ __forceinline__ Lanes<T, V> load(const T *p) {
    Lanes<T, V> o;
    if constexpr (sizeof(T) * V == 16) {
        if constexpr (sizeof(T) == 4) {
            float4 x = RO ? __ldg(reinterpret_cast<const float4 *>(p)) : *reinterpret_cast<const float4 *>(p);
            o.v[0] = x.x; o.v[1] = x.y; o.v[2] = x.z; o.v[3] = x.w;
        } else {
            double2 x = RO ? __ldg(reinterpret_cast<const double2 *>(p)) : *reinterpret_cast<const double2 *>(p);
            o.v[0] = x.x; o.v[1] = x.y;
        }
    } else if constexpr (sizeof(T) * V == 8 && sizeof(T) == 4) {
        float2 x = RO ? __ldg(reinterpret_cast<const float2 *>(p)) : *reinterpret_cast<const float2 *>(p);
        o.v[0] = x.x; o.v[1] = x.y;
    } else if constexpr (sizeof(T) * V == 32) {
        double2 a = RO ? __ldg(reinterpret_cast<const double2 *>(p)) : *reinterpret_cast<const double2 *>(p);
        double2 b = RO ? __ldg(reinterpret_cast<const double2 *>(p) + 1) : *(reinterpret_cast<const double2 *>(p) + 1);
        o.v[0] = a.x; o.v[1] = a.y; o.v[2] = b.x; o.v[3] = b.y;
    } else {
#pragma unroll
        for (int l = 0; l < V; l++) o.v[l] = RO ? __ldg(p + l) : p[l];
    }
    return o;
}

template <class T, int V>
__device__ __forceinline__ void store(T *p, const Lanes<T, V> &o) {
    if constexpr (sizeof(T) * V == 16) {
        if constexpr (sizeof(T) == 4) {
            *reinterpret_cast<float4 *>(p) = make_float4(o.v[0], o.v[1], o.v[2], o.v[3]);
        } else {
            *reinterpret_cast<double2 *>(p) = make_double2(o.v[0], o.v[1]);
        }
    } else if constexpr (sizeof(T) * V == 8 && sizeof(T) == 4) {
        *reinterpret_cast<float2 *>(p) = make_float2(o.v[0], o.v[1]);
    } else if constexpr (sizeof(T) * V == 32) {
        reinterpret_cast<double2 *>(p)[0] = make_double2(o.v[0], o.v[1]);
        reinterpret_cast<double2 *>(p)[1] = make_double2(o.v[2], o.v[3]);
    } else {
#pragma unroll
        for (int l = 0; l < V; l++) p[l] = o.v[l];
    }
}

// ------------------------------------------------------------ arguments
template <class T>
struct StepArgs {
    const T *cur;              // p^n        [chunks][cells_p][V]
    T *nxt;                    // p^{n-1} in, p^{n+1} out
    T *out;                    // where the special cells' p^{n+1} goes: nxt, or a third buffer when two
                               // steps share one pass over the fields
    const uint32_t *interior;  // [nz][ny][nxw] one bit per padded cell
    const uint4 *sp;           // [n_special] {padded cell (ascending), meta, first slot, tap row or NO_TAP};
                               // meta: bits 0-5 air-neighbour flags, bits 6-10 slot count
    const T *slots;            // [n_slots][4] inv_d, cv, k, w
    T *su, *sg;                // [chunks][n_slots][V] branch velocity u and its integral g
    const T *tapw;             // [n_tap_rows][lanes_total] merged tap weight per source
    const T *sig;              // [lanes_total][sig_stride] or one shared row (sig_stride 0)
    const uint32_t *recv;      // [n_recv] padded receiver cells
    T *ring;                   // [chunks][RING][n_recv][V], or two such rings (ring_stride apart) used by
                               // alternate chunks, so that one is folded while the next chunk fills the other
    long long ring_stride;     // elements between the two rings; 0: one ring
    const long long *base;     // step index of the chunk's first step
    long long cells_p;         // padded cells per chunk
    long long sig_stride;
    int nxp, ny, nz, nxw;
    int n_special, n_slots, n_recv, chunks, lanes_total;
    int tiles_x, tiles_y, tiles_z, zt;
    int interior_blocks, special_blocks, record_blocks;
    T l2, lam, half_dt;
};

// The interior update of one cell, WGSL order (fdtd.wgsl:52-61), which is
// also the CPU order (fdtd.rs:706 with lap of fdtd.rs:685-696 and K = 6).
template <class T, int V>
__device__ __forceinline__ Lanes<T, V> interior_update(const Lanes<T, V> &c, const Lanes<T, V> &old, const Lanes<T, V> &xm,
                                                       const Lanes<T, V> &xp, const Lanes<T, V> &ym, const Lanes<T, V> &yp,
                                                       const Lanes<T, V> &zm, const Lanes<T, V> &zp, T l2) {
    Lanes<T, V> o;
#pragma unroll
    for (int l = 0; l < V; l++) {
        T s = radd(xm.v[l], xp.v[l]);
        s = radd(s, ym.v[l]);
        s = radd(s, yp.v[l]);
        s = radd(s, zm.v[l]);
        s = radd(s, zp.v[l]);
        T six = T(6);
        T two = T(2);
        o.v[l] = radd(rsub(rmul(two, c.v[l]), old.v[l]), rmul(l2, rsub(s, rmul(six, c.v[l]))));
    }
    return o;
}

// One special cell k of chunk c at step n (the special role of fdtd_step).
// The cell's loads are issued together before any arithmetic -- its
// neighbours, and the constants and branch states of up to SLOT_REGS slots,
// kept in registers for both passes of the boundary solve -- because the
// boundary solve is otherwise a chain of dependent loads per cell.
constexpr int SLOT_REGS = 3;  // beta0 + two branches: the usual node

template <class T, int V>
struct SlotRegs {
    T inv_d, cv, kb, w;
    Lanes<T, V> u, g;
};

template <class T, int V, class A>
__device__ __forceinline__ void load_slot(const A &a, const T *SU, const T *SG, long long j, SlotRegs<T, V> &r) {
    if constexpr (sizeof(T) == 4) {
        const float4 c = __ldg(reinterpret_cast<const float4 *>(a.slots) + j);
        r.inv_d = c.x, r.cv = c.y, r.kb = c.z, r.w = c.w;
    } else {
        const double2 c0 = __ldg(reinterpret_cast<const double2 *>(a.slots) + 2 * j);
        const double2 c1 = __ldg(reinterpret_cast<const double2 *>(a.slots) + 2 * j + 1);
        r.inv_d = c0.x, r.cv = c0.y, r.kb = c1.x, r.w = c1.y;
    }
    r.u = load<T, V, false>(SU + j * V);
    r.g = load<T, V, false>(SG + j * V);
}

// Field access of the special-cell update for values stored as computed
// (FP32, FP64): p^n at a cell (dz: its plane relative to the cell's, which
// FP16 storage needs for the slab scale), p^n at its neighbour d (-x, +x,
// -y, +y, -z, +z; off: the neighbour's cell offset), p^(n-1), and the store
// of p^(n+1).
template <class T, int V>
struct PlainField {
    static constexpr bool STREAM = false;
    const T *P;
    T *Q;  // p^(n-1)
    T *O;  // p^(n+1): Q itself, or a separate buffer
    __device__ __forceinline__ Lanes<T, V> p(long long cell, int) const { return load<T, V, true>(P + cell * V); }
    __device__ __forceinline__ Lanes<T, V> nb(long long cell, int, long long off) const {
        return load<T, V, true>(P + (cell + off) * V);
    }
    __device__ __forceinline__ Lanes<T, V> old(long long cell) const { return load<T, V, false>(Q + cell * V); }
    __device__ __forceinline__ void put(long long cell, const Lanes<T, V> &v) const { store<T, V>(O + cell * V, v); }
};

// The special-cell update of chunk c at step n from its record rec, with
// field access f (PlainField, or the FP16 form with slab scales) and the
// step's arguments a (StepArgs or HalfArgs).
template <class T, int V, bool RUST_ORDER, int SR, class A, class F>
__device__ __forceinline__ void special_core(const A &a, const F &f, const uint4 rec, int c, long long n) {
    const long long nxy = (long long)a.nxp * a.ny;
    const long long cell = rec.x;
    const uint32_t m = rec.y;
    const long long j0 = rec.z;
    const uint32_t tap = rec.w;
    const int ns = (int)((m >> META_SLOT_SHIFT) & META_SLOT_MASK);
    T *SU = a.su + (long long)c * a.n_slots * V;
    T *SG = a.sg + (long long)c * a.n_slots * V;
    // All loads first.
    const Lanes<T, V> pc = f.p(cell, 0);
    const Lanes<T, V> pp = f.old(cell);
    const long long offs[6] = {-1, 1, -(long long)a.nxp, (long long)a.nxp, -nxy, nxy};
    // The laplacian over air neighbours in the -x,+x,-y,+y,-z,+z order.
    // Fields in global memory load every neighbour before summing (one
    // round of memory latency); fields staged in shared memory (F::STREAM)
    // sum each neighbour as it is read, which holds fewer registers.  The
    // sums and their order are the same.
    Lanes<T, V> sum;
#pragma unroll
    for (int l = 0; l < V; l++) sum.v[l] = T(0);
    T kk = T(0);
    SlotRegs<T, V> sr[SR > 0 ? SR : 1];
    if constexpr (F::STREAM) {
#pragma unroll
        for (int d = 0; d < 6; d++) {
            if ((m >> d) & 1u) {
                const Lanes<T, V> v = f.nb(cell, d, offs[d]);
#pragma unroll
                for (int l = 0; l < V; l++) sum.v[l] = radd(sum.v[l], v.v[l]);
                kk = radd(kk, T(1));
            }
        }
#pragma unroll
        for (int q = 0; q < SR; q++)
            if (q < ns) load_slot<T, V, A>(a, SU, SG, j0 + q, sr[q]);
    } else {
        Lanes<T, V> nb[6];
#pragma unroll
        for (int d = 0; d < 6; d++)
            if ((m >> d) & 1u) nb[d] = f.nb(cell, d, offs[d]);
#pragma unroll
        for (int q = 0; q < SR; q++)
            if (q < ns) load_slot<T, V, A>(a, SU, SG, j0 + q, sr[q]);
#pragma unroll
        for (int d = 0; d < 6; d++) {
            if ((m >> d) & 1u) {
#pragma unroll
                for (int l = 0; l < V; l++) sum.v[l] = radd(sum.v[l], nb[d].v[l]);
                kk = radd(kk, T(1));
            }
        }
    }
    Lanes<T, V> lap, next;
#pragma unroll
    for (int l = 0; l < V; l++) lap.v[l] = rmul(a.l2, rsub(sum.v[l], rmul(kk, pc.v[l])));
    const T hf = T(0.5), two = T(2), one = T(1);
    if (ns == 0) {
#pragma unroll
        for (int l = 0; l < V; l++) next.v[l] = radd(rsub(rmul(two, pc.v[l]), pp.v[l]), lap.v[l]);
    } else {
        T s1 = T(0);
        Lanes<T, V> s2;
#pragma unroll
        for (int l = 0; l < V; l++) s2.v[l] = T(0);
        for (int q = 0; q < ns; q++) {
            SlotRegs<T, V> r;
            if (q < SR) {
#pragma unroll
                for (int i = 0; i < SR; i++)
                    if (i == q) r = sr[i];
            } else {
                load_slot<T, V, A>(a, SU, SG, j0 + q, r);
            }
#pragma unroll
            for (int l = 0; l < V; l++) {
                T e = rmul(radd(radd(rsub(rmul(r.cv, r.u.v[l]), rmul(r.kb, r.g.v[l])), rmul(hf, pc.v[l])), rmul(r.w, pp.v[l])),
                           r.inv_d);
                s2.v[l] = RUST_ORDER ? radd(s2.v[l], rsub(e, r.u.v[l])) : rsub(radd(s2.v[l], e), r.u.v[l]);
            }
            s1 = radd(s1, rmul(rsub(hf, r.w), r.inv_d));
        }
        const T den = radd(one, rmul(a.lam, s1));
#pragma unroll
        for (int l = 0; l < V; l++)
            next.v[l] = rdiv(rsub(radd(rsub(rmul(two, pc.v[l]), pp.v[l]), lap.v[l]), rmul(a.lam, s2.v[l])), den);
        for (int q = 0; q < ns; q++) {
            SlotRegs<T, V> r;
            if (q < SR) {
#pragma unroll
                for (int i = 0; i < SR; i++)
                    if (i == q) r = sr[i];
            } else {
                load_slot<T, V, A>(a, SU, SG, j0 + q, r);
            }
#pragma unroll
            for (int l = 0; l < V; l++) {
                T e = rmul(radd(radd(rsub(rmul(r.cv, r.u.v[l]), rmul(r.kb, r.g.v[l])), rmul(hf, pc.v[l])), rmul(r.w, pp.v[l])),
                           r.inv_d);
                T un = radd(rmul(rmul(rsub(hf, r.w), r.inv_d), next.v[l]), e);
                r.g.v[l] = radd(r.g.v[l], rmul(a.half_dt, radd(un, r.u.v[l])));
                r.u.v[l] = un;
            }
            store<T, V>(SU + (j0 + q) * V, r.u);
            store<T, V>(SG + (j0 + q) * V, r.g);
        }
    }
    if (tap != NO_TAP) {
#pragma unroll
        for (int l = 0; l < V; l++) {
            const int s = c * V + l;
            const T sv = a.sig[(long long)s * a.sig_stride + n];
            next.v[l] = radd(next.v[l], rmul(sv, a.tapw[(long long)tap * a.lanes_total + s]));
        }
    }
    f.put(cell, next);
}

template <class T, int V, bool RUST_ORDER, int SR = SLOT_REGS>
__device__ __forceinline__ void special_cell(const StepArgs<T> &a, long long k, long long n) {
    const int c = (int)(k / a.n_special);
    k -= (long long)c * a.n_special;
    const uint4 rec = __ldg(a.sp + k);
    const PlainField<T, V> f{a.cur + (long long)c * a.cells_p * V, a.nxt + (long long)c * a.cells_p * V,
                             a.out + (long long)c * a.cells_p * V};
    special_core<T, V, RUST_ORDER, SR>(a, f, rec, c, n);
}

// One receiver r of chunk c into ring slot t (the record role of fdtd_step).
template <class T, int V>
__device__ __forceinline__ void record_one(const StepArgs<T> &a, long long k, int t) {
    const int c = (int)(k / a.n_recv);
    const long long r = k - (long long)c * a.n_recv;
    const T *P = a.cur + (long long)c * a.cells_p * V;
    const Lanes<T, V> v = load<T, V, true>(P + (long long)a.recv[r] * V);
    T *ring = a.ring + ((*a.base / RING) & 1) * a.ring_stride;
    store<T, V>(ring + (((long long)c * RING + t) * a.n_recv + r) * V, v);
}

// ------------------------------------------------------------------ step
// RUST_ORDER selects the CPU reference's association of the branch sum
// (s2 + (e - u), fdtd.rs:588) instead of the shader's ((s2 + e) - u,
// fdtd.wgsl:94).
template <class T, int V, bool RUST_ORDER>
__device__ __forceinline__ void step_block(const StepArgs<T> &a, int b, int t) {
    const long long nxy = (long long)a.nxp * a.ny;
    if (b < a.interior_blocks) {
        // ---------------------------------------------------- interior
        const int per_chunk = a.tiles_x * a.tiles_y * a.tiles_z;
        const int c = b / per_chunk;
        int r = b - c * per_chunk;
        const int tz = r / (a.tiles_x * a.tiles_y);
        r -= tz * a.tiles_x * a.tiles_y;
        const int ty = r / a.tiles_x;
        const int tx = r - ty * a.tiles_x;
        const int lane = threadIdx.x & 31;
        const int y = 1 + ty * TILE_Y + (threadIdx.x >> 5);
        if (y >= a.ny - 1) return;
        const int x = tx * 32 + lane;
        const int zs = 1 + tz * a.zt;
        const int ze = min(zs + a.zt, a.nz - 1);
        const T *P = a.cur + (long long)c * a.cells_p * V;
        T *Q = a.nxt + (long long)c * a.cells_p * V;
        long long i = ((long long)zs * a.ny + y) * a.nxp + x;
        const uint32_t *mrow = a.interior + ((long long)zs * a.ny + y) * a.nxw + tx;
        const long long mstep = (long long)a.ny * a.nxw;
        Lanes<T, V> zm, zc, zp;
        bool have = false;
        for (int z = zs; z < ze; ++z, i += nxy, mrow += mstep) {
            const uint32_t word = __ldg(mrow);
            if (word == 0u) {  // uniform per warp: a solid or special-only row segment
                have = false;
                continue;
            }
            if (!have) {
                zm = load<T, V, true>(P + (i - nxy) * V);
                zc = load<T, V, true>(P + i * V);
                have = true;
            }
            zp = load<T, V, true>(P + (i + nxy) * V);
            if ((word >> lane) & 1u) {
                Lanes<T, V> xm = load<T, V, true>(P + (i - 1) * V);
                Lanes<T, V> xp = load<T, V, true>(P + (i + 1) * V);
                Lanes<T, V> ym = load<T, V, true>(P + (i - a.nxp) * V);
                Lanes<T, V> yp = load<T, V, true>(P + (i + a.nxp) * V);
                Lanes<T, V> old = load<T, V, false>(Q + i * V);
                store<T, V>(Q + i * V, interior_update<T, V>(zc, old, xm, xp, ym, yp, zm, zp, a.l2));
            }
            zm = zc;
            zc = zp;
        }
        return;
    }
    b -= a.interior_blocks;
    const long long n = *a.base + t;
    if (b < a.special_blocks) {
        // ----------------------------------------------------- special
        const long long k = (long long)b * BLOCK + threadIdx.x;
        if (k >= (long long)a.n_special * a.chunks) return;
        special_cell<T, V, RUST_ORDER, 0>(a, k, *a.base + t);  // lean: shares the kernel with the interior role
        return;
    }
    b -= a.special_blocks;
    // --------------------------------------------------------- record
    const long long k = (long long)b * BLOCK + threadIdx.x;
    if (k >= (long long)a.n_recv * a.chunks) return;
    record_one<T, V>(a, k, t);
}

template <class T, int V, bool RUST_ORDER>
__global__ void __launch_bounds__(BLOCK) fdtd_step(StepArgs<T> a, int t) {
    step_block<T, V, RUST_ORDER>(a, blockIdx.x, t);
}

// The special and record roles alone (interior_blocks == 0), for the branch
// that runs beside the TMA interior kernel.  MINB caps the registers so that
// MINB blocks fit an SM: a lighter branch leaves room for interior CTAs on
// the same SMs.
template <int V, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) special_branch(StepArgs<float> a, int t) {
    constexpr int SR = MINB >= 4 ? (V == 4 ? 0 : 1) : MINB == 3 ? 2 : SLOT_REGS;  // slots held in registers
    int b = blockIdx.x;
    if (b < a.special_blocks) {
        const long long k = (long long)b * BLOCK + threadIdx.x;
        if (k >= (long long)a.n_special * a.chunks) return;
        special_cell<float, V, false, SR>(a, k, *a.base + t);
        return;
    }
    b -= a.special_blocks;
    const long long k = (long long)b * BLOCK + threadIdx.x;
    if (k >= (long long)a.n_recv * a.chunks) return;
    record_one<float, V>(a, k, t);
}

// ----------------------------------------------------------- many rooms
// Several rooms advance in one launch per step.  The grid is the rooms'
// blocks laid end to end (the work-tile table: room r owns blocks
// [first, first + blocks)); a block finds its room, then runs the same three
// roles on that room's arguments.  Rooms keep their own lanes per chunk and
// their own step count: past its last step a room's blocks do nothing.
template <class T>
struct RoomStep {
    StepArgs<T> a[2];  // by buffer parity
    int lanes;         // V of the room's chunks: 1, 2 or 4
    int blocks;
    long long steps;
};

template <class T, bool RUST_ORDER>
__global__ void __launch_bounds__(BLOCK) fdtd_step_rooms(const RoomStep<T> *rooms, int n_rooms, int t, int parity) {
    int b = blockIdx.x, r = 0;
    while (r < n_rooms - 1 && b >= rooms[r].blocks) {
        b -= rooms[r].blocks;
        r++;
    }
    const RoomStep<T> &room = rooms[r];
    if (*room.a[0].base + t >= room.steps) return;
    const StepArgs<T> &a = room.a[parity];
    switch (room.lanes) {
        case 1: step_block<T, 1, RUST_ORDER>(a, b, t); break;
        case 2: step_block<T, 2, RUST_ORDER>(a, b, t); break;
        default: step_block<T, 4, RUST_ORDER>(a, b, t); break;
    }
}

// ------------------------------------------------------------- twiddles
// tw[t][f] = exp(-j 2 pi frac(f dt n)) for n = base + t, phase in FP64
// exactly as fdtd.rs:680 forms it.
// The chunk folded starts at step *base - lag: lag = RING folds the previous
// chunk (beside the steps of the current one); nothing before step 0.
template <class T>
__global__ void twiddle_chunk(const double *freqs, int nf, double dt, const long long *base, int count, long long steps,
                              T *tw, int lag) {
    const long long b0 = *base - lag;
    if (b0 < 0) return;
    count = (int)min((long long)count, steps - b0);  // a room that stops inside the chunk
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= count * nf) return;
    const int t = idx / nf, f = idx - t * nf;
    const double x = freqs[f] * dt * (double)(b0 + t);
    const double ph = -6.283185307179586 * (x - trunc(x));
    double s, c;
    sincos(ph, &s, &c);
    tw[2 * idx] = (T)c;
    tw[2 * idx + 1] = (T)s;
}

// ------------------------------------------------------------------ DFT
// acc[c][r][f][l] += sum_t ring[c][t][r][l] * tw[t][f], the partial sum of a
// chunk in A (the samples' type T, or FP64 for FP64 accumulation of FP32
// samples), added into FP64.  One thread per (chunk, receiver, freq).
template <class T, int V, class A = T>
__global__ void __launch_bounds__(BLOCK) dft_chunk(const T *ring, const A *tw, double *acc, int n_recv, int nf, int chunks,
                                                   int count, const long long *base, long long steps, int lag,
                                                   long long ring_stride) {
    const long long b0 = *base - lag;
    if (b0 < 0) return;
    count = (int)min((long long)count, steps - b0);
    ring += ((b0 / RING) & 1) * ring_stride;
    const long long idx = (long long)blockIdx.x * BLOCK + threadIdx.x;
    const long long total = (long long)chunks * n_recv * nf;
    if (idx >= total) return;
    const long long rf = idx % ((long long)n_recv * nf);
    const int c = (int)(idx / ((long long)n_recv * nf));
    const int r = (int)(rf / nf), f = (int)(rf - (long long)r * nf);
    A re[V], im[V];
#pragma unroll
    for (int l = 0; l < V; l++) re[l] = im[l] = A(0);
    const T *src = ring + ((long long)c * RING * n_recv + r) * V;
    for (int t = 0; t < count; t++) {
        const Lanes<T, V> v = load<T, V, true>(src + (long long)t * n_recv * V);
        const A wr = __ldg(tw + 2 * (t * nf + f)), wi = __ldg(tw + 2 * (t * nf + f) + 1);
#pragma unroll
        for (int l = 0; l < V; l++) {
            re[l] = fma((A)v.v[l], wr, re[l]);
            im[l] = fma((A)v.v[l], wi, im[l]);
        }
    }
    double *out = acc + idx * V * 2;
#pragma unroll
    for (int l = 0; l < V; l++) {
        out[2 * l] += (double)re[l];
        out[2 * l + 1] += (double)im[l];
    }
}

// The same fold for FP32 samples and sums, shaped as the small matrix
// product it is: the chunk's twiddles are staged in shared memory once per
// block ([t][f], frequencies padded to DFT_FB with zeros), and each thread
// takes one (chunk, receiver) and DFT_FB frequencies, so every sample it
// loads (coalesced across the receivers of a warp) feeds 2 x V x DFT_FB FMAs.
// Each output still sums its steps in order with the same FMAs, so the
// spectra are dft_chunk's bit for bit.  Used when the twiddles fit in
// DFT_SMEM_MAX bytes.
constexpr int DFT_FB = 4;
constexpr int DFT_SMEM_MAX = 96 * 1024;
__host__ __device__ constexpr int dft_nfp(int nf) { return (nf + DFT_FB - 1) / DFT_FB * DFT_FB; }

template <int V>
__global__ void __launch_bounds__(BLOCK) dft_chunk_tiled(const float *ring, const float *tw, double *acc, int n_recv,
                                                         int nf, int chunks, int count, const long long *base,
                                                         long long steps, int lag, long long ring_stride) {
    extern __shared__ float2 s_tw[];
    const long long b0 = *base - lag;
    if (b0 < 0) return;  // the same for every thread: no barrier is left waiting
    count = (int)min((long long)count, steps - b0);
    ring += ((b0 / RING) & 1) * ring_stride;
    const int nfp = dft_nfp(nf);
    // Staged with one 8-byte load per twiddle, eight loads in flight per
    // thread.
    const float2 *tw2 = reinterpret_cast<const float2 *>(tw);
#pragma unroll 8
    for (int i = threadIdx.x; i < count * nfp; i += BLOCK) {
        const int t = i / nfp, f = i - t * nfp;
        s_tw[i] = f < nf ? __ldg(tw2 + t * nf + f) : make_float2(0.0f, 0.0f);
    }
    __syncthreads();
    const int fblocks = nfp / DFT_FB;
    const long long idx = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (idx >= (long long)chunks * fblocks * n_recv) return;
    const int r = (int)(idx % n_recv);
    const long long rest = idx / n_recv;
    const int fb = (int)(rest % fblocks), c = (int)(rest / fblocks);
    float re[DFT_FB][V], im[DFT_FB][V];
#pragma unroll
    for (int k = 0; k < DFT_FB; k++)
#pragma unroll
        for (int l = 0; l < V; l++) re[k][l] = im[k][l] = 0.0f;
    const float *src = ring + ((long long)c * RING * n_recv + r) * V;
    const float2 *w = s_tw + fb * DFT_FB;
#pragma unroll 8
    for (int t = 0; t < count; t++) {
        const Lanes<float, V> v = load<float, V, true>(src + (long long)t * n_recv * V);
#pragma unroll
        for (int k = 0; k < DFT_FB; k++) {
            const float2 wk = w[t * nfp + k];
#pragma unroll
            for (int l = 0; l < V; l++) {
                re[k][l] = fmaf(v.v[l], wk.x, re[k][l]);
                im[k][l] = fmaf(v.v[l], wk.y, im[k][l]);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < DFT_FB; k++) {
        const int f = fb * DFT_FB + k;
        if (f >= nf) break;
        double *out = acc + (((long long)c * n_recv + r) * nf + f) * V * 2;
#pragma unroll
        for (int l = 0; l < V; l++) {
            out[2 * l] += (double)re[k][l];
            out[2 * l + 1] += (double)im[k][l];
        }
    }
}

// ir[s][r][n0 + t] = ring[c][t][r][l] (s = c*V + l): the time series of
// run_cpu_ir (fdtd.rs:628-641).
template <class T, int V>
__global__ void ir_chunk(const T *ring, T *ir, int n_recv, int chunks, int n_sources, long long steps,
                         const long long *base, int count, int lag, long long ring_stride) {
    const int full = count;
    const long long b0 = *base - lag;
    if (b0 < 0) return;
    count = (int)min((long long)count, steps - b0);
    ring += ((b0 / RING) & 1) * ring_stride;
    const long long idx = (long long)blockIdx.x * BLOCK + threadIdx.x;
    const long long total = (long long)chunks * V * n_recv * full;
    if (idx >= total) return;
    const int t = (int)(idx % full);
    if (t >= count) return;
    long long rest = idx / full;
    const int r = (int)(rest % n_recv);
    rest /= n_recv;
    const int s = (int)rest;  // c * V + l
    if (s >= n_sources) return;
    const int c = s / V, l = s - c * V;
    ir[((long long)s * n_recv + r) * steps + b0 + t] = ring[(((long long)c * RING + t) * n_recv + r) * V + l];
}

// Per-speaker transfer functions from a plan's spectra accumulators, as
// complex64 in the results.bin transfer layout (result.rs:444-456): mics
// [m][speaker][f], then per plane [speaker][point][f].  One thread per
// (speaker, receiver, frequency): the sum over the speaker's right-hand sides
// of factor[lane][f] x acc[lane][r][f] in FP64 (the factor carries the
// component weight, the to_transfer scale and the calibration), rounded once
// to FP32.  acc is [chunk][r][f][lane in chunk][2]; plane_first[p] is the
// first receiver of plane p (plane_first[0] = n_mics, plane_first[n_planes] =
// n_recv).
__global__ void __launch_bounds__(BLOCK) speaker_transfers(const double *acc, int n_recv, int nf, int V,
                                                           const int *spk_start, const int *spk_lanes,
                                                           const double2 *factor, int n_speakers,
                                                           const long long *plane_first, int n_planes, float2 *out) {
    const long long idx = (long long)blockIdx.x * BLOCK + threadIdx.x;
    const long long per_spk = (long long)n_recv * nf;
    if (idx >= per_spk * n_speakers) return;
    const int s = (int)(idx / per_spk);
    const long long rf = idx - (long long)s * per_spk;
    const int r = (int)(rf / nf), f = (int)(rf - (long long)r * nf);
    double re = 0.0, im = 0.0;
    for (int j = spk_start[s]; j < spk_start[s + 1]; j++) {
        const int lane = spk_lanes[j];
        const int c = lane / V, l = lane - c * V;
        const double *a = acc + ((((long long)c * n_recv + r) * nf + f) * V + l) * 2;
        const double2 k = factor[(long long)lane * nf + f];
        re += k.x * a[0] - k.y * a[1];
        im += k.x * a[1] + k.y * a[0];
    }
    const long long n_mics = plane_first[0];
    long long o;
    if (r < n_mics) {
        o = ((long long)r * n_speakers + s) * nf + f;
    } else {
        int p = 0;
        while (p + 1 < n_planes && r >= plane_first[p + 1]) p++;
        const long long first = plane_first[p], points = plane_first[p + 1] - first;
        o = n_mics * n_speakers * nf + (first - n_mics) * n_speakers * nf + ((long long)s * points + (r - first)) * nf + f;
    }
    out[o] = make_float2((float)re, (float)im);
}

__global__ void advance_base(long long *base, int by) { *base += by; }

}  // namespace wk
