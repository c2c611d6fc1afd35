// grid_build.cuh -- FdtdGrid::build_dx (core/wavey-solver/src/fdtd.rs:289-378)
// on the device, for box and prism rooms with pillars, absorbing blocks and
// rigid solids, and for rooms imported as triangle meshes: the same
// classification, neighbour flags, face lookup and boundary slots as the
// host builders (wavey_gb300/csrc/host/grid.cpp, mesh.cpp), in the same FP64
// operations, so the arrays are identical.  Boundary nodes are numbered in
// cell order by a scan over the cells.
//
//   grid_column_fill  mesh rooms, one thread per (x, y) column: column_fill
//                  (fdtd.rs:385-422), the crossings of one upward ray
//   grid_classify  one thread per cell: rigid solid?  air?  (fdtd.rs:308-337)
//   grid_flags     one thread per cell: air bit and air-neighbour bits (fdtd.rs:349-356)
//   grid_nodes     one thread per cell: slot count of a boundary node -- the
//                  surface behind each missing face within 1.5 dx (fdtd.rs:357-363)
//                  and boundary_slots (fdtd.rs:539-571); with `write`, its node
//                  index, cell, first slot and slot constants
//   scan_*         exclusive scan of the per-cell node and slot counts, and the air count
#pragma once
#include <cstdint>

#include "../../include/wavey_host.h"

namespace wk {

struct GbRect {
    int axis;
    double c, lo[3], hi[3];
};

// Triangles binned by their extent across one axis (for rays along it):
// cell (i, j) of a nu x nv grid of side h from (u0, v0) lists the triangles,
// in triangle order, at list[start[j * nu + i] .. start[j * nu + i + 1]).
struct GbBins {
    int u, v;
    double u0, v0, h;
    long long nu, nv;
    const uint32_t *start, *list;
};

struct GbRoom {
    double x0, y0, x1, y1, height;
    int n_pillars, n_blocks, n_solids, n_rects;
    const double *pillars, *blocks, *solids;  // device copies
    const GbRect *rects;
    const wh_fit *fits;                       // one per rect (mesh rooms: one per surface)
    long long nx, ny, nz;
    double origin[3], dx, dt;
    // Mesh rooms (mesh != 0): triangles {v0, v1 - v0, v2 - v0}, each
    // triangle's surface, per-axis bins, and column_fill's inside flags.
    int mesh;
    long long n_tri;
    const double *tri;
    const uint32_t *tri_surface;
    GbBins bins[3];
    const uint8_t *inside;
};

// Moeller-Trumbore, two-sided (wavey-geom bvh.rs:238-259), each operation
// rounded on its own as the host builder computes it.  e = [v0, e1, e2].
__device__ __forceinline__ bool gb_ray_triangle(const double o[3], const double d[3], const double *e, double *t) {
    auto cross = [](const double *a, const double *b, double *out) {
        out[0] = __dsub_rn(__dmul_rn(a[1], b[2]), __dmul_rn(b[1], a[2]));
        out[1] = __dsub_rn(__dmul_rn(a[2], b[0]), __dmul_rn(b[2], a[0]));
        out[2] = __dsub_rn(__dmul_rn(a[0], b[1]), __dmul_rn(b[0], a[1]));
    };
    auto dot = [](const double *a, const double *b) {
        return __dadd_rn(__dadd_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2]));
    };
    double p[3], q[3], s[3];
    cross(d, e + 6, p);
    const double det = dot(e + 3, p);
    if (fabs(det) < 1e-14) return false;
    const double inv = __ddiv_rn(1.0, det);
    for (int a = 0; a < 3; a++) s[a] = __dsub_rn(o[a], e[a]);
    const double u = __dmul_rn(dot(s, p), inv);
    if (!(u >= -1e-10 && u <= 1.0 + 1e-10)) return false;
    cross(s, e + 3, q);
    const double v = __dmul_rn(dot(d, q), inv);
    if (v < -1e-10 || __dadd_rn(u, v) > 1.0 + 1e-10) return false;
    *t = __dmul_rn(dot(e + 6, q), inv);
    return true;
}

// The bin a ray along b's axis through p falls in, or -1.
__device__ __forceinline__ long long gb_bin(const GbBins &b, const double p[3]) {
    const double a = p[b.u], c = p[b.v];
    if (a < b.u0 || c < b.v0) return -1;
    const long long i = (long long)floor((a - b.u0) / b.h), j = (long long)floor((c - b.v0) / b.h);
    if (i >= b.nu || j >= b.nv) return -1;
    return j * b.nu + i;
}

__device__ __forceinline__ void gb_center(const GbRoom &r, long long x, long long y, long long z, double p[3]) {
    p[0] = __dadd_rn(r.origin[0], __dmul_rn((double)x, r.dx));
    p[1] = __dadd_rn(r.origin[1], __dmul_rn((double)y, r.dx));
    p[2] = __dadd_rn(r.origin[2], __dmul_rn((double)z, r.dx));
}

__device__ __forceinline__ bool gb_in_box(const double *b, const double p[3]) {
    return p[0] >= b[0] && p[1] >= b[1] && p[2] >= b[2] && p[0] <= b[3] && p[1] <= b[4] && p[2] <= b[5];
}

__device__ __forceinline__ bool gb_in_rect(double x0, double y0, double x1, double y1, double x, double y) {
    return x >= x0 && x < x1 && y >= y0 && y < y1;
}

constexpr int GB_MAX_CROSSINGS = 128;
constexpr int GB_ERR_CROSSINGS = 1;

// column_fill (fdtd.rs:385-422): one upward ray per (x, y) column, moved off
// the cell centres by (0.0001372, 0.0002918) dx, from one cell below the
// grid; crossings sorted by parameter, a crossing of one surface side at the
// same height as the previous one (within 1e-9) counted once; a cell is
// inside after an odd number of crossings below its centre.
__global__ void __launch_bounds__(256) grid_column_fill(GbRoom r, uint8_t *inside, int *err) {
    const long long col = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= r.nx * r.ny) return;
    const long long x = col % r.nx, y = col / r.nx;
    double cen[3];
    gb_center(r, x, y, 0, cen);
    const double start = __dsub_rn(r.origin[2], r.dx);
    const double o[3] = {__dadd_rn(cen[0], __dmul_rn(0.0001372, r.dx)), __dadd_rn(cen[1], __dmul_rn(0.0002918, r.dx)),
                         __dadd_rn(start, 0.0)};
    const double up[3] = {0.0, 0.0, 1.0};
    double ht[GB_MAX_CROSSINGS];
    bool hu[GB_MAX_CROSSINGS];
    int n = 0;
    const long long b = gb_bin(r.bins[2], o);
    if (b >= 0) {
        for (uint32_t k = r.bins[2].start[b]; k < r.bins[2].start[b + 1]; k++) {
            const uint32_t t = r.bins[2].list[k];
            const double *e = r.tri + 9 * (long long)t;
            double th;
            if (!gb_ray_triangle(o, up, e, &th) || !(th > 0.0)) continue;
            if (n == GB_MAX_CROSSINGS) {
                atomicExch(err, GB_ERR_CROSSINGS);
                return;
            }
            // cross(e1, e2).z > 0: the triangle faces up.  Insertion keeps
            // equal parameters in triangle order (a stable sort).
            const bool u = __dsub_rn(__dmul_rn(e[3], e[7]), __dmul_rn(e[6], e[4])) > 0.0;
            int j = n++;
            while (j > 0 && ht[j - 1] > th) {
                ht[j] = ht[j - 1];
                hu[j] = hu[j - 1];
                j--;
            }
            ht[j] = th;
            hu[j] = u;
        }
    }
    // Crossings of one side at the same height count once.
    int m = 0;
    for (int k = 0; k < n; k++) {
        if (m > 0 && __dsub_rn(ht[k], ht[m - 1]) < 1e-9 && hu[m - 1] == hu[k]) continue;
        ht[m] = ht[k];
        hu[m] = hu[k];
        m++;
    }
    int k = 0;
    const long long nxy = r.nx * r.ny;
    for (long long z = 0; z < r.nz; z++) {
        double p[3];
        gb_center(r, x, y, z, p);
        const double tz = __dsub_rn(p[2], start);
        while (k < m && ht[k] < tz) k++;
        inside[z * nxy + col] = (k % 2 == 1);
    }
}

// room.rs:151-157 (strict 0 < z < h and the plan region) minus the blocks.
__device__ bool gb_room_contains(const GbRoom &r, const double p[3]) {
    if (!(p[2] > 0.0 && p[2] < r.height)) return false;
    if (!gb_in_rect(r.x0, r.y0, r.x1, r.y1, p[0], p[1])) return false;
    for (int i = 0; i < r.n_pillars; i++) {
        const double *q = r.pillars + 4 * i;
        if (gb_in_rect(q[0], q[1], q[2], q[3], p[0], p[1])) return false;
    }
    for (int i = 0; i < r.n_blocks; i++)
        if (gb_in_box(r.blocks + 6 * i, p)) return false;
    return true;
}

__global__ void __launch_bounds__(256) grid_classify(GbRoom r, uint8_t *solid, uint8_t *air) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long cells = r.nx * r.ny * r.nz;
    if (i >= cells) return;
    const long long x = i % r.nx, y = (i / r.nx) % r.ny, z = i / (r.nx * r.ny);
    double p[3];
    gb_center(r, x, y, z, p);
    bool s = false;
    for (int k = 0; k < r.n_solids && !s; k++) s = gb_in_box(r.solids + 6 * k, p);
    solid[i] = s;
    air[i] = !s && x > 0 && y > 0 && z > 0 && x < r.nx - 1 && y < r.ny - 1 && z < r.nz - 1 &&
             (r.mesh ? r.inside[i] != 0 : gb_room_contains(r, p));
}

__global__ void __launch_bounds__(256) grid_flags(GbRoom r, const uint8_t *air, uint8_t *flags) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long cells = r.nx * r.ny * r.nz;
    if (i >= cells || !air[i]) return;
    const long long nxy = r.nx * r.ny;
    const long long off[6] = {-1, 1, -r.nx, r.nx, -nxy, nxy};
    uint8_t fl = WAVEY_AIR;
    for (int k = 0; k < 6; k++)
        if (air[i + off[k]]) fl |= (uint8_t)(1u << k);  // air cells are interior: i + off stays in the grid
    flags[i] = fl;
}

__device__ bool gb_fits_equal(const wh_fit &a, const wh_fit &b) {
    if (a.beta0 != b.beta0 || a.n_branches != b.n_branches || a.band_lo != b.band_lo || a.band_hi != b.band_hi ||
        a.rms_error != b.rms_error || a.max_error != b.max_error)
        return false;
    for (int i = 0; i < a.n_branches; i++)
        if (a.r[i] != b.r[i] || a.m[i] != b.m[i] || a.k[i] != b.k[i]) return false;
    return true;
}

// The surfaces behind the missing faces of air cell (x, y, z), in face order.
__device__ int gb_faces(const GbRoom &r, const uint8_t *solid, long long x, long long y, long long z, uint8_t fl,
                        int faces[6]) {
    const long long nxy = r.nx * r.ny, i = (z * r.ny + y) * r.nx + x;
    const long long off[6] = {-1, 1, -r.nx, r.nx, -nxy, nxy};
    double p[3];
    gb_center(r, x, y, z, p);
    const double reach = __dmul_rn(r.dx, 1.5);
    int nf = 0;
    for (int k = 0; k < 6; k++) {
        if (fl & (1u << k)) continue;
        if (solid[i + off[k]]) continue;  // rigid: no admittance
        const int axis = k / 2;
        const double sgn = (k & 1) ? 1.0 : -1.0;
        int best = -1;
        double tbest = reach;
        if (r.mesh) {
            // The closest triangle along the face direction, 0 < t < 1.5 dx
            // (fdtd.rs:357-362); the first in triangle order at equal t.
            const double dir[3] = {axis == 0 ? sgn : 0.0, axis == 1 ? sgn : 0.0, axis == 2 ? sgn : 0.0};
            const GbBins &bn = r.bins[axis];
            const long long b = gb_bin(bn, p);
            if (b >= 0)
                for (uint32_t j = bn.start[b]; j < bn.start[b + 1]; j++) {
                    const uint32_t t = bn.list[j];
                    double th;
                    if (gb_ray_triangle(p, dir, r.tri + 9 * (long long)t, &th) && th > 0.0 && th < tbest) {
                        tbest = th;
                        best = (int)r.tri_surface[t];
                    }
                }
            if (best >= 0) faces[nf++] = best;
            continue;
        }
        for (int q = 0; q < r.n_rects; q++) {
            const GbRect &rc = r.rects[q];
            if (rc.axis != axis) continue;
            const double t = __dmul_rn(__dsub_rn(rc.c, p[axis]), sgn);
            if (!(t > 0.0 && t < tbest)) continue;
            bool inside = true;
            for (int a = 0; a < 3 && inside; a++)
                if (a != axis) inside = p[a] >= rc.lo[a] && p[a] <= rc.hi[a];
            if (!inside) continue;
            best = q;
            tbest = t;
        }
        if (best >= 0) faces[nf++] = best;
    }
    return nf;
}

// boundary_slots (fdtd.rs:539-571): identical fits grouped in first-seen
// order, n identical faces dividing r, m, k by n; writes up to 30 slots when
// out is not null and returns their count.
__device__ int gb_slots(const GbRoom &r, const int *faces, int nfaces, double *out) {
    int cs[6], cn[6], ncounts = 0;
    for (int f = 0; f < nfaces; f++) {
        const int s = faces[f];
        int k = 0;
        while (k < ncounts && !gb_fits_equal(r.fits[cs[k]], r.fits[s])) k++;
        if (k < ncounts) {
            cn[k]++;
        } else {
            cs[ncounts] = s;
            cn[ncounts] = 1;
            ncounts++;
        }
    }
    int ns = 0;
    const double dt = r.dt;
    auto add = [&](double rr, double m, double k, double n) {
        if (out) {
            rr = __ddiv_rn(rr, n);
            m = __ddiv_rn(m, n);
            k = __ddiv_rn(k, n);
            double d, cv, w;
            if (m > 0.0) {
                d = __dadd_rn(__dadd_rn(__ddiv_rn(m, dt), __ddiv_rn(rr, 2.0)), __ddiv_rn(__dmul_rn(k, dt), 4.0));
                cv = __dsub_rn(__dsub_rn(__ddiv_rn(m, dt), __ddiv_rn(rr, 2.0)), __ddiv_rn(__dmul_rn(k, dt), 4.0));
                w = 0.25;
            } else {
                d = __dadd_rn(rr, __ddiv_rn(__dmul_rn(k, dt), 2.0));
                cv = __ddiv_rn(__dmul_rn(-k, dt), 2.0);
                w = 0.0;
            }
            double *o = out + 4 * ns;
            o[0] = __ddiv_rn(1.0, d);
            o[1] = cv;
            o[2] = k;
            o[3] = w;
        }
        ns++;
    };
    for (int q = 0; q < ncounts; q++) {
        const wh_fit &fit = r.fits[cs[q]];
        const double n = (double)cn[q];
        if (fit.beta0 > 0.0) add(__ddiv_rn(1.0, fit.beta0), 0.0, 0.0, n);
        for (int b = 0; b < fit.n_branches; b++) add(fit.r[b], fit.m[b], fit.k[b], n);
    }
    return ns;
}

// Pass 1 (write = false): slot count per cell into cnt (0: not a boundary
// node).  Pass 2 (write = true): node index and slot offset from the scans.
__global__ void __launch_bounds__(256) grid_nodes(GbRoom r, const uint8_t *solid, const uint8_t *flags,
                                                   uint32_t *cnt, bool write, const uint32_t *node_at,
                                                   const unsigned long long *slot_at, uint32_t *bidx, uint32_t *bcell,
                                                   uint32_t *bstart, double *slots) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long cells = r.nx * r.ny * r.nz;
    if (i >= cells) return;
    const uint8_t fl = flags[i];
    if (!(fl & WAVEY_AIR) || (fl & 63) == 63) {
        if (!write) cnt[i] = 0;
        return;
    }
    if (write && cnt[i] == 0) return;
    const long long x = i % r.nx, y = (i / r.nx) % r.ny, z = i / (r.nx * r.ny);
    int faces[6];
    const int nf = gb_faces(r, solid, x, y, z, fl, faces);
    if (!write) {
        cnt[i] = (uint32_t)gb_slots(r, faces, nf, nullptr);
        return;
    }
    const uint32_t node = node_at[i];
    const unsigned long long s0 = slot_at[i];
    bidx[i] = node;
    bcell[node] = (uint32_t)i;
    bstart[node] = (uint32_t)s0;
    gb_slots(r, faces, nf, slots + 4 * s0);
}

// Exclusive scans over the cells of (cnt > 0) and cnt, in blocks of 1024:
// per-block totals, a scan of the totals, then each block's own scan.
constexpr int SCAN_BLOCK = 1024;

__global__ void __launch_bounds__(SCAN_BLOCK) scan_totals(const uint32_t *cnt, const uint8_t *flags, long long n,
                                                          unsigned long long *node_tot, unsigned long long *slot_tot,
                                                          unsigned long long *air_tot) {
    __shared__ unsigned long long sn[SCAN_BLOCK / 32], ss[SCAN_BLOCK / 32], sa[SCAN_BLOCK / 32];
    const long long i = (long long)blockIdx.x * SCAN_BLOCK + threadIdx.x;
    const uint32_t c = i < n ? cnt[i] : 0u;
    unsigned long long a = c > 0 ? 1 : 0, b = c, air = (i < n && (flags[i] & WAVEY_AIR)) ? 1 : 0;
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
        air += __shfl_down_sync(0xffffffffu, air, o);
    }
    if ((threadIdx.x & 31) == 0) {
        sn[threadIdx.x / 32] = a;
        ss[threadIdx.x / 32] = b;
        sa[threadIdx.x / 32] = air;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long ta = 0, tb = 0, tc = 0;
        for (int w = 0; w < SCAN_BLOCK / 32; w++) {
            ta += sn[w];
            tb += ss[w];
            tc += sa[w];
        }
        node_tot[blockIdx.x] = ta;
        slot_tot[blockIdx.x] = tb;
        air_tot[blockIdx.x] = tc;
    }
}

// One block: exclusive scan of the block totals in place (sequential chunks
// per thread, then a scan of the chunk sums); also writes the grand totals.
__global__ void __launch_bounds__(SCAN_BLOCK) scan_block_totals(unsigned long long *node_tot,
                                                                unsigned long long *slot_tot,
                                                                const unsigned long long *air_tot, long long nb,
                                                                unsigned long long *grand) {
    __shared__ unsigned long long cn[SCAN_BLOCK], cs[SCAN_BLOCK], ca[SCAN_BLOCK];
    const long long per = (nb + SCAN_BLOCK - 1) / SCAN_BLOCK;
    const long long a0 = (long long)threadIdx.x * per, a1 = min(a0 + per, nb);
    unsigned long long sa = 0, sb = 0, sc = 0;
    for (long long k = a0; k < a1; k++) {
        sa += node_tot[k];
        sb += slot_tot[k];
        sc += air_tot[k];
    }
    cn[threadIdx.x] = sa;
    cs[threadIdx.x] = sb;
    ca[threadIdx.x] = sc;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long ra = 0, rb = 0, rc = 0;
        for (int t = 0; t < SCAN_BLOCK; t++) {
            const unsigned long long va = cn[t], vb = cs[t];
            cn[t] = ra;
            cs[t] = rb;
            ra += va;
            rb += vb;
            rc += ca[t];
        }
        grand[0] = ra;
        grand[1] = rb;
        grand[2] = rc;
    }
    __syncthreads();
    unsigned long long ra = cn[threadIdx.x], rb = cs[threadIdx.x];
    for (long long k = a0; k < a1; k++) {
        const unsigned long long va = node_tot[k], vb = slot_tot[k];
        node_tot[k] = ra;
        slot_tot[k] = rb;
        ra += va;
        rb += vb;
    }
}

// Each block's own exclusive scan, offset by its block prefix.
__global__ void __launch_bounds__(SCAN_BLOCK) scan_apply(const uint32_t *cnt, long long n,
                                                         const unsigned long long *node_pre,
                                                         const unsigned long long *slot_pre, uint32_t *node_at,
                                                         unsigned long long *slot_at) {
    __shared__ unsigned long long wn[SCAN_BLOCK / 32], ws[SCAN_BLOCK / 32];
    const long long i = (long long)blockIdx.x * SCAN_BLOCK + threadIdx.x;
    const uint32_t c = i < n ? cnt[i] : 0u;
    const int lane = threadIdx.x & 31, warp = threadIdx.x / 32;
    unsigned long long a = c > 0 ? 1 : 0, b = c;  // inclusive warp scan
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long ua = __shfl_up_sync(0xffffffffu, a, o), ub = __shfl_up_sync(0xffffffffu, b, o);
        if (lane >= o) {
            a += ua;
            b += ub;
        }
    }
    if (lane == 31) {
        wn[warp] = a;
        ws[warp] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long ra = 0, rb = 0;
        for (int w = 0; w < SCAN_BLOCK / 32; w++) {
            const unsigned long long va = wn[w], vb = ws[w];
            wn[w] = ra;
            ws[w] = rb;
            ra += va;
            rb += vb;
        }
    }
    __syncthreads();
    if (i < n && c > 0) {
        node_at[i] = (uint32_t)(node_pre[blockIdx.x] + wn[warp] + a - 1);
        slot_at[i] = slot_pre[blockIdx.x] + ws[warp] + b - c;
    }
}

}  // namespace wk
