// grid.cpp -- voxelised box rooms, boundary slots and source/receiver nodes.
//
// Restates for box-shaped rooms:
//   FdtdGrid::build_dx       wavey-solver/src/fdtd.rs:289-378
//   build_with spacing rule  wavey-solver/src/fdtd.rs:282-286
//   boundary_slots           wavey-solver/src/fdtd.rs:539-571
//   nearest_air              wavey-solver/src/fdtd.rs:245-272
//   taps_at                  wavey-solver/src/fdtd.rs:467-492
//   baffle_point / air_along wavey-solver/src/fdtd.rs:497-534
//   source_components        wavey-solver/src/fdtd.rs:730-743
//   Room::contains (prism)   wavey-geom/src/room.rs:151-157 with the even-odd
//                            polygon test of wavey-geom/src/regions.rs:237-249
//                            (a rectangle then holds [x0, x1) x [y0, y1))
//
// The face lookup `room.bvh.intersect(center, dir, 0, 1.5 dx)` is restated
// analytically: every room surface here is an axis-aligned rectangle, so the
// surface behind a missing face is the nearest rectangle crossed by the axis
// ray with 0 < t < 1.5 dx.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "grid_core.hpp"

namespace {

struct Rect {
    int axis;       // plane normal axis
    double c;       // plane coordinate
    double lo[3];   // closed extent on the other two axes (the normal axis entry is unused)
    double hi[3];
};

// Surfaces in build_room order (see wavey_host.h).
std::vector<Rect> room_rects(const wh_room *r) {
    std::vector<Rect> s;
    auto add = [&](int axis, double c, double x0, double y0, double z0, double x1, double y1, double z1) {
        Rect q{axis, c, {x0, y0, z0}, {x1, y1, z1}};
        s.push_back(q);
    };
    const double h = r->height;
    add(2, 0.0, r->x0, r->y0, 0, r->x1, r->y1, 0);   // floor
    add(2, h, r->x0, r->y0, 0, r->x1, r->y1, 0);     // ceiling
    add(1, r->y0, r->x0, 0, 0.0, r->x1, 0, h);       // wall y = y0
    add(0, r->x1, 0, r->y0, 0.0, 0, r->y1, h);       // wall x = x1
    add(1, r->y1, r->x0, 0, 0.0, r->x1, 0, h);       // wall y = y1
    add(0, r->x0, 0, r->y0, 0.0, 0, r->y1, h);       // wall x = x0
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

inline bool in_box(const double *b, const double p[3]) {
    return p[0] >= b[0] && p[1] >= b[1] && p[2] >= b[2] && p[0] <= b[3] && p[1] <= b[4] && p[2] <= b[5];
}

inline bool in_rect_half_open(double x0, double y0, double x1, double y1, double x, double y) {
    return x >= x0 && x < x1 && y >= y0 && y < y1;
}

bool prism_contains(const wh_room *r, const double p[3]) {
    if (!(p[2] > 0.0 && p[2] < r->height)) return false;
    if (!in_rect_half_open(r->x0, r->y0, r->x1, r->y1, p[0], p[1])) return false;
    for (int i = 0; i < r->n_pillars; i++) {
        const double *q = r->pillars + 4 * i;
        if (in_rect_half_open(q[0], q[1], q[2], q[3], p[0], p[1])) return false;
    }
    return true;
}

bool room_contains(const wh_room *r, const double p[3]) {
    if (!prism_contains(r, p)) return false;
    for (int i = 0; i < r->n_blocks; i++)
        if (in_box(r->blocks + 6 * i, p)) return false;
    return true;
}

}  // namespace

extern "C" int32_t wh_room_surface_count(const wh_room *room) {
    return 6 + 4 * room->n_pillars + 6 * room->n_blocks;
}

extern "C" int wh_room_contains(const wh_room *room, const double p[3]) { return room_contains(room, p) ? 1 : 0; }

extern "C" double wh_grid_spacing(const wh_room *room, double c, double f_max, double ppw) {
    double cab = INFINITY;
    for (int i = 0; i < room->n_solids; i++) {
        const double *s = room->solids + 6 * i;
        double m = std::min(std::min(s[3] - s[0], s[4] - s[1]), s[5] - s[2]);
        cab = std::min(cab, m / 8.0);
    }
    return std::min(c / (f_max * ppw), cab);
}

extern "C" int wh_grid_build(const wh_room *room, const wh_fit *fits, int32_t n_fits, double c, double dx, wh_grid **out) {
    if (!room || !out || !(dx > 0.0) || !(c > 0.0) || !(room->height > 0.0) || room->x1 <= room->x0 || room->y1 <= room->y0)
        return WAVEY_E_INVALID;
    const std::vector<Rect> rects = room_rects(room);
    if ((int)rects.size() != n_fits || !fits) return WAVEY_E_INVALID;
    *out = nullptr;
    // Bounds: the plan rectangle from z = 0 to the ceiling (room.rs:185-190).
    const double lo[3] = {room->x0, room->y0, 0.0}, hi[3] = {room->x1, room->y1, room->height};
    wh_grid *g = nullptr;
    int st = wavey_grid::alloc_grid(lo, hi, c, dx, &g);
    if (st != WAVEY_OK) return st;
    const int64_t nx = g->n[0], ny = g->n[1], nz = g->n[2];
    const size_t cells = g->flags.size();
    // Solid (cabinet) and air classification, fdtd.rs:308-337.
    std::vector<uint8_t> solid(cells, 0), air(cells, 0);
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < nz; z++)
        for (int64_t y = 0; y < ny; y++)
            for (int64_t x = 0; x < nx; x++) {
                int64_t i = g->index(x, y, z);
                double p[3];
                g->center(x, y, z, p);
                bool s = false;
                for (int k = 0; k < room->n_solids && !s; k++) s = in_box(room->solids + 6 * k, p);
                solid[i] = s;
                air[i] = !s && x > 0 && y > 0 && z > 0 && x < nx - 1 && y < ny - 1 && z < nz - 1 && room_contains(room, p);
            }
    // The surface behind a missing face: the nearest rectangle crossed by the
    // axis ray with 0 < t < 1.5 dx.
    const double reach = dx * 1.5;
    const int nrect = (int)rects.size();
    auto behind = [&](const double p[3], int k) -> int {
        int axis = k / 2;
        double sgn = (k & 1) ? 1.0 : -1.0;
        int best = -1;
        double tbest = reach;
        for (int q = 0; q < nrect; q++) {
            const Rect &r = rects[q];
            if (r.axis != axis) continue;
            double t = (r.c - p[axis]) * sgn;
            if (!(t > 0.0 && t < tbest)) continue;
            bool inside = true;
            for (int a = 0; a < 3 && inside; a++)
                if (a != axis) inside = p[a] >= r.lo[a] && p[a] <= r.hi[a];
            if (!inside) continue;
            best = q;
            tbest = t;
        }
        return best;
    };
    st = wavey_grid::finish_grid(g, air, solid, fits, behind);
    if (st != WAVEY_OK) return st;
    *out = g;
    return WAVEY_OK;
}

extern "C" void wh_grid_view_of(const wh_grid *g, wh_grid_view *v) {
    v->nx = g->n[0];
    v->ny = g->n[1];
    v->nz = g->n[2];
    for (int a = 0; a < 3; a++) v->origin[a] = g->origin[a];
    v->dx = g->dx;
    v->dt = g->dt;
    v->flags = g->flags.data();
    v->bidx = g->bidx.data();
    v->n_boundary = (int64_t)g->bcell.size();
    v->bcell = g->bcell.data();
    v->bstart = g->bstart.data();
    v->slots = g->slots.data();
    v->n_slots = (int64_t)(g->slots.size() / 4);
    v->air_cells = g->air;
}

extern "C" void wh_grid_free(wh_grid *g) { delete g; }

extern "C" int wh_grid_alloc(const int64_t n[3], const double origin[3], double dx, double dt, int64_t air_cells,
                             int64_t n_boundary, int64_t n_slots, wh_grid **out) {
    if (!n || !origin || !out || n[0] < 3 || n[1] < 3 || n[2] < 3 || n_boundary < 0 || n_slots < 0 ||
        n_boundary >= (int64_t)WAVEY_NO_BOUNDARY)
        return WAVEY_E_INVALID;
    const uint64_t cells = (uint64_t)n[0] * (uint64_t)n[1] * (uint64_t)n[2];
    if (cells > WAVEY_MAX_CELLS) return WAVEY_E_LIMIT;
    *out = nullptr;
    wh_grid *g = new (std::nothrow) wh_grid();
    if (!g) return WAVEY_E_NOMEM;
    for (int a = 0; a < 3; a++) {
        g->n[a] = n[a];
        g->origin[a] = origin[a];
    }
    g->dx = dx;
    g->dt = dt;
    g->air = air_cells;
    try {
        g->flags.assign(cells, 0);
        g->bidx.assign(cells, WAVEY_NO_BOUNDARY);
        g->bcell.assign((size_t)n_boundary, 0);
        g->bstart.assign((size_t)n_boundary + 1, 0);
        g->slots.assign((size_t)n_slots * 4, 0.0);
    } catch (...) {
        delete g;
        return WAVEY_E_NOMEM;
    }
    *out = g;
    return WAVEY_OK;
}

extern "C" void wh_grid_arrays(wh_grid *g, uint8_t **flags, uint32_t **bidx, uint32_t **bcell, uint32_t **bstart,
                               double **slots) {
    *flags = g->flags.data();
    *bidx = g->bidx.data();
    *bcell = g->bcell.data();
    *bstart = g->bstart.data();
    *slots = g->slots.data();
}

extern "C" int64_t wh_nearest_air(const wh_grid *g, const double p[3]) {
    int64_t c[3];
    for (int a = 0; a < 3; a++) c[a] = (int64_t)std::round((p[a] - g->origin[a]) / g->dx);
    for (int64_t r = 0; r < 17; r++) {
        bool have = false;
        double bd = 0.0;
        int64_t bi = -1;
        for (int64_t dz = -r; dz <= r; dz++)
            for (int64_t dy = -r; dy <= r; dy++)
                for (int64_t dx = -r; dx <= r; dx++) {
                    int64_t x = c[0] + dx, y = c[1] + dy, z = c[2] + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= g->n[0] || y >= g->n[1] || z >= g->n[2]) continue;
                    int64_t i = g->index(x, y, z);
                    if (!g->is_air(i)) continue;
                    double q[3];
                    g->center(x, y, z, q);
                    double ex = q[0] - p[0], ey = q[1] - p[1], ez = q[2] - p[2];
                    double d = ex * ex + ey * ey + ez * ez;
                    if (!have || d < bd) {
                        have = true;
                        bd = d;
                        bi = i;
                    }
                }
        if (have) return bi;
    }
    return -1;
}

extern "C" int32_t wh_taps_at(const wh_grid *g, const double p[3], int64_t cells[8], double weights[8]) {
    double q[3], f[3], b[3];
    for (int a = 0; a < 3; a++) {
        q[a] = (p[a] - g->origin[a]) / g->dx;
        b[a] = std::floor(q[a]);
        f[a] = q[a] - b[a];
    }
    int n = 0;
    for (int dx = 0; dx < 2; dx++) {
        double wx = dx ? f[0] : 1.0 - f[0];
        for (int dy = 0; dy < 2; dy++) {
            double wy = dy ? f[1] : 1.0 - f[1];
            for (int dz = 0; dz < 2; dz++) {
                double wz = dz ? f[2] : 1.0 - f[2];
                int64_t x = (int64_t)b[0] + dx, y = (int64_t)b[1] + dy, z = (int64_t)b[2] + dz;
                if (x < 0 || y < 0 || z < 0 || x >= g->n[0] || y >= g->n[1] || z >= g->n[2]) continue;
                int64_t i = g->index(x, y, z);
                double w = wx * wy * wz;
                if (g->is_air(i) && w > 1e-9) {
                    cells[n] = i;
                    weights[n] = w;
                    n++;
                }
            }
        }
    }
    double sum = -0.0;
    for (int k = 0; k < n; k++) sum += weights[k];
    if (sum < 0.25) {
        int64_t i = wh_nearest_air(g, p);
        if (i < 0) return -1;
        cells[0] = i;
        weights[0] = 1.0;
        return 1;
    }
    for (int k = 0; k < n; k++) weights[k] = weights[k] / sum;
    return n;
}

extern "C" int32_t wh_source_components(const wh_grid *g, int64_t c, int32_t order, int64_t comp_cells[4][2],
                                        double comp_w[4][2], int32_t comp_n[4]) {
    const int64_t cells = g->n[0] * g->n[1] * g->n[2];
    if (c < 0 || c >= cells) return -1;
    comp_cells[0][0] = c;
    comp_w[0][0] = 1.0;
    comp_n[0] = 1;
    if (order < 1) return 1;
    const int64_t steps[3] = {1, g->n[0], g->n[0] * g->n[1]};
    for (int s = 0; s < 3; s++) {
        int64_t plus = c + steps[s], minus = c - steps[s];
        if (minus < 0) return -1;
        if (plus >= cells || !g->is_air(plus) || !g->is_air(minus)) return -1;
        comp_cells[1 + s][0] = plus;
        comp_w[1 + s][0] = 1.0;
        comp_cells[1 + s][1] = minus;
        comp_w[1 + s][1] = -1.0;
        comp_n[1 + s] = 2;
    }
    return 4;
}

extern "C" void wh_baffle_point(const wh_grid *g, const double p[3], const double axis[3], double out[3]) {
    const double step = g->dx * 0.05;
    const int64_t count = (int64_t)(2.0 / step);
    for (int64_t k = 0; k < count; k++) {
        double q[3], r[3];
        for (int a = 0; a < 3; a++) q[a] = p[a] + axis[a] * ((double)k * step);
        bool neg = false;
        for (int a = 0; a < 3; a++) {
            r[a] = std::round((q[a] - g->origin[a]) / g->dx);
            neg = neg || r[a] < 0.0;
        }
        if (neg) continue;
        int64_t x = (int64_t)r[0], y = (int64_t)r[1], z = (int64_t)r[2];
        if (x < g->n[0] && y < g->n[1] && z < g->n[2] && g->is_air(g->index(x, y, z))) {
            double back = std::min(g->dx * 0.5, (double)k * step);
            for (int a = 0; a < 3; a++) out[a] = q[a] - axis[a] * back;
            return;
        }
    }
    for (int a = 0; a < 3; a++) out[a] = p[a];
}

extern "C" int64_t wh_air_along(const wh_grid *g, const double p[3], const double axis[3]) {
    const double step = g->dx * 0.5;
    const int64_t count = (int64_t)(2.0 / step);
    for (int64_t k = 0; k < count; k++) {
        double r[3];
        for (int a = 0; a < 3; a++) r[a] = std::round((p[a] + axis[a] * ((double)k * step) - g->origin[a]) / g->dx);
        if (r[0] < 0.0 || r[1] < 0.0 || r[2] < 0.0) continue;
        int64_t x = (int64_t)r[0], y = (int64_t)r[1], z = (int64_t)r[2];
        if (x < g->n[0] && y < g->n[1] && z < g->n[2]) {
            int64_t i = g->index(x, y, z);
            if (g->is_air(i)) return i;
        }
    }
    return wh_nearest_air(g, p);
}
