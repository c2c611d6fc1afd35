// grid_core.hpp -- the part of FdtdGrid::build_dx that does not depend on the
// room's shape, shared by the box-room builder (grid.cpp) and the mesh-room
// builder (mesh.cpp):
//   neighbour flags              wavey-solver/src/fdtd.rs:340-356
//   surfaces behind missing faces, one lookup per face (fdtd.rs:357-363)
//   boundary_slots               wavey-solver/src/fdtd.rs:539-571
//   node numbering in cell order wavey-solver/src/fdtd.rs:368-375
// Internal to libwavey_host.so.
#pragma once

#include <cmath>
#include <cstdint>
#include <new>
#include <vector>

#include "../../../include/wavey_host.h"
#include "../../../include/wavey_status.h"

struct wh_grid {
    int64_t n[3];
    double origin[3];
    double dx, dt;
    std::vector<uint8_t> flags;
    std::vector<uint32_t> bidx;
    std::vector<uint32_t> bcell, bstart;
    std::vector<double> slots;
    int64_t air = 0;

    int64_t index(int64_t x, int64_t y, int64_t z) const { return (z * n[1] + y) * n[0] + x; }
    void center(int64_t x, int64_t y, int64_t z, double out[3]) const {
        out[0] = origin[0] + (double)x * dx;
        out[1] = origin[1] + (double)y * dx;
        out[2] = origin[2] + (double)z * dx;
    }
    bool is_air(int64_t i) const { return flags[i] & WAVEY_AIR; }
};

namespace wavey_grid {

struct Slot {
    double inv_d, cv, k, w;
};

// The six neighbour directions in flag-bit order: -x, +x, -y, +y, -z, +z.
static const int DIRS[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};

inline bool fits_equal(const wh_fit &a, const wh_fit &b) {
    if (a.beta0 != b.beta0 || a.n_branches != b.n_branches || a.band_lo != b.band_lo || a.band_hi != b.band_hi ||
        a.rms_error != b.rms_error || a.max_error != b.max_error)
        return false;
    for (int i = 0; i < a.n_branches; i++)
        if (a.r[i] != b.r[i] || a.m[i] != b.m[i] || a.k[i] != b.k[i]) return false;
    return true;
}

// fdtd.rs:539-571: faces with the same fit share slots, admittance x count.
inline void boundary_slots(const int *faces, int nfaces, const wh_fit *fits, double dt, std::vector<Slot> &slots) {
    slots.clear();
    int cs[6], cn[6], ncounts = 0;
    for (int f = 0; f < nfaces; f++) {
        int s = faces[f], k = 0;
        while (k < ncounts && !fits_equal(fits[cs[k]], fits[s])) k++;
        if (k < ncounts)
            cn[k]++;
        else {
            cs[ncounts] = s;
            cn[ncounts] = 1;
            ncounts++;
        }
    }
    for (int q = 0; q < ncounts; q++) {
        const wh_fit &fit = fits[cs[q]];
        double n = (double)cn[q];
        auto add = [&](double r, double m, double k) {
            r = r / n;
            m = m / n;
            k = k / n;
            double d, cv, w;
            if (m > 0.0) {
                d = m / dt + r / 2.0 + k * dt / 4.0;
                cv = m / dt - r / 2.0 - k * dt / 4.0;
                w = 0.25;
            } else {
                d = r + k * dt / 2.0;
                cv = -k * dt / 2.0;
                w = 0.0;
            }
            slots.push_back({1.0 / d, cv, k, w});
        };
        if (fit.beta0 > 0.0) add(1.0 / fit.beta0, 0.0, 0.0);
        for (int b = 0; b < fit.n_branches; b++) add(fit.r[b], fit.m[b], fit.k[b]);
    }
}

// Allocates the grid's arrays for spacing dx over the bounds [lo, hi] with
// one solid layer of padding (fdtd.rs:290-306).  Returns a WAVEY_* status.
inline int alloc_grid(const double lo[3], const double hi[3], double c, double dx, wh_grid **out) {
    *out = nullptr;
    wh_grid *g = new (std::nothrow) wh_grid();
    if (!g) return WAVEY_E_NOMEM;
    g->dx = dx;
    g->dt = WAVEY_COURANT * dx / c;
    for (int a = 0; a < 3; a++) {
        g->origin[a] = lo[a] - dx * 0.5;
        g->n[a] = (int64_t)std::ceil((hi[a] - lo[a]) / dx) + 2;
    }
    const uint64_t cells = (uint64_t)g->n[0] * (uint64_t)g->n[1] * (uint64_t)g->n[2];
    if (cells > WAVEY_MAX_CELLS) {
        delete g;
        return WAVEY_E_LIMIT;
    }
    try {
        g->flags.assign(cells, 0);
        g->bidx.assign(cells, WAVEY_NO_BOUNDARY);
    } catch (...) {
        delete g;
        return WAVEY_E_NOMEM;
    }
    *out = g;
    return WAVEY_OK;
}

// Neighbour flags, faces, slots and node numbering from the air and solid
// classification.  surface_behind(p, k) gives the surface index behind the
// missing face k of the air cell centred at p (the reference's
// `room.bvh.intersect(p, dir, 0, 1.5 dx)`), or -1 when nothing is hit.
// On failure the grid is deleted.  Returns a WAVEY_* status.
template <class SurfaceBehind>
int finish_grid(wh_grid *g, const std::vector<uint8_t> &air, const std::vector<uint8_t> &solid, const wh_fit *fits,
                SurfaceBehind surface_behind) {
    const int64_t nx = g->n[0], ny = g->n[1], nz = g->n[2];
    // Neighbour flags per air cell, in parallel: each cell writes its own byte.
#pragma omp parallel for schedule(static)
    for (int64_t z = 1; z < nz - 1; z++)
        for (int64_t y = 1; y < ny - 1; y++)
            for (int64_t x = 1; x < nx - 1; x++) {
                int64_t i = g->index(x, y, z);
                if (!air[i]) continue;
                uint8_t fl = WAVEY_AIR;
                for (int k = 0; k < 6; k++)
                    if (air[g->index(x + DIRS[k][0], y + DIRS[k][1], z + DIRS[k][2])]) fl |= (uint8_t)(1u << k);
                g->flags[i] = fl;
            }
    // Surfaces behind the missing faces and the slots of each boundary node.
    // Planes are done in parallel, then concatenated in plane order, so
    // boundary nodes are numbered in cell order as in the reference.
    struct PlaneNodes {
        std::vector<uint32_t> cell, nslots;
        std::vector<double> slots;
        int64_t air = 0;
    };
    std::vector<PlaneNodes> planes(nz);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t z = 1; z < nz - 1; z++) {
        PlaneNodes &pn = planes[z];
        std::vector<Slot> sl;
        std::vector<int> flist;
        for (int64_t y = 1; y < ny - 1; y++)
            for (int64_t x = 1; x < nx - 1; x++) {
                int64_t i = g->index(x, y, z);
                if (!air[i]) continue;
                pn.air++;
                uint8_t fl = g->flags[i];
                if ((fl & 63) == 63) continue;
                double p[3];
                g->center(x, y, z, p);
                flist.clear();
                for (int k = 0; k < 6; k++) {
                    if (fl & (1u << k)) continue;
                    int64_t j = g->index(x + DIRS[k][0], y + DIRS[k][1], z + DIRS[k][2]);
                    if (solid[j]) continue;  // cabinet face: rigid, no branch
                    int s = surface_behind(p, k);
                    if (s >= 0) flist.push_back(s);
                }
                boundary_slots(flist.data(), (int)flist.size(), fits, g->dt, sl);
                if (!sl.empty()) {
                    pn.cell.push_back((uint32_t)i);
                    pn.nslots.push_back((uint32_t)sl.size());
                    for (const Slot &q : sl) {
                        pn.slots.push_back(q.inv_d);
                        pn.slots.push_back(q.cv);
                        pn.slots.push_back(q.k);
                        pn.slots.push_back(q.w);
                    }
                }
            }
    }
    size_t n_nodes = 0, n_vals = 0;
    for (const PlaneNodes &pn : planes) {
        n_nodes += pn.cell.size();
        n_vals += pn.slots.size();
    }
    if (n_nodes >= (size_t)WAVEY_NO_BOUNDARY) {
        delete g;
        return WAVEY_E_LIMIT;
    }
    try {
        g->bcell.reserve(n_nodes);
        g->bstart.reserve(n_nodes + 1);
        g->slots.reserve(n_vals);
    } catch (...) {
        delete g;
        return WAVEY_E_NOMEM;
    }
    for (PlaneNodes &pn : planes) {
        g->air += pn.air;
        size_t v = 0;
        for (size_t k = 0; k < pn.cell.size(); k++) {
            g->bidx[pn.cell[k]] = (uint32_t)g->bcell.size();
            g->bcell.push_back(pn.cell[k]);
            g->bstart.push_back((uint32_t)(g->slots.size() / 4));
            g->slots.insert(g->slots.end(), pn.slots.begin() + v, pn.slots.begin() + v + 4 * pn.nslots[k]);
            v += 4 * pn.nslots[k];
        }
        PlaneNodes().cell.swap(pn.cell);
        std::vector<double>().swap(pn.slots);
    }
    g->bstart.push_back((uint32_t)(g->slots.size() / 4));
    return WAVEY_OK;
}

}  // namespace wavey_grid
