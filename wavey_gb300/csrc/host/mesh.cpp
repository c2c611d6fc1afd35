// mesh.cpp -- rooms from polygon meshes (imported OBJ rooms) and their
// voxelisation for the FDTD grid.
//
// Restates:
//   room_from_mesh             wavey-geom/src/room.rs:399-461 (surfaces per
//                              material group and plane, normals into the room)
//   Builder::tri               wavey-geom/src/room.rs:235-249
//   parity_inside / contains   wavey-geom/src/room.rs:151-157, 355-367
//   ray_triangle_edges         wavey-geom/src/bvh.rs:238-259 (two-sided
//                              Moeller-Trumbore, the same operations in the
//                              same order, so hit parameters agree bit for bit)
//   Bvh::intersect / all_hits  wavey-geom/src/bvh.rs:64-88
//   column_fill                wavey-solver/src/fdtd.rs:385-422
//   FdtdGrid::build_dx         wavey-solver/src/fdtd.rs:289-378 (mesh branch)
//
// Differences that do not change a grid: polygons with more than three
// vertices are cut into triangles by ear clipping here (the reference uses the
// earcut crate), so the diagonals inside a polygon may differ; a ray that
// crosses a polygon hits exactly one of its triangles either way (or two at
// the same parameter on a shared diagonal, which column_fill counts once and
// the face lookup resolves to the same surface).  Ray queries run over
// per-axis bins of triangles instead of a BVH: every triangle the ray can hit
// is tested, in triangle order, so the closest hit is the same; among hits at
// exactly the same parameter the first triangle wins (the reference's BVH
// visit order decides there).
#include <algorithm>
#include <array>
#include <cmath>
#include <new>
#include <vector>

#include "grid_core.hpp"

namespace {

struct V3 {
    double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline double comp(const V3 &a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
// glam's DVec3 operations, term for term.
inline double dot(V3 a, V3 b) { return (a.x * b.x) + (a.y * b.y) + (a.z * b.z); }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
inline double length(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 normalize(V3 a) { return a * (1.0 / length(a)); }
inline V3 vmin(V3 a, V3 b) { return {std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)}; }
inline V3 vmax(V3 a, V3 b) { return {std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)}; }

// bvh.rs:238-259.  e = [v0, v1 - v0, v2 - v0].
inline bool ray_triangle(const V3 &o, const V3 &d, const std::array<V3, 3> &e, double *t) {
    const V3 p = cross(d, e[2]);
    const double det = dot(e[1], p);
    if (std::fabs(det) < 1e-14) return false;
    const double inv = 1.0 / det;
    const V3 s = o - e[0];
    const double u = dot(s, p) * inv;
    if (!(u >= -1e-10 && u <= 1.0 + 1e-10)) return false;
    const V3 q = cross(s, e[1]);
    const double v = dot(d, q) * inv;
    if (v < -1e-10 || u + v > 1.0 + 1e-10) return false;
    *t = dot(e[2], q) * inv;
    return true;
}

std::vector<std::array<V3, 3>> edges_of(const std::vector<V3> &pos) {
    std::vector<std::array<V3, 3>> e(pos.size() / 3);
    for (size_t i = 0; i < e.size(); i++) {
        const V3 a = pos[3 * i], b = pos[3 * i + 1], c = pos[3 * i + 2];
        e[i] = {a, b - a, c - a};
    }
    return e;
}

// Number of hits along o + t d with t_min < t (every triangle counts, as in
// Bvh::all_hits over coincident triangles).
size_t count_hits(const std::vector<std::array<V3, 3>> &edges, V3 o, V3 d, double t_min) {
    size_t n = 0;
    for (const auto &e : edges) {
        double t;
        if (ray_triangle(o, d, e, &t) && t > t_min) n++;
    }
    return n;
}

// room.rs:355-367: inside when at least two of three skew rays cross the
// surface an odd number of times.
bool parity_inside(const std::vector<std::array<V3, 3>> &edges, V3 p) {
    static const double DIRS[3][3] = {
        {0.5772156649, 0.6180339887, 0.5338319},
        {-0.6931471806, 0.4142135624, -0.3010299957},
        {0.2360679775, -0.7320508076, 0.6457513111},
    };
    int odd = 0;
    for (const auto &d : DIRS) {
        const V3 dir = normalize(V3{d[0], d[1], d[2]});
        if (count_hits(edges, p, dir, 1e-9) % 2 == 1) odd++;
    }
    return odd >= 2;
}

// Newell normal of a polygon (room.rs:377-381).
V3 newell(const std::vector<V3> &poly) {
    V3 n{0.0, 0.0, 0.0};
    for (size_t i = 0; i < poly.size(); i++) {
        const V3 a = poly[i], b = poly[(i + 1) % poly.size()];
        n = n + V3{(a.y - b.y) * (a.z + b.z), (a.z - b.z) * (a.x + b.x), (a.x - b.x) * (a.y + b.y)};
    }
    return n;
}

// Triangles of a planar polygon, keeping its winding (room.rs:371-397): ear
// clipping in the plane of the dominant normal axis.
std::vector<std::array<V3, 3>> triangulate(const std::vector<V3> &poly) {
    std::vector<std::array<V3, 3>> out;
    if (poly.size() < 3) return out;
    if (poly.size() == 3) {
        out.push_back({poly[0], poly[1], poly[2]});
        return out;
    }
    const V3 nn = newell(poly);
    const double len = length(nn);
    if (!(len > 0.0)) return out;
    const V3 n = nn * (1.0 / len);
    // 2-D coordinates with the polygon counter-clockwise about +n.
    const double ax = std::fabs(n.x), ay = std::fabs(n.y), az = std::fabs(n.z);
    const int drop = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
    const int u = (drop + 1) % 3, v = (drop + 2) % 3;
    const double sgn = comp(n, drop) >= 0.0 ? 1.0 : -1.0;
    std::vector<double> px(poly.size()), py(poly.size());
    for (size_t i = 0; i < poly.size(); i++) {
        px[i] = comp(poly[i], u);
        py[i] = comp(poly[i], v) * sgn;
    }
    std::vector<int> idx(poly.size());
    for (size_t i = 0; i < idx.size(); i++) idx[i] = (int)i;
    auto cross2 = [&](int a, int b, int c) {
        return (px[b] - px[a]) * (py[c] - py[a]) - (py[b] - py[a]) * (px[c] - px[a]);
    };
    auto inside = [&](int a, int b, int c, int p) {
        return cross2(a, b, p) >= 0.0 && cross2(b, c, p) >= 0.0 && cross2(c, a, p) >= 0.0;
    };
    while (idx.size() > 3) {
        const size_t m = idx.size();
        size_t ear = m;
        double best = -INFINITY;
        size_t fallback = 0;
        for (size_t k = 0; k < m && ear == m; k++) {
            const int a = idx[(k + m - 1) % m], b = idx[k], c = idx[(k + 1) % m];
            const double cr = cross2(a, b, c);
            if (cr > best) {
                best = cr;
                fallback = k;
            }
            if (cr <= 0.0) continue;
            bool empty = true;
            for (size_t j = 0; j < m && empty; j++) {
                const int q = idx[j];
                if (q == a || q == b || q == c) continue;
                if (inside(a, b, c, q)) empty = false;
            }
            if (empty) ear = k;
        }
        if (ear == m) ear = fallback;  // degenerate remainder: clip the most convex corner
        const int a = idx[(ear + m - 1) % m], b = idx[ear], c = idx[(ear + 1) % m];
        out.push_back({poly[a], poly[b], poly[c]});
        idx.erase(idx.begin() + (ptrdiff_t)ear);
    }
    out.push_back({poly[idx[0]], poly[idx[1]], poly[idx[2]]});
    for (auto &t : out)
        if (dot(cross(t[1] - t[0], t[2] - t[0]), n) < 0.0) std::swap(t[1], t[2]);
    return out;
}

// Triangles binned by their extent across one axis, for rays along that axis.
struct AxisBins {
    int axis = 0, u = 1, v = 2;
    double u0 = 0, v0 = 0, h = 1;
    int64_t nu = 1, nv = 1;
    std::vector<std::vector<uint32_t>> cells;

    void build(const std::vector<V3> &pos, int ax, V3 lo, V3 hi, double size) {
        axis = ax;
        u = (ax + 1) % 3;
        v = (ax + 2) % 3;
        const double pad = 1e-6 * (1.0 + length(hi - lo));
        u0 = comp(lo, u) - 2.0 * pad;
        v0 = comp(lo, v) - 2.0 * pad;
        const double eu = comp(hi, u) - comp(lo, u) + 4.0 * pad, ev = comp(hi, v) - comp(lo, v) + 4.0 * pad;
        h = std::max(size, std::max(eu, ev) / 4096.0);
        nu = std::max<int64_t>(1, (int64_t)std::ceil(eu / h));
        nv = std::max<int64_t>(1, (int64_t)std::ceil(ev / h));
        cells.assign((size_t)(nu * nv), {});
        for (size_t t = 0; t < pos.size() / 3; t++) {
            double a0 = INFINITY, a1 = -INFINITY, b0 = INFINITY, b1 = -INFINITY;
            for (int k = 0; k < 3; k++) {
                a0 = std::min(a0, comp(pos[3 * t + k], u));
                a1 = std::max(a1, comp(pos[3 * t + k], u));
                b0 = std::min(b0, comp(pos[3 * t + k], v));
                b1 = std::max(b1, comp(pos[3 * t + k], v));
            }
            const int64_t i0 = clampu(a0 - pad), i1 = clampu(a1 + pad);
            const int64_t j0 = clampv(b0 - pad), j1 = clampv(b1 + pad);
            for (int64_t j = j0; j <= j1; j++)
                for (int64_t i = i0; i <= i1; i++) cells[(size_t)(j * nu + i)].push_back((uint32_t)t);
        }
    }
    int64_t clampu(double a) const { return std::min(nu - 1, std::max<int64_t>(0, (int64_t)std::floor((a - u0) / h))); }
    int64_t clampv(double b) const { return std::min(nv - 1, std::max<int64_t>(0, (int64_t)std::floor((b - v0) / h))); }
    // Triangles a ray along the axis through p may hit (in triangle order).
    const std::vector<uint32_t> *at(const V3 &p) const {
        const double a = comp(p, u), b = comp(p, v);
        if (a < u0 || b < v0) return nullptr;
        const int64_t i = (int64_t)std::floor((a - u0) / h), j = (int64_t)std::floor((b - v0) / h);
        if (i >= nu || j >= nv) return nullptr;
        return &cells[(size_t)(j * nu + i)];
    }
};

}  // namespace

struct wh_mesh_room {
    std::vector<V3> pos;               // three per triangle, winding matching its surface's normal
    std::vector<uint32_t> tri_surface;  // surface of each triangle
    struct Surface {
        int32_t group;
        V3 normal;
        double d, area;
        int32_t kind;  // 0 wall, 1 floor, 2 ceiling
    };
    std::vector<Surface> surfaces;
    std::vector<std::array<V3, 3>> edges;
    V3 lo{0, 0, 0}, hi{0, 0, 0};
};

extern "C" int wh_mesh_room_build(const double *verts, int64_t n_verts, const uint32_t *face_verts,
                                  const int64_t *face_start, const int32_t *face_group, int64_t n_faces,
                                  wh_mesh_room **out) {
    if (!out || n_verts < 0 || n_faces < 0 || (n_verts > 0 && !verts) || (n_faces > 0 && (!face_start || !face_group)))
        return WAVEY_E_INVALID;
    *out = nullptr;
    // Triangles of every polygon with their group (room.rs:403-411).
    std::vector<std::array<V3, 3>> tris;
    std::vector<int32_t> groups;
    try {
        for (int64_t f = 0; f < n_faces; f++) {
            const int64_t a = face_start[f], b = face_start[f + 1];
            if (a < 0 || b < a || (b > a && !face_verts)) return WAVEY_E_INVALID;
            std::vector<V3> poly;
            for (int64_t k = a; k < b; k++) {
                const uint32_t i = face_verts[k];
                if ((int64_t)i >= n_verts) return WAVEY_E_INVALID;
                poly.push_back({verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]});
            }
            for (const auto &t : triangulate(poly))
                if (length(cross(t[1] - t[0], t[2] - t[0])) > 1e-12) {
                    tris.push_back(t);
                    groups.push_back(face_group[f]);
                }
        }
    } catch (...) {
        return WAVEY_E_NOMEM;
    }
    if (tris.empty()) return WAVEY_E_INVALID;
    wh_mesh_room *r = new (std::nothrow) wh_mesh_room();
    if (!r) return WAVEY_E_NOMEM;
    try {
        std::vector<V3> flat;
        for (const auto &t : tris) flat.insert(flat.end(), t.begin(), t.end());
        const std::vector<std::array<V3, 3>> probe = edges_of(flat);
        V3 lo{INFINITY, INFINITY, INFINITY}, hi{-INFINITY, -INFINITY, -INFINITY};
        for (const V3 &p : flat) {
            lo = vmin(lo, p);
            hi = vmax(hi, p);
        }
        const double eps = length(hi - lo) * 1e-5;
        // Surface per (group, plane); normals into the room (room.rs:418-447).
        struct Plane {
            int32_t group;
            V3 n;
            double d;
            size_t s;
        };
        std::vector<Plane> planes;
        for (size_t k = 0; k < tris.size(); k++) {
            const auto &t = tris[k];
            const int32_t g = groups[k];
            // Centroid as (t0 + t1 + t2) / 3.0, divided, not multiplied by 1/3.
            const V3 cc{((t[0].x + t[1].x) + t[2].x) / 3.0, ((t[0].y + t[1].y) + t[2].y) / 3.0,
                        ((t[0].z + t[1].z) + t[2].z) / 3.0};
            V3 n = normalize(cross(t[1] - t[0], t[2] - t[0]));
            if (!parity_inside(probe, cc + n * eps)) n = -n;
            const double d = dot(n, cc);
            size_t s = (size_t)-1;
            for (const Plane &pl : planes)
                if (pl.group == g && dot(pl.n, n) > 1.0 - 1e-6 && std::fabs(pl.d - d) < 1e-4) {
                    s = pl.s;
                    break;
                }
            if (s == (size_t)-1) {
                const int32_t kind = n.z > 0.7 ? 1 : (n.z < -0.7 ? 2 : 0);
                r->surfaces.push_back({g, n, dot(n, cc), 0.0, kind});
                s = r->surfaces.size() - 1;
                planes.push_back({g, n, d, s});
            }
            // Builder::tri: drop slivers, wind to match the surface normal.
            V3 a = t[0], b = t[1], c2 = t[2];
            const V3 nn = cross(b - a, c2 - a);
            const double area = length(nn) * 0.5;
            if (area < 1e-12) continue;
            if (dot(nn, r->surfaces[s].normal) < 0.0) std::swap(b, c2);
            r->pos.push_back(a);
            r->pos.push_back(b);
            r->pos.push_back(c2);
            r->surfaces[s].area += area;
            r->tri_surface.push_back((uint32_t)s);
        }
        r->edges = edges_of(r->pos);
        r->lo = {INFINITY, INFINITY, INFINITY};
        r->hi = {-INFINITY, -INFINITY, -INFINITY};
        for (const V3 &p : r->pos) {
            r->lo = vmin(r->lo, p);
            r->hi = vmax(r->hi, p);
        }
    } catch (...) {
        delete r;
        return WAVEY_E_NOMEM;
    }
    *out = r;
    return WAVEY_OK;
}

extern "C" void wh_mesh_room_free(wh_mesh_room *room) { delete room; }

extern "C" int32_t wh_mesh_room_surface_count(const wh_mesh_room *room) { return (int32_t)room->surfaces.size(); }

extern "C" int64_t wh_mesh_room_triangle_count(const wh_mesh_room *room) { return (int64_t)room->tri_surface.size(); }

extern "C" void wh_mesh_room_surface(const wh_mesh_room *room, int32_t s, int32_t *group, int32_t *kind,
                                     double normal[3], double *d, double *area) {
    const auto &q = room->surfaces[(size_t)s];
    if (group) *group = q.group;
    if (kind) *kind = q.kind;
    if (normal) {
        normal[0] = q.normal.x;
        normal[1] = q.normal.y;
        normal[2] = q.normal.z;
    }
    if (d) *d = q.d;
    if (area) *area = q.area;
}

extern "C" void wh_mesh_room_triangles(const wh_mesh_room *room, double *positions, uint32_t *tri_surface) {
    for (size_t i = 0; i < room->pos.size(); i++) {
        positions[3 * i] = room->pos[i].x;
        positions[3 * i + 1] = room->pos[i].y;
        positions[3 * i + 2] = room->pos[i].z;
    }
    std::copy(room->tri_surface.begin(), room->tri_surface.end(), tri_surface);
}

extern "C" void wh_mesh_room_bounds(const wh_mesh_room *room, double lo[3], double hi[3]) {
    lo[0] = room->lo.x;
    lo[1] = room->lo.y;
    lo[2] = room->lo.z;
    hi[0] = room->hi.x;
    hi[1] = room->hi.y;
    hi[2] = room->hi.z;
}

extern "C" int wh_mesh_room_contains(const wh_mesh_room *room, const double p[3]) {
    return parity_inside(room->edges, V3{p[0], p[1], p[2]}) ? 1 : 0;
}

// room.rs:165-178: divergence theorem with inward normals.
extern "C" double wh_mesh_room_volume(const wh_mesh_room *room) {
    double s = 0.0;
    for (size_t t = 0; t < room->pos.size() / 3; t++) {
        const V3 a = room->pos[3 * t], b = room->pos[3 * t + 1], c = room->pos[3 * t + 2];
        s += dot(a, cross(b - a, c - a)) / 6.0;
    }
    return -s;
}

extern "C" int wh_grid_build_mesh(const wh_mesh_room *room, const double *solids, int32_t n_solids, const wh_fit *fits,
                                  int32_t n_fits, double c, double dx, wh_grid **out) {
    if (!room || !out || !(dx > 0.0) || !(c > 0.0) || n_solids < 0 || (n_solids > 0 && !solids) || !fits ||
        n_fits != (int32_t)room->surfaces.size())
        return WAVEY_E_INVALID;
    *out = nullptr;
    const double lo[3] = {room->lo.x, room->lo.y, room->lo.z}, hi[3] = {room->hi.x, room->hi.y, room->hi.z};
    wh_grid *g = nullptr;
    int st = wavey_grid::alloc_grid(lo, hi, c, dx, &g);
    if (st != WAVEY_OK) return st;
    const int64_t nx = g->n[0], ny = g->n[1], nz = g->n[2];
    const size_t cells = g->flags.size();
    std::vector<uint8_t> solid, inside, air;
    AxisBins bins[3];
    try {
        solid.assign(cells, 0);
        inside.assign(cells, 0);
        air.assign(cells, 0);
        for (int a = 0; a < 3; a++) bins[a].build(room->pos, a, room->lo, room->hi, 4.0 * dx);
    } catch (...) {
        delete g;
        return WAVEY_E_NOMEM;
    }
    // column_fill (fdtd.rs:385-422): one upward ray per (x, y) column,
    // moved off the cell centres; crossings of one surface side at the same
    // height count once.
    const V3 off{0.0001372 * dx, 0.0002918 * dx, 0.0};
    const double start = g->origin[2] - dx;
    const V3 up_dir{0.0, 0.0, 1.0};
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t col = 0; col < nx * ny; col++) {
        const int64_t x = col % nx, y = col / nx;
        double cen[3];
        g->center(x, y, 0, cen);
        const V3 o = V3{cen[0], cen[1], start} + off;
        struct Crossing {
            double t;
            bool up;
        };
        std::vector<Crossing> hits;
        if (const std::vector<uint32_t> *cand = bins[2].at(o))
            for (uint32_t t : *cand) {
                double th;
                if (ray_triangle(o, up_dir, room->edges[t], &th) && th > 0.0) {
                    const V3 a = room->pos[3 * t], b = room->pos[3 * t + 1], cc = room->pos[3 * t + 2];
                    hits.push_back({th, cross(b - a, cc - a).z > 0.0});
                }
            }
        std::stable_sort(hits.begin(), hits.end(), [](const Crossing &a, const Crossing &b) { return a.t < b.t; });
        std::vector<Crossing> crossings;
        for (const Crossing &h : hits) {
            if (!crossings.empty() && h.t - crossings.back().t < 1e-9 && crossings.back().up == h.up) continue;
            crossings.push_back(h);
        }
        size_t k = 0;
        for (int64_t z = 0; z < nz; z++) {
            double p[3];
            g->center(x, y, z, p);
            const double tz = p[2] - start;
            while (k < crossings.size() && crossings[k].t < tz) k++;
            inside[(size_t)g->index(x, y, z)] = (k % 2 == 1);
        }
    }
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < nz; z++)
        for (int64_t y = 0; y < ny; y++)
            for (int64_t x = 0; x < nx; x++) {
                const int64_t i = g->index(x, y, z);
                double p[3];
                g->center(x, y, z, p);
                bool s = false;
                for (int k = 0; k < n_solids && !s; k++) {
                    const double *b = solids + 6 * k;
                    s = p[0] >= b[0] && p[1] >= b[1] && p[2] >= b[2] && p[0] <= b[3] && p[1] <= b[4] && p[2] <= b[5];
                }
                solid[(size_t)i] = s;
                air[(size_t)i] = !s && x > 0 && y > 0 && z > 0 && x < nx - 1 && y < ny - 1 && z < nz - 1 &&
                                 inside[(size_t)i];
            }
    // The surface between an air cell and its missing neighbour: the closest
    // triangle along the face direction with 0 < t < 1.5 dx (fdtd.rs:357-362).
    const double reach = dx * 1.5;
    auto behind = [&](const double p[3], int k) -> int {
        const int axis = k / 2;
        V3 dir{0.0, 0.0, 0.0};
        (axis == 0 ? dir.x : (axis == 1 ? dir.y : dir.z)) = (k & 1) ? 1.0 : -1.0;
        const V3 o{p[0], p[1], p[2]};
        const std::vector<uint32_t> *cand = bins[axis].at(o);
        if (!cand) return -1;
        double tmax = reach;
        int best = -1;
        for (uint32_t t : *cand) {
            double th;
            if (ray_triangle(o, dir, room->edges[t], &th) && th > 0.0 && th < tmax) {
                tmax = th;
                best = (int)room->tri_surface[t];
            }
        }
        return best;
    };
    st = wavey_grid::finish_grid(g, air, solid, fits, behind);
    if (st != WAVEY_OK) return st;
    *out = g;
    return WAVEY_OK;
}
