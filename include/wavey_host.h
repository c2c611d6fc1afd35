/*
 * wavey_host.h -- host-side inputs and outputs of the FDTD wave solver.
 *
 * C-ABI of libwavey_host.so: everything wavey-solver computes on the host
 * around the GPU run, restated in C++ so that callers without the Rust crate
 * (tests, benchmarks, C/C++/Python hosts) can build the same grids, taps,
 * signals and transfer functions that the reference hands to its GPU
 * backend.  A Rust host keeps its own `FdtdGrid` and only needs
 * wavey_cuda.h.
 *
 * All functions are thread-safe (no global state).  Functions returning int
 * return 0 on success and a negative WAVEY_E_* code otherwise.
 */
#ifndef WAVEY_HOST_H
#define WAVEY_HOST_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* fdtd.rs:138 and fdtd.rs:140 */
#define WAVEY_COURANT 0.5773502691896257
#define WAVEY_MAX_CELLS 600000000ull
#define WAVEY_NO_BOUNDARY 0xFFFFFFFFu
#define WAVEY_AIR 64u

/* ---------------------------------------------------------------- materials
 * Replaces wavey-materials: Spectrum::eval (spectrum.rs:24-44),
 * Material::absorption_at (material.rs:70-76), fit_real_impedance
 * (material.rs:96-111) and fit_admittance (impedance_fit.rs:158-235).
 */
typedef struct {
    /* n == 0: scalar `value`; else a table over log-frequency. */
    int32_t n;
    double value;
    const double *freqs_hz;
    const double *values;
} wh_spectrum;

/* One fitted boundary admittance, AdmittanceFit (impedance_fit.rs:34-44).
 * Up to WH_MAX_BRANCHES mass-spring-damper branches. */
#define WH_MAX_BRANCHES 4
typedef struct {
    double beta0;
    int32_t n_branches;
    double r[WH_MAX_BRANCHES], m[WH_MAX_BRANCHES], k[WH_MAX_BRANCHES];
    double band_lo, band_hi;
    double rms_error, max_error;
} wh_fit;

double wh_spectrum_eval(const wh_spectrum *s, double f);
double wh_fit_real_impedance(double alpha);
/* Statistical (Paris) absorption of a fitted admittance, 256-point rule
 * (impedance_fit.rs:63-65). */
double wh_fit_absorption(const wh_fit *fit, double f);
/* Normalised admittance beta(f) (impedance_fit.rs:48-55): out[0]=re, out[1]=im. */
void wh_fit_admittance_at(const wh_fit *fit, double f, double out[2]);
int wh_fit_admittance(const wh_spectrum *absorption, double band_lo, double band_hi, int32_t max_branches, wh_fit *out);

/* ------------------------------------------------------------------- rooms
 * Box-shaped rooms: the prism rooms `build_room` makes from a rectangular
 * plan with rectangular pillars (wavey-geom room.rs:281-349), plus optional
 * axis-aligned absorbing blocks (balcony steps) and rigid solids (cabinets,
 * fdtd.rs:424-461).
 *
 * Surface order (material index), as build_room orders them for a plan
 * drawn counter-clockwise: 0 floor, 1 ceiling, 2 wall y=y0, 3 wall x=x1,
 * 4 wall y=y1, 5 wall x=x0; then per pillar its faces y=py0, x=px0, y=py1,
 * x=px1; then per block its faces x=bx0, x=bx1, y=by0, y=by1, z=bz0, z=bz1.
 */
typedef struct {
    double x0, y0, x1, y1;   /* plan rectangle */
    double height;           /* floor at z = 0, ceiling at z = height */
    int32_t n_pillars;       /* floor-to-ceiling rectangular holes in the plan */
    const double *pillars;   /* [n_pillars][4] = x0, y0, x1, y1 */
    int32_t n_blocks;        /* absorbing boxes removed from the air */
    const double *blocks;    /* [n_blocks][6] = x0, y0, z0, x1, y1, z1 */
    int32_t n_solids;        /* rigid boxes: their faces get no admittance slot */
    const double *solids;    /* [n_solids][6] */
} wh_room;

int32_t wh_room_surface_count(const wh_room *room);
/* Strict inside test of the room (room.rs:151-157 for the prism part). */
int wh_room_contains(const wh_room *room, const double p[3]);

/* -------------------------------------------------------------- mesh rooms
 * Rooms imported as polygon meshes (OBJ rooms), room_from_mesh
 * (wavey-geom room.rs:399-461): polygons are cut into triangles, each
 * (material group, plane) becomes one surface with its normal into the room
 * (found by the ray-parity inside test, room.rs:355-367), and surfaces are
 * numbered in discovery order.  A surface's material is its group's.
 */
typedef struct wh_mesh_room wh_mesh_room;

/* verts: [n_verts][3]; polygon f is face_verts[face_start[f] ..
 * face_start[f + 1]) with material group face_group[f]. */
int wh_mesh_room_build(const double *verts, int64_t n_verts, const uint32_t *face_verts, const int64_t *face_start,
                       const int32_t *face_group, int64_t n_faces, wh_mesh_room **out);
void wh_mesh_room_free(wh_mesh_room *room);
int32_t wh_mesh_room_surface_count(const wh_mesh_room *room);
int64_t wh_mesh_room_triangle_count(const wh_mesh_room *room);
/* Surface s: its material group, kind (0 wall, 1 floor, 2 ceiling), unit
 * normal into the room, plane offset d = n.p and area.  Any output may be
 * NULL. */
void wh_mesh_room_surface(const wh_mesh_room *room, int32_t s, int32_t *group, int32_t *kind, double normal[3],
                          double *d, double *area);
/* positions [triangles][3][3] (wound to their surface's normal) and the
 * surface of each triangle (Room::tri_surface). */
void wh_mesh_room_triangles(const wh_mesh_room *room, double *positions, uint32_t *tri_surface);
void wh_mesh_room_bounds(const wh_mesh_room *room, double lo[3], double hi[3]);
/* Room::contains for mesh rooms (room.rs:151-157, parity_inside). */
int wh_mesh_room_contains(const wh_mesh_room *room, const double p[3]);
/* Room::volume (room.rs:165-178). */
double wh_mesh_room_volume(const wh_mesh_room *room);

/* ------------------------------------------------------------------- grids
 * FdtdGrid (fdtd.rs:196-209) with the boundary nodes in CSR form.
 */
typedef struct wh_grid wh_grid;

typedef struct {
    int64_t nx, ny, nz;
    double origin[3];
    double dx, dt;
    const uint8_t *flags;     /* [cells] bit 6 air, bits 0-5 air neighbours */
    const uint32_t *bidx;     /* [cells] boundary node index or WAVEY_NO_BOUNDARY */
    int64_t n_boundary;
    const uint32_t *bcell;    /* [n_boundary] cell of each boundary node */
    const uint32_t *bstart;   /* [n_boundary + 1] slot range per node */
    const double *slots;      /* [n_slots][4] = inv_d, cv, k, w (fdtd.rs:178-187) */
    int64_t n_slots;
    int64_t air_cells;
} wh_grid_view;

/* FdtdGrid::build_dx (fdtd.rs:289-378) with `fits` holding one fit per
 * surface.  Fails with WAVEY_E_LIMIT above MAX_CELLS. */
int wh_grid_build(const wh_room *room, const wh_fit *fits, int32_t n_fits, double c, double dx, wh_grid **out);
/* FdtdGrid::build_dx (fdtd.rs:289-378) for a mesh room: air by column_fill
 * (fdtd.rs:385-422, one upward ray per grid column), the surface behind
 * each missing face by the closest triangle along the face direction within
 * 1.5 dx (fdtd.rs:357-362).  solids: optional rigid boxes [n_solids][6]
 * (x0, y0, z0, x1, y1, z1) whose faces carry no admittance.  fits: one per
 * surface (wh_mesh_room_surface_count). */
int wh_grid_build_mesh(const wh_mesh_room *room, const double *solids, int32_t n_solids, const wh_fit *fits,
                       int32_t n_fits, double c, double dx, wh_grid **out);
/* FdtdGrid::build_with spacing rule (fdtd.rs:282-286): c / (f_max * ppw),
 * at most the smallest solid side / 8. */
double wh_grid_spacing(const wh_room *room, double c, double f_max, double ppw);
void wh_grid_view_of(const wh_grid *g, wh_grid_view *out);
void wh_grid_free(wh_grid *g);
/* An empty grid of the given shape with room for n_boundary nodes and
 * n_slots slots, for a builder outside this library to fill (the CUDA grid
 * builder, wavey_cuda_grid_build / wavey_cuda_grid_read): flags zeroed, bidx
 * WAVEY_NO_BOUNDARY; wh_grid_arrays gives the writable arrays.  No
 * counterpart in the reference. */
int wh_grid_alloc(const int64_t n[3], const double origin[3], double dx, double dt, int64_t air_cells,
                  int64_t n_boundary, int64_t n_slots, wh_grid **out);
void wh_grid_arrays(wh_grid *g, uint8_t **flags, uint32_t **bidx, uint32_t **bcell, uint32_t **bstart,
                    double **slots);

/* fdtd.rs:245-272; returns the cell or -1. */
int64_t wh_nearest_air(const wh_grid *g, const double p[3]);
/* fdtd.rs:467-492; writes up to 8 taps, returns their count or -1. */
int32_t wh_taps_at(const wh_grid *g, const double p[3], int64_t cells[8], double weights[8]);
/* fdtd.rs:730-743; components of order 0 or 1 at cell c.  Writes
 * comp_cells/comp_w as 4 components of 2 taps (monopole uses 1), returns
 * the component count or -1 when a neighbour is not air. */
int32_t wh_source_components(const wh_grid *g, int64_t c, int32_t order, int64_t comp_cells[4][2],
                             double comp_w[4][2], int32_t comp_n[4]);
/* fdtd.rs:497-512 and fdtd.rs:516-534 */
void wh_baffle_point(const wh_grid *g, const double p[3], const double axis[3], double out[3]);
int64_t wh_air_along(const wh_grid *g, const double p[3], const double axis[3]);

/* ----------------------------------------------------------- time / freqs */
/* fdtd.rs:601-610 */
void wh_source_signal(double f_max, double dt, int64_t steps, double *out);
/* freq.rs:15-22, 1/n-octave grid; returns the count (writes at most cap). */
int32_t wh_frequency_grid(double f_min, double f_max, int32_t n, double *out, int32_t cap);
/* fdtd.rs:142-175 */
double wh_crossover_weight(double crossover_hz, double f);
double wh_phase_error_deg_per_m(double f, double c, double dx);
/* fdtd.rs:866-869 */
double wh_auto_duration(const double *rt, int32_t n);

/* --------------------------------------------------------- post-processing */
/* to_transfer (fdtd.rs:819-840).  spectra/out are [n_recv][nf] complex as
 * interleaved (re, im); h0 is [nf] complex. */
void wh_to_transfer(const double *spectra, int64_t n_recv, const double *signal, int64_t steps, double dt, double dx,
                    const double *freqs, int64_t nf, double c, double r_ref, const double *h0, double *out);
/* blend (fdtd.rs:847-863) */
void wh_blend(const double ism[2], const double wave[2], double w, double out[2]);
/* Directional fit (fdtd.rs:749-807).  The 400 golden-spiral directions in
 * the speaker's frame come from wh_fit_directions; the caller evaluates the
 * directivity there (d_samples, complex) and on axis (d_axis).  to_room is a
 * column-major 3x3 rotation.  out_a = a0, ax, ay, az (complex). */
#define WH_FIT_DIRECTIONS 400
void wh_fit_directions(double out[WH_FIT_DIRECTIONS][3]);
void wh_fit_first_order(const double *d_samples, const double d_axis[2], const double to_room[9], double out_a[8],
                        double *residual);
/* component_weights (fdtd.rs:812-815): out = 4 complex weights. */
void wh_component_weights(const double a0[2], const double a[6], double k, double dx, double out[8]);
/* SpeakerInstance::rotation (wavey-speaker instance.rs:44-48), column-major. */
void wh_speaker_rotation(double yaw_deg, double pitch_deg, double roll_deg, double out[9]);

#ifdef __cplusplus
}
#endif
#endif
