// mlc_kernels.cuh -- launch interface between the step driver and the kernels.
//
// Every kernel serves all members of a context in one launch: blockIdx.z (or
// blockIdx.y for the reduction) selects the member, whose descriptor Dom<R>
// (extents, parameters, pointers) sits in a device array.  Grids cover the
// largest member; blocks outside a smaller member's extent return at once.
// Buffer roles are read from each member's device clock plus the offsets a
// launch passes (uvoff acoustic substeps, advoff advection rounds since the
// step began), so one recorded graph replays every step.
#pragma once
#include <cuda_runtime.h>

#include "mlc_device.cuh"

namespace mlc {

// Columns of a column-solve block (one row segment, one thread a column):
// FP64 members and mixed members.
#ifndef MLC_DV_W
#define MLC_DV_W 128
#endif
constexpr int kSolveColsD = MLC_DV_W;
constexpr int kSolveColsF = 128;

// Extents of a launch (maxima over the members) and the launch shapes.
struct LaunchGeom {
  int jx, iy, kz, nmem;
  int col_x, col_y;      // column kernels
  int solve_x, solve_y;  // kept in the tune report; the solves use fixed 128-column blocks
  int vert_x, vert_y;    // adv_vertical
  int htile;             // adv_horizontal tile shape (hshape)
  int nadv_r;            // advected fields of type R per member
  int nadv_d;            // advected FP64 fields per member (mixed: theta_v, Exner)
  int red_blocks;        // reduction blocks of the largest member
  int solve_df;          // mixed solve: recurrence in double-float (1) or FP32 (0)
  // work lists of an uneven batch (device arrays; null: grids over the
  // largest member) and their lengths, one per tiling
  const WorkItem *wl_pt;     // col_x x col_y tiles, level chunks
  const WorkItem *wl_v4;     // 128 x 4 tiles, level chunks
  const WorkItem *wl_solve;  // 128-column row segments
  const WorkItem *wl_vert;   // vert_x x vert_y column tiles, R fields
  const WorkItem *wl_vinc;   // the same, the two double-float fields
  const WorkItem *wl_h;      // horizontal WAF tiles (shape htile), levels
  const WorkItem *wl_hinc;   // increment-form WAF tiles, levels
  int n_pt, n_v4, n_solve, n_vert, n_vinc, n_h, n_hinc;
};

template <class R> struct Launch {
  // one-off kernel attributes (large dynamic shared memory); call before capture
  static cudaError_t configure_sound();
  static cudaError_t configure_advect();
  // ---- sound (Main/mod_moloch.F90:545-765) ----
  static void sound_prep(const LaunchGeom &L, const Dom<R> *d, int advoff, cudaStream_t s);
  static void sound_div(const LaunchGeom &L, const Dom<R> *d, int uvoff, cudaStream_t s);
  static void sound_solve(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, bool last,
                          cudaStream_t s);
  static void sound_momentum(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff,
                             cudaStream_t s);
  // ---- advection (Main/mod_moloch.F90:767-1042) ----
  static void adv_prep(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s);
  static void adv_vertical(const LaunchGeom &L, const Dom<R> *d, int advoff, cudaStream_t s);
  static void adv_horizontal(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff,
                             cudaStream_t s);
  // theta_v and Exner of a mixed member (double-float, increment form)
  static void adv_vertical_inc(const LaunchGeom &L, const Dom<R> *d, int advoff, cudaStream_t s);
  static void adv_horizontal_inc(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff,
                                 cudaStream_t s);
  static void adv_species_copy(const LaunchGeom &L, const Dom<R> *d, int advoff, cudaStream_t s);
  static void adv_curvature(const LaunchGeom &L, const Dom<R> *d, int advoff, cudaStream_t s);
  static void adv_back(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s);
  // ---- step end (Main/mod_moloch.F90:340-446, mod_bdycod.F90) ----
  static void bdy_ring(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s);
  static void end_relax(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s);
  static void bdy_spectral(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s);
  static void end_cross(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s);
  // the step split at the physics: k_end_ps and the cross-point work up to
  // mkslice (post = false), or status_update with the tendencies (post = true)
  static void end_cross_split(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, bool post,
                              cudaStream_t s);
  static void end_uvstag(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s);
  // status_update of the TKE (ibltyp = 2): tendency (split step) and floor
  static void end_tke(const LaunchGeom &L, const Dom<R> *d, bool whole_step, cudaStream_t s);
  static void end_reduce(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff,
                         cudaStream_t s);
  // ---- layout conversion (one member, from the host) ----
  static void unpack3(const double *src, R *dst, const Geom &g, int nj, int ni, int nk,
                      cudaStream_t s);
  static void pack3(const R *src, double *dst, const Geom &g, int nj, int ni, int nk,
                    cudaStream_t s);
  // double-float planes (hi, lo) of nplane elements each
  static void unpack3_df(const double *src, double *dst, const Geom &g, int nj, int ni, int nk,
                         size_t nplane, cudaStream_t s);
  static void pack3_df(const double *src, double *dst, const Geom &g, int nj, int ni, int nk,
                       size_t nplane, cudaStream_t s);
};

// Reduction blocks the mass budget uses for a geometry.
int reduce_blocks(const Geom &g);

}  // namespace mlc
