// mlc_kernels.cuh -- launch interface between the step driver and the kernels.
#pragma once
#include <cuda_runtime.h>

#include "mlc_device.cuh"

namespace mlc {

// Advected fields of one advection step: each is read from `cur`, its two
// vertical WAF passes go to `wz`, and the horizontal passes write `out`.
constexpr int kMaxAdv = 24;
template <class R>
struct AdvTable {
  const R *cur[kMaxAdv];
  R *wz[kMaxAdv];
  R *out[kMaxAdv];
  int n;
};

// Buffers of one substep of the acoustic loop.
template <class R>
struct SoundBufs {
  const R *u_in, *v_in;  // state at the start of the substep (ud, vd)
  R *u_out, *v_out;      // state at its end
};

template <class R> struct Launch {
  // one-off kernel attributes (large dynamic shared memory); call before capture
  static cudaError_t configure_sound();
  static cudaError_t configure_advect();
  // ---- sound (Main/mod_moloch.F90:545-765) ----
  static void sound_prep(const Geom &g, const State<R> &st, const Work<R> &wk, cudaStream_t s);
  static void sound_div(const Geom &g, const Scal &c, const Stat<R> &sa, const State<R> &st,
                        const Work<R> &wk, const SoundBufs<R> &b, cudaStream_t s);
  static void sound_solve(const Geom &g, const Scal &c, const Stat<R> &sa, const State<R> &st,
                          const Work<R> &wk, bool last, cudaStream_t s);
  static void sound_momentum(const Geom &g, const Scal &c, const Stat<R> &sa, const State<R> &st,
                             const Work<R> &wk, const SoundBufs<R> &b, cudaStream_t s);
  // ---- advection (Main/mod_moloch.F90:767-1042) ----
  static void adv_prep(const Geom &g, const State<R> &st, const Work<R> &wk, cudaStream_t s);
  static void adv_vertical(const Geom &g, const Scal &c, const Stat<R> &sa, const Work<R> &wk,
                           const AdvTable<R> &t, cudaStream_t s);
  static void adv_horizontal(const Geom &g, const Scal &c, const Stat<R> &sa, const State<R> &st,
                             const AdvTable<R> &t, cudaStream_t s);
  // the same two passes for FP64 fields advected with this domain's winds
  static void adv_vertical_f64(const Geom &g, const Scal &c, const Stat<R> &sa, const Work<R> &wk,
                               const AdvTable<double> &t, cudaStream_t s);
  static void adv_horizontal_f64(const Geom &g, const Scal &c, const Stat<R> &sa,
                                 const State<R> &st, const AdvTable<double> &t, cudaStream_t s);
  static void adv_curvature(const Geom &g, const Scal &c, const Stat<R> &sa, const State<R> &st,
                            cudaStream_t s);
  static void adv_back(const Geom &g, const State<R> &st, const Work<R> &wk, cudaStream_t s);
  // ---- step end (Main/mod_moloch.F90:340-446, mod_bdycod.F90) ----
  static void end_tvirt(const Geom &g, const Scal &c, const State<R> &st, cudaStream_t s);
  static void bdy_ring(const Geom &g, const Scal &c, const State<R> &st, const Bdy<R> &bd,
                       const Clock *clk, cudaStream_t s);
  static void bdy_relax(const Geom &g, const Scal &c, const Stat<R> &sa, const State<R> &st,
                        const Bdy<R> &bd, const Clock *clk, cudaStream_t s);
  static void end_cross(const Geom &g, const Scal &c, const Stat<R> &sa, const State<R> &st,
                        cudaStream_t s);
  static void end_uvstag(const Geom &g, const State<R> &st, cudaStream_t s);
  static void end_reduce(const Geom &g, const Scal &c, const Stat<R> &sa, const State<R> &st,
                         double *partials, int nblocks, DiagDev *diag, Clock *clk,
                         cudaStream_t s);
  // ---- layout conversion ----
  static void unpack3(const double *src, R *dst, const Geom &g, int nj, int ni, int nk,
                      cudaStream_t s);
  static void pack3(const R *src, double *dst, const Geom &g, int nj, int ni, int nk,
                    cudaStream_t s);
};

// Blocks the reduction of end_reduce uses for a geometry.
int reduce_blocks(const Geom &g);

}  // namespace mlc
