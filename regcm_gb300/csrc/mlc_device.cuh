// mlc_device.cuh -- device-side data layout and parameter blocks.
//
// Layout in HBM.  Every 3-D field of a domain, whatever its staggering, is
// stored as planes of iy rows x P columns (P = jx rounded up to 128 bytes),
// j fastest, then i, then k: element (j,i,k) of the reference's 1-based
// arrays sits at (j-1) + (i-1)*P + (k-1)*P*iy.  Cross-point fields leave
// column jx and row iy unused.  Rows start on 128-byte boundaries, so a warp
// reading 32 consecutive j is one or two full cache lines, and one pitch and
// plane stride serve every field of the domain.  w and fmzf hold kz+1 planes;
// species arrays (qx, trac) are consecutive kz-plane blocks.
#pragma once
#include <cstddef>
#include <cstdint>

#include "mlc_constants.h"

namespace mlc {

struct Geom {
  int jx, iy, kz, nqx, ntr;
  int P;        // row pitch in elements
  size_t PS;    // plane stride = P*iy
  __host__ __device__ size_t at(int j, int i, int k) const {
    return (size_t)(j - 1) + (size_t)(i - 1) * (size_t)P + (size_t)(k - 1) * PS;
  }
  __host__ __device__ size_t at2(int j, int i) const {
    return (size_t)(j - 1) + (size_t)(i - 1) * (size_t)P;
  }
  __host__ __device__ size_t field3() const { return PS * (size_t)kz; }
};

// Scalars of one domain (all derived on the host once, in FP64).
struct Scal {
  double dx, rdx, dtsec, dt, dtstepa, dtsound, rdzita, dtbdys, rtb;
  int nadv, nsound, divdamp, divfilter, top_nudge, apply_bdy, lrotllr, ipptls;
  int present_qc, present_qi, nspgx, nztop, debug_level;
  int hb_cr, hb_ud, hb_vd;  // relaxation zone non-empty (ba%havebound)
  int curvature;            // curvature terms are not identically zero
};

// Time-invariant device arrays.  Metric arrays use the field type R.
template <class R>
struct Stat {
  const R *fmz, *fmzf, *rfmzu, *rfmzv;   // 3-D
  const double *fmz_d, *fmzf_d;          // FP64 fmz, fmzf for the solve of an FP64 member
  const double *cfz;                     // cp*fmzf*dtsound*rdzita for the solve of a mixed member
  const R *zrfmu, *zrfmd;                // 3-D: (dtrdz*fmz)/fmzf(k), /fmzf(k+1)
  const double *zeta, *dz;               // 3-D, FP64 (surface pressure, budget)
  const R *hx, *hy;                      // 2-D
  const R *msfu, *msfv, *msfx, *mx2, *rmu, *rmv, *coru, *corv;  // 2-D
  const int32_t *ibnd_cr, *ibnd_ud, *ibnd_vd;                   // 2-D
  const double *hefc;      // (nspgx, kz)
  const double *fcx;       // (nspgx)
  const double *tnudge, *ffilt, *gzitakh, *xkdamp, *xknu;      // (kz), 1-based via [k-1]
  const double *gzitak;    // (kz+1)
  const double *rlat;      // (iy)
};

// Prognostic and diagnostic state.
// The Exner function and theta_v are FP64 in both precision modes: in the
// implicit w equation cp*theta_v*fmzf*dPi/dzeta nearly cancels g, and FP32
// rounding of either factor (6e-8 relative) would leave a w forcing of
// ~3e-6 m/s per substep, large against w itself.
template <class R>
struct State {
  R *u, *v, *w, *t, *tvirt, *ux, *vx, *p, *rho, *qsat;
  double *pai, *tetav;
  R *qx, *trac;  // species blocks
  double *ps;    // 2-D, FP64
};

// Boundary data b0/b1 for one domain.
template <class R>
struct Bdy {
  const R *xtb[2], *xqb[2], *xlb[2], *xib[2], *dub[2], *dvb[2], *chib[2];
  const double *xpaib[2], *xpsb[2];
};

// Per-step device scratch that kernels of one step share.
template <class R>
struct Work {
  R *s;        // (kz+1) planes
  R *zdiv2;    // raw divergence (kz planes)
  double *tetavf;  // (kz+1) planes, levels 2..kz used (FP64: feeds the solve)
  R *u2, *v2;  // second buffers of the acoustic ping-pong
  R *wx;       // w at half levels
};

// Boundary clock and buffer roles kept on the device, so a recorded step
// graph replays unchanged: the last kernel of a step advances the clock and
// flips the ping-pong roles.
struct Clock {
  double xbctime;
  int nonfinite;     // sticky: set when a non-finite ps is seen
  int bad_step;      // step counter value at the first non-finite ps
  int step;          // steps completed since the last reset
  int uv_role;       // half of the u/v pairs holding the state at step start
  int adv_role;      // half of the advected-field pairs holding the state
  int pad;
};

// Mass budget and ps extrema of the last step (FP64).
struct DiagDev {
  double drymass, dryadv, qmass, qadv, ps_max, ps_min;
  int nonfinite, pad;
};

// ---- one member (domain) as the kernels see it -----------------------------
// Both halves of every ping-pong pair are listed; the roles in *clk pick the
// current half.  Members of one launch may have different extents.
constexpr int kMaxFields = 24;
template <class R>
struct Dom {
  Geom g;
  Scal c;
  Stat<R> sa;
  Bdy<R> bd;
  R *u[2], *v[2], *ux[2], *vx[2], *qx[2], *trac[2], *wx[2];
  double *pai[2], *tetav[2];
  R *w, *t, *tvirt, *p, *rho, *qsat;
  double *ps;
  R *s, *zdiv2;
  double *tetavf;
  R *wz[kMaxFields];     // per advected R field
  double *wz_d[2];       // per advected FP64 field (theta_v, Exner) of a mixed member
  Clock *clk;
  DiagDev *diag;
  double *partials;
  int red_blocks, rows_per_block;
  int active;            // 0: an empty slot, every block returns at once
};

// The state with the roles the launch works on.
template <class R>
__host__ __device__ __forceinline__ State<R> state_of(const Dom<R> &D, int uv, int adv) {
  State<R> st;
  st.u = D.u[uv]; st.v = D.v[uv]; st.w = D.w; st.t = D.t; st.tvirt = D.tvirt;
  st.ux = D.ux[adv]; st.vx = D.vx[adv]; st.p = D.p; st.rho = D.rho; st.qsat = D.qsat;
  st.pai = D.pai[adv]; st.tetav = D.tetav[adv]; st.qx = D.qx[adv]; st.trac = D.trac[adv];
  st.ps = D.ps;
  return st;
}

}  // namespace mlc
