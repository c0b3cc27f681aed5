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
  int nmem;       // ensemble members advanced by one launch (1 = one domain)
  size_t mstride; // bytes between consecutive members' arenas
  // launch shapes (picked by the autotuner; defaults in mlc_context.cu)
  int col_x, col_y;      // column kernels (threads along j, i)
  int solve_x, solve_y;  // sound_solve
  int vert_x, vert_y;    // adv_vertical
  int htile;             // adv_horizontal tile: 0 32x8, 1 32x4, 2 64x4, 3 16x8
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
  const double *fmz_d, *fmzf_d;          // FP64 copies for the vertical solve
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

// Boundary clock kept on the device so a captured step graph stays valid.
struct Clock {
  double xbctime;
  int nonfinite;     // sticky: set when a non-finite ps is seen
  int bad_step;      // step counter value at the first non-finite ps
  int step;          // steps completed since the last reset
  int pad;
};

// Mass budget and ps extrema of the last step (FP64).
struct DiagDev {
  double drymass, dryadv, qmass, qadv, ps_max, ps_min;
  int nonfinite, pad;
};

// ---- ensemble members -----------------------------------------------------
// Every array of member m lives at member 0's address plus m * mstride, so a
// kernel that serves all members rebases its pointer arguments once.
template <class T>
__device__ __forceinline__ T *mshift(T *p, size_t off) {
  return p ? reinterpret_cast<T *>(reinterpret_cast<char *>(p) + off) : p;
}
template <class T>
__device__ __forceinline__ const T *mshift(const T *p, size_t off) {
  return p ? reinterpret_cast<const T *>(reinterpret_cast<const char *>(p) + off) : p;
}

template <class R>
__device__ __forceinline__ void rebase(Stat<R> &s, size_t o) {
  if (!o) return;
  s.fmz = mshift(s.fmz, o); s.fmzf = mshift(s.fmzf, o); s.rfmzu = mshift(s.rfmzu, o);
  s.rfmzv = mshift(s.rfmzv, o); s.fmz_d = mshift(s.fmz_d, o); s.fmzf_d = mshift(s.fmzf_d, o);
  s.zrfmu = mshift(s.zrfmu, o); s.zrfmd = mshift(s.zrfmd, o); s.zeta = mshift(s.zeta, o);
  s.dz = mshift(s.dz, o); s.hx = mshift(s.hx, o); s.hy = mshift(s.hy, o);
  s.msfu = mshift(s.msfu, o); s.msfv = mshift(s.msfv, o); s.msfx = mshift(s.msfx, o);
  s.mx2 = mshift(s.mx2, o); s.rmu = mshift(s.rmu, o); s.rmv = mshift(s.rmv, o);
  s.coru = mshift(s.coru, o); s.corv = mshift(s.corv, o); s.ibnd_cr = mshift(s.ibnd_cr, o);
  s.ibnd_ud = mshift(s.ibnd_ud, o); s.ibnd_vd = mshift(s.ibnd_vd, o); s.hefc = mshift(s.hefc, o);
  s.fcx = mshift(s.fcx, o); s.tnudge = mshift(s.tnudge, o); s.ffilt = mshift(s.ffilt, o);
  s.gzitakh = mshift(s.gzitakh, o); s.xkdamp = mshift(s.xkdamp, o); s.xknu = mshift(s.xknu, o);
  s.gzitak = mshift(s.gzitak, o); s.rlat = mshift(s.rlat, o);
}

template <class R>
__device__ __forceinline__ void rebase(State<R> &s, size_t o) {
  if (!o) return;
  s.u = mshift(s.u, o); s.v = mshift(s.v, o); s.w = mshift(s.w, o); s.t = mshift(s.t, o);
  s.tvirt = mshift(s.tvirt, o); s.ux = mshift(s.ux, o); s.vx = mshift(s.vx, o);
  s.p = mshift(s.p, o); s.rho = mshift(s.rho, o); s.qsat = mshift(s.qsat, o);
  s.pai = mshift(s.pai, o); s.tetav = mshift(s.tetav, o); s.qx = mshift(s.qx, o);
  s.trac = mshift(s.trac, o); s.ps = mshift(s.ps, o);
}

template <class R>
__device__ __forceinline__ void rebase(Bdy<R> &b, size_t o) {
  if (!o) return;
  for (int q = 0; q < 2; ++q) {
    b.xtb[q] = mshift(b.xtb[q], o); b.xqb[q] = mshift(b.xqb[q], o); b.xlb[q] = mshift(b.xlb[q], o);
    b.xib[q] = mshift(b.xib[q], o); b.dub[q] = mshift(b.dub[q], o); b.dvb[q] = mshift(b.dvb[q], o);
    b.chib[q] = mshift(b.chib[q], o); b.xpaib[q] = mshift(b.xpaib[q], o);
    b.xpsb[q] = mshift(b.xpsb[q], o);
  }
}

}  // namespace mlc
