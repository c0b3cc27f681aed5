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

// Scalars of one domain (all derived on the host once, in FP64; the f-suffixed
// copies are the same values rounded to FP32 once, for the FP32 kernels).
struct Scal {
  double dx, rdx, dtsec, dt, dtstepa, dtsound, rdzita, dtbdys, rtb;
  float dxf, rdxf, dtsecf, dtstepaf, dtsoundf, rdzitaf;
  float gdts_hi, gdts_lo;   // g*dtsound as a double-float
  double dtrdxs, dxrdt;     // dtsound*rdx, dx/dtsound (acoustic substep)
  float dtrdxsf, dxrdtf;
  int nadv, nsound, divdamp, divfilter, top_nudge, apply_bdy, lrotllr, ipptls;
  int present_qc, present_qi, nspgx, nztop, debug_level;
  int hb_cr, hb_ud, hb_vd;  // relaxation zone non-empty (ba%havebound)
  int curvature;            // curvature terms are not identically zero
  int spectral;             // spectral nudging on
  int km2, lm2;             // sine modes in x and y (2*km, 2*lm)
  int tke;                  // ibltyp = 2: TKE advected, bounded and updated
  double dtrad;             // spectral nudging interval
};
// sine modes of spectral nudging per direction, at most
constexpr int kMaxModes = 32;

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
  // the 1-D arrays, hefc, fcx and dz in the field type (aliases for FP64)
  const R *gzitak_r, *gzitakh_r, *xkdamp_r, *xknu_r, *ffilt_r, *tnudge_r, *hefc_r, *fcx_r, *dz_r;
  // a mixed member's dz - dz_r (dz as the double-float {dz_r, dz_lo}, for the
  // mass budget); null for an FP64 member
  const R *dz_lo;
  // an FP64 member's constant factors of the acoustic substep, formed once at
  // bind time in the kernels' own operand order (null for a mixed member):
  //   sound_div: dtrdx*rfmzu*rmu (u points; rotated: dtrdx*rfmzu),
  //              dtrdy*rfmzv*rmv (v points), fmz*mfac (cross points)
  //   sound_momentum: dxrdt*xkdamp(k)*msfu and dxrdt*xkdamp(k)*msfv
  //              (rotated: dxrdt*xkdamp(k)), g*dts*hx*gzitakh(k) and
  //              g*dts*hy*gzitakh(k) (3-D), coru*dts and corv*dts (2-D)
  const double *dv_cu, *dv_cv, *dv_cf, *mo_du, *mo_dv, *mo_gu, *mo_gv, *mo_cu, *mo_cv;
  //   sound_solve (3-D, cross points): (bw*dtrdz)*fmz with bw the relaxation
  //              weight 1 - hefc of the point's zone (1 outside), zcs2*fmz
  //              and dtrdz*fmz
  const double *sv_a, *sv_b, *sv_c;
  // spectral nudging: sine bases bvx (km2 rows of jx) and bvy (lm2 rows of
  // iy), the level weights cnudge (kz)
  const R *bvx, *bvy, *cnudge;
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
  R *tke;        // (kz+1) planes, ibltyp = 2 (else null)
};

// Boundary data b0/b1 for one domain.  Temperature and Exner are FP64 (a
// mixed member: double-float planes): the relaxation pulls t and pai toward
// them every step, so a rounded copy would leave a persistent offset in the
// relaxation zone.
template <class R>
struct Bdy {
  const R *xqb[2], *xlb[2], *xib[2], *dub[2], *dvb[2], *chib[2];
  const double *xtb[2], *xpaib[2], *xpsb[2];
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
  int fault;         // sticky: a bounded device wait gave up (1 = TMA tile load)
  double tspectral;  // seconds of boundary updates, for the spectral nudging interval
  unsigned red_done; // blocks of the step's budget reduction that have finished (0 between steps)
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
  // turbulent kinetic energy at the interfaces (kz+1 planes) and its
  // advected copy at the levels (a ping-pong pair); null unless ibltyp = 2
  R *tke, *tkex[2];
  R *s, *zdiv2;
  double *tetavf;
  R *wz[kMaxFields];     // per advected R field
  double *wz_d[2];       // per advected FP64 field (theta_v, Exner) of a mixed member
  Clock *clk;
  DiagDev *diag;
  double *partials;
  R *spec;               // spectral nudging: per field and level, iy rows of km2 coefficients
  // an FP64 member's s(k)*zrfmu(k) - s(k+1)*zrfmd(k) of the advection round
  // (the vertical WAF update's divergence factor, the same for every field)
  double *vdiv;
  // an FP64 member's flux factors of interface k+1 at level k's offset:
  // zamu = s*dtrdz, zmi = zamu - is and zmih = zmi/2 (the vertical WAF's)
  double *vzamu, *vzmih, *vzmi;
  // physics tendencies of the open step (null: zero), fields of the state's
  // layout: tten, uten, vten, then nqx qxten, then ntr chiten
  const R *tend;
  int red_blocks;
  int active;            // 0: an empty slot, every block returns at once
  // test hook of the bounded waits (0 = off): the horizontal WAF's blocks
  // wait this many polls on an mbarrier no copy completes, then record the
  // fault, as they do for a copy that never lands
  int stall_polls;
  // TMA tensor maps (CUtensorMap, 128 B each, 64-B aligned) of the wz fields,
  // [horizontal tile shape][field], for the horizontal WAF's halo tiles
  const void *tmap;
};
constexpr int kTileShapes = 4;
constexpr int kTmapBytes = 128;
// Tensor maps per tile shape: the kMaxFields wz fields of the R table, then
// the planes the increment form of a mixed member reads: theta_v and Exner
// of both buffer halves (hi, lo) and their vertical increments (hi, lo)
//   kMaxFields + 0..3  theta_v[0].hi, theta_v[0].lo, theta_v[1].hi, theta_v[1].lo
//   kMaxFields + 4..7  Exner[0].hi, ..., Exner[1].lo
//   kMaxFields + 8..11 increment of theta_v (hi, lo), of Exner (hi, lo)
constexpr int kIncMaps = 12;
constexpr int kTmapSlots = kMaxFields + kIncMaps;

// Tile shapes of the horizontal WAF (LaunchGeom::htile).  A warp is one row
// of 32*v columns, lane l holding columns v*l .. v*l+v-1; a block is nw rows.
// Every warp computes its whole range and writes all but two columns at each
// end (the zonal fluxes of a column need the intermediate field two columns
// either side), so consecutive tiles overlap by four columns.
//   0 = 32x8, 1 = 64x8, 2 = 64x4, 3 = 32x4 (columns x rows)
struct HShape {
  int v, nw;
};
__host__ __device__ constexpr HShape hshape(int elem_bytes, int idx) {
  return (void)elem_bytes,
         idx == 1 ? HShape{2, 8} : idx == 2 ? HShape{2, 4} : idx == 3 ? HShape{1, 4} : HShape{1, 8};
}
// The increment-form WAF (theta_v and Exner of a mixed member, two planes per
// field) runs the same lanes in blocks of four rows.
__host__ __device__ constexpr HShape hshape_inc(int idx) {
  return HShape{hshape(4, idx).v, 4};
}
// Column offset (j - 1) of the first tile's first column: at most -2, so the
// first written column is j <= 1, and a multiple of v (aligned lane vectors).
__host__ __device__ constexpr int hshape_ob0(int v) { return -(v > 2 ? v : 2); }
// Columns the halo tile's TMA box starts left of the warp range, so that the
// copy starts on 16 bytes (tile offsets step by 32*v - 4, a multiple of 16
// bytes); the box is 32*v + 2*off columns by nw + 4 rows.
__host__ __device__ constexpr int hshape_off(int elem_bytes, int v) {
  return ((hshape_ob0(v) % (16 / elem_bytes)) + 16 / elem_bytes) % (16 / elem_bytes);
}

// A per-domain constant in the kernel's field type: the FP64 value for an
// FP64 member, its FP32 copy for a mixed one (no conversion on the device).
template <class R>
__device__ __forceinline__ R pick(double d, float f) {
  if constexpr (sizeof(R) == sizeof(double)) return d;
  else return f;
}

// ---- double-float values of a mixed member ----------------------------------
// theta_v, Exner, theta_v at half levels, the vertical increments of the
// increment-form advection, cp*fmzf*dtrdz and the boundary Exner values of a
// mixed member are kept as unevaluated sums hi + lo of two floats (about 48
// significant bits) in two planes of the field's 8-byte-per-element
// allocation: hi in elements [0, n), lo in [n, 2n) of the float view.
// Arithmetic on them uses error-free transformations - TwoSum (Knuth, The Art
// of Computer Programming vol. 2, 4.2.2), Fast2Sum (Dekker 1971) and
// TwoProduct with a fused multiply-add - so the FP32 path runs no FP64
// instruction.  The code relies on IEEE FP32 addition (no fast-math).
struct F2 {
  float hi, lo;
};
__device__ __forceinline__ F2 two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ F2 fast_two_sum(float a, float b) {  // needs |a| >= |b|
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ F2 two_prod(float a, float b) {
  const float p = a * b;
  return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ F2 df_add(F2 a, F2 b) {
  const F2 s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ F2 df_add_f(F2 a, float b) {
  const F2 s = two_sum(a.hi, b);
  return fast_two_sum(s.hi, s.lo + a.lo);
}
__device__ __forceinline__ F2 df_mul(F2 a, F2 b) {
  const F2 p = two_prod(a.hi, b.hi);
  return fast_two_sum(p.hi, p.lo + (a.hi * b.lo + a.lo * b.hi));
}
__device__ __forceinline__ F2 df_mul_f(F2 a, float b) {
  const F2 p = two_prod(a.hi, b);
  return fast_two_sum(p.hi, fmaf(a.lo, b, p.lo));
}
// a / b for a double-float a and an FP32 b: one correction of the FP32 quotient
// with the exact remainder (a - q*b by TwoProduct)
__device__ __forceinline__ F2 df_div_f(F2 a, float b) {
  const float q1 = a.hi / b;
  const F2 p = two_prod(q1, b);
  const float r = ((a.hi - p.hi) - p.lo) + a.lo;
  return fast_two_sum(q1, r / b);
}
// a / b for double-floats, the same way
__device__ __forceinline__ F2 df_div(F2 a, F2 b) {
  const float q1 = a.hi / b.hi;
  const F2 p = df_mul(F2{q1, 0.f}, b);
  const float r = ((a.hi - p.hi) - p.lo) + a.lo;
  return fast_two_sum(q1, r / b.hi);
}
// 1 / b for a double-float b: the hardware's approximate FP32 reciprocal rc
// (__fdividef, within 2 ulp) and one Newton step rc + rc*(1 - b*rc) with the
// residual formed by TwoProduct (the double-length reciprocal of Karp and
// Markstein, ACM TOMS 23(4), 1997).  Relative error about 2^-44 for b of
// normal FP32 range; about a third of df_div's instructions (no IEEE FP32
// division).
__device__ __forceinline__ F2 df_recip(F2 b) {
  const float rc = __fdividef(1.f, b.hi);
  const F2 p = two_prod(rc, b.hi);
  const float e = ((1.f - p.hi) - p.lo) - rc * b.lo;
  return fast_two_sum(rc, rc * e);
}
// a - b rounded to FP32 (the hi difference is exact for values within 2x)
__device__ __forceinline__ float df_diff(F2 a, F2 b) { return (a.hi - b.hi) + (a.lo - b.lo); }
__device__ __forceinline__ float df_f(F2 a) { return a.hi + a.lo; }

// Planes of n double-float elements over an 8-byte-per-element allocation.
struct DF {
  float *p;
  size_t n;
  __device__ __forceinline__ DF(const double *a, size_t n_)
      : p(reinterpret_cast<float *>(const_cast<double *>(a))), n(n_) {}
  __device__ __forceinline__ DF(float *p_, size_t n_) : p(p_), n(n_) {}
  __device__ __forceinline__ F2 ld(size_t o) const { return {p[o], p[o + n]}; }
  __device__ __forceinline__ void st(size_t o, F2 v) const { p[o] = v.hi; p[o + n] = v.lo; }
  __device__ __forceinline__ float hi(size_t o) const { return p[o]; }
};

// ---- work lists of an uneven batch ------------------------------------------
// A launch over members of different extents covers, by default, the largest
// member's tiles for every member (blockIdx.z is the member; blocks outside a
// smaller member return at once).  With a work list the launch has one block
// per entry instead, and each entry names the member and the block's tile in
// the kernel's own coordinates, so only the members' own tiles are launched:
//   point kernels   a = tile along j, b = tile along i, c = level chunk
//   column solves   a = 128-column segment, b = row index (i - 2)
//   vertical WAF    a = column tile along j, b = tile along i, c = field
//   horizontal WAF  a = tile along j, b = tile along i, c = level - 1
// The lists are built on the host whenever the members or the launch shapes
// change (all values below 2^15: extents <= 32768, levels <= 128, members
// <= 4096, fields <= 24).
struct WorkItem {
  int16_t m, a, b, c;
};
// blockIdx.x of a grid of tiles_j x ti tiles (y: c, z: member) as a work item
__device__ __forceinline__ WorkItem grid_item(int tiles_j) {
  return {(int16_t)blockIdx.z, (int16_t)(blockIdx.x % (unsigned)tiles_j),
          (int16_t)(blockIdx.x / (unsigned)tiles_j), (int16_t)blockIdx.y};
}
__device__ __forceinline__ WorkItem work_item(const WorkItem *wl, int tiles_j) {
  return wl ? wl[blockIdx.x] : grid_item(tiles_j);
}

// Point kernels run one thread per grid point (j, i, k): blocks of
// (blockDim.x, blockDim.y) points along (j, i); grid x = the tiles along j
// times the tiles along i, y = the level, z = the member.  j0, i0 are the
// first j and i the kernel covers.
struct Pt {
  int j, i, k;
};
// Levels one thread of a point kernel runs (its per-thread setup - the
// member's descriptor, roles and 2-D metric - is shared by them); grid y
// counts chunks of this many levels and Pt::k is the chunk's first level.
constexpr int kPtLevels = 4;
__device__ __forceinline__ Pt point_of(int tiles_j, int j0, int i0) {
  const int bj = (int)(blockIdx.x % (unsigned)tiles_j), bi = (int)(blockIdx.x / (unsigned)tiles_j);
  return {bj * (int)blockDim.x + (int)threadIdx.x + j0, bi * (int)blockDim.y + (int)threadIdx.y + i0,
          (int)blockIdx.y * kPtLevels + 1};
}
// the same for the tile of a work item
__device__ __forceinline__ Pt point_at(const WorkItem &w, int j0, int i0) {
  return {(int)w.a * (int)blockDim.x + (int)threadIdx.x + j0,
          (int)w.b * (int)blockDim.y + (int)threadIdx.y + i0, (int)w.c * kPtLevels + 1};
}

// The state with the roles the launch works on.
template <class R>
__host__ __device__ __forceinline__ State<R> state_of(const Dom<R> &D, int uv, int adv) {
  State<R> st;
  st.u = D.u[uv]; st.v = D.v[uv]; st.w = D.w; st.t = D.t; st.tvirt = D.tvirt;
  st.ux = D.ux[adv]; st.vx = D.vx[adv]; st.p = D.p; st.rho = D.rho; st.qsat = D.qsat;
  st.pai = D.pai[adv]; st.tetav = D.tetav[adv]; st.qx = D.qx[adv]; st.trac = D.trac[adv];
  st.ps = D.ps;
  st.tke = D.tke;
  return st;
}

}  // namespace mlc
