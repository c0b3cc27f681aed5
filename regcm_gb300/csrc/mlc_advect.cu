// mlc_advect.cu -- WAF flux-form advection of every advected field
// (Main/mod_moloch.F90:767-1042, subroutines advection and wafone, with the
// interpolations of :1445-1569 and local_flow_param :1571-1590).
//
//   adv_prep        u,v -> ux,vx (4th order, 2nd at the edges) and w -> wx.
//   adv_vertical    per column and field: both vertical WAF passes
//                   (do_vadvtwice) with the column in shared memory.
//   adv_horizontal  per (32 x 8) tile, level and field: meridional then zonal
//                   WAF.  The tile stages wz with a 2-point halo in shared
//                   memory, builds the meridional fluxes and the intermediate
//                   p0 on a 2-column halo, then the zonal fluxes and the
//                   result, so each field is read and written once.  The
//                   result goes to a second buffer because the halo columns
//                   of a tile still need the field's old values.
//   adv_curvature   curvature terms on ux, vx (skipped when they are zero at
//                   every point: with uniform map factors the reference adds
//                   an exact zero).
//   adv_back        ux,vx -> u,v and wx -> w (4th order, 2nd at the edges).
// Operand order follows the reference expression by expression.  The ratios
// dtrdz*fmz/fmzf of the vertical passes are per-domain constants read from
// arrays computed once with the same expression.
#include <type_traits>

#include "mlc_kernels.cuh"
#include "mlc_tma.cuh"

namespace mlc {

namespace {


// Main/mod_moloch.F90:1571-1590; minnum is the 4-byte real holding minden.
template <class R> struct FlowEps;
template <> struct FlowEps<double> {
  static __device__ __forceinline__ double den() { return 1.0e-30; }
  static __device__ __forceinline__ double num() { return (double)1.0e-30f; }
};

// The bit pattern of x through an opaque move, for the sign, region and
// upwind tests that run on the integer pipe: a plain reinterpretation lets the
// compiler turn an integer test of the pattern back into an FP64 comparison
// (an instruction of the 1/64-rate FP64 pipe on GB300)
__device__ __forceinline__ long long bits_of(double x) {
  long long b;
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
  return b;
}

// -x for an FP64 operand of a fused multiply-add, as a flip of the sign bit
// in the integer pipe (exact, like the negation itself), so that no FP64
// instruction forms it (on GB300 every FP64 instruction is 1/64-rate work)
__device__ __forceinline__ double neg_d(double x) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ULL);
}

// x0 + m*(a*b - c*d + e*f) of the horizontal updates.  For FP64 the products
// are fused explicitly (the second and third into fused multiply-adds), so the
// rounding does not depend on how the compiler contracts the expression in
// each tile instantiation: the tile shapes give bit-identical FP64 results.
// FP32 leaves the contraction to the compiler.  rot: m = 1, no product.
// chain: the rotated-pole form is x0 + a*b - c*d + e*f, left to right (the
// zonal update), else x0 + (a*b - c*d + e*f) (the meridional one).
template <class T>
__device__ __forceinline__ T stencil_update(T x0, T m, bool rot, bool chain, T a, T b, T c, T d, T e,
                                            T f) {
  if constexpr (sizeof(T) == sizeof(double)) {
    if (rot && chain) return __fma_rn(e, f, __fma_rn(neg_d(c), d, __fma_rn(a, b, x0)));
    const T t = __fma_rn(e, f, __fma_rn(neg_d(c), d, __dmul_rn(a, b)));
    return __fma_rn(m, t, x0);  // rot: m = 1, x0 + t exactly as the sum
  } else {
    const T z = e * f;
    if (rot && chain) return x0 + a * b - c * d + z;
    return rot ? x0 + (a * b - c * d + z) : x0 + m * (a * b - c * d + z);
  }
}

// The upwind tests zamu >= 0 and zamu > 0.  For FP64 they are made on the
// bit pattern by the integer pipe (each FP64 compare is an instruction of the
// 1/64-rate FP64 pipe on GB300), with the comparisons' exact results for
// -0, infinities and NaN; FP32 compares directly.
template <class T>
__device__ __forceinline__ bool nonneg(T x) {
  if constexpr (sizeof(T) == sizeof(double)) {
    const long long b = bits_of(x);
    return (b >= 0 && b <= 0x7ff0000000000000LL) || b == (long long)0x8000000000000000ULL;
  } else {
    return x >= T(0);
  }
}
template <class T>
__device__ __forceinline__ bool positive(T x) {
  if constexpr (sizeof(T) == sizeof(double)) {
    const long long b = bits_of(x);
    return b > 0 && b <= 0x7ff0000000000000LL;
  } else {
    return x > T(0);
  }
}

// WAF flux  hvel*((1+phi)*a + (1-phi)*c)  with  phi = is + zamu*b - is*b  and
// the limiter  b = max(0, min(2, max(r, min(2r, 1))))  of  r = num/den
// (local_flow_param, Main/mod_moloch.F90:1571-1590; the flux lines
// :877-883, :986-993, :1017-1024).  In every use den = c - a, so
//   (1+phi)*a + (1-phi)*c = (a + c) - phi*den,
//   phi*den = is*den + (zamu - is)*B,   B = b*den.
// With d = |den| > 0 and q = num*sign(den) (so r = q/d), multiplying the
// limiter by d > 0 gives
//   B = sign(den) * max(0, min(2d, max(q, min(2q, d)))),
// whose candidates 0, q, 2q, d, 2d are exact: B is one of 0, 2*num, den, num,
// 2*den exactly, the value of b*den in each region of r, ties included.  No
// division.  FP32 takes the branch-free clamp; FP64 tests the regions of r in
// turn (0, 1/2, 1, 2), which usually stops early - on GB300 each FP64 min, max
// or compare is an instruction of the 1/64-rate FP64 pipe - and keeps the
// reference's guard of denominators below minden exactly.  is = +1 (up) or
// -1 enters as a choice of constants and of den's sign (is*den exactly), not
// as a multiplication.
template <class T>
__device__ __forceinline__ T waf_b(T den, T num) {
  T B;
  if constexpr (sizeof(T) == sizeof(float)) {
    // FP32: the branch-free clamp, signs moved by bit operations; the guard
    // of tiny denominators is left out - it changes B only where
    // |den| < 1e-15, by less than 2|den|, far below FP32 rounding of the
    // flux
    const unsigned sg = __float_as_uint(den) & 0x80000000u;
    const float q = __uint_as_float(__float_as_uint(num) ^ sg);
    const float d = fabsf(den);
    const float bd = fmaxf(0.f, fminf(d + d, fmaxf(q, fminf(q + q, d))));
    B = __uint_as_float(__float_as_uint(bd) ^ sg);
  } else {
    // FP64: the region tests on the integer pipe.  Non-negative doubles order
    // like their bit patterns read as integers, and for a normal d (d >= minden
    // here) d/2 and 2d are d's pattern -/+ 2^52; q = sign(den)*num by a sign-bit
    // XOR.  The tests are the comparisons above exactly (a NaN num fails every
    // comparison and takes the last region in both forms); only the flux itself
    // uses the FP64 pipe.
    const long long bden = bits_of(den), bnum = bits_of(num);
    const long long mag = 0x7fffffffffffffffLL, one_exp = 1LL << 52;
    const long long ad = bden & mag;                    // |den|
    const long long bq = bnum ^ (bden & ~mag);          // q, as a signed pattern
    const long long eden = __double_as_longlong(FlowEps<T>::den());
    const long long enum_ = __double_as_longlong(FlowEps<T>::num());
    if (ad < eden) B = (bnum & mag) < enum_ ? den : T(0);  // r = 1 or r = 0
    else if ((bnum & mag) > 0x7ff0000000000000LL) B = den + den;  // num is NaN
    else if (bq <= 0) B = T(0);                          // q <= 0 (and -0)
    else if (bq < ad - one_exp) B = num + num;           // q < d/2
    else if (bq <= ad) B = den;                          // q <= d
    else if (bq < ad + one_exp) B = num;                 // q < 2d
    else B = den + den;
  }
  return B;
}
template <class T>
__device__ __forceinline__ T waf_flux(T hvel, bool up, T zamu, T a, T c, T num) {
  const T den = c - a;
  const T B = waf_b<T>(den, num);
  if constexpr (sizeof(T) == sizeof(double)) {
    // is*den as a choice of den's sign (no FP64 multiply); the fused
    // multiply-add and the final product are explicit, so that the compiler
    // cannot fuse them into the caller's arithmetic differently in each tile
    // instantiation (the tile shapes give bit-identical results)
    const T sden = up ? den : -den;
    const T zmi = zamu - (up ? T(1) : T(-1));
    return __dmul_rn(hvel, (a + c) - __fma_rn(zmi, B, sden));
  } else {
    const T is = up ? T(1) : T(-1);
    return hvel * ((a + c) - (is * den + (zamu - is) * B));
  }
}
// The same flux as vel*(x - zmih*B) with vel = 2*hvel (the wind itself),
// x = a upwind of a positive zamu (is = +1) else c, and zmih = (zamu - is)/2:
// (a + c) - is*den = 2x exactly, so in exact arithmetic
//   hvel*((a + c) - (is*den + (zamu - is)*B)) = vel*(x - zmih*B),
// one fused multiply-add and one product, with the wind and zmih of an
// interface formed once for every field.
//
// FP64 keeps the doubling out of the FP64 pipe: in the regions where B is
// 2*num or 2*den the flux takes zmi = 2*zmih (exact) as the factor of num or
// den instead, zmih*(2*sel) = zmi*sel exactly, so only the differences, one
// fused multiply-add and one product are FP64 instructions.
__device__ __forceinline__ double waf_sel(double den, double num, bool &dbl) {
  // the regions of waf_b, tested on the bit patterns
  const long long bden = bits_of(den), bnum = bits_of(num);
  const long long mag = 0x7fffffffffffffffLL, one_exp = 1LL << 52;
  const long long ad = bden & mag;
  const long long bq = bnum ^ (bden & ~mag);
  const long long eden = __double_as_longlong(FlowEps<double>::den());
  const long long enum_ = __double_as_longlong(FlowEps<double>::num());
  dbl = false;
  if (ad < eden) return (bnum & mag) < enum_ ? den : 0.0;
  if ((bnum & mag) > 0x7ff0000000000000LL) { dbl = true; return den; }
  if (bq <= 0) return 0.0;
  if (bq < ad - one_exp) { dbl = true; return num; }
  if (bq <= ad) return den;
  if (bq < ad + one_exp) return num;
  dbl = true;
  return den;
}
// a - a for the limiter's region tests: +0 for a finite a, else a NaN (every
// NaN takes the same region), formed on the integer pipe in FP64
template <class T>
__device__ __forceinline__ T self_diff(T a) {
  if constexpr (sizeof(T) == sizeof(double)) {
    const long long b = bits_of(a);
    const long long e = 0x7ff0000000000000LL;
    return (b & e) == e ? __longlong_as_double(0x7ff8000000000000LL) : 0.0;
  } else {
    return a - a;
  }
}
// The same with den = c - a and the upwind value x given (a caller that
// streams the differences of neighbouring interfaces forms each once: an
// interface's den is the num of the interfaces on either side)
template <class T>
__device__ __forceinline__ T waf_flux_d(T vel, bool up, T zmih, T zmi, T x, T den, T num) {
  if constexpr (sizeof(T) == sizeof(double)) {
    bool dbl;
    const double sel = waf_sel(den, num, dbl);
    return __dmul_rn(vel, __fma_rn(neg_d(dbl ? zmi : zmih), sel, x));
  } else {
    (void)zmi;
    const T B = waf_b<T>(den, num);
    return vel * fmaf(-zmih, B, x);
  }
}
template <class T>
__device__ __forceinline__ T waf_flux_h(T vel, bool up, T zmih, T zmi, T a, T c, T num) {
  const T den = c - a;
  const T x = up ? a : c;
  if constexpr (sizeof(T) == sizeof(double)) {
    bool dbl;
    const double sel = waf_sel(den, num, dbl);
    return __dmul_rn(vel, __fma_rn(neg_d(dbl ? zmi : zmih), sel, x));
  } else {
    (void)zmi;
    const T B = waf_b<T>(den, num);
    return vel * fmaf(-zmih, B, x);
  }
}
// zmi = zamu - is and zmih = zmi/2 of an interface (the halving is exact)
template <class T>
__device__ __forceinline__ T waf_zmi(T zamu, bool up) {
  if constexpr (sizeof(T) == sizeof(double)) return __dadd_rn(zamu, up ? -1.0 : 1.0);
  else return zamu - (up ? 1.f : -1.f);
}
template <class T>
__device__ __forceinline__ T waf_zmih(T zamu, bool up) {
  if constexpr (sizeof(T) == sizeof(double)) return __dmul_rn(waf_zmi<T>(zamu, up), 0.5);
  else return waf_zmi<T>(zamu, up) * 0.5f;
}

// The advected fields of a member, in the reference's order (tetav, pai,
// ux, vx, wx, qv, qx(iqfrst:nqx) when ipptls > 0, tkex when ibltyp = 2,
// trac; advection, Main/mod_moloch.F90:781-807).  Table 0 holds the fields of type R: all of
// them in FP64, all but theta_v and Exner in a mixed member, whose two FP64
// fields form table 1.  cur is the field's current half, out the other.
template <class R>
__device__ __forceinline__ int n_table_r(const Dom<R> &D) {
  const int nfix = sizeof(R) == sizeof(double) ? 2 : 0;
  return nfix + 4 + (D.c.ipptls > 0 ? D.g.nqx - 1 : 0) + D.c.tke + D.g.ntr;
}

template <class R>
__device__ __forceinline__ void field_r(const Dom<R> &D, int f, int adv, const R *&cur, R *&out) {
  if (sizeof(R) == sizeof(double)) {
    if (f == 0) { cur = (const R *)D.tetav[adv]; out = (R *)D.tetav[adv ^ 1]; return; }
    if (f == 1) { cur = (const R *)D.pai[adv]; out = (R *)D.pai[adv ^ 1]; return; }
    f -= 2;
  }
  const size_t F = D.g.field3();
  switch (f) {
    case 0: cur = D.ux[adv]; out = D.ux[adv ^ 1]; return;
    case 1: cur = D.vx[adv]; out = D.vx[adv ^ 1]; return;
    case 2: cur = D.wx[adv]; out = D.wx[adv ^ 1]; return;
    case 3: cur = D.qx[adv]; out = D.qx[adv ^ 1]; return;
    default: break;
  }
  f -= 4;
  const int nq = D.c.ipptls > 0 ? D.g.nqx - 1 : 0;
  if (f < nq) {
    cur = D.qx[adv] + (size_t)(f + 1) * F;
    out = D.qx[adv ^ 1] + (size_t)(f + 1) * F;
    return;
  }
  f -= nq;
  if (D.c.tke) {
    if (f == 0) {
      cur = D.tkex[adv];
      out = D.tkex[adv ^ 1];
      return;
    }
    f -= 1;
  }
  cur = D.trac[adv] + (size_t)f * F;
  out = D.trac[adv ^ 1] + (size_t)f * F;
}

// The field set `set` of a member: 0 = the R table, 1 = the FP64 table.
template <class R, class T>
__device__ __forceinline__ void field_t(const Dom<R> &D, int set, int f, int adv, const T *&cur,
                                        T *&out, T *&wz) {
  if constexpr (sizeof(T) == sizeof(R)) {
    const R *c0;
    R *o0;
    field_r<R>(D, f, adv, c0, o0);
    cur = (const T *)c0;
    out = (T *)o0;
    wz = (T *)D.wz[f];
  } else {
    (void)set;
    cur = f == 0 ? D.tetav[adv] : D.pai[adv];
    out = f == 0 ? D.tetav[adv ^ 1] : D.pai[adv ^ 1];
    wz = D.wz_d[f];
  }
}

template <class R>
__global__ void k_adv_prep(const Dom<R> *__restrict__ doms, int uvoff, int advoff, int tiles_j,
    const WorkItem *__restrict__ wl) {
  const WorkItem wi = work_item(wl, tiles_j);
  const Dom<R> &D = doms[wi.m];
  if (!D.active) return;
  const Geom g = D.g;
  const int uv = (D.clk->uv_role + uvoff) & 1, adv = (D.clk->adv_role + advoff) & 1;
  const R *__restrict__ u = D.u[uv];
  const R *__restrict__ v = D.v[uv];
  const R *__restrict__ w = D.w;
  R *__restrict__ ux = D.ux[adv];
  R *__restrict__ vx = D.vx[adv];
  R *__restrict__ wx = D.wx[adv];
  const Pt q_ = point_at(wi, 1, 1);
  const int j = q_.j, k0 = q_.k;
  if (k0 > g.kz) return;
  const int i = q_.i;
  const int jx = g.jx, iy = g.iy, kz = g.kz;
  if (j > jx - 1 || i > iy - 1) return;
  const size_t ij = g.at2(j, i), PS = g.PS, S = (size_t)g.P;
#pragma unroll
  for (int k = k0; k < k0 + kPtLevels && k <= g.kz; ++k) {
    const size_t o = ij + (size_t)(k - 1) * PS;
    // uvstagtouvx :1535-1549
    R a;
    if (j == 1) a = R(0.5) * (u[o] + u[o + 1]);
    else if (j == jx - 1) a = R(0.5) * (u[o + 1] + u[o]);
    else a = R(0.5625) * (u[o + 1] + u[o]) - R(0.0625) * (u[o + 2] + u[o - 1]);
    ux[o] = a;
    // :1553-1566
    if (i == 1) a = R(0.5) * (v[o] + v[o + S]);
    else if (i == iy - 1) a = R(0.5) * (v[o + S] + v[o]);
    else a = R(0.5625) * (v[o + S] + v[o]) - R(0.0625) * (v[o + 2 * S] + v[o - S]);
    vx[o] = a;
    // zstagtoh :1445-1459
    if (k == 1) a = R(0.5) * (w[o + PS] + w[o]);
    else if (k == kz) a = R(0.5) * (w[o + PS] + w[o]);
    else a = R(0.5625) * (w[o + PS] + w[o]) - R(0.0625) * (w[o + 2 * PS] + w[o - PS]);
    wx[o] = a;
    if (D.c.tke) {
      // zstagtoh(tke, tkex) (Main/mod_moloch.F90:782-784)
      const R *__restrict__ tk = D.tke;
      if (k == 1 || k == kz) a = R(0.5) * (tk[o + PS] + tk[o]);
      else a = R(0.5625) * (tk[o + PS] + tk[o]) - R(0.0625) * (tk[o + 2 * PS] + tk[o - PS]);
      D.tkex[adv][o] = a;
    }
    if constexpr (sizeof(R) == sizeof(double)) {
      // the vertical WAF update's factor s(k)*zu(k) - s(k+1)*zd(k), and the
      // flux factors of interface k+1 - zamu = s*dtrdz, zmi = zamu - is and
      // zmih = zmi/2 - once for all fields (FP64 arithmetic is the FP64
      // path's bound)
      const double skp = D.s[o + PS];
      D.vdiv[o] = __fma_rn(neg_d(skp), D.sa.zrfmd[o], __dmul_rn(D.s[o], D.sa.zrfmu[o]));
      const double dtrdz = 0.5 * (D.c.dtstepa * D.c.rdzita);
      const double zamu = __dmul_rn(skp, dtrdz);
      const double zmi = waf_zmi<double>(zamu, nonneg(zamu));
      D.vzamu[o] = zamu;
      D.vzmi[o] = zmi;
      D.vzmih[o] = __dmul_rn(zmi, 0.5);
    }
  }
}

// Two vertical WAF passes (do_vadvtwice, :858-922), one thread per column
// and field, streaming the levels upward through registers.  Pass 1's flux
// at interface k+1 needs the input at levels k-1..k+2 and its update at k the
// fluxes at k and k+1; pass 2 needs pass 1's output at m-1..m+2, so it runs
// two levels behind pass 1 in the same loop.  Every value is loaded once and
// the column never touches shared memory.  R is the type of the winds and
// metric, T that of the advected field and of the arithmetic.  Fluxes and
// updates are the reference's expressions, operand for operand.
template <class T>
__device__ __forceinline__ T vflux(T dtrdz, T skp, T cm1, T ck, T cp1, T cp2, int k, int kz) {
  // interface k+1 between levels k and k+1; the upwind difference col(k1) -
  // col(k1p1) with the reference's clamps k1p1 = min(k+2, kz), k1 = max(k-1, 1)
  const T zamu = skp * dtrdz;
  const bool up = nonneg(zamu);
  T num;
  if (up) num = k + 2 <= kz ? cp1 - cp2 : cp1 - cp1;
  else num = k >= 2 ? cm1 - ck : ck - ck;
  const T zmi = waf_zmi<T>(zamu, up);
  return waf_flux_h<T>(skp, up, zmi * T(0.5), zmi, cp1, ck, num);
}
// the same with the interface's factors given (an FP64 member, k_adv_prep)
struct VIf {
  double zamu, zmih, zmi;
};
__device__ __forceinline__ double vflux_p(double skp, const VIf &t, double cm1, double ck, double cp1,
                                          double cp2, int k, int kz) {
  const bool up = nonneg(t.zamu);
  double num;
  if (up) num = k + 2 <= kz ? cp1 - cp2 : cp1 - cp1;
  else num = k >= 2 ? cm1 - ck : ck - ck;
  return waf_flux_h<double>(skp, up, t.zmih, t.zmi, cp1, ck, num);
}
template <class T>
__device__ __forceinline__ T vupdate(T pk, T fb, T fa, T sk, T skp, T zu, T zd) {
  const T zdv = (sk * zu - skp * zd) * pk;
  return pk - fb * zu + fa * zd + zdv;
}
// the same with the factor sk*zu - skp*zd given (FP64: from adv_prep), the
// products fused explicitly
template <class T>
__device__ __forceinline__ T vupdate_f(T pk, T fb, T fa, T dv, T zu, T zd) {
  return __fma_rn(dv, pk, __fma_rn(fa, zd, __fma_rn(neg_d(fb), zu, pk)));
}

// Blocks of 256 threads an SM the vertical WAF is compiled for, FP64 and FP32
// (0: no bound, the compiler's own register choice).
#ifndef MLC_VERT_MINB_D
#define MLC_VERT_MINB_D 0
#endif
#ifndef MLC_VERT_MINB_F
#define MLC_VERT_MINB_F 4
#endif
template <class T>
constexpr int vert_min_blocks() {
  return sizeof(T) == sizeof(double) ? (MLC_VERT_MINB_D > 0 ? MLC_VERT_MINB_D : 1) : MLC_VERT_MINB_F;
}
// Levels an FP32 column loads ahead of the one it computes (1 or 2; two
// measured no faster on the moist 512x512x41 step, 0.256 ms a step both).
#ifndef MLC_VPF_F
#define MLC_VPF_F 1
#endif
// grid: x = column tiles along j times the fields (field fastest, so the
// blocks reading one column's s and metric run together), y = row tiles,
// z = member; block (vert_x, vert_y) columns along (j, i)
template <class R, class T>
__global__ void __launch_bounds__(256, vert_min_blocks<T>())
    k_adv_vertical(const Dom<R> *__restrict__ doms, int nf, int set, int advoff,
                               const WorkItem *__restrict__ wl) {
  constexpr int kVpf = sizeof(T) == sizeof(float) ? MLC_VPF_F : 1;  // levels loaded ahead
  const WorkItem wi = wl ? wl[blockIdx.x]
                          : WorkItem{(int16_t)blockIdx.z, (int16_t)(blockIdx.x / (unsigned)nf),
                                     (int16_t)blockIdx.y, (int16_t)(blockIdx.x % (unsigned)nf)};
  const Dom<R> &D = doms[wi.m];
  if (!D.active) return;
  const int f = wi.c;
  const int bj = wi.a;
  if (set == 0 && f >= n_table_r(D)) return;  // a member with fewer species
  const Geom g = D.g;
  const int kz = g.kz;
  const int j = bj * (int)blockDim.x + (int)threadIdx.x + 1;
  const int i = (int)wi.b * (int)blockDim.y + (int)threadIdx.y + 1;
  if (j > g.jx - 1 || i > g.iy - 1) return;
  const Scal &c = D.c;
  const int adv = (D.clk->adv_role + advoff) & 1;
  const T *src;
  T *outp, *dst;
  field_t<R, T>(D, set, f, adv, src, outp, dst);
  (void)outp;
  const size_t ij = g.at2(j, i);
  src += ij;
  dst += ij;
  const R *__restrict__ sp = D.s + ij;
  const R *__restrict__ zup = D.sa.zrfmu + ij;
  const R *__restrict__ zdp = D.sa.zrfmd + ij;
  const unsigned PS = (unsigned)g.PS;  // a domain's fields stay below 2^31 elements
  const T dtrdz = T(0.5) * (pick<T>(c.dtstepa, c.dtstepaf) * pick<T>(c.rdzita, c.rdzitaf));

  // windows: pass-1 input at k-1..k+2, pass-1 output at k-3..k-1, s at
  // k-2..k+1, metric at k-2..k-1, the pass-1 flux at interface k and the
  // pass-2 flux at interface k-2
  T c0m1 = T(0), c0k = src[0], c0p1 = src[PS];
  T c1m3 = T(0), c1m2 = T(0), c1m1 = T(0);
  T sm2 = T(0), sm1 = T(0), sk = T(sp[0]);
  T zum2 = T(0), zdm2 = T(0), zum1 = T(0), zdm1 = T(0);
  T f1k = T(0), f2m = T(0);
  // differences c(k) - c(k+1) of the pass-1 input at interfaces k-1, k (d1p,
  // d1c) and of the pass-2 input at m-1, m (d2p, d2c): an interface's den is
  // the num of its neighbours, so each difference is formed once
  T d1p = T(0), d1c = T(0), d2p = T(0), d2c = T(0);
  // FP64 member: the update's divergence factor, precomputed per level
  constexpr bool kPre = sizeof(R) == sizeof(double) && sizeof(T) == sizeof(double);
  const double *__restrict__ dvp = kPre ? D.vdiv + ij : nullptr;
  T dvm2 = T(0), dvm1 = T(0), n_dv = kPre ? T(dvp[0]) : T(0);
  // FP64 member: the interface factors (zamu, hvel, zmi) of interfaces k+1,
  // k and k-1 (pass 1 at k, pass 2 at k-2), the next level's loaded ahead
  const double *__restrict__ zap = kPre ? D.vzamu + ij : nullptr;
  const double *__restrict__ zmp = kPre ? D.vzmih + ij : nullptr;
  const double *__restrict__ z2p = kPre ? D.vzmi + ij : nullptr;
  VIf tkm1{0, 0, 0}, tkm2{0, 0, 0};
  VIf n_t = kPre ? VIf{zap[0], zmp[0], z2p[0]} : VIf{0, 0, 0};
  // the next level's loads, issued one level ahead (kVpf = 2: the level
  // after it too, in m_*)
  T n_s = T(sp[PS]), n_c = src[2 * PS], n_zu = T(zup[0]), n_zd = T(zdp[0]);
  T m_s = T(0), m_c = T(0), m_zu = T(0), m_zd = T(0), m_dv = T(0);
  VIf m_t{0, 0, 0};
  if constexpr (kVpf == 2) {
    if (kz >= 2) {
      m_s = T(sp[2 * PS]);
      m_zu = T(zup[PS]);
      m_zd = T(zdp[PS]);
      if constexpr (kPre) {
        m_dv = T(dvp[PS]);
        m_t = VIf{zap[PS], zmp[PS], z2p[PS]};
      }
    }
    if (kz >= 4) m_c = src[3 * PS];
  }
  // level k; every bound check is known to hold inside the column
  // (4 <= k <= kz-3, kz-4 with two levels ahead), so the interior steps
  // carry none
  auto step = [&](int k, auto interior) {
    constexpr bool I = decltype(interior)::value;
    const unsigned o = (unsigned)(k - 1) * PS;
    const T skp1 = n_s, c0p2 = (I || k + 2 <= kz) ? n_c : T(0), zuk = n_zu, zdk = n_zd;
    const T dvk = n_dv;
    const VIf tk = n_t;
    if constexpr (kVpf == 2) {
      // the level after next: s at k+3, the metric at k+2, c at k+4
      n_s = m_s; n_zu = m_zu; n_zd = m_zd; n_c = m_c;
      if constexpr (kPre) { n_dv = m_dv; n_t = m_t; }
      if (I || k + 2 <= kz) {
        if constexpr (kPre) {
          m_dv = T(dvp[o + 2 * PS]);
          m_t = VIf{zap[o + 2 * PS], zmp[o + 2 * PS], z2p[o + 2 * PS]};
        }
        m_s = T(sp[o + 3 * PS]);
        m_zu = T(zup[o + 2 * PS]);
        m_zd = T(zdp[o + 2 * PS]);
        if (I || k + 4 <= kz) m_c = src[o + 4 * PS];
      }
    } else if (I || k < kz) {
      if constexpr (kPre) {
        n_dv = T(dvp[o + PS]);
        n_t = VIf{zap[o + PS], zmp[o + PS], z2p[o + PS]};
      }
      n_s = T(sp[o + 2 * PS]);
      n_zu = T(zup[o + PS]);
      n_zd = T(zdp[o + PS]);
      if (I || k + 3 <= kz) n_c = src[o + 3 * PS];
    }
    T f1kp;
    const T d1n = c0p1 - c0p2;  // the next interface's den, this one's upwind num
    if constexpr (kPre) {
      if (I) {
        const bool up = nonneg(tk.zamu);
        f1kp = waf_flux_d<double>(skp1, up, tk.zmih, tk.zmi, up ? c0p1 : c0k, d1c, up ? d1n : d1p);
      } else {
        f1kp = k <= kz - 1 ? vflux_p(skp1, tk, c0m1, c0k, c0p1, c0p2, k, kz) : T(0);
      }
    } else if (I) {
      const T zamu = skp1 * dtrdz;
      const bool up = nonneg(zamu);
      const T zmi = waf_zmi<T>(zamu, up);
      f1kp = waf_flux_d<T>(skp1, up, zmi * T(0.5), zmi, up ? c0p1 : c0k, d1c, up ? d1n : d1p);
    } else {
      f1kp = k <= kz - 1 ? vflux<T>(dtrdz, skp1, c0m1, c0k, c0p1, c0p2, k, kz) : T(0);
    }
    T c1k;
    if constexpr (kPre) c1k = vupdate_f<T>(c0k, f1k, f1kp, dvk, zuk, zdk);
    else c1k = vupdate<T>(c0k, f1k, f1kp, sk, skp1, zuk, zdk);
    const T d2n = c1m1 - c1k;
    if (I || k >= 3) {  // pass 2 at level m = k-2
      T f2n;
      if constexpr (kPre) {
        if (I) {
          const bool up = nonneg(tkm2.zamu);
          f2n = waf_flux_d<double>(sm1, up, tkm2.zmih, tkm2.zmi, up ? c1m1 : c1m2, d2c, up ? d2n : d2p);
        } else {
          f2n = vflux_p(sm1, tkm2, c1m3, c1m2, c1m1, c1k, k - 2, kz);
        }
      } else if (I) {
        const T zamu = sm1 * dtrdz;
        const bool up = nonneg(zamu);
        const T zmi = waf_zmi<T>(zamu, up);
        f2n = waf_flux_d<T>(sm1, up, zmi * T(0.5), zmi, up ? c1m1 : c1m2, d2c, up ? d2n : d2p);
      } else {
        f2n = vflux<T>(dtrdz, sm1, c1m3, c1m2, c1m1, c1k, k - 2, kz);
      }
      if constexpr (kPre) dst[o - 2 * PS] = vupdate_f<T>(c1m2, f2m, f2n, dvm2, zum2, zdm2);
      else dst[o - 2 * PS] = vupdate<T>(c1m2, f2m, f2n, sm2, sm1, zum2, zdm2);
      f2m = f2n;
    }
    c0m1 = c0k; c0k = c0p1; c0p1 = c0p2;
    c1m3 = c1m2; c1m2 = c1m1; c1m1 = c1k;
    d1p = d1c; d1c = d1n; d2p = d2c; d2c = d2n;
    sm2 = sm1; sm1 = sk; sk = skp1;
    zum2 = zum1; zdm2 = zdm1; zum1 = zuk; zdm1 = zdk;
    dvm2 = dvm1; dvm1 = dvk;
    tkm2 = tkm1; tkm1 = tk;
    f1k = f1kp;
  };
  using edge = std::integral_constant<bool, false>;
  using mid = std::integral_constant<bool, true>;
  const int k1 = min(3, kz), k2 = max(4, kz - (kVpf == 2 ? 3 : 2));
  for (int k = 1; k <= k1; ++k) step(k, edge{});
#pragma unroll 4
  for (int k = 4; k < k2; ++k) step(k, mid{});
  for (int k = k2; k <= kz; ++k) step(k, edge{});
  // pass 2 at levels kz-1 (flux through interface kz) and kz (none above)
  const unsigned ot = (unsigned)(kz - 1) * PS;
  T f2n;
  if constexpr (kPre) f2n = vflux_p(sm1, tkm2, c1m3, c1m2, c1m1, c1m1, kz - 1, kz);
  else f2n = vflux<T>(dtrdz, sm1, c1m3, c1m2, c1m1, c1m1, kz - 1, kz);
  if constexpr (kPre) {
    dst[ot - PS] = vupdate_f<T>(c1m2, f2m, f2n, dvm2, zum2, zdm2);
    dst[ot] = vupdate_f<T>(c1m1, f2n, T(0), dvm1, zum1, zdm1);
  } else {
    dst[ot - PS] = vupdate<T>(c1m2, f2m, f2n, sm2, sm1, zum2, zdm2);
    dst[ot] = vupdate<T>(c1m1, f2n, T(0), sm1, sk, zum1, zdm1);
  }
}

// ---- lane vectors ---------------------------------------------------------
template <int B> struct VecOf;
template <> struct VecOf<4> { using t = unsigned; };
template <> struct VecOf<8> { using t = uint2; };
template <> struct VecOf<16> { using t = uint4; };

// v consecutive elements at p, which is aligned to min(v * sizeof(T), 16)
template <class T, int V>
__device__ __forceinline__ void ld_vec(T (&x)[V], const T *p) {
  constexpr int B = V * (int)sizeof(T);
  if constexpr (B <= 16) {
    const typename VecOf<B>::t w = *reinterpret_cast<const typename VecOf<B>::t *>(p);
    memcpy(x, &w, B);
  } else {
#pragma unroll
    for (int h = 0; h < B / 16; ++h) {
      const uint4 w = reinterpret_cast<const uint4 *>(p)[h];
      memcpy(reinterpret_cast<char *>(x) + 16 * h, &w, 16);
    }
  }
}
template <class T, int V>
__device__ __forceinline__ void st_vec(T *p, const T (&x)[V]) {
  constexpr int B = V * (int)sizeof(T);
  if constexpr (B <= 16) {
    typename VecOf<B>::t w;
    memcpy(&w, x, B);
    *reinterpret_cast<typename VecOf<B>::t *>(p) = w;
  } else {
#pragma unroll
    for (int h = 0; h < B / 16; ++h) {
      uint4 w;
      memcpy(&w, reinterpret_cast<const char *>(x) + 16 * h, 16);
      reinterpret_cast<uint4 *>(p)[h] = w;
    }
  }
}
// the lane's v elements of row r (1-based) of a plane, or zeros
template <class T, int V>
__device__ __forceinline__ void ld_row(T (&x)[V], const T *plane, int e0, int r, unsigned P, bool ok) {
  if (ok) {
    ld_vec<T, V>(x, plane + (unsigned)e0 + (unsigned)(r - 1) * P);
  } else {
#pragma unroll
    for (int q = 0; q < V; ++q) x[q] = T(0);
  }
}
// element q+1 of the lane's columns: the lane's own, or the next lane's first
template <class T, int V>
__device__ __forceinline__ void next_col(T (&e)[V], const T (&x)[V]) {
#pragma unroll
  for (int q = 0; q + 1 < V; ++q) e[q] = x[q + 1];
  e[V - 1] = __shfl_down_sync(0xffffffffu, x[0], 1);
}

// Meridional then zonal WAF at one level for a tile of nw rows, every field
// of the R table (:984-1038; ROTLLR :926-983).  Warp w owns row I0+w; lane l
// owns v consecutive columns of it.  The winds, Courant numbers and metric
// coefficients of the lane's points are formed once, in registers, and then
// for each field in turn: its halo tile (rows I0-2 .. I0+nw+1, landed by TMA,
// double-buffered) gives the meridional fluxes of the warp's row, shared
// with the row above through shared memory (the last warp also forms the
// flux of row I0+nw); the intermediate p0 follows; the zonal fluxes take
// their neighbours' p0 from the adjacent lanes by shuffles, and the result
// goes to the field's other buffer (the halo of other tiles still needs the
// old values).  A warp's range is 32*v columns, of which it writes the
// middle 32*v - 4 (a column's zonal update needs p0 two columns either
// side); tiles overlap by four columns.  Per field the expressions are the
// reference's, operand for operand.
// Resident warps an SM the WAF tile kernels are compiled for; the register
// budget follows (65536 / (32 * warps) a thread).  Measured on the moist
// 512x512x41 step: FP32 horizontal WAF at 40 warps (48 registers, 12 bytes
// spilled) 0.455 ms a step, at 32 (64 registers) 0.464, at 16 warps (90
// registers) 0.72; the increment form at 32
// warps (64 registers, 32 bytes spilled) 0.27 against 0.29 at 24 and 0.37 at
// 20.  FP64 at 16 warps (128 registers): the FP64 pipe is the bound, but 8
// warps an SM leave it idle (6.98 against 7.83 ms).
#ifndef MLC_HWAF_WARPS
#define MLC_HWAF_WARPS 40
#endif
#ifndef MLC_HWAF_WARPS_D
#define MLC_HWAF_WARPS_D 16
#endif
#ifndef MLC_HINC_WARPS
#define MLC_HINC_WARPS 32
#endif
template <class R>
constexpr int waf_min_blocks(int warps, int nw) {
  return warps / nw > 1 ? warps / nw : 1;
}
template <class R, int V, int NW>
__global__ void __launch_bounds__(32 * NW, waf_min_blocks<R>(sizeof(R) == sizeof(float)
                                                                   ? MLC_HWAF_WARPS
                                                                   : MLC_HWAF_WARPS_D, NW))
    k_adv_horizontal(const Dom<R> *__restrict__ doms,
                                                           int tiles_j, int uvoff, int advoff,
    const WorkItem *__restrict__ wl) {
  using T = R;
  constexpr int W = 32 * V;       // columns of a warp's range
  constexpr int S = W - 4;        // columns it writes: range columns 2 .. W-3
  constexpr int OB0 = hshape_ob0(V);
  constexpr int OFF = hshape_off((int)sizeof(T), V);
  constexpr int BW = W + 2 * OFF;  // halo tile row: range column c sits at c + OFF
  constexpr unsigned kBox = (unsigned)((NW + 4) * BW * sizeof(T));
  constexpr unsigned kBuf = (kBox + 127u) / 128u * 128u;
  constexpr int kStages = 4;  // halo tiles in flight: the next three fields land while one is used
  constexpr int shape = V == 1 ? (NW == 8 ? 0 : 3) : (NW == 8 ? 1 : 2);
  static_assert(hshape((int)sizeof(T), shape).v == V && hshape((int)sizeof(T), shape).nw == NW,
                "tile shape table");
  __shared__ __align__(128) unsigned char wzraw[kStages][kBuf];  // TMA destinations
  __shared__ __align__(16) T zp_s[2][NW + 1][W];           // meridional fluxes, rows I0 .. I0+NW
  __shared__ __align__(8) uint64_t mbar[kStages];
  __shared__ const T *cur_s[kMaxFields];                   // each field's current and other half
  __shared__ T *out_s[kMaxFields];
  // grid: x = tiles along j and i, y = level, z = member
  const WorkItem wi = work_item(wl, tiles_j);
  const Dom<R> &D = doms[wi.m];
  if (!D.active) return;
  const int k = wi.c + 1;
  const Geom g = D.g;
  const int jx = g.jx, iy = g.iy;
  if (k > g.kz) return;
  const int bj = wi.a, bi = wi.b;
  const int ob = bj * S + OB0;  // column offset (j - 1) of the range's first column
  const int I0 = bi * NW + 1;
  if (ob + 3 > jx - 1 || I0 > iy - 1) return;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const int uv = (D.clk->uv_role + uvoff) & 1, adv = (D.clk->adv_role + advoff) & 1;
  const int lane = (int)(threadIdx.x & 31u), wp = (int)(threadIdx.x >> 5);
  const int tid = (int)threadIdx.x;
  const int i = I0 + wp;
  const int e0 = ob + V * lane;                  // column offset of the lane's first column
  const bool inrow = e0 >= 0 && e0 + V <= g.P;   // the lane's columns lie inside a row
  const unsigned P = (unsigned)g.P;
  const unsigned ko = (unsigned)(k - 1) * (unsigned)g.PS;  // a field stays below 2^31 elements
  const T *__restrict__ uk = D.u[uv] + ko;
  const T *__restrict__ vk = D.v[uv] + ko;
  const T dta = pick<T>(c.dtstepa, c.dtstepaf);
  const T dtrdx = dta * pick<T>(c.rdx, c.rdxf), dtrdy = dta * pick<T>(c.rdx, c.rdxf);
  const bool rot = c.lrotllr != 0;
  const int nf = n_table_r(D);
  const char *tmaps = static_cast<const char *>(D.tmap) + (size_t)shape * kTmapSlots * kTmapBytes;
  auto tile = [&](int b) { return reinterpret_cast<T(*)[BW]>(wzraw[b]); };
  auto issue = [&](int fld, int b) {  // one thread: the halo tile of field fld into buffer b
    fence_proxy_async();
    mbar_expect_tx(&mbar[b], kBox);
    tma_load_3d(wzraw[b], tmaps + (size_t)fld * kTmapBytes, ob - OFF, I0 - 3, k - 1, &mbar[b]);
  };
  if (tid == 0) {
    for (int q = 0; q < kStages; ++q) mbar_init(&mbar[q], 1);
    fence_mbar_init();
  }
  if (tid < nf) {
    const T *cur0;
    T *out0, *wz0;
    field_t<R, T>(D, 0, tid, adv, cur0, out0, wz0);
    cur_s[tid] = cur0 + ko;
    out_s[tid] = out0 + ko;
  }
  __syncthreads();
  if (D.stall_polls > 0) {
    // test hook: wait on a barrier that no copy completes (none is issued
    // yet), give up after the member's poll count and record the fault the
    // way the tile waits below do; the block leaves with nothing in flight
    const bool landed = mbar_wait_polls(&mbar[0], 0u, D.stall_polls);
    if (__syncthreads_or(!landed) && tid == 0) atomicOr(&D.clk->fault, 1);
    return;
  }
  if (tid == 0)
    for (int q = 0; q < kStages && q < nf; ++q) issue(q, q);

  // ---- the lane's coefficients (while the first tiles land) ----
  int jq[V];
#pragma unroll
  for (int q = 0; q < V; ++q) jq[q] = e0 + q + 1;
  const bool rowM = i >= 2 && i <= iy - 1;  // meridional flux rows
  const bool rowP = i >= 2 && i <= iy - 2;  // p0, zonal flux and update rows
  const bool okM = inrow && rowM, okP = inrow && rowP;
  // The fluxes of row I0+NW (the tile's north face): with two columns a lane
  // the last two warps take 32 columns each, one a lane, so that no warp
  // forms more than three flux rows' worth before the block barrier (the
  // last warp alone would form four); with one column a lane the last warp
  // takes them.  ec0 is the range column of the lane's first one there.
  constexpr int VE = V == 2 && NW >= 2 ? 1 : V;
  const bool eWarp = VE == 1 && V == 2 ? wp >= NW - 2 : wp == NW - 1;
  const int ec0 = VE == 1 && V == 2 ? (wp - (NW - 2)) * 32 + lane : V * lane;
  const int eE0 = ob + ec0;
  T vv[V], zmy[V], vve[VE], zmye[VE];
  bool mv[V], me[VE];  // meridional flux defined at the column (row i, row I0+NW)
  {
    T a[V], b[V];
    ld_row<T, V>(a, vk, e0, i, P, okM);
    ld_row<T, V>(b, sa.msfv, e0, i, P, okM && !rot);
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const bool ok = okM && jq[q] >= 1 && jq[q] <= jx - 1;
      mv[q] = ok;
      vv[q] = ok ? a[q] : T(0);  // the flux's wind v (= 2*hvel)
      zmy[q] = ok ? (rot ? a[q] * dtrdy : a[q] * b[q] * dtrdy) : T(0);
    }
    const int ie = I0 + NW;
    const bool okE = eWarp && eE0 >= 0 && eE0 + VE <= g.P && ie >= 2 && ie <= iy - 1;
    T ae[VE], be[VE];
    ld_row<T, VE>(ae, vk, eE0, ie, P, okE);
    ld_row<T, VE>(be, sa.msfv, eE0, ie, P, okE && !rot);
#pragma unroll
    for (int q = 0; q < VE; ++q) {
      const int je = eE0 + q + 1;
      const bool ok = okE && je >= 1 && je <= jx - 1;
      me[q] = ok;
      vve[q] = ok ? ae[q] : T(0);
      zmye[q] = ok ? (rot ? ae[q] * dtrdy : ae[q] * be[q] * dtrdy) : T(0);
    }
  }
  T zs[V], zn[V], dvy[V], m2[V], uu[V], zmx[V], zw[V], ze[V], dvx[V];
  bool pv[V], xv[V], rv[V];  // p0, zonal flux, interior update defined at the column
  {
    T fz[V], vi[V], vn[V], ri[V], rn[V], fi[V], fn[V], mf[V], ui[V], rmui[V], msu[V];
    ld_row<T, V>(fz, sa.fmz + ko, e0, i, P, okP);
    ld_row<T, V>(vi, vk, e0, i, P, okP);
    ld_row<T, V>(vn, vk, e0, i + 1, P, okP);
    ld_row<T, V>(ri, sa.rmv, e0, i, P, okP);
    ld_row<T, V>(rn, sa.rmv, e0, i + 1, P, okP);
    ld_row<T, V>(fi, (rot ? sa.rfmzv : sa.rfmzu) + ko, e0, i, P, okP);
    ld_row<T, V>(fn, (rot ? sa.rfmzv : sa.rfmzu) + ko, e0, i + 1, P, okP);
    ld_row<T, V>(mf, rot ? sa.msfx : sa.mx2, e0, i, P, okP);
    ld_row<T, V>(ui, uk, e0, i, P, okP);
    ld_row<T, V>(rmui, sa.rmu, e0, i, P, okP && !rot);
    ld_row<T, V>(msu, sa.msfu, e0, i, P, okP);
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const int j = jq[q];
      pv[q] = okP && j >= 1 && j <= jx - 1;
      xv[q] = okP && j >= 2 && j <= jx - 1;
      rv[q] = okP && j >= 2 && j <= jx - 2;
      if (rot) {
        const T zhxvtn = dtrdy * rn[q] * mf[q];
        const T zhxvts = dtrdy * ri[q] * mf[q];
        zn[q] = zhxvtn * fz[q] * fn[q];
        zs[q] = zhxvts * fz[q] * fi[q];
        dvy[q] = vn[q] * zn[q] - vi[q] * zs[q];
        m2[q] = T(1);
      } else {
        // rfmzu as in the reference (Main/mod_moloch.F90:1000-1001)
        zn[q] = dtrdy * fz[q] * fn[q];
        zs[q] = dtrdy * fz[q] * fi[q];
        dvy[q] = vn[q] * rn[q] * zn[q] - vi[q] * ri[q] * zs[q];
        m2[q] = mf[q];
      }
      uu[q] = xv[q] ? ui[q] : T(0);  // the zonal flux's wind u (= 2*hvel)
      zmx[q] = xv[q] ? ui[q] * msu[q] * dtrdx : T(0);
    }
    // the zonal update also needs u, rfmzu and rmu one column east
    T fzu[V], fze[V], ue[V], rme[V];
    ld_row<T, V>(fzu, sa.rfmzu + ko, e0, i, P, okP);
    next_col<T, V>(fze, fzu);
    next_col<T, V>(ue, ui);
    next_col<T, V>(rme, rmui);
#pragma unroll
    for (int q = 0; q < V; ++q) {
      if (rot) {
        const T zcostx = dtrdx * mf[q];
        zw[q] = zcostx * fz[q] * fzu[q];
        ze[q] = zcostx * fz[q] * fze[q];
        dvx[q] = ue[q] * ze[q] - ui[q] * zw[q];
      } else {
        zw[q] = dtrdx * fz[q] * fzu[q];
        ze[q] = dtrdx * fz[q] * fze[q];
        dvx[q] = ue[q] * rme[q] * ze[q] - ui[q] * rmui[q] * zw[q];
      }
    }
  }
  // the three fluxes' factors in the form vel*(x - zmih*B), once for every
  // field: the upwind flags (zamu > 0) and zmih
  bool upy[V], upe[VE], upx[V];
  T z2y[V], z2e[VE], z2x[V];  // zmi = 2*zmih (FP64 only)
#pragma unroll
  for (int q = 0; q < V; ++q) {
    upy[q] = positive(zmy[q]);
    upx[q] = positive(zmx[q]);
    z2y[q] = waf_zmi<T>(zmy[q], upy[q]);
    z2x[q] = waf_zmi<T>(zmx[q], upx[q]);
    zmy[q] = z2y[q] * T(0.5);
    zmx[q] = z2x[q] * T(0.5);
  }
#pragma unroll
  for (int q = 0; q < VE; ++q) {
    upe[q] = positive(zmye[q]);
    z2e[q] = waf_zmi<T>(zmye[q], upe[q]);
    zmye[q] = z2e[q] * T(0.5);
  }
  // rows of the halo tile (global row r at tile row r - I0 + 2) the upwind
  // differences use, with the reference's clamps ih = min(i+1, imax),
  // ihm1 = max(ih-1, imin)
  auto mrows = [&](int r, int &ta, int &tb, int &tc) {
    ta = max(r - 2, 1) - I0 + 2;
    const int rb = min(r + 1, iy - 1);
    tb = rb - I0 + 2;
    tc = max(rb - 1, 1) - I0 + 2;
  };
  int tA, tB, tC, eA, eB, eC;
  mrows(i, tA, tB, tC);
  mrows(I0 + NW, eA, eB, eC);
  // columns the lane may write: range columns 2 .. W-3 inside the domain
  bool wv[V];
  bool wall = true;
#pragma unroll
  for (int q = 0; q < V; ++q) {
    const int cc = V * lane + q;
    wv[q] = inrow && i <= iy - 1 && cc >= 2 && cc <= W - 3 && jq[q] >= 1 && jq[q] <= jx - 1;
    wall = wall && wv[q];
  }
  const bool rowin = inrow && i <= iy - 1;

  for (int f = 0; f < nf; ++f) {
    const T *pp = cur_s[f];
    T *out = out_s[f];
    // the field's old values at the lane's points, in flight during the
    // meridional pass
    T ppk[V];
    ld_row<T, V>(ppk, pp, e0, i, P, rowin);
    const int b = f % kStages;
    const bool landed = mbar_wait_bounded(&mbar[b], (unsigned)((f / kStages) & 1));
    T(*wt)[BW] = tile(b);
    T(*zp)[W] = zp_s[f & 1];
    // meridional fluxes zpby(j,i): j in jce, i in ici1..ice2
    T wzi[V];
    {
      T wa[V], wA[V], wB[V], wC[V], x[V];
      ld_vec<T, V>(wa, &wt[i - I0 + 1][OFF + V * lane]);
      ld_vec<T, V>(wzi, &wt[i - I0 + 2][OFF + V * lane]);
      ld_vec<T, V>(wA, &wt[tA][OFF + V * lane]);
      ld_vec<T, V>(wB, &wt[tB][OFF + V * lane]);
      ld_vec<T, V>(wC, &wt[tC][OFF + V * lane]);
#pragma unroll
      for (int q = 0; q < V; ++q) {
        const bool up = upy[q];
        const T y = waf_flux_h<T>(vv[q], up, zmy[q], z2y[q], wa[q], wzi[q],
                                  (up ? wa[q] : wB[q]) - (up ? wA[q] : wC[q]));
        x[q] = mv[q] ? y : T(0);  // zero outside the flux points
      }
      st_vec<T, V>(&zp[wp][V * lane], x);
      if (eWarp) {
        T xa[VE], xc[VE], eA_[VE], eB_[VE], eC_[VE], xe[VE];
        ld_vec<T, VE>(xa, &wt[NW + 1][OFF + ec0]);
        ld_vec<T, VE>(xc, &wt[NW + 2][OFF + ec0]);
        ld_vec<T, VE>(eA_, &wt[eA][OFF + ec0]);
        ld_vec<T, VE>(eB_, &wt[eB][OFF + ec0]);
        ld_vec<T, VE>(eC_, &wt[eC][OFF + ec0]);
#pragma unroll
        for (int q = 0; q < VE; ++q) {
          const bool up = upe[q];
          const T y = waf_flux_h<T>(vve[q], up, zmye[q], z2e[q], xa[q], xc[q],
                                    (up ? xa[q] : eB_[q]) - (up ? eA_[q] : eC_[q]));
          xe[q] = me[q] ? y : T(0);
        }
        st_vec<T, VE>(&zp[NW][ec0], xe);
      }
    }
    if (__syncthreads_or(!landed)) {
      if (tid == 0) {
        atomicOr(&D.clk->fault, 1);
        // let copies still in flight land before the shared memory is released
        for (int g2 = f; g2 < f + kStages && g2 < nf; ++g2)
          mbar_wait_bounded(&mbar[g2 % kStages], (unsigned)((g2 / kStages) & 1));
      }
      return;
    }
    // buffer b is read for the last time above: fetch the field kStages on
    if (tid == 0 && f + kStages < nf) issue(f + kStages, b);
    // p0(j,i): j in jce, i in ici
    T p0[V];
    {
      T ys[V], yn[V];
      ld_vec<T, V>(ys, &zp[wp][V * lane]);
      ld_vec<T, V>(yn, &zp[wp + 1][V * lane]);
#pragma unroll
      for (int q = 0; q < V; ++q) {
        const T x = stencil_update<T>(wzi[q], m2[q], rot, false, ys[q], zs[q], yn[q], zn[q], dvy[q], ppk[q]);
        p0[q] = pv[q] ? x : T(0);
      }
    }
    // zonal fluxes zpbw(j,i): j in jci1..jce2, i in ici; p0 at range
    // columns c-2 .. c+1 (the lane's own, two from the lane to the west, one
    // from the lane to the east)
    T pw1 = __shfl_up_sync(0xffffffffu, p0[V - 1], 1);
    auto p0at = [&](int q) -> T {  // p0 of lane column q, q in -1 .. V-1
      return q < 0 ? pw1 : p0[q];
    };
    // differences p0(c) - p0(c-1) at the lane's columns, and those of the
    // columns either side from the neighbouring lanes: a column's den is the
    // num of its neighbours (upwind the one to the west, downwind the east)
    T dq[V];
#pragma unroll
    for (int q = 0; q < V; ++q) dq[q] = p0at(q) - p0at(q - 1);
    const T dw = __shfl_up_sync(0xffffffffu, dq[V - 1], 1);
    const T de = __shfl_down_sync(0xffffffffu, dq[0], 1);
    auto dat = [&](int q) -> T { return q < 0 ? dw : q >= V ? de : dq[q]; };
    T zx[V];
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const int j = jq[q];
      const bool up = upx[q];
      const T a = p0at(q - 1), cq = p0at(q);
      // jhm1 = max(j-2, jmin) upwind; jh = min(j+1, jmax) downwind:
      // upwind a - p0(jhm1), which is a - a at j = 2; downwind p0(jh) - p0(jh-1)
      const T num = up ? (j == 2 ? self_diff<T>(a) : dat(q - 1)) : (j == jx - 1 ? dq[q] : dat(q + 1));
      const T x = waf_flux_d<T>(uu[q], up, zmx[q], z2x[q], up ? a : cq, dq[q], num);
      zx[q] = xv[q] ? x : T(0);
    }
    T zxe[V];
    next_col<T, V>(zxe, zx);
    // result: interior update, ring copied
    T res[V];
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const T x = stencil_update<T>(p0[q], m2[q], rot, true, zx[q], zw[q], zxe[q], ze[q], dvx[q], ppk[q]);
      res[q] = rv[q] ? x : ppk[q];
    }
    if (wall) {
      st_vec<T, V>(out + (unsigned)e0 + (unsigned)(i - 1) * P, res);
    } else if (rowin) {
#pragma unroll
      for (int q = 0; q < V; ++q)
        if (wv[q]) out[(unsigned)(e0 + q) + (unsigned)(i - 1) * P] = res[q];
    }
  }
}

// Species that are not advected (ipptls = 0: qx(iqfrst:nqx)) keep their
// values when the advected fields move to the other half of their pairs.
template <class R>
__global__ void k_species_copy(const Dom<R> *__restrict__ doms, int advoff, int tiles_j,
    const WorkItem *__restrict__ wl) {
  const WorkItem wi = work_item(wl, tiles_j);
  const Dom<R> &D = doms[wi.m];
  if (!D.active) return;
  const Geom g = D.g;
  const Pt q = point_at(wi, 1, 1);
  if (D.c.ipptls > 0 || q.j > g.jx - 1 || q.i > g.iy - 1 || q.k > g.kz) return;
  const int adv = (D.clk->adv_role + advoff) & 1;
  const size_t F = g.field3();
#pragma unroll
  for (int k = q.k; k < q.k + kPtLevels && k <= g.kz; ++k) {
    const size_t o = g.at(q.j, q.i, k);
    for (int n = 1; n < g.nqx; ++n) D.qx[adv ^ 1][o + (size_t)n * F] = D.qx[adv][o + (size_t)n * F];
  }
}

// :809-825
template <class R>
__global__ void k_adv_curvature(const Dom<R> *__restrict__ doms, int advoff, int tiles_j,
    const WorkItem *__restrict__ wl) {
  const WorkItem wi = work_item(wl, tiles_j);
  const Dom<R> &D = doms[wi.m];
  if (!D.active || !D.c.curvature) return;
  const Geom g = D.g;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const int adv = (D.clk->adv_role + advoff) & 1;
  R *__restrict__ ux = D.ux[adv];
  R *__restrict__ vx = D.vx[adv];
  const Pt q_ = point_at(wi, 2, 2);
  const int j = q_.j, k0 = q_.k;
  if (k0 > g.kz) return;
  const int i = q_.i;
  if (j > g.jx - 2 || i > g.iy - 2) return;
  const size_t ij = g.at2(j, i);
  const R dta = pick<R>(c.dtstepa, c.dtstepaf);
  R tanx, tany;
  if (c.lrotllr) {
    const double dlat = kDegrad * 0.5 * (sa.rlat[i - 1] + sa.rlat[i]);
    tanx = R(sin(dlat)) * sa.msfx[ij] * R(kRearthRad);
    tany = tanx;
  } else {
    tanx = (sa.msfu[ij - 1] - sa.msfu[ij]) * pick<R>(c.rdx, c.rdxf);
    tany = (sa.msfv[ij - (size_t)g.P] - sa.msfv[ij]) * pick<R>(c.rdx, c.rdxf);
  }
#pragma unroll
  for (int k = k0; k < k0 + kPtLevels && k <= g.kz; ++k) {
    const size_t o = ij + (size_t)(k - 1) * g.PS;
    R a = ux[o];
    const R b = vx[o];
    a = a + a * b * tanx * dta;
    ux[o] = a;
    vx[o] = b - a * a * tany * dta;
  }
}

// uvxtouvstag :1477-1522 and htozstag :1461-1475
template <class R>
__global__ void k_adv_back(const Dom<R> *__restrict__ doms, int uvoff, int advoff, int tiles_j,
    const WorkItem *__restrict__ wl) {
  const WorkItem wi = work_item(wl, tiles_j);
  const Dom<R> &D = doms[wi.m];
  if (!D.active) return;
  const Geom g = D.g;
  const int uv = (D.clk->uv_role + uvoff) & 1, adv = (D.clk->adv_role + advoff) & 1;
  const R *__restrict__ ux = D.ux[adv];
  const R *__restrict__ vx = D.vx[adv];
  const R *__restrict__ wx = D.wx[adv];
  R *__restrict__ u = D.u[uv];
  R *__restrict__ v = D.v[uv];
  R *__restrict__ w = D.w;
  const Pt q_ = point_at(wi, 1, 1);
  const int j = q_.j, k0 = q_.k;
  if (k0 > g.kz) return;
  const int i = q_.i;
  const int jx = g.jx, iy = g.iy, kz = g.kz;
  if (j > jx || i > iy) return;
  const size_t ij = g.at2(j, i), PS = g.PS, S = (size_t)g.P;
  const bool do_u = (j >= 2 && j <= jx - 1 && i >= 2 && i <= iy - 2);
  const bool do_v = (j >= 2 && j <= jx - 2 && i >= 2 && i <= iy - 1);
  const bool do_w = (j <= jx - 1 && i <= iy - 1);
#pragma unroll
  for (int k = k0; k < k0 + kPtLevels && k <= g.kz; ++k) {
    const size_t o = ij + (size_t)(k - 1) * PS;
    if (do_u) {
      R a;
      if (j == jx - 1) a = R(0.5) * (ux[o - 1] + ux[o]);
      else if (j == 2) a = R(0.5) * (ux[o] + ux[o - 1]);
      else a = R(0.5625) * (ux[o] + ux[o - 1]) - R(0.0625) * (ux[o + 1] + ux[o - 2]);
      u[o] = a;
    }
    if (do_v) {
      R a;
      if (i == iy - 1) a = R(0.5) * (vx[o - S] + vx[o]);
      else if (i == 2) a = R(0.5) * (vx[o] + vx[o - S]);
      else a = R(0.5625) * (vx[o] + vx[o - S]) - R(0.0625) * (vx[o + S] + vx[o - 2 * S]);
      v[o] = a;
    }
    if (do_w && k >= 2) {
      R a;
      if (k == 2) a = R(0.5) * (wx[o] + wx[o - PS]);
      else if (k == kz) a = R(0.5) * (wx[o] + wx[o - PS]);
      else a = R(0.5625) * (wx[o] + wx[o - PS]) - R(0.0625) * (wx[o + PS] + wx[o - 2 * PS]);
      w[o] = a;
      if (D.c.tke) {
        // htozstag(tkex, tke) (Main/mod_moloch.F90:831-834)
        const R *__restrict__ tx = D.tkex[adv];
        if (k == 2 || k == kz) a = R(0.5) * (tx[o] + tx[o - PS]);
        else a = R(0.5625) * (tx[o] + tx[o - PS]) - R(0.0625) * (tx[o + PS] + tx[o - 2 * PS]);
        D.tke[o] = a;
      }
    }
  }
}

// ---- increment form for the FP64 fields (theta_v, Exner) of a mixed member --
//
// The WAF update is linear in the advected field once the limiter regions
// are fixed, and the regions depend on differences only.  So every flux can
// be formed from values relative to a reference r:
//   F(a - r, c - r, num) = F(a, c, num) - 2*hvel*r,
// and a cell's update relative to its own value needs only neighbour
// differences and the cell's own increment, all small numbers that FP32
// carries to ~1e-7 of the increment (not of the field).  FP64 is left for the
// neighbour differences, for the terms where the scheme does not preserve a
// constant field (the model top of the vertical pass, where the flux through
// kz+1 is zero but s(kz+1) is not; non-uniform map factors in the horizontal
// passes) and for the final sum field + increment.  Fluxes are formed once
// per interface, relative to the cell below (south, west) of it, and moved to
// the other cell's reference by -2*hvel*(its value - the first cell's).

// Both vertical passes (Main/mod_moloch.F90:858-922) in increment form, one
// thread per column, streaming the levels upward like k_adv_vertical with
// pass 2 two levels behind pass 1.  e is the pass input's increment over the
// field (zero for pass 1), dzs(k) = field(k+1) - field(k).  The flux through
// interface k+1 is formed relative to cell k and moved to cell k+1 by
// -s(k+1)*dzs(k).  Writes the increment dz = (field after the passes) -
// field, as a double-float: the bottom and top cells carry a double-float
// constant part (no flux through levels 1 and kz+1, where s need not vanish).
__device__ __forceinline__ float vflux_inc(float dtrdz, float skp, float em1, float ek, float ekp1,
                                           float ekp2, float dzm1, float dzk, float dzp1, int k,
                                           int kz) {
  const float zamu = skp * dtrdz;
  const bool up = zamu >= 0.f;
  float num;
  if (up) num = k + 2 <= kz ? (ekp1 - ekp2) - dzp1 : 0.f;
  else num = k >= 2 ? (em1 - ek) - dzm1 : 0.f;
  return waf_flux<float>(0.5f * skp, up, zamu, dzk + ekp1, ek, num);
}
// the cell update without the bottom/top constant parts; flb is the flux
// through interface k (relative to cell k-1), fla the flux through k+1
__device__ __forceinline__ float vupdate_inc(float ek, float flb, float fla, float sk, float skp,
                                             float zu, float zd, float dzm1, int k, int kz) {
  const float fb = k >= 2 ? flb - sk * dzm1 : 0.f;
  const float fa = k <= kz - 1 ? fla : 0.f;
  return -fb * zu + fa * zd + (sk * zu - skp * zd) * ek;
}

template <class R>
__global__ void k_adv_vertical_inc(const Dom<R> *__restrict__ doms, int advoff,
                                   const WorkItem *__restrict__ wl) {
  const WorkItem wi = wl ? wl[blockIdx.x]
                          : WorkItem{(int16_t)blockIdx.z, (int16_t)(blockIdx.x >> 1), (int16_t)blockIdx.y,
                                     (int16_t)(blockIdx.x & 1u)};
  const Dom<R> &D = doms[wi.m];
  if (!D.active) return;
  const int f = wi.c;
  const int bj = wi.a;
  const Geom g = D.g;
  const int kz = g.kz;
  const int j = bj * (int)blockDim.x + (int)threadIdx.x + 1;
  const int i = (int)wi.b * (int)blockDim.y + (int)threadIdx.y + 1;
  if (j > g.jx - 1 || i > g.iy - 1) return;
  const Scal &c = D.c;
  const int adv = (D.clk->adv_role + advoff) & 1;
  const size_t F = g.field3();
  const size_t ij = g.at2(j, i);
  // double-float planes: offsets count floats of the hi plane
  const DF src0(f == 0 ? D.tetav[adv] : D.pai[adv], F);
  const DF dst0(D.wz_d[f], F);
  const DF src{src0.p + ij, F};
  const DF dst{dst0.p + ij, F};
  const R *__restrict__ sp = D.s + ij;
  const R *__restrict__ zup = D.sa.zrfmu + ij;
  const R *__restrict__ zdp = D.sa.zrfmd + ij;
  const unsigned PS = (unsigned)g.PS;
  const float dtrdz = 0.5f * (c.dtstepaf * c.rdzitaf);

  // the bottom cell's and top cell's FP32 parts and double-float constant parts
  float eb32 = 0.f, et32 = 0.f;
  F2 hb{0.f, 0.f}, ht{0.f, 0.f};
  const F2 src1 = src.ld(0);
  // windows: field at k+1, dzs at k-3..k, pass-1 output at k-3..k-1, s at
  // k-2..k+1, metric at k-2..k-1, pass-1 flux at k (relative to k-1), pass-2
  // flux at k-2
  F2 xp1 = src.ld(PS);
  float dm3 = 0.f, dm2 = 0.f, dm1 = 0.f, dk = df_diff(xp1, src1);
  float e1m3 = 0.f, e1m2 = 0.f, e1m1 = 0.f;
  float sm2 = 0.f, sm1 = 0.f, sk = float(sp[0]);
  float zum2 = 0.f, zdm2 = 0.f, zum1 = 0.f, zdm1 = 0.f;
  float f1k = 0.f, f2m = 0.f;
  unsigned o = 0;
  F2 n_x = src.ld(2 * PS);
  float n_s = float(sp[PS]), n_zu = float(zup[0]), n_zd = float(zdp[0]);
  for (int k = 1; k <= kz; ++k, o += PS) {
    const float skp1 = n_s, zuk = n_zu, zdk = n_zd;
    const F2 xp2 = n_x;  // field at k+2 (k+2 <= kz)
    if (k < kz) {
      n_s = float(sp[o + 2 * PS]);
      n_zu = float(zup[o + PS]);
      n_zd = float(zdp[o + PS]);
      if (k + 3 <= kz) n_x = src.ld(o + 3 * PS);
    }
    const float dp1 = k + 2 <= kz ? df_diff(xp2, xp1) : 0.f;  // dzs(k+1)
    // pass 1 (input increment zero)
    const float f1kp = k <= kz - 1 ? vflux_inc(dtrdz, skp1, 0.f, 0.f, 0.f, 0.f, dm1, dk, dp1, k, kz) : 0.f;
    const float u1 = vupdate_inc(0.f, f1k, f1kp, sk, skp1, zuk, zdk, dm1, k, kz);
    float e1k;
    if (k == kz) {
      et32 += u1;
      ht = df_add(ht, df_mul(src.ld(o), two_prod(-skp1, zdk)));
      e1k = et32 + df_f(ht);
    } else if (k == 1) {
      eb32 += u1;
      hb = df_add(hb, df_mul(src1, two_prod(sk, zuk)));
      e1k = eb32 + df_f(hb);
    } else {
      e1k = 0.f + u1;
    }
    if (k >= 3) {  // pass 2 at level m = k-2
      const int m = k - 2;
      const float f2n = vflux_inc(dtrdz, sm1, e1m3, e1m2, e1m1, e1k, dm3, dm2, dm1, m, kz);
      const float u2 = vupdate_inc(e1m2, f2m, f2n, sm2, sm1, zum2, zdm2, dm3, m, kz);
      F2 d;
      if (m == 1) {
        eb32 += u2;
        hb = df_add(hb, df_mul(src1, two_prod(sm2, zum2)));
        d = df_add_f(hb, eb32);
      } else {
        d = F2{e1m2 + u2, 0.f};
      }
      dst.st(o - 2 * PS, d);
      f2m = f2n;
    }
    dm3 = dm2; dm2 = dm1; dm1 = dk; dk = dp1;
    xp1 = xp2;
    e1m3 = e1m2; e1m2 = e1m1; e1m1 = e1k;
    sm2 = sm1; sm1 = sk; sk = skp1;
    zum2 = zum1; zdm2 = zdm1; zum1 = zuk; zdm1 = zdk;
    f1k = f1kp;
  }
  // pass 2 at levels kz-1 and kz; dm3 = dzs(kz-2), dm2 = dzs(kz-1) now
  const unsigned ot = (unsigned)(kz - 1) * PS;
  const float f2n = vflux_inc(dtrdz, sm1, e1m3, e1m2, e1m1, 0.f, dm3, dm2, dm1, kz - 1, kz);
  const float u2 = vupdate_inc(e1m2, f2m, f2n, sm2, sm1, zum2, zdm2, dm3, kz - 1, kz);
  dst.st(ot - PS, F2{e1m2 + u2, 0.f});
  const float ut = vupdate_inc(e1m1, f2n, 0.f, sm1, sk, zum1, zdm1, dm2, kz, kz);
  et32 += ut;
  ht = df_add(ht, df_mul(src.ld(ot), two_prod(-sk, zdm1)));
  dst.st(ot, df_add_f(ht, et32));
}

// Meridional then zonal WAF (:984-1038; ROTLLR :926-983) in increment form
// for theta_v and Exner of a mixed member, at one level for a tile of nw rows,
// with the lane geometry of k_adv_horizontal: warp w owns row I0+w, lane l
// owns v consecutive columns, coefficients in registers, the meridional
// fluxes shared between rows through shared memory and the zonal neighbours
// taken from adjacent lanes.  pp is the field at the start of the advection
// step (double-float), dz its vertical increment; out = pp + dz + (meridional
// + zonal increments).  Fluxes are formed relative to the cell south (west)
// of the interface, from FP32 increments and neighbour differences.
template <class R, int V, int NW>
__global__ void __launch_bounds__(32 * NW, waf_min_blocks<R>(MLC_HINC_WARPS, NW))
    k_adv_horizontal_inc(const Dom<R> *__restrict__ doms,
                                                               int tiles_j, int uvoff,
                                                               int advoff,
                                                               const WorkItem *__restrict__ wl) {
  constexpr int W = 32 * V, S = W - 4;
  constexpr int OB0 = hshape_ob0(V);
  constexpr int OFF = hshape_off(4, V);
  constexpr int BW = W + 2 * OFF;  // tile row: range column c sits at c + OFF
  constexpr unsigned kBox = (unsigned)((NW + 4) * BW * 4);
  constexpr unsigned kBuf = (kBox + 127u) / 128u * 128u;
  constexpr int shape = V == 1 ? 0 : 1;
  static_assert(hshape_inc(shape).v == V && hshape_inc(shape).nw == NW, "tile shape table");
  // per field: the halo tiles (rows I0-2 .. I0+NW+1) of pp hi, pp lo, dz hi,
  // dz lo, landed by TMA, all issued at the start
  __shared__ __align__(128) unsigned char tiles[2][4][kBuf];
  __shared__ __align__(16) float fy_s[2][NW + 1][W];  // meridional fluxes, rows I0 .. I0+NW
  __shared__ __align__(8) uint64_t mbar[2];
  const WorkItem wi = work_item(wl, tiles_j);
  const Dom<R> &D = doms[wi.m];
  if (!D.active) return;
  const int k = wi.c + 1;
  const Geom g = D.g;
  const int jx = g.jx, iy = g.iy;
  if (k > g.kz) return;
  const int bj = wi.a, bi = wi.b;
  const int ob = bj * S + OB0;
  const int I0 = bi * NW + 1;
  if (ob + 3 > jx - 1 || I0 > iy - 1) return;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const int uv = (D.clk->uv_role + uvoff) & 1, adv = (D.clk->adv_role + advoff) & 1;
  const int lane = (int)(threadIdx.x & 31u), wp = (int)(threadIdx.x >> 5);
  const int i = I0 + wp;
  const int e0 = ob + V * lane;
  const bool inrow = e0 >= 0 && e0 + V <= g.P;
  const unsigned P = (unsigned)g.P;
  const unsigned ko = (unsigned)(k - 1) * (unsigned)g.PS;
  const size_t F = g.field3();
  const float *__restrict__ uk = D.u[uv] + ko;
  const float *__restrict__ vk = D.v[uv] + ko;
  const float dta = c.dtstepaf;
  const float dtrdx = dta * c.rdxf, dtrdy = dta * c.rdxf;
  const bool rot = c.lrotllr != 0;
  using T = float;
  const int tid = (int)threadIdx.x;
  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) {
    const char *tm = static_cast<const char *>(D.tmap) + ((size_t)shape * kTmapSlots + kMaxFields) * kTmapBytes;
    for (int f = 0; f < 2; ++f) {
      mbar_expect_tx(&mbar[f], 4u * kBox);
      const int pslot = 4 * f + 2 * adv, dslot = 8 + 2 * f;
      const int slot[4] = {pslot, pslot + 1, dslot, dslot + 1};
      for (int q = 0; q < 4; ++q)
        tma_load_3d(tiles[f][q], tm + (size_t)slot[q] * kTmapBytes, ob - OFF, I0 - 3, k - 1, &mbar[f]);
    }
  }

  int jq[V];
#pragma unroll
  for (int q = 0; q < V; ++q) jq[q] = e0 + q + 1;
  const bool rowM = i >= 2 && i <= iy - 1;
  const bool rowP = i >= 2 && i <= iy - 2;
  const bool okM = inrow && rowM, okP = inrow && rowP;
  const int ie = I0 + NW;
  const bool okE = wp == NW - 1 && inrow && ie >= 2 && ie <= iy - 1;
  // ---- coefficients ----
  T vv[V], zmy[V], vve[V], zmye[V];
  bool mv[V], me[V];
  {
    T a[V], b[V];
    ld_row<T, V>(a, vk, e0, i, P, okM);
    ld_row<T, V>(b, sa.msfv, e0, i, P, okM && !rot);
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const bool ok = okM && jq[q] >= 1 && jq[q] <= jx - 1;
      mv[q] = ok;
      vv[q] = ok ? a[q] : T(0);
      zmy[q] = ok ? (rot ? a[q] * dtrdy : a[q] * b[q] * dtrdy) : T(0);
    }
    ld_row<T, V>(a, vk, e0, ie, P, okE);
    ld_row<T, V>(b, sa.msfv, e0, ie, P, okE && !rot);
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const bool ok = okE && jq[q] >= 1 && jq[q] <= jx - 1;
      me[q] = ok;
      vve[q] = ok ? a[q] : T(0);
      zmye[q] = ok ? (rot ? a[q] * dtrdy : a[q] * b[q] * dtrdy) : T(0);
    }
  }
  T zs[V], zn[V], vsv[V], cy[V], m2[V], uu[V], zmx[V], zw[V], ze[V], uwv[V], cx[V];
  bool pv[V], xv[V], rv[V], cyf[V], cxf[V];
  {
    T fz[V], vi[V], vn[V], ri[V], rn[V], fi[V], fn[V], mf[V], ui[V], rmui[V], msu[V];
    ld_row<T, V>(fz, sa.fmz + ko, e0, i, P, okP);
    ld_row<T, V>(vi, vk, e0, i, P, okP);
    ld_row<T, V>(vn, vk, e0, i + 1, P, okP);
    ld_row<T, V>(ri, sa.rmv, e0, i, P, okP);
    ld_row<T, V>(rn, sa.rmv, e0, i + 1, P, okP);
    ld_row<T, V>(fi, (rot ? sa.rfmzv : sa.rfmzu) + ko, e0, i, P, okP);
    ld_row<T, V>(fn, (rot ? sa.rfmzv : sa.rfmzu) + ko, e0, i + 1, P, okP);
    ld_row<T, V>(mf, rot ? sa.msfx : sa.mx2, e0, i, P, okP);
    ld_row<T, V>(ui, uk, e0, i, P, okP);
    ld_row<T, V>(rmui, sa.rmu, e0, i, P, okP && !rot);
    ld_row<T, V>(msu, sa.msfu, e0, i, P, okP);
    T fzu[V], fze[V], ue[V], rme[V];
    ld_row<T, V>(fzu, sa.rfmzu + ko, e0, i, P, okP);
    next_col<T, V>(fze, fzu);
    next_col<T, V>(ue, ui);
    next_col<T, V>(rme, rmui);
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const int j = jq[q];
      pv[q] = okP && j >= 1 && j <= jx - 1;
      xv[q] = okP && j >= 2 && j <= jx - 1;
      rv[q] = okP && j >= 2 && j <= jx - 2;
      vsv[q] = vi[q];
      uwv[q] = ui[q];
      if (rot) {
        const T zhxvtn = dtrdy * rn[q] * mf[q];
        const T zhxvts = dtrdy * ri[q] * mf[q];
        zn[q] = zhxvtn * fz[q] * fn[q];
        zs[q] = zhxvts * fz[q] * fi[q];
        m2[q] = T(1);
        cyf[q] = false;
        cy[q] = T(0);
        const T zcostx = dtrdx * mf[q];
        zw[q] = zcostx * fz[q] * fzu[q];
        ze[q] = zcostx * fz[q] * fze[q];
        cxf[q] = false;
        cx[q] = T(0);
      } else {
        zn[q] = dtrdy * fz[q] * fn[q];
        zs[q] = dtrdy * fz[q] * fi[q];
        m2[q] = mf[q];
        // the map-factor terms a constant field does not cancel
        cyf[q] = ri[q] != 1.f || rn[q] != 1.f;
        cy[q] = mf[q] * (vi[q] * zs[q] * (1.f - ri[q]) - vn[q] * zn[q] * (1.f - rn[q]));
        zw[q] = dtrdx * fz[q] * fzu[q];
        ze[q] = dtrdx * fz[q] * fze[q];
        cxf[q] = rmui[q] != 1.f || rme[q] != 1.f;
        cx[q] = mf[q] * (ui[q] * zw[q] * (1.f - rmui[q]) - ue[q] * ze[q] * (1.f - rme[q]));
      }
      uu[q] = xv[q] ? ui[q] : T(0);
      zmx[q] = xv[q] ? ui[q] * msu[q] * dtrdx : T(0);
    }
  }
  const bool rowin = inrow && i <= iy - 1;
  bool wv[V];
  bool wall = true;
#pragma unroll
  for (int q = 0; q < V; ++q) {
    const int cc = V * lane + q;
    wv[q] = rowin && cc >= 2 && cc <= W - 3 && jq[q] >= 1 && jq[q] <= jx - 1;
    wall = wall && wv[q];
  }
  // the meridional flux through the south face of row r (relative to pp(r-1))
  // from dz and pp differences of rows r-2 .. r+1; the reference's clamps
  // ih = min(r+1, imax), ihm1 = max(ih-1, imin)
  auto mflux = [&](T (&x)[V], const T (&vvr)[V], const T (&zm)[V], const bool (&ok)[V], int r,
                   const T (&zm2)[V], const T (&zm1)[V], const T (&z0)[V], const T (&zp1)[V],
                   const T (&dym2)[V], const T (&dym1)[V], const T (&dy0)[V]) {
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const bool up = zm[q] > 0.f;
      float num;
      if (up) num = r >= 3 ? (zm1[q] - zm2[q]) + dym2[q] : (zm1[q] - zm1[q]) + 0.f;
      else num = r <= iy - 2 ? (zp1[q] - z0[q]) + dy0[q] : (z0[q] - zm1[q]) + dym1[q];
      const float y = waf_flux<float>(0.5f * vvr[q], up, zm[q], zm1[q], z0[q] + dym1[q], num);
      x[q] = ok[q] ? y : 0.f;
    }
  };

  for (int f = 0; f < 2; ++f) {
    float *outh = reinterpret_cast<float *>(f == 0 ? D.tetav[adv ^ 1] : D.pai[adv ^ 1]);
    float (*fy)[W] = fy_s[f];
    const bool landed = mbar_wait_bounded(&mbar[f], 0u);
    const float(*tph)[BW] = reinterpret_cast<const float(*)[BW]>(tiles[f][0]);
    const float(*tpl)[BW] = reinterpret_cast<const float(*)[BW]>(tiles[f][1]);
    const float(*tzh)[BW] = reinterpret_cast<const float(*)[BW]>(tiles[f][2]);
    const float(*tzl)[BW] = reinterpret_cast<const float(*)[BW]>(tiles[f][3]);
    const int cl = OFF + V * lane;
    // rows i-2 .. i+1 (tile rows wp .. wp+3) of pp (hi, lo) and dz (rounded
    // to FP32); zero outside the cross points
    T ph[4][V], pl[4][V], zz[4][V], dzi_h[V], dzi_l[V];
#pragma unroll
    for (int rr = 0; rr < 4; ++rr) {
      ld_vec<T, V>(ph[rr], &tph[wp + rr][cl]);
      ld_vec<T, V>(pl[rr], &tpl[wp + rr][cl]);
      T zh[V], zl[V];
      ld_vec<T, V>(zh, &tzh[wp + rr][cl]);
      ld_vec<T, V>(zl, &tzl[wp + rr][cl]);
#pragma unroll
      for (int q = 0; q < V; ++q) zz[rr][q] = zh[q] + zl[q];
      if (rr == 2) {
#pragma unroll
        for (int q = 0; q < V; ++q) { dzi_h[q] = zh[q]; dzi_l[q] = zl[q]; }
      }
    }
    // dy(r) = pp(r+1) - pp(r) for r = i-2, i-1, i
    T dy[3][V];
#pragma unroll
    for (int rr = 0; rr < 3; ++rr)
#pragma unroll
      for (int q = 0; q < V; ++q)
        dy[rr][q] = (ph[rr + 1][q] - ph[rr][q]) + (pl[rr + 1][q] - pl[rr][q]);
    {
      T x[V];
      mflux(x, vv, zmy, mv, i, zz[0], zz[1], zz[2], zz[3], dy[0], dy[1], dy[2]);
      st_vec<T, V>(&fy[wp][V * lane], x);
    }
    if (wp == NW - 1) {  // the flux of row I0+NW: rows ie-2 .. ie+1 = i-1 .. i+2
      T h4[V], l4[V], zh[V], zl[V], z4[V], dy3[V];
      ld_vec<T, V>(h4, &tph[NW + 3][cl]);
      ld_vec<T, V>(l4, &tpl[NW + 3][cl]);
      ld_vec<T, V>(zh, &tzh[NW + 3][cl]);
      ld_vec<T, V>(zl, &tzl[NW + 3][cl]);
#pragma unroll
      for (int q = 0; q < V; ++q) {
        z4[q] = zh[q] + zl[q];
        dy3[q] = (h4[q] - ph[3][q]) + (l4[q] - pl[3][q]);
      }
      T x[V];
      mflux(x, vve, zmye, me, ie, zz[1], zz[2], zz[3], z4, dy[1], dy[2], dy3);
      st_vec<T, V>(&fy[NW][V * lane], x);
    }
    if (__syncthreads_or(!landed)) {
      if (tid == 0) {
        atomicOr(&D.clk->fault, 1);
        // let copies still in flight land before the shared memory is released
        mbar_wait_bounded(&mbar[f], 0u);
        if (f == 0) mbar_wait_bounded(&mbar[1], 0u);
      }
      return;
    }
    // p0 - pp: ey = dz + hy, hy the meridional increment
    T hy[V], ey[V];
    {
      T ys[V], yn[V];
      ld_vec<T, V>(ys, &fy[wp][V * lane]);
      ld_vec<T, V>(yn, &fy[wp + 1][V * lane]);
#pragma unroll
      for (int q = 0; q < V; ++q) {
        const float fs = ys[q] - vsv[q] * dy[1][q];  // moved to pp(i)
        const float fn = yn[q];
        float h = m2[q] * (fs * zs[q] - fn * zn[q]);
        if (rot) h = fs * zs[q] - fn * zn[q];
        else if (cyf[q]) h += ph[2][q] * cy[q];
        hy[q] = pv[q] ? h : 0.f;
        ey[q] = zz[2][q] + hy[q];
      }
    }
    // dx(j) = pp(j+1) - pp(j) at row i for the lane's columns; the east
    // neighbour's pp from the next lane
    T dx[V], dxw2, dxw1;
    {
      T eh[V], el[V];
      next_col<T, V>(eh, ph[2]);
      next_col<T, V>(el, pl[2]);
#pragma unroll
      for (int q = 0; q < V; ++q) dx[q] = (eh[q] - ph[2][q]) + (el[q] - pl[2][q]);
      dxw2 = __shfl_up_sync(0xffffffffu, dx[V >= 2 ? V - 2 : 0], V >= 2 ? 1 : 2);
      dxw1 = __shfl_up_sync(0xffffffffu, dx[V - 1], 1);
    }
    const float ew2 = __shfl_up_sync(0xffffffffu, ey[V >= 2 ? V - 2 : 0], V >= 2 ? 1 : 2);
    const float ew1 = __shfl_up_sync(0xffffffffu, ey[V - 1], 1);
    const float ee1 = __shfl_down_sync(0xffffffffu, ey[0], 1);
    auto eyat = [&](int q) -> float {
      return q == -2 ? ew2 : q == -1 ? ew1 : q == V ? ee1 : ey[q < 0 ? 0 : q >= V ? V - 1 : q];
    };
    auto dxat = [&](int q) -> float {
      return q == -2 ? dxw2 : q == -1 ? dxw1 : dx[q < 0 ? 0 : q >= V ? V - 1 : q];
    };
    // zonal fluxes at the lane's columns, relative to pp(j-1)
    T fx[V];
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const int j = jq[q];
      const bool up = zmx[q] > 0.f;
      const float a = eyat(q - 1), cq = eyat(q);
      float num;
      if (up) num = j >= 3 ? (a - eyat(q - 2)) + dxat(q - 2) : (a - a) + 0.f;
      else num = j <= jx - 2 ? (eyat(q + 1) - cq) + dxat(q) : (cq - a) + dxat(q - 1);
      const float y = waf_flux<float>(0.5f * uu[q], up, zmx[q], a, cq + dxat(q - 1), num);
      fx[q] = xv[q] ? y : 0.f;
    }
    T fxe[V];
    next_col<T, V>(fxe, fx);
    // result
    T rh[V], rl[V];
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const F2 ppk{ph[2][q], pl[2][q]};
      F2 x = ppk;
      if (rv[q]) {
        const float fw = fx[q] - uwv[q] * dxat(q - 1);  // moved to pp(j)
        const float fe = fxe[q];
        float hx;
        if (rot) {
          hx = fw * zw[q] - fe * ze[q];
        } else {
          hx = m2[q] * (fw * zw[q] - fe * ze[q]);
          if (cxf[q]) hx += ppk.hi * cx[q];
        }
        x = df_add_f(df_add(ppk, F2{dzi_h[q], dzi_l[q]}), hy[q] + hx);
      }
      rh[q] = x.hi;
      rl[q] = x.lo;
    }
    float *oh = outh + ko + (unsigned)(i - 1) * P;
    if (wall) {
      st_vec<T, V>(oh + (unsigned)e0, rh);
      st_vec<T, V>(oh + F + (unsigned)e0, rl);
    } else if (rowin) {
#pragma unroll
      for (int q = 0; q < V; ++q)
        if (wv[q]) {
          oh[(unsigned)(e0 + q)] = rh[q];
          oh[F + (unsigned)(e0 + q)] = rl[q];
        }
    }
  }
}

// grid of a point kernel over nj x ni points per level
inline dim3 pt_grid(const LaunchGeom &L, int nj, int ni, int &tiles_j) {
  tiles_j = (nj + L.col_x - 1) / L.col_x;
  if (L.wl_pt) return dim3((unsigned)L.n_pt, 1, 1);  // one block per work item
  const int ti = (ni + L.col_y - 1) / L.col_y;
  return dim3((unsigned)(tiles_j * ti), (unsigned)((L.kz + kPtLevels - 1) / kPtLevels),
              (unsigned)L.nmem);
}

}  // namespace

template <class R>
void Launch<R>::adv_prep(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s) {
  const dim3 b((unsigned)L.col_x, (unsigned)L.col_y);
  int tj;
  const dim3 grd = pt_grid(L, L.jx - 1, L.iy - 1, tj);
  k_adv_prep<R><<<grd, b, 0, s>>>(d, uvoff, advoff, tj, L.wl_pt);
}

template <class R, class T>
void launch_vertical(const LaunchGeom &L, const Dom<R> *d, int nf, int set, int advoff,
                     cudaStream_t s) {
  // one thread per column: blocks of vert_x x vert_y columns along (j, i)
  const dim3 b((unsigned)L.vert_x, (unsigned)L.vert_y);
  const WorkItem *wl = set == 0 ? L.wl_vert : L.wl_vinc;
  const int nw = set == 0 ? L.n_vert : L.n_vinc;
  const dim3 grd = wl ? dim3((unsigned)nw, 1, 1)
                      : dim3((unsigned)(((L.jx - 1 + L.vert_x - 1) / L.vert_x) * nf),
                             (unsigned)((L.iy - 1 + L.vert_y - 1) / L.vert_y), (unsigned)L.nmem);
  k_adv_vertical<R, T><<<grd, b, 0, s>>>(d, nf, set, advoff, wl);
}

template <class R, int V, int NW>
void launch_tile(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s) {
  // tiles along j: tile bj writes j = bj*S + ob0 + 3 .. bj*S + ob0 + S + 2
  constexpr int S = 32 * V - 4;
  const int tj = (L.jx - 3 - hshape_ob0(V) + S - 1) / S, ti = (L.iy - 1 + NW - 1) / NW;
  const dim3 grd = L.wl_h ? dim3((unsigned)L.n_h, 1, 1)
                          : dim3((unsigned)(tj * ti), (unsigned)L.kz, (unsigned)L.nmem);
  k_adv_horizontal<R, V, NW><<<grd, 32 * NW, 0, s>>>(d, tj, uvoff, advoff, L.wl_h);
}

template <class R>
void launch_horizontal(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s) {
  constexpr int eb = (int)sizeof(R);
  switch (L.htile) {
    case 1: launch_tile<R, hshape(eb, 1).v, hshape(eb, 1).nw>(L, d, uvoff, advoff, s); break;
    case 2: launch_tile<R, hshape(eb, 2).v, hshape(eb, 2).nw>(L, d, uvoff, advoff, s); break;
    case 3: launch_tile<R, hshape(eb, 3).v, hshape(eb, 3).nw>(L, d, uvoff, advoff, s); break;
    default: launch_tile<R, hshape(eb, 0).v, hshape(eb, 0).nw>(L, d, uvoff, advoff, s); break;
  }
}

template <class R>
void launch_vertical_inc(const LaunchGeom &L, const Dom<R> *d, int advoff, cudaStream_t s) {
  const dim3 b((unsigned)L.vert_x, (unsigned)L.vert_y);
  const dim3 grd = L.wl_vinc ? dim3((unsigned)L.n_vinc, 1, 1)
                             : dim3((unsigned)(((L.jx - 1 + L.vert_x - 1) / L.vert_x) * 2),
                                    (unsigned)((L.iy - 1 + L.vert_y - 1) / L.vert_y), (unsigned)L.nmem);
  k_adv_vertical_inc<R><<<grd, b, 0, s>>>(d, advoff, L.wl_vinc);
}

template <class R, int V, int NW>
void launch_tile_inc(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s) {
  constexpr int S = 32 * V - 4;
  const int tj = (L.jx - 3 - hshape_ob0(V) + S - 1) / S, ti = (L.iy - 1 + NW - 1) / NW;
  const dim3 grd = L.wl_hinc ? dim3((unsigned)L.n_hinc, 1, 1)
                             : dim3((unsigned)(tj * ti), (unsigned)L.kz, (unsigned)L.nmem);
  k_adv_horizontal_inc<R, V, NW><<<grd, 32 * NW, 0, s>>>(d, tj, uvoff, advoff, L.wl_hinc);
}

template <class R>
void launch_horizontal_inc(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff,
                           cudaStream_t s) {
  if (hshape_inc(L.htile).v == 2) launch_tile_inc<R, 2, hshape_inc(1).nw>(L, d, uvoff, advoff, s);
  else launch_tile_inc<R, 1, hshape_inc(0).nw>(L, d, uvoff, advoff, s);
}

template <class R>
void Launch<R>::adv_vertical(const LaunchGeom &L, const Dom<R> *d, int advoff, cudaStream_t s) {
  launch_vertical<R, R>(L, d, L.nadv_r, 0, advoff, s);
}

template <class R>
void Launch<R>::adv_horizontal(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff,
                               cudaStream_t s) {
  launch_horizontal<R>(L, d, uvoff, advoff, s);
}

// The FP64 fields of a mixed member (L.nadv_d = 2) use the increment form.
template <class R>
void Launch<R>::adv_vertical_inc(const LaunchGeom &L, const Dom<R> *d, int advoff, cudaStream_t s) {
  if constexpr (sizeof(R) == sizeof(float)) launch_vertical_inc<R>(L, d, advoff, s);
}

template <class R>
void Launch<R>::adv_horizontal_inc(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff,
                                   cudaStream_t s) {
  if constexpr (sizeof(R) == sizeof(float)) launch_horizontal_inc<R>(L, d, uvoff, advoff, s);
}

template <class R>
void Launch<R>::adv_species_copy(const LaunchGeom &L, const Dom<R> *d, int advoff, cudaStream_t s) {
  const dim3 b((unsigned)L.col_x, (unsigned)L.col_y);
  int tj;
  const dim3 grd = pt_grid(L, L.jx - 1, L.iy - 1, tj);
  k_species_copy<R><<<grd, b, 0, s>>>(d, advoff, tj, L.wl_pt);
}

template <class R>
void Launch<R>::adv_curvature(const LaunchGeom &L, const Dom<R> *d, int advoff, cudaStream_t s) {
  const dim3 b((unsigned)L.col_x, (unsigned)L.col_y);
  int tj;
  const dim3 grd = pt_grid(L, L.jx - 3, L.iy - 3, tj);
  k_adv_curvature<R><<<grd, b, 0, s>>>(d, advoff, tj, L.wl_pt);
}

template <class R>
void Launch<R>::adv_back(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s) {
  const dim3 b((unsigned)L.col_x, (unsigned)L.col_y);
  int tj;
  const dim3 grd = pt_grid(L, L.jx, L.iy, tj);
  k_adv_back<R><<<grd, b, 0, s>>>(d, uvoff, advoff, tj, L.wl_pt);
}

template <class R>
cudaError_t Launch<R>::configure_advect() {
  return cudaSuccess;
}

template struct Launch<double>;
template struct Launch<float>;

}  // namespace mlc
