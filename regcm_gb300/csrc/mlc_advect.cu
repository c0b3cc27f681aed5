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
#include "mlc_kernels.cuh"

namespace mlc {

namespace {


// Main/mod_moloch.F90:1571-1590; minnum is the 4-byte real holding minden.
template <class R> struct FlowEps;
template <> struct FlowEps<double> {
  static __device__ __forceinline__ double den() { return 1.0e-30; }
  static __device__ __forceinline__ double num() { return (double)1.0e-30f; }
};
template <> struct FlowEps<float> {
  static __device__ __forceinline__ float den() { return 1.0e-15f; }
  static __device__ __forceinline__ float num() { return 1.0e-15f; }
};

// WAF flux  hvel*((1+phi)*a + (1-phi)*c)  with  phi = is + zamu*b - is*b  and
// the limiter  b = max(0, min(2, max(r, min(2r, 1))))  of  r = num/den
// (local_flow_param, Main/mod_moloch.F90:1571-1590; the flux lines
// :877-883, :986-993, :1017-1024).  In every use den = c - a, so
//   (1+phi)*a + (1-phi)*c = (a + c) - phi*den,
//   phi*den = is*den + (zamu - is)*B,   B = b*den,
// and B is 0, 2*num, den, num or 2*den as r falls in (-inf,0], (0,1/2),
// [1/2,1], (1,2) or [2,inf): the division num/den is never formed.  The
// result equals the reference's to rounding (b is continuous in r, so the
// region tests need no exact ties), at a third of the FP64 instructions.
template <class T>
__device__ __forceinline__ T waf_flux(T hvel, T is, T zamu, T a, T c, T num) {
  const T den = c - a;
  const T aden = fabs(den);
  T B;
  if (aden < FlowEps<T>::den()) {
    B = fabs(num) < FlowEps<T>::num() ? den : T(0);  // r = 1 or r = 0
  } else {
    const T q = den < T(0) ? -num : num;  // r = q / |den|
    if (q <= T(0)) B = T(0);
    else if (q < T(0.5) * aden) B = num + num;
    else if (q <= aden) B = den;
    else if (q < T(2) * aden) B = num;
    else B = den + den;
  }
  return hvel * ((a + c) - (is * den + (zamu - is) * B));
}

// The advected fields of a member, in the reference's order (tetav, pai,
// ux, vx, wx, qv, qx(iqfrst:nqx) when ipptls > 0, trac; advection,
// Main/mod_moloch.F90:781-807).  Table 0 holds the fields of type R: all of
// them in FP64, all but theta_v and Exner in a mixed member, whose two FP64
// fields form table 1.  cur is the field's current half, out the other.
template <class R>
__device__ __forceinline__ int n_table_r(const Dom<R> &D) {
  const int nfix = sizeof(R) == sizeof(double) ? 2 : 0;
  return nfix + 4 + (D.c.ipptls > 0 ? D.g.nqx - 1 : 0) + D.g.ntr;
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
__global__ void k_adv_prep(const Dom<R> *__restrict__ doms, int uvoff, int advoff) {
  const Dom<R> &D = doms[blockIdx.z];
  if (!D.active) return;
  const Geom g = D.g;
  const int uv = (D.clk->uv_role + uvoff) & 1, adv = (D.clk->adv_role + advoff) & 1;
  const R *__restrict__ u = D.u[uv];
  const R *__restrict__ v = D.v[uv];
  const R *__restrict__ w = D.w;
  R *__restrict__ ux = D.ux[adv];
  R *__restrict__ vx = D.vx[adv];
  R *__restrict__ wx = D.wx[adv];
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int i = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int jx = g.jx, iy = g.iy, kz = g.kz;
  if (j > jx - 1 || i > iy - 1) return;
  const size_t ij = g.at2(j, i), PS = g.PS, S = (size_t)g.P;
  for (int k = 1; k <= kz; ++k) {
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
  }
}

// Two vertical WAF passes for one column of one field (:858-922).  R is the
// type of the winds and metric, T the type of the advected field and of the
// arithmetic (T = R except for the FP64 Exner field of a mixed domain).
template <class R, class T>
__global__ void k_adv_vertical(const Dom<R> *__restrict__ doms, int nf, int set, int advoff) {
  extern __shared__ unsigned char smem_raw[];
  T *smem = reinterpret_cast<T *>(smem_raw);
  const int nth = blockDim.x * blockDim.y;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  // grid: x = field x tiles along j, y = tiles along i, z = member
  const Dom<R> &D = doms[blockIdx.z];
  if (!D.active) return;
  const int tiles_j = gridDim.x / nf;
  const int f = blockIdx.x / tiles_j;
  const int bj = blockIdx.x - f * tiles_j;
  if (set == 0 && f >= n_table_r(D)) return;  // a member with fewer species
  const Geom g = D.g;
  const int kz = g.kz;
  T *col = smem;                                 // field column, levels 1..kz
  T *flx = smem + (size_t)(kz + 2) * nth;        // wfw, interfaces 1..kz+1
  T *sc = smem + (size_t)2 * (kz + 2) * nth;     // s, levels 1..kz+1
#define COL(a, k) a[(size_t)(k) * nth + tid]
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const R *__restrict__ s = D.s;
  const int adv = (D.clk->adv_role + advoff) & 1;
  const T *src;
  T *outp, *dst;
  field_t<R, T>(D, set, f, adv, src, outp, dst);
  (void)outp;
  const int j = bj * blockDim.x + threadIdx.x + 1;
  const int i = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (j > g.jx - 1 || i > g.iy - 1) return;
  const size_t ij = g.at2(j, i), PS = g.PS;
  const T dtrdz = T(0.5) * (T(c.dtstepa) * T(c.rdzita));

  for (int k = 1; k <= kz; ++k) COL(col, k) = src[ij + (size_t)(k - 1) * PS];
  for (int k = 1; k <= kz + 1; ++k) COL(sc, k) = T(s[ij + (size_t)(k - 1) * PS]);
  for (int pass = 0; pass < 2; ++pass) {
    COL(flx, 1) = T(0);
    COL(flx, kz + 1) = T(0);
    for (int k = 1; k <= kz - 1; ++k) {
      const T skp = COL(sc, k + 1);
      const T zamu = skp * dtrdz;
      T is;
      int k1, k1p1;
      if (zamu >= T(0)) {
        is = T(1); k1 = k + 1; k1p1 = k1 + 1;
        if (k1p1 > kz) k1p1 = kz;
      } else {
        is = T(-1); k1 = k - 1; k1p1 = k;
        if (k1 < 1) k1 = 1;
      }
      COL(flx, k + 1) = waf_flux<T>(T(0.5) * skp, is, zamu, COL(col, k + 1), COL(col, k),
                                    COL(col, k1) - COL(col, k1p1));
    }
    for (int k = 1; k <= kz; ++k) {
      const size_t o = ij + (size_t)(k - 1) * PS;
      const T zrfmu = T(sa.zrfmu[o]);
      const T zrfmd = T(sa.zrfmd[o]);
      const T pk = COL(col, k);
      const T zdv = (COL(sc, k) * zrfmu - COL(sc, k + 1) * zrfmd) * pk;
      COL(col, k) = pk - COL(flx, k) * zrfmu + COL(flx, k + 1) * zrfmd + zdv;
    }
  }

  for (int k = 1; k <= kz; ++k) dst[ij + (size_t)(k - 1) * PS] = COL(col, k);
#undef COL
}

// Meridional then zonal WAF for one tile (:984-1038; ROTLLR :926-983).
template <class R, class T, int kTJ, int kTI>
__global__ void __launch_bounds__(kTJ *kTI) k_adv_horizontal(const Dom<R> *__restrict__ doms,
                                                            int nf, int tiles_j, int set,
                                                            int uvoff, int advoff) {
  constexpr int WJ = kTJ + 4;  // columns J0-2 .. J0+TJ+1
  __shared__ T wz_s[kTI + 4][WJ];      // rows I0-2 .. I0+TI+1
  __shared__ T zpby_s[kTI + 1][WJ];    // rows I0 .. I0+TI
  __shared__ T p0_s[kTI][WJ];          // rows I0 .. I0+TI-1
  __shared__ T zpbw_s[kTI][kTJ + 1];   // columns J0 .. J0+TJ
  // grid: x = tiles along j and i, y = field x level, z = member
  const Dom<R> &D = doms[blockIdx.z];
  if (!D.active) return;
  const int f = blockIdx.y % nf;
  if (set == 0 && f >= n_table_r(D)) return;
  const int k = blockIdx.y / nf + 1;
  const int bj = blockIdx.x % tiles_j, bi = blockIdx.x / tiles_j;
  const Geom g = D.g;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const int jx = g.jx, iy = g.iy, kz = g.kz;
  if (k > kz) return;
  const int J0c = bj * kTJ + 1, I0c = bi * kTI + 1;
  if (J0c > jx - 1 || I0c > iy - 1) return;
  const int uv = (D.clk->uv_role + uvoff) & 1, adv = (D.clk->adv_role + advoff) & 1;
  const R *__restrict__ u = D.u[uv];
  const R *__restrict__ v = D.v[uv];
  const T *cur0;
  T *out0, *wz0;
  field_t<R, T>(D, set, f, adv, cur0, out0, wz0);
  const int J0 = J0c, I0 = I0c;
  const int tid = threadIdx.y * kTJ + threadIdx.x;
  const int nth = kTJ * kTI;
  const size_t PS = g.PS, ko = (size_t)(k - 1) * PS;
  const T *pp = cur0 + ko;
  const T *wz = wz0 + ko;
  T *out = out0 + ko;
  const R *uk = u + ko;
  const R *vk = v + ko;
  const T dta = T(c.dtstepa);
  const T dtrdx = dta * T(c.rdx), dtrdy = dta * T(c.rdx);
  const bool rot = c.lrotllr != 0;
  const int imin = 1, imax = iy - 1, jmin = 1, jmax = jx - 1;

  // stage wz (cross points only; others are never read for valid outputs)
  for (int e = tid; e < (kTI + 4) * WJ; e += nth) {
    const int rr = e / WJ, cc = e % WJ;
    const int i = I0 - 2 + rr, j = J0 - 2 + cc;
    T x = T(0);
    if (i >= 1 && i <= iy - 1 && j >= 1 && j <= jx - 1) x = wz[g.at2(j, i)];
    wz_s[rr][cc] = x;
  }
  __syncthreads();
  // meridional fluxes zpby(j,i): j in jce, i in ici1..ice2
  for (int e = tid; e < (kTI + 1) * WJ; e += nth) {
    const int rr = e / WJ, cc = e % WJ;
    const int i = I0 + rr, j = J0 - 2 + cc;
    T x = T(0);
    if (j >= 1 && j <= jx - 1 && i >= 2 && i <= iy - 1) {
      const size_t ij = g.at2(j, i);
      const T vv = T(vk[ij]);
      const T zamu = rot ? vv * dtrdy : vv * T(sa.msfv[ij]) * dtrdy;
      T is;
      int ih;
      if (zamu > T(0)) { is = T(1); ih = i - 1; }
      else { is = T(-1); ih = min(i + 1, imax); }
      const int ihm1 = max(ih - 1, imin);
      // shared-memory row of global row i is i - (I0 - 2)
      const int b = 2 - I0;
      x = waf_flux<T>(T(0.5) * vv, is, zamu, wz_s[i - 1 + b][cc], wz_s[i + b][cc],
                      wz_s[ih + b][cc] - wz_s[ihm1 + b][cc]);
    }
    zpby_s[rr][cc] = x;
  }
  __syncthreads();
  // p0(j,i): j in jce, i in ici
  for (int e = tid; e < kTI * WJ; e += nth) {
    const int rr = e / WJ, cc = e % WJ;
    const int i = I0 + rr, j = J0 - 2 + cc;
    T x = T(0);
    if (j >= 1 && j <= jx - 1 && i >= 2 && i <= iy - 2) {
      const size_t ij = g.at2(j, i), ijN = ij + (size_t)g.P;
      const T fz = T(sa.fmz[ko + ij]);
      const T ppk = pp[ij];
      const T wzk = wz_s[rr + 2][cc];
      if (rot) {
        const T zhxvtn = dtrdy * T(sa.rmv[ijN]) * T(sa.msfx[ij]);
        const T zhxvts = dtrdy * T(sa.rmv[ij]) * T(sa.msfx[ij]);
        const T zrfmn = zhxvtn * fz * T(sa.rfmzv[ko + ijN]);
        const T zrfms = zhxvts * fz * T(sa.rfmzv[ko + ij]);
        const T zdv = (T(vk[ijN]) * zrfmn - T(vk[ij]) * zrfms) * ppk;
        x = wzk + (zpby_s[rr][cc] * zrfms - zpby_s[rr + 1][cc] * zrfmn + zdv);
      } else {
        // rfmzu as in the reference (Main/mod_moloch.F90:1000-1001)
        const T zrfmn = dtrdy * fz * T(sa.rfmzu[ko + ijN]);
        const T zrfms = dtrdy * fz * T(sa.rfmzu[ko + ij]);
        const T zdv = (T(vk[ijN]) * T(sa.rmv[ijN]) * zrfmn - T(vk[ij]) * T(sa.rmv[ij]) * zrfms) * ppk;
        x = wzk + T(sa.mx2[ij]) * (zpby_s[rr][cc] * zrfms - zpby_s[rr + 1][cc] * zrfmn + zdv);
      }
    }
    p0_s[rr][cc] = x;
  }
  __syncthreads();
  // zonal fluxes zpbw(j,i): j in jci1..jce2, i in ici
  for (int e = tid; e < kTI * (kTJ + 1); e += nth) {
    const int rr = e / (kTJ + 1), cc = e % (kTJ + 1);
    const int i = I0 + rr, j = J0 + cc;
    T x = T(0);
    if (j >= 2 && j <= jx - 1 && i >= 2 && i <= iy - 2) {
      const size_t ij = g.at2(j, i);
      const T uu = T(uk[ij]);
      const T zamu = uu * T(sa.msfu[ij]) * dtrdx;
      T is;
      int jh;
      if (zamu > T(0)) { is = T(1); jh = j - 1; }
      else { is = T(-1); jh = min(j + 1, jmax); }
      const int jhm1 = max(jh - 1, jmin);
      const int b = 2 - J0;  // p0_s column of global column j is j - (J0 - 2)
      x = waf_flux<T>(T(0.5) * uu, is, zamu, p0_s[rr][j - 1 + b], p0_s[rr][j + b],
                      p0_s[rr][jh + b] - p0_s[rr][jhm1 + b]);
    }
    zpbw_s[rr][cc] = x;
  }
  __syncthreads();
  // result on the tile: interior update, ring copied
  {
    const int rr = threadIdx.y, cc = threadIdx.x;
    const int i = I0 + rr, j = J0 + cc;
    if (i <= iy - 1 && j <= jx - 1) {
      const size_t ij = g.at2(j, i);
      const T ppk = pp[ij];
      T x = ppk;
      if (j >= 2 && j <= jx - 2 && i >= 2 && i <= iy - 2) {
        const T fz = T(sa.fmz[ko + ij]);
        const T p0k = p0_s[rr][cc + 2];
        if (rot) {
          const T zcostx = dtrdx * T(sa.msfx[ij]);
          const T zrfmw = zcostx * fz * T(sa.rfmzu[ko + ij]);
          const T zrfme = zcostx * fz * T(sa.rfmzu[ko + ij + 1]);
          const T zdv = (T(uk[ij + 1]) * zrfme - T(uk[ij]) * zrfmw) * ppk;
          x = p0k + zpbw_s[rr][cc] * zrfmw - zpbw_s[rr][cc + 1] * zrfme + zdv;
        } else {
          const T zrfmw = dtrdx * fz * T(sa.rfmzu[ko + ij]);
          const T zrfme = dtrdx * fz * T(sa.rfmzu[ko + ij + 1]);
          const T zdv = (T(uk[ij + 1]) * T(sa.rmu[ij + 1]) * zrfme - T(uk[ij]) * T(sa.rmu[ij]) * zrfmw) * ppk;
          x = p0k + T(sa.mx2[ij]) * (zpbw_s[rr][cc] * zrfmw - zpbw_s[rr][cc + 1] * zrfme + zdv);
        }
      }
      out[ij] = x;
    }
  }
}

// Species that are not advected (ipptls = 0: qx(iqfrst:nqx)) keep their
// values when the advected fields move to the other half of their pairs.
template <class R>
__global__ void k_species_copy(const Dom<R> *__restrict__ doms, int advoff) {
  const Dom<R> &D = doms[blockIdx.z];
  if (!D.active) return;
  const Geom g = D.g;
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int i = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (D.c.ipptls > 0 || j > g.jx - 1 || i > g.iy - 1) return;
  const int adv = (D.clk->adv_role + advoff) & 1;
  const size_t F = g.field3(), ij = g.at2(j, i);
  for (int n = 1; n < g.nqx; ++n)
    for (int k = 1; k <= g.kz; ++k) {
      const size_t o = ij + (size_t)(k - 1) * g.PS + (size_t)n * F;
      D.qx[adv ^ 1][o] = D.qx[adv][o];
    }
}

// :809-825
template <class R>
__global__ void k_adv_curvature(const Dom<R> *__restrict__ doms, int advoff) {
  const Dom<R> &D = doms[blockIdx.z];
  if (!D.active || !D.c.curvature) return;
  const Geom g = D.g;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const int adv = (D.clk->adv_role + advoff) & 1;
  R *__restrict__ ux = D.ux[adv];
  R *__restrict__ vx = D.vx[adv];
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int i = blockIdx.y * blockDim.y + threadIdx.y + 2;
  if (j > g.jx - 2 || i > g.iy - 2) return;
  const size_t ij = g.at2(j, i);
  const R dta = R(c.dtstepa);
  R tanx, tany;
  if (c.lrotllr) {
    const double dlat = kDegrad * 0.5 * (sa.rlat[i - 1] + sa.rlat[i]);
    tanx = R(sin(dlat)) * sa.msfx[ij] * R(kRearthRad);
    tany = tanx;
  } else {
    tanx = (sa.msfu[ij - 1] - sa.msfu[ij]) * R(c.rdx);
    tany = (sa.msfv[ij - (size_t)g.P] - sa.msfv[ij]) * R(c.rdx);
  }
  for (int k = 1; k <= g.kz; ++k) {
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
__global__ void k_adv_back(const Dom<R> *__restrict__ doms, int uvoff, int advoff) {
  const Dom<R> &D = doms[blockIdx.z];
  if (!D.active) return;
  const Geom g = D.g;
  const int uv = (D.clk->uv_role + uvoff) & 1, adv = (D.clk->adv_role + advoff) & 1;
  const R *__restrict__ ux = D.ux[adv];
  const R *__restrict__ vx = D.vx[adv];
  const R *__restrict__ wx = D.wx[adv];
  R *__restrict__ u = D.u[uv];
  R *__restrict__ v = D.v[uv];
  R *__restrict__ w = D.w;
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int i = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int jx = g.jx, iy = g.iy, kz = g.kz;
  if (j > jx || i > iy) return;
  const size_t ij = g.at2(j, i), PS = g.PS, S = (size_t)g.P;
  const bool do_u = (j >= 2 && j <= jx - 1 && i >= 2 && i <= iy - 2);
  const bool do_v = (j >= 2 && j <= jx - 2 && i >= 2 && i <= iy - 1);
  const bool do_w = (j <= jx - 1 && i <= iy - 1);
  for (int k = 1; k <= kz; ++k) {
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

// Both vertical passes (Main/mod_moloch.F90:858-922).  Writes the increment
// dz = (field after the passes) - field, in FP64.
template <class R>
__global__ void k_adv_vertical_inc(const Dom<R> *__restrict__ doms, int advoff) {
  extern __shared__ float vsm[];
  const int nth = blockDim.x * blockDim.y;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const Dom<R> &D = doms[blockIdx.z];
  if (!D.active) return;
  const int tiles_j = gridDim.x / 2;
  const int f = blockIdx.x / tiles_j;
  const int bj = blockIdx.x - f * tiles_j;
  const Geom g = D.g;
  const int kz = g.kz;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const int adv = (D.clk->adv_role + advoff) & 1;
  const double *__restrict__ src = f == 0 ? D.tetav[adv] : D.pai[adv];
  double *__restrict__ dst = D.wz_d[f];
  const R *__restrict__ s = D.s;
  const int j = bj * blockDim.x + threadIdx.x + 1;
  const int i = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (j > g.jx - 1 || i > g.iy - 1) return;
#define DZ(k) vsm[(size_t)(k) * nth + tid]                  // v(k+1) - v(k), k = 1..kz-1
#define E(k) vsm[(size_t)(kz + 1 + (k)) * nth + tid]        // increment, k = 1..kz
  const size_t ij = g.at2(j, i), PS = g.PS;
  const float dtrdz = 0.5f * (float(c.dtstepa) * float(c.rdzita));
  double vlo = src[ij];
  const double v1 = vlo;
  for (int k = 1; k <= kz - 1; ++k) {
    const double vhi = src[ij + (size_t)k * PS];
    DZ(k) = float(vhi - vlo);
    vlo = vhi;
  }
  const double vtop = vlo;
  for (int k = 1; k <= kz; ++k) E(k) = 0.f;
  // FP32 parts of the bottom and top cells, and their FP64 constant parts
  float eb32 = 0.f, et32 = 0.f;
  double hb = 0.0, ht = 0.0;
  for (int pass = 0; pass < 2; ++pass) {
    float fb = 0.f;                    // flux below cell k, relative to cell k
    float e_km1 = 0.f, e_k = E(1), e_kp1 = kz >= 2 ? E(2) : 0.f;
    float sk = float(s[ij]);
    for (int k = 1; k <= kz; ++k) {
      const size_t o = ij + (size_t)(k - 1) * PS;
      const float e_kp2 = k + 2 <= kz ? E(k + 2) : 0.f;
      const float skp = float(s[o + PS]);
      float fa = 0.f, fup = 0.f;       // flux above (relative to k), same moved to k+1
      if (k <= kz - 1) {
        const float zamu = skp * dtrdz;
        const float dzk = DZ(k);
        float is, num;
        if (zamu >= 0.f) {
          is = 1.f;
          num = k + 2 <= kz ? (e_kp1 - e_kp2) - DZ(k + 1) : 0.f;
        } else {
          is = -1.f;
          num = k >= 2 ? (e_km1 - e_k) - DZ(k - 1) : 0.f;
        }
        fa = waf_flux<float>(0.5f * skp, is, zamu, dzk + e_kp1, e_k, num);
        fup = fa - skp * dzk;
      }
      const float zrfmu = float(sa.zrfmu[o]), zrfmd = float(sa.zrfmd[o]);
      const float upd = -fb * zrfmu + fa * zrfmd + (sk * zrfmu - skp * zrfmd) * e_k;
      float en;
      if (k == 1 || k == kz) {
        // constant part: k = kz has no flux through kz+1, k = 1 none through 1
        const double kap = k == kz ? -(double)skp * (double)zrfmd : (double)sk * (double)zrfmu;
        const double vk = k == kz ? vtop : v1;
        if (k == kz) { et32 += upd; ht += vk * kap; en = et32 + float(ht); }
        else { eb32 += upd; hb += vk * kap; en = eb32 + float(hb); }
      } else {
        en = e_k + upd;
      }
      E(k) = en;                       // old E(k) lives on in e_km1 below
      e_km1 = e_k; e_k = e_kp1; e_kp1 = e_kp2;
      fb = fup;
      sk = skp;
    }
  }
  for (int k = 1; k <= kz; ++k) {
    double d;
    if (k == kz) d = (double)et32 + ht;
    else if (k == 1) d = (double)eb32 + hb;
    else d = (double)E(k);
    dst[ij + (size_t)(k - 1) * PS] = d;
  }
#undef DZ
#undef E
}

// Meridional then zonal WAF of one tile (:984-1038; ROTLLR :926-983) in
// increment form.  pp is the field at the start of the advection step, dz
// its vertical increment; out = pp + dz + (meridional + zonal increments).
template <class R, int kTJ, int kTI>
__global__ void __launch_bounds__(kTJ *kTI) k_adv_horizontal_inc(const Dom<R> *__restrict__ doms,
                                                                int tiles_j, int uvoff,
                                                                int advoff) {
  constexpr int WJ = kTJ + 4;          // columns J0-2 .. J0+TJ+1
  __shared__ double pp_s[kTI + 4][WJ];  // rows I0-2 .. I0+TI+1
  __shared__ float dz_s[kTI + 4][WJ];   // vertical increment
  __shared__ float dy_s[kTI + 3][WJ];   // pp(i+1) - pp(i), rows I0-2 .. I0+TI
  __shared__ float fy_s[kTI + 1][WJ];   // meridional flux at i, relative to pp(i-1)
  __shared__ float ey_s[kTI][WJ];       // p0 - pp, rows I0 .. I0+TI-1
  __shared__ float hy_s[kTI][WJ];       // meridional increment alone
  __shared__ float dx_s[kTI][kTJ + 3];  // pp(j+1) - pp(j), columns J0-2 .. J0+TJ
  __shared__ float fx_s[kTI][kTJ + 1];  // zonal flux at j, relative to pp(j-1)
  const Dom<R> &D = doms[blockIdx.z];
  if (!D.active) return;
  const int f = blockIdx.y & 1;
  const int k = (blockIdx.y >> 1) + 1;
  const int bj = blockIdx.x % tiles_j, bi = blockIdx.x / tiles_j;
  const Geom g = D.g;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const int jx = g.jx, iy = g.iy, kz = g.kz;
  if (k > kz) return;
  const int J0 = bj * kTJ + 1, I0 = bi * kTI + 1;
  if (J0 > jx - 1 || I0 > iy - 1) return;
  const int uv = (D.clk->uv_role + uvoff) & 1, adv = (D.clk->adv_role + advoff) & 1;
  const size_t PS = g.PS, ko = (size_t)(k - 1) * PS;
  const double *__restrict__ pp = (f == 0 ? D.tetav[adv] : D.pai[adv]) + ko;
  double *__restrict__ out = (f == 0 ? D.tetav[adv ^ 1] : D.pai[adv ^ 1]) + ko;
  const double *__restrict__ dzg = D.wz_d[f] + ko;
  const R *__restrict__ uk = D.u[uv] + ko;
  const R *__restrict__ vk = D.v[uv] + ko;
  const int tid = threadIdx.y * kTJ + threadIdx.x;
  const int nth = kTJ * kTI;
  const float dta = float(c.dtstepa);
  const float dtrdx = dta * float(c.rdx), dtrdy = dta * float(c.rdx);
  const bool rot = c.lrotllr != 0;
  const int imin = 1, imax = iy - 1, jmin = 1, jmax = jx - 1;

  for (int e = tid; e < (kTI + 4) * WJ; e += nth) {
    const int rr = e / WJ, cc = e % WJ;
    const int i = I0 - 2 + rr, j = J0 - 2 + cc;
    double x = 0.0, z = 0.0;
    if (i >= 1 && i <= iy - 1 && j >= 1 && j <= jx - 1) {
      const size_t ij = g.at2(j, i);
      x = pp[ij];
      z = dzg[ij];
    }
    pp_s[rr][cc] = x;
    dz_s[rr][cc] = float(z);
  }
  __syncthreads();
  for (int e = tid; e < (kTI + 3) * WJ; e += nth) {
    const int rr = e / WJ, cc = e % WJ;
    dy_s[rr][cc] = float(pp_s[rr + 1][cc] - pp_s[rr][cc]);
  }
  for (int e = tid; e < kTI * (kTJ + 3); e += nth) {
    const int rr = e / (kTJ + 3), cc = e % (kTJ + 3);
    dx_s[rr][cc] = float(pp_s[rr + 2][cc + 1] - pp_s[rr + 2][cc]);
  }
  __syncthreads();
  // meridional fluxes at interface rows i = I0 .. I0+TI, relative to pp(i-1)
  for (int e = tid; e < (kTI + 1) * WJ; e += nth) {
    const int rr = e / WJ, cc = e % WJ;
    const int i = I0 + rr, j = J0 - 2 + cc;
    float x = 0.f;
    if (j >= 1 && j <= jx - 1 && i >= 2 && i <= iy - 1) {
      const size_t ij = g.at2(j, i);
      const float vv = float(vk[ij]);
      const float zamu = rot ? vv * dtrdy : vv * float(sa.msfv[ij]) * dtrdy;
      float is;
      int ih;
      if (zamu > 0.f) { is = 1.f; ih = i - 1; }
      else { is = -1.f; ih = min(i + 1, imax); }
      const int ihm1 = max(ih - 1, imin);
      const int b = 2 - I0;  // tile row of global row i is i + b
      const float dpp = ih != ihm1 ? dy_s[ihm1 + b][cc] : 0.f;
      const float num = (dz_s[ih + b][cc] - dz_s[ihm1 + b][cc]) + dpp;
      x = waf_flux<float>(0.5f * vv, is, zamu, dz_s[i - 1 + b][cc],
                          dz_s[i + b][cc] + dy_s[i - 1 + b][cc], num);
    }
    fy_s[rr][cc] = x;
  }
  __syncthreads();
  // p0 - pp on rows I0 .. I0+TI-1
  for (int e = tid; e < kTI * WJ; e += nth) {
    const int rr = e / WJ, cc = e % WJ;
    const int i = I0 + rr, j = J0 - 2 + cc;
    float hy = 0.f;
    if (j >= 1 && j <= jx - 1 && i >= 2 && i <= iy - 2) {
      const size_t ij = g.at2(j, i), ijN = ij + (size_t)g.P;
      const float fz = float(sa.fmz[ko + ij]);
      const float vs = float(vk[ij]), vn = float(vk[ijN]);
      const float fs = fy_s[rr][cc] - vs * dy_s[rr + 1][cc];  // moved to pp(i)
      const float fn = fy_s[rr + 1][cc];
      if (rot) {
        const float zhxvtn = dtrdy * float(sa.rmv[ijN]) * float(sa.msfx[ij]);
        const float zhxvts = dtrdy * float(sa.rmv[ij]) * float(sa.msfx[ij]);
        const float zrfmn = zhxvtn * fz * float(sa.rfmzv[ko + ijN]);
        const float zrfms = zhxvts * fz * float(sa.rfmzv[ko + ij]);
        hy = fs * zrfms - fn * zrfmn;
      } else {
        const float zrfmn = dtrdy * fz * float(sa.rfmzu[ko + ijN]);
        const float zrfms = dtrdy * fz * float(sa.rfmzu[ko + ij]);
        const float mx2 = float(sa.mx2[ij]);
        const float rs = float(sa.rmv[ij]), rn = float(sa.rmv[ijN]);
        hy = mx2 * (fs * zrfms - fn * zrfmn);
        if (rs != 1.f || rn != 1.f)
          hy += float(pp_s[rr + 2][cc] *
                      (double)(mx2 * (vs * zrfms * (1.f - rs) - vn * zrfmn * (1.f - rn))));
      }
    }
    hy_s[rr][cc] = hy;
    ey_s[rr][cc] = dz_s[rr + 2][cc] + hy;
  }
  __syncthreads();
  // zonal fluxes at interface columns j = J0 .. J0+TJ, relative to pp(j-1)
  for (int e = tid; e < kTI * (kTJ + 1); e += nth) {
    const int rr = e / (kTJ + 1), cc = e % (kTJ + 1);
    const int i = I0 + rr, j = J0 + cc;
    float x = 0.f;
    if (j >= 2 && j <= jx - 1 && i >= 2 && i <= iy - 2) {
      const size_t ij = g.at2(j, i);
      const float uu = float(uk[ij]);
      const float zamu = uu * float(sa.msfu[ij]) * dtrdx;
      float is;
      int jh;
      if (zamu > 0.f) { is = 1.f; jh = j - 1; }
      else { is = -1.f; jh = min(j + 1, jmax); }
      const int jhm1 = max(jh - 1, jmin);
      const int b = 2 - J0;  // ey_s / dx_s column of global column j is j + b
      const float dpp = jh != jhm1 ? dx_s[rr][jhm1 + b] : 0.f;
      const float num = (ey_s[rr][jh + b] - ey_s[rr][jhm1 + b]) + dpp;
      x = waf_flux<float>(0.5f * uu, is, zamu, ey_s[rr][j - 1 + b],
                          ey_s[rr][j + b] + dx_s[rr][j - 1 + b], num);
    }
    fx_s[rr][cc] = x;
  }
  __syncthreads();
  {
    const int rr = threadIdx.y, cc = threadIdx.x;
    const int i = I0 + rr, j = J0 + cc;
    if (i <= iy - 1 && j <= jx - 1) {
      const size_t ij = g.at2(j, i);
      const double ppk = pp_s[rr + 2][cc + 2];
      double x = ppk;
      if (j >= 2 && j <= jx - 2 && i >= 2 && i <= iy - 2) {
        const float fz = float(sa.fmz[ko + ij]);
        const float uw = float(uk[ij]), ue = float(uk[ij + 1]);
        const float fw = fx_s[rr][cc] - uw * dx_s[rr][cc + 1];  // moved to pp(j)
        const float fe = fx_s[rr][cc + 1];
        float hx;
        if (rot) {
          const float zcostx = dtrdx * float(sa.msfx[ij]);
          const float zrfmw = zcostx * fz * float(sa.rfmzu[ko + ij]);
          const float zrfme = zcostx * fz * float(sa.rfmzu[ko + ij + 1]);
          hx = fw * zrfmw - fe * zrfme;
        } else {
          const float zrfmw = dtrdx * fz * float(sa.rfmzu[ko + ij]);
          const float zrfme = dtrdx * fz * float(sa.rfmzu[ko + ij + 1]);
          const float mx2 = float(sa.mx2[ij]);
          const float rw = float(sa.rmu[ij]), re = float(sa.rmu[ij + 1]);
          hx = mx2 * (fw * zrfmw - fe * zrfme);
          if (rw != 1.f || re != 1.f)
            hx += float(ppk * (double)(mx2 * (uw * zrfmw * (1.f - rw) - ue * zrfme * (1.f - re))));
        }
        x = ppk + dzg[ij] + (double)(hy_s[rr][cc + 2] + hx);
      }
      out[ij] = x;
    }
  }
}

inline dim3 grid2(int nj, int ni, dim3 b, int nmem) {
  return dim3((unsigned)((nj + b.x - 1) / b.x), (unsigned)((ni + b.y - 1) / b.y), (unsigned)nmem);
}

}  // namespace

template <class R>
void Launch<R>::adv_prep(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s) {
  const dim3 b((unsigned)L.col_x, (unsigned)L.col_y);
  k_adv_prep<R><<<grid2(L.jx - 1, L.iy - 1, b, L.nmem), b, 0, s>>>(d, uvoff, advoff);
}

template <class R, class T>
void launch_vertical(const LaunchGeom &L, const Dom<R> *d, int nf, int set, int advoff,
                     cudaStream_t s) {
  const dim3 b((unsigned)L.vert_x, (unsigned)L.vert_y);
  const size_t smem = (size_t)3 * (L.kz + 2) * b.x * b.y * sizeof(T);
  dim3 grd = grid2(L.jx - 1, L.iy - 1, b, L.nmem);
  grd.x *= (unsigned)nf;
  k_adv_vertical<R, T><<<grd, b, smem, s>>>(d, nf, set, advoff);
}

template <class R, class T, int TJ, int TI>
void launch_tile(const LaunchGeom &L, const Dom<R> *d, int nf, int set, int uvoff, int advoff,
                 cudaStream_t s) {
  const int tj = (L.jx - 1 + TJ - 1) / TJ, ti = (L.iy - 1 + TI - 1) / TI;
  const dim3 grd((unsigned)(tj * ti), (unsigned)(nf * L.kz), (unsigned)L.nmem);
  k_adv_horizontal<R, T, TJ, TI><<<grd, dim3(TJ, TI), 0, s>>>(d, nf, tj, set, uvoff, advoff);
}

template <class R, class T>
void launch_horizontal(const LaunchGeom &L, const Dom<R> *d, int nf, int set, int uvoff,
                       int advoff, cudaStream_t s) {
  switch (L.htile) {
    case 1: launch_tile<R, T, 32, 4>(L, d, nf, set, uvoff, advoff, s); break;
    case 2: launch_tile<R, T, 64, 4>(L, d, nf, set, uvoff, advoff, s); break;
    case 3: launch_tile<R, T, 16, 8>(L, d, nf, set, uvoff, advoff, s); break;
    default: launch_tile<R, T, 32, 8>(L, d, nf, set, uvoff, advoff, s); break;
  }
}

template <class R>
void launch_vertical_inc(const LaunchGeom &L, const Dom<R> *d, int advoff, cudaStream_t s) {
  const dim3 b((unsigned)L.vert_x, (unsigned)L.vert_y);
  const size_t smem = (size_t)2 * (L.kz + 2) * b.x * b.y * sizeof(float);
  dim3 grd = grid2(L.jx - 1, L.iy - 1, b, L.nmem);
  grd.x *= 2u;
  k_adv_vertical_inc<R><<<grd, b, smem, s>>>(d, advoff);
}

template <class R, int TJ, int TI>
void launch_tile_inc(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s) {
  const int tj = (L.jx - 1 + TJ - 1) / TJ, ti = (L.iy - 1 + TI - 1) / TI;
  const dim3 grd((unsigned)(tj * ti), (unsigned)(2 * L.kz), (unsigned)L.nmem);
  k_adv_horizontal_inc<R, TJ, TI><<<grd, dim3(TJ, TI), 0, s>>>(d, tj, uvoff, advoff);
}

template <class R>
void launch_horizontal_inc(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff,
                           cudaStream_t s) {
  switch (L.htile) {
    case 1: launch_tile_inc<R, 32, 4>(L, d, uvoff, advoff, s); break;
    case 2: launch_tile_inc<R, 64, 4>(L, d, uvoff, advoff, s); break;
    case 3: launch_tile_inc<R, 16, 8>(L, d, uvoff, advoff, s); break;
    default: launch_tile_inc<R, 32, 8>(L, d, uvoff, advoff, s); break;
  }
}

// The FP64 fields of a mixed member (L.nadv_d = 2) use the increment form.
template <class R>
void Launch<R>::adv_vertical(const LaunchGeom &L, const Dom<R> *d, int advoff, cudaStream_t s) {
  launch_vertical<R, R>(L, d, L.nadv_r, 0, advoff, s);
  if constexpr (sizeof(R) == sizeof(float))
    if (L.nadv_d) launch_vertical_inc<R>(L, d, advoff, s);
}

template <class R>
void Launch<R>::adv_horizontal(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff,
                               cudaStream_t s) {
  launch_horizontal<R, R>(L, d, L.nadv_r, 0, uvoff, advoff, s);
  if constexpr (sizeof(R) == sizeof(float))
    if (L.nadv_d) launch_horizontal_inc<R>(L, d, uvoff, advoff, s);
}

template <class R>
void Launch<R>::adv_species_copy(const LaunchGeom &L, const Dom<R> *d, int advoff, cudaStream_t s) {
  const dim3 b((unsigned)L.col_x, (unsigned)L.col_y);
  k_species_copy<R><<<grid2(L.jx - 1, L.iy - 1, b, L.nmem), b, 0, s>>>(d, advoff);
}

template <class R>
void Launch<R>::adv_curvature(const LaunchGeom &L, const Dom<R> *d, int advoff, cudaStream_t s) {
  const dim3 b((unsigned)L.col_x, (unsigned)L.col_y);
  k_adv_curvature<R><<<grid2(L.jx - 3, L.iy - 3, b, L.nmem), b, 0, s>>>(d, advoff);
}

template <class R>
void Launch<R>::adv_back(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s) {
  const dim3 b((unsigned)L.col_x, (unsigned)L.col_y);
  k_adv_back<R><<<grid2(L.jx, L.iy, b, L.nmem), b, 0, s>>>(d, uvoff, advoff);
}

template <class R>
cudaError_t Launch<R>::configure_advect() {
  cudaError_t e = cudaFuncSetAttribute(k_adv_vertical<R, R>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if constexpr (sizeof(R) == sizeof(float))
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_adv_vertical_inc<R>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  return e;
}

template struct Launch<double>;
template struct Launch<float>;

}  // namespace mlc
