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
//   phi*den = is*den + (zamu - is)*B,   B = b*den.
// With d = |den| > 0 and q = num*sign(den) (so r = q/d), multiplying the
// limiter by d > 0 gives
//   B = sign(den) * max(0, min(2d, max(q, min(2q, d)))),
// whose candidates 0, q, 2q, d, 2d are exact: B is one of 0, 2*num, den, num,
// 2*den exactly, the value of b*den in each region of r, ties included.  No
// division.  FP32 takes the branch-free clamp; FP64 tests the regions of r in
// turn (0, 1/2, 1, 2), which usually stops early - on GB300 each FP64 min, max
// or compare is an instruction of the 1/64-rate FP64 pipe.  Both give the same
// B, and the flux equals the reference's to rounding.
template <class T>
__device__ __forceinline__ T waf_flux(T hvel, T is, T zamu, T a, T c, T num) {
  const T den = c - a;
  const T d = fabs(den);
  const T q = den < T(0) ? -num : num;
  T B;
  if (d < FlowEps<T>::den()) {
    B = fabs(num) < FlowEps<T>::num() ? den : T(0);  // r = 1 or r = 0
  } else if constexpr (sizeof(T) == sizeof(float)) {
    const T bd = fmax(T(0), fmin(d + d, fmax(q, fmin(q + q, d))));
    B = den < T(0) ? -bd : bd;
  } else {
    if (q <= T(0)) B = T(0);
    else if (q < T(0.5) * d) B = num + num;
    else if (q <= d) B = den;
    else if (q < T(2) * d) B = num;
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
__global__ void k_adv_prep(const Dom<R> *__restrict__ doms, int uvoff, int advoff, int tiles_j) {
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
  const Pt q_ = point_of(tiles_j, 1, 1);
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
  }
}

// Two vertical WAF passes for the columns of one field (:858-922).  A block
// holds blockDim.x consecutive columns (j) of one row i with their levels in
// shared memory, laid out [level][column]; its blockDim.y thread rows share
// the levels.  Within a pass every interface flux depends only on the pass
// input and every cell update only on its two fluxes, so each pass is two
// level-parallel phases.  R is the type of the winds and metric, T that of
// the advected field and of the arithmetic.
template <class R, class T>
__global__ void k_adv_vertical(const Dom<R> *__restrict__ doms, int nf, int set, int advoff) {
  extern __shared__ unsigned char smem_raw[];
  T *smem = reinterpret_cast<T *>(smem_raw);
  const int CX = blockDim.x, KT = blockDim.y;
  const int tx = threadIdx.x, ty = threadIdx.y;
  // grid: x = field x column tiles along j, y = row i, z = member
  const Dom<R> &D = doms[blockIdx.z];
  if (!D.active) return;
  const int tiles_j = gridDim.x / nf;
  const int f = blockIdx.x / tiles_j;
  const int bj = blockIdx.x - f * tiles_j;
  if (set == 0 && f >= n_table_r(D)) return;  // a member with fewer species
  const Geom g = D.g;
  const int kz = g.kz;
  const int i = blockIdx.y + 1;
  if (i > g.iy - 1 || bj * CX + 1 > g.jx - 1) return;
  const int j = bj * CX + tx + 1;
  const bool on = j <= g.jx - 1;
  const size_t L = (size_t)(kz + 2) * CX;
  T *col = smem;          // field, levels 1..kz
  T *flx = smem + L;      // wfw, interfaces 1..kz+1
  T *sc = smem + 2 * L;   // s, levels 1..kz+1
  T *zu = smem + 3 * L;   // dtrdz*fmz/fmzf(k)
  T *zd = smem + 4 * L;   // dtrdz*fmz/fmzf(k+1)
#define A(a, k) a[(size_t)(k) * CX + tx]
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const R *__restrict__ s = D.s;
  const int adv = (D.clk->adv_role + advoff) & 1;
  const T *src;
  T *outp, *dst;
  field_t<R, T>(D, set, f, adv, src, outp, dst);
  (void)outp;
  const size_t ij = on ? g.at2(j, i) : 0, PS = g.PS;
  const T dtrdz = T(0.5) * (pick<T>(c.dtstepa, c.dtstepaf) * pick<T>(c.rdzita, c.rdzitaf));

  if (on)
    for (int k = 1 + ty; k <= kz + 1; k += KT) {
      const size_t o = ij + (size_t)(k - 1) * PS;
      A(sc, k) = T(s[o]);
      if (k <= kz) {
        A(col, k) = src[o];
        A(zu, k) = T(sa.zrfmu[o]);
        A(zd, k) = T(sa.zrfmd[o]);
      }
    }
  if (ty == 0) {
    A(flx, 1) = T(0);
    A(flx, kz + 1) = T(0);
  }
  __syncthreads();
  for (int pass = 0; pass < 2; ++pass) {
    if (on)
      for (int k = 1 + ty; k <= kz - 1; k += KT) {
        const T skp = A(sc, k + 1);
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
        A(flx, k + 1) = waf_flux<T>(T(0.5) * skp, is, zamu, A(col, k + 1), A(col, k),
                                    A(col, k1) - A(col, k1p1));
      }
    __syncthreads();
    if (on)
      for (int k = 1 + ty; k <= kz; k += KT) {
        const T zrfmu = A(zu, k), zrfmd = A(zd, k);
        const T pk = A(col, k);
        const T zdv = (A(sc, k) * zrfmu - A(sc, k + 1) * zrfmd) * pk;
        A(col, k) = pk - A(flx, k) * zrfmu + A(flx, k + 1) * zrfmd + zdv;
      }
    __syncthreads();
  }
  if (on)
    for (int k = 1 + ty; k <= kz; k += KT) dst[ij + (size_t)(k - 1) * PS] = A(col, k);
#undef A
}

// ---- TMA tile loads and mbarriers (inline PTX, sm_90+) ----------------------
__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// orders this thread's earlier generic-proxy accesses of shared memory before
// a following async-proxy (TMA) write to it
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// one tiled copy of the box at (x, y, z) of the tensor map into shared memory
__device__ __forceinline__ void tma_load_3d(void *dst, const void *tmap, int x, int y, int z,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
  return ok != 0;
}
// gives up after a bounded number of polls (a copy that never lands must not
// hang the GPU); the caller records the fault
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity) {
  for (int it = 0; it < (1 << 18); ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

template <int TJ, int TI>
constexpr int tile_shape_index() {
  return (TJ == 32 && TI == 8) ? 0 : (TJ == 32 && TI == 4) ? 1 : (TJ == 64 && TI == 4) ? 2 : 3;
}

// Meridional then zonal WAF for one tile at one level, every field of the R
// table (:984-1038; ROTLLR :926-983).  The winds, Courant numbers and metric
// coefficients of the tile are formed once, in shared memory, and then each
// field in turn is staged with a 2-point halo, its meridional fluxes and the
// intermediate p0 are built on a 2-column halo, then its zonal fluxes and
// the result, so each field is read and written once.  The result goes to
// the field's other buffer because the halo columns of a tile still need its
// old values.  Per field the expressions are the reference's, operand for
// operand; only the field-independent factors are computed once.
template <class R, int kTJ, int kTI>
__global__ void __launch_bounds__(kTJ *kTI) k_adv_horizontal(const Dom<R> *__restrict__ doms,
                                                            int tiles_j, int uvoff, int advoff) {
  using T = R;
  constexpr int WJ = kTJ + 4;            // columns J0-2 .. J0+TJ+1
  // halo tiles of two fields (TMA destinations, double-buffered): rows
  // I0-2 .. I0+TI+1; column J0-2+cc of the kernel sits at cc + OFF, the copy
  // starting OFF columns further left so that it starts on 16 bytes
  constexpr int OFF = sizeof(T) == sizeof(float) ? 2 : 0;
  constexpr int BW = WJ + 2 * OFF;
  constexpr unsigned kBox = (unsigned)((kTI + 4) * BW * sizeof(T));
  __shared__ __align__(128) T wzt[2][kTI + 4][BW];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ T zpby_s[kTI + 1][WJ];      // rows I0 .. I0+TI
  __shared__ T p0_s[kTI][WJ];            // rows I0 .. I0+TI-1
  __shared__ T zpbw_s[kTI][kTJ + 1];     // columns J0 .. J0+TJ
  // field-independent factors of the tile
  __shared__ T vy_s[kTI + 1][WJ], zmy_s[kTI + 1][WJ];   // v, Courant number at rows I0..I0+TI
  __shared__ T zs_s[kTI][WJ], zn_s[kTI][WJ], dvy_s[kTI][WJ], m2_s[kTI][WJ];
  __shared__ T ux_s[kTI][kTJ + 1], zmx_s[kTI][kTJ + 1];  // u, Courant number at columns J0..J0+TJ
  __shared__ T zw_s[kTI][kTJ], ze_s[kTI][kTJ], dvx_s[kTI][kTJ];
  // grid: x = tiles along j and i, y = level, z = member
  const Dom<R> &D = doms[blockIdx.z];
  if (!D.active) return;
  const int k = blockIdx.y + 1;
  const int bj = blockIdx.x % tiles_j, bi = blockIdx.x / tiles_j;
  const Geom g = D.g;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const int jx = g.jx, iy = g.iy, kz = g.kz;
  if (k > kz) return;
  const int J0 = bj * kTJ + 1, I0 = bi * kTI + 1;
  if (J0 > jx - 1 || I0 > iy - 1) return;
  const int uv = (D.clk->uv_role + uvoff) & 1, adv = (D.clk->adv_role + advoff) & 1;
  const int tid = threadIdx.y * kTJ + threadIdx.x;
  const int nth = kTJ * kTI;
  const size_t PS = g.PS, ko = (size_t)(k - 1) * PS;
  const R *__restrict__ uk = D.u[uv] + ko;
  const R *__restrict__ vk = D.v[uv] + ko;
  const T dta = pick<T>(c.dtstepa, c.dtstepaf);
  const T dtrdx = dta * pick<T>(c.rdx, c.rdxf), dtrdy = dta * pick<T>(c.rdx, c.rdxf);
  const bool rot = c.lrotllr != 0;
  const int imin = 1, imax = iy - 1, jmin = 1, jmax = jx - 1;
  const int nf = n_table_r(D);
  const char *tmaps = static_cast<const char *>(D.tmap) +
                      (size_t)tile_shape_index<kTJ, kTI>() * kMaxFields * kTmapBytes;
  auto issue = [&](int fld, int b) {  // one thread: the halo tile of field fld into buffer b
    fence_proxy_async();
    mbar_expect_tx(&mbar[b], kBox);
    tma_load_3d(&wzt[b][0][0], tmaps + (size_t)fld * kTmapBytes, J0 - 3 - OFF, I0 - 3, k - 1,
                &mbar[b]);
  };
  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) {
    issue(0, 0);
    if (nf > 1) issue(1, 1);
  }

  // ---- field-independent factors (while the first tiles land) ----
  for (int e = tid; e < (kTI + 1) * WJ; e += nth) {
    const int rr = e / WJ, cc = e % WJ;
    const int i = I0 + rr, j = J0 - 2 + cc;
    T vv = T(0), zamu = T(0);
    if (j >= 1 && j <= jx - 1 && i >= 2 && i <= iy - 1) {
      const size_t ij = g.at2(j, i);
      vv = T(vk[ij]);
      zamu = rot ? vv * dtrdy : vv * T(sa.msfv[ij]) * dtrdy;
    }
    vy_s[rr][cc] = vv;
    zmy_s[rr][cc] = zamu;
  }
  for (int e = tid; e < kTI * WJ; e += nth) {
    const int rr = e / WJ, cc = e % WJ;
    const int i = I0 + rr, j = J0 - 2 + cc;
    T zs = T(0), zn = T(0), dv = T(0), m2 = T(1);
    if (j >= 1 && j <= jx - 1 && i >= 2 && i <= iy - 2) {
      const size_t ij = g.at2(j, i), ijN = ij + (size_t)g.P;
      const T fz = T(sa.fmz[ko + ij]);
      if (rot) {
        const T zhxvtn = dtrdy * T(sa.rmv[ijN]) * T(sa.msfx[ij]);
        const T zhxvts = dtrdy * T(sa.rmv[ij]) * T(sa.msfx[ij]);
        zn = zhxvtn * fz * T(sa.rfmzv[ko + ijN]);
        zs = zhxvts * fz * T(sa.rfmzv[ko + ij]);
        dv = T(vk[ijN]) * zn - T(vk[ij]) * zs;
      } else {
        // rfmzu as in the reference (Main/mod_moloch.F90:1000-1001)
        zn = dtrdy * fz * T(sa.rfmzu[ko + ijN]);
        zs = dtrdy * fz * T(sa.rfmzu[ko + ij]);
        dv = T(vk[ijN]) * T(sa.rmv[ijN]) * zn - T(vk[ij]) * T(sa.rmv[ij]) * zs;
        m2 = T(sa.mx2[ij]);
      }
    }
    zs_s[rr][cc] = zs; zn_s[rr][cc] = zn; dvy_s[rr][cc] = dv; m2_s[rr][cc] = m2;
  }
  for (int e = tid; e < kTI * (kTJ + 1); e += nth) {
    const int rr = e / (kTJ + 1), cc = e % (kTJ + 1);
    const int i = I0 + rr, j = J0 + cc;
    T uu = T(0), zamu = T(0);
    if (j >= 2 && j <= jx - 1 && i >= 2 && i <= iy - 2) {
      const size_t ij = g.at2(j, i);
      uu = T(uk[ij]);
      zamu = uu * T(sa.msfu[ij]) * dtrdx;
    }
    ux_s[rr][cc] = uu;
    zmx_s[rr][cc] = zamu;
  }
  {
    const int rr = threadIdx.y, cc = threadIdx.x;
    const int i = I0 + rr, j = J0 + cc;
    T zw = T(0), ze = T(0), dv = T(0);
    if (j >= 2 && j <= jx - 2 && i >= 2 && i <= iy - 2) {
      const size_t ij = g.at2(j, i);
      const T fz = T(sa.fmz[ko + ij]);
      if (rot) {
        const T zcostx = dtrdx * T(sa.msfx[ij]);
        zw = zcostx * fz * T(sa.rfmzu[ko + ij]);
        ze = zcostx * fz * T(sa.rfmzu[ko + ij + 1]);
        dv = T(uk[ij + 1]) * ze - T(uk[ij]) * zw;
      } else {
        zw = dtrdx * fz * T(sa.rfmzu[ko + ij]);
        ze = dtrdx * fz * T(sa.rfmzu[ko + ij + 1]);
        dv = T(uk[ij + 1]) * T(sa.rmu[ij + 1]) * ze - T(uk[ij]) * T(sa.rmu[ij]) * zw;
      }
    }
    zw_s[rr][cc] = zw; ze_s[rr][cc] = ze; dvx_s[rr][cc] = dv;
  }

  for (int f = 0; f < nf; ++f) {
    const T *cur0;
    T *out0, *wz0;
    field_t<R, T>(D, 0, f, adv, cur0, out0, wz0);
    const T *pp = cur0 + ko;
    const T *wz = wz0 + ko;
    T *out = out0 + ko;
    (void)wz;
    // the field's halo tile (zero outside the cross points)
    const int b = f & 1;
    const bool landed = mbar_wait_bounded(&mbar[b], (unsigned)((f >> 1) & 1));
    if (__syncthreads_or(!landed)) {  // also orders the factors above before their use
      if (tid == 0) {
        atomicOr(&D.clk->fault, 1);
        // let copies still in flight land before the shared memory is released
        mbar_wait_bounded(&mbar[b], (unsigned)((f >> 1) & 1));
        if (f + 1 < nf) mbar_wait_bounded(&mbar[b ^ 1], (unsigned)(((f + 1) >> 1) & 1));
      }
      return;
    }
    T (*wz_s)[BW] = wzt[b];
    // meridional fluxes zpby(j,i): j in jce, i in ici1..ice2
    for (int e = tid; e < (kTI + 1) * WJ; e += nth) {
      const int rr = e / WJ, cc = e % WJ;
      const int i = I0 + rr, j = J0 - 2 + cc;
      T x = T(0);
      if (j >= 1 && j <= jx - 1 && i >= 2 && i <= iy - 1) {
        const T vv = vy_s[rr][cc];
        const T zamu = zmy_s[rr][cc];
        T is;
        int ih;
        if (zamu > T(0)) { is = T(1); ih = i - 1; }
        else { is = T(-1); ih = min(i + 1, imax); }
        const int ihm1 = max(ih - 1, imin);
        const int bo = 2 - I0;  // shared-memory row of global row i is i + bo
        x = waf_flux<T>(T(0.5) * vv, is, zamu, wz_s[i - 1 + bo][cc + OFF], wz_s[i + bo][cc + OFF],
                        wz_s[ih + bo][cc + OFF] - wz_s[ihm1 + bo][cc + OFF]);
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
        const T ppk = pp[g.at2(j, i)];
        const T wzk = wz_s[rr + 2][cc + OFF];
        const T zdv = dvy_s[rr][cc] * ppk;
        const T zrfms = zs_s[rr][cc], zrfmn = zn_s[rr][cc];
        if (rot) x = wzk + (zpby_s[rr][cc] * zrfms - zpby_s[rr + 1][cc] * zrfmn + zdv);
        else x = wzk + m2_s[rr][cc] * (zpby_s[rr][cc] * zrfms - zpby_s[rr + 1][cc] * zrfmn + zdv);
      }
      p0_s[rr][cc] = x;
    }
    __syncthreads();
    // buffer b is read for the last time above: fetch the field after next
    if (tid == 0 && f + 2 < nf) issue(f + 2, b);
    // zonal fluxes zpbw(j,i): j in jci1..jce2, i in ici
    for (int e = tid; e < kTI * (kTJ + 1); e += nth) {
      const int rr = e / (kTJ + 1), cc = e % (kTJ + 1);
      const int i = I0 + rr, j = J0 + cc;
      T x = T(0);
      if (j >= 2 && j <= jx - 1 && i >= 2 && i <= iy - 2) {
        const T uu = ux_s[rr][cc];
        const T zamu = zmx_s[rr][cc];
        T is;
        int jh;
        if (zamu > T(0)) { is = T(1); jh = j - 1; }
        else { is = T(-1); jh = min(j + 1, jmax); }
        const int jhm1 = max(jh - 1, jmin);
        const int bo = 2 - J0;  // p0_s column of global column j is j + bo
        x = waf_flux<T>(T(0.5) * uu, is, zamu, p0_s[rr][j - 1 + bo], p0_s[rr][j + bo],
                        p0_s[rr][jh + bo] - p0_s[rr][jhm1 + bo]);
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
          const T p0k = p0_s[rr][cc + 2];
          const T zrfmw = zw_s[rr][cc], zrfme = ze_s[rr][cc];
          const T zdv = dvx_s[rr][cc] * ppk;
          if (rot) x = p0k + zpbw_s[rr][cc] * zrfmw - zpbw_s[rr][cc + 1] * zrfme + zdv;
          else x = p0k + m2_s[rr][cc + 2] * (zpbw_s[rr][cc] * zrfmw - zpbw_s[rr][cc + 1] * zrfme + zdv);
        }
        out[ij] = x;
      }
    }
  }
}

// Species that are not advected (ipptls = 0: qx(iqfrst:nqx)) keep their
// values when the advected fields move to the other half of their pairs.
template <class R>
__global__ void k_species_copy(const Dom<R> *__restrict__ doms, int advoff, int tiles_j) {
  const Dom<R> &D = doms[blockIdx.z];
  if (!D.active) return;
  const Geom g = D.g;
  const Pt q = point_of(tiles_j, 1, 1);
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
__global__ void k_adv_curvature(const Dom<R> *__restrict__ doms, int advoff, int tiles_j) {
  const Dom<R> &D = doms[blockIdx.z];
  if (!D.active || !D.c.curvature) return;
  const Geom g = D.g;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const int adv = (D.clk->adv_role + advoff) & 1;
  R *__restrict__ ux = D.ux[adv];
  R *__restrict__ vx = D.vx[adv];
  const Pt q_ = point_of(tiles_j, 2, 2);
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
__global__ void k_adv_back(const Dom<R> *__restrict__ doms, int uvoff, int advoff, int tiles_j) {
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
  const Pt q_ = point_of(tiles_j, 1, 1);
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
  const int CX = blockDim.x, KT = blockDim.y;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const Dom<R> &D = doms[blockIdx.z];
  if (!D.active) return;
  const int tiles_j = gridDim.x / 2;
  const int f = blockIdx.x / tiles_j;
  const int bj = blockIdx.x - f * tiles_j;
  const Geom g = D.g;
  const int kz = g.kz;
  const int i = blockIdx.y + 1;
  if (i > g.iy - 1 || bj * CX + 1 > g.jx - 1) return;
  const int j = bj * CX + tx + 1;
  const bool on = j <= g.jx - 1;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const int adv = (D.clk->adv_role + advoff) & 1;
  const size_t F = g.field3();
  const DF src(f == 0 ? D.tetav[adv] : D.pai[adv], F);
  const DF dst(D.wz_d[f], F);
  const R *__restrict__ s = D.s;
  const size_t L = (size_t)(kz + 2) * CX;
  float *dzs = vsm;           // v(k+1) - v(k), k = 1..kz-1
  float *e = vsm + L;         // increment of the pass input, k = 1..kz
  float *flo = vsm + 2 * L;   // flux at k+1 relative to cell k, k = 1..kz-1
  float *sc = vsm + 3 * L;    // s, levels 1..kz+1
  float *zu = vsm + 4 * L;
  float *zd = vsm + 5 * L;
#define A(a, k) a[(size_t)(k) * CX + tx]
  const size_t ij = on ? g.at2(j, i) : 0, PS = g.PS;
  const float dtrdz = 0.5f * (c.dtstepaf * c.rdzitaf);
  if (on)
    for (int k = 1 + ty; k <= kz + 1; k += KT) {
      const size_t o = ij + (size_t)(k - 1) * PS;
      A(sc, k) = float(s[o]);
      if (k <= kz) {
        A(e, k) = 0.f;
        A(zu, k) = float(sa.zrfmu[o]);
        A(zd, k) = float(sa.zrfmd[o]);
        if (k <= kz - 1) A(dzs, k) = df_diff(src.ld(o + PS), src.ld(o));
      }
    }
  __syncthreads();
  // the threads owning the bottom and top cells keep their FP32 parts and
  // double-float constant parts in registers over both passes
  float eb32 = 0.f, et32 = 0.f;
  F2 hb{0.f, 0.f}, ht{0.f, 0.f};
  for (int pass = 0; pass < 2; ++pass) {
    if (on)
      for (int k = 1 + ty; k <= kz - 1; k += KT) {
        const float skp = A(sc, k + 1);
        const float zamu = skp * dtrdz;
        const float ek = A(e, k), ekp1 = A(e, k + 1);
        float is, num;
        if (zamu >= 0.f) {
          is = 1.f;
          num = k + 2 <= kz ? (ekp1 - A(e, k + 2)) - A(dzs, k + 1) : 0.f;
        } else {
          is = -1.f;
          num = k >= 2 ? (A(e, k - 1) - ek) - A(dzs, k - 1) : 0.f;
        }
        A(flo, k) = waf_flux<float>(0.5f * skp, is, zamu, A(dzs, k) + ekp1, ek, num);
      }
    __syncthreads();
    if (on)
      for (int k = 1 + ty; k <= kz; k += KT) {
        const float sk = A(sc, k), skp = A(sc, k + 1);
        const float zrfmu = A(zu, k), zrfmd = A(zd, k);
        const float ek = A(e, k);
        // flux below, moved to cell k; flux above, relative to cell k
        const float fb = k >= 2 ? A(flo, k - 1) - sk * A(dzs, k - 1) : 0.f;
        const float fa = k <= kz - 1 ? A(flo, k) : 0.f;
        const float upd = -fb * zrfmu + fa * zrfmd + (sk * zrfmu - skp * zrfmd) * ek;
        float en;
        if (k == kz) {
          // no flux through kz+1: constant part -v*s(kz+1)*zrfmd, exact product
          et32 += upd;
          ht = df_add(ht, df_mul(src.ld(ij + (size_t)(kz - 1) * PS), two_prod(-skp, zrfmd)));
          en = et32 + df_f(ht);
        } else if (k == 1) {
          // no flux through level 1: constant part v*s(1)*zrfmu (s(1) = 0 inside)
          eb32 += upd;
          hb = df_add(hb, df_mul(src.ld(ij), two_prod(sk, zrfmu)));
          en = eb32 + df_f(hb);
        } else {
          en = ek + upd;
        }
        A(e, k) = en;
      }
    __syncthreads();
  }
  if (on)
    for (int k = 1 + ty; k <= kz; k += KT) {
      F2 d;
      if (k == kz) d = df_add_f(ht, et32);
      else if (k == 1) d = df_add_f(hb, eb32);
      else d = F2{A(e, k), 0.f};
      dst.st(ij + (size_t)(k - 1) * PS, d);
    }
#undef A
}

// Meridional then zonal WAF of one tile (:984-1038; ROTLLR :926-983) in
// increment form.  pp is the field at the start of the advection step, dz
// its vertical increment; out = pp + dz + (meridional + zonal increments).
template <class R, int kTJ, int kTI>
__global__ void __launch_bounds__(kTJ *kTI) k_adv_horizontal_inc(const Dom<R> *__restrict__ doms,
                                                                int tiles_j, int uvoff,
                                                                int advoff) {
  constexpr int WJ = kTJ + 4;          // columns J0-2 .. J0+TJ+1
  __shared__ float pph_s[kTI + 4][WJ];  // rows I0-2 .. I0+TI+1: pp as hi + lo
  __shared__ float ppl_s[kTI + 4][WJ];
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
  const size_t F = g.field3();
  const DF pp(f == 0 ? D.tetav[adv] : D.pai[adv], F);
  const DF out(f == 0 ? D.tetav[adv ^ 1] : D.pai[adv ^ 1], F);
  const DF dzg(D.wz_d[f], F);
  const R *__restrict__ uk = D.u[uv] + ko;
  const R *__restrict__ vk = D.v[uv] + ko;
  const int tid = threadIdx.y * kTJ + threadIdx.x;
  const int nth = kTJ * kTI;
  const float dta = c.dtstepaf;
  const float dtrdx = dta * c.rdxf, dtrdy = dta * c.rdxf;
  const bool rot = c.lrotllr != 0;
  const int imin = 1, imax = iy - 1, jmin = 1, jmax = jx - 1;

  for (int e = tid; e < (kTI + 4) * WJ; e += nth) {
    const int rr = e / WJ, cc = e % WJ;
    const int i = I0 - 2 + rr, j = J0 - 2 + cc;
    F2 x{0.f, 0.f};
    float z = 0.f;
    if (i >= 1 && i <= iy - 1 && j >= 1 && j <= jx - 1) {
      const size_t ij = g.at2(j, i) + ko;
      x = pp.ld(ij);
      z = df_f(dzg.ld(ij));
    }
    pph_s[rr][cc] = x.hi;
    ppl_s[rr][cc] = x.lo;
    dz_s[rr][cc] = z;
  }
  __syncthreads();
  for (int e = tid; e < (kTI + 3) * WJ; e += nth) {
    const int rr = e / WJ, cc = e % WJ;
    dy_s[rr][cc] = (pph_s[rr + 1][cc] - pph_s[rr][cc]) + (ppl_s[rr + 1][cc] - ppl_s[rr][cc]);
  }
  for (int e = tid; e < kTI * (kTJ + 3); e += nth) {
    const int rr = e / (kTJ + 3), cc = e % (kTJ + 3);
    dx_s[rr][cc] = (pph_s[rr + 2][cc + 1] - pph_s[rr + 2][cc]) +
                   (ppl_s[rr + 2][cc + 1] - ppl_s[rr + 2][cc]);
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
          hy += pph_s[rr + 2][cc] * (mx2 * (vs * zrfms * (1.f - rs) - vn * zrfmn * (1.f - rn)));
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
      const F2 ppk{pph_s[rr + 2][cc + 2], ppl_s[rr + 2][cc + 2]};
      F2 x = ppk;
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
            hx += ppk.hi * (mx2 * (uw * zrfmw * (1.f - rw) - ue * zrfme * (1.f - re)));
        }
        x = df_add_f(df_add(ppk, dzg.ld(ij + ko)), hy_s[rr][cc + 2] + hx);
      }
      out.st(ij + ko, x);
    }
  }
}

// grid of a point kernel over nj x ni points per level
inline dim3 pt_grid(const LaunchGeom &L, int nj, int ni, int &tiles_j) {
  tiles_j = (nj + L.col_x - 1) / L.col_x;
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
  k_adv_prep<R><<<grd, b, 0, s>>>(d, uvoff, advoff, tj);
}

template <class R, class T>
void launch_vertical(const LaunchGeom &L, const Dom<R> *d, int nf, int set, int advoff,
                     cudaStream_t s) {
  // vert_x columns along j per block, vert_y threads along the levels
  const dim3 b((unsigned)L.vert_x, (unsigned)L.vert_y);
  const size_t smem = (size_t)5 * (L.kz + 2) * b.x * sizeof(T);
  const dim3 grd((unsigned)(((L.jx - 1 + L.vert_x - 1) / L.vert_x) * nf), (unsigned)(L.iy - 1),
                 (unsigned)L.nmem);
  k_adv_vertical<R, T><<<grd, b, smem, s>>>(d, nf, set, advoff);
}

template <class R, int TJ, int TI>
void launch_tile(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s) {
  const int tj = (L.jx - 1 + TJ - 1) / TJ, ti = (L.iy - 1 + TI - 1) / TI;
  const dim3 grd((unsigned)(tj * ti), (unsigned)L.kz, (unsigned)L.nmem);
  k_adv_horizontal<R, TJ, TI><<<grd, dim3(TJ, TI), 0, s>>>(d, tj, uvoff, advoff);
}

template <class R>
void launch_horizontal(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s) {
  switch (L.htile) {
    case 1: launch_tile<R, 32, 4>(L, d, uvoff, advoff, s); break;
    case 2: launch_tile<R, 64, 4>(L, d, uvoff, advoff, s); break;
    case 3: launch_tile<R, 16, 8>(L, d, uvoff, advoff, s); break;
    default: launch_tile<R, 32, 8>(L, d, uvoff, advoff, s); break;
  }
}

template <class R>
void launch_vertical_inc(const LaunchGeom &L, const Dom<R> *d, int advoff, cudaStream_t s) {
  const dim3 b((unsigned)L.vert_x, (unsigned)L.vert_y);
  const size_t smem = (size_t)6 * (L.kz + 2) * b.x * sizeof(float);
  const dim3 grd((unsigned)(((L.jx - 1 + L.vert_x - 1) / L.vert_x) * 2), (unsigned)(L.iy - 1),
                 (unsigned)L.nmem);
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
  launch_horizontal<R>(L, d, uvoff, advoff, s);
  if constexpr (sizeof(R) == sizeof(float))
    if (L.nadv_d) launch_horizontal_inc<R>(L, d, uvoff, advoff, s);
}

template <class R>
void Launch<R>::adv_species_copy(const LaunchGeom &L, const Dom<R> *d, int advoff, cudaStream_t s) {
  const dim3 b((unsigned)L.col_x, (unsigned)L.col_y);
  int tj;
  const dim3 grd = pt_grid(L, L.jx - 1, L.iy - 1, tj);
  k_species_copy<R><<<grd, b, 0, s>>>(d, advoff, tj);
}

template <class R>
void Launch<R>::adv_curvature(const LaunchGeom &L, const Dom<R> *d, int advoff, cudaStream_t s) {
  const dim3 b((unsigned)L.col_x, (unsigned)L.col_y);
  int tj;
  const dim3 grd = pt_grid(L, L.jx - 3, L.iy - 3, tj);
  k_adv_curvature<R><<<grd, b, 0, s>>>(d, advoff, tj);
}

template <class R>
void Launch<R>::adv_back(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s) {
  const dim3 b((unsigned)L.col_x, (unsigned)L.col_y);
  int tj;
  const dim3 grd = pt_grid(L, L.jx, L.iy, tj);
  k_adv_back<R><<<grd, b, 0, s>>>(d, uvoff, advoff, tj);
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
