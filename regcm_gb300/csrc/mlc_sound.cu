// mlc_sound.cu -- the acoustic substeps of the MOLOCH step
// (Main/mod_moloch.F90:531-765, subroutines sound, divergence_damping,
// divergence_diffusion).
//
// One substep is three kernels:
//   sound_div       per column of cross points: raw horizontal divergence
//                   zdiv2 (Eq. 16) and the generalized vertical velocity s
//                   (Eq. 10), s(kz+1) and the surface w.
//   sound_solve     per interior column, one thread per column: the 5-point
//                   divergence filter, the vertical divergence term, the
//                   implicit w-Exner tridiagonal system (Eq. 19, Thomas
//                   algorithm with the column held in shared memory), the
//                   Exner update and, after the last substep, the completed s.
//   sound_momentum  u and v (Eq. 17/18): divergence damping, Coriolis with
//                   the substep's initial winds, pressure gradient with the new
//                   Exner function, terrain term, relaxation-zone weight.  It
//                   writes the other half of a ping-pong pair, which is how the
//                   reference's ud/vd copies are kept without a copy.
// Every expression keeps the reference's operands and association order; the
// only departures are FMA contraction by the compiler and the relaxation
// weight bdywt recomputed from ibnd and hefc instead of read from an array
// (the same value, Main/mod_bdycod.F90:4033-4047).
#include "mlc_kernels.cuh"
#include "mlc_tma.cuh"

namespace mlc {

namespace {


__device__ __forceinline__ double relax_weight(const int32_t *ibnd, const double *hefc, int nsp,
                                               size_t ij, int k) {
  int ib = ibnd[ij];
  return ib > 0 ? 1.0 - hefc[(size_t)(ib - 1) + (size_t)(k - 1) * nsp] : 1.0;
}

template <class R>
__global__ void k_sound_prep(const Dom<R> *__restrict__ doms, int advoff, int tiles_j,
    const WorkItem *__restrict__ wl) {
  const WorkItem wi = work_item(wl, tiles_j);
  const Dom<R> &D = doms[wi.m];
  if (!D.active) return;
  const Geom g = D.g;
  const Pt q = point_at(wi, 1, 1);
  if (q.j > g.jx - 1 || q.i > g.iy - 1 || q.k > g.kz) return;
  const int adv = (D.clk->adv_role + advoff) & 1;
  const double *__restrict__ tetav = D.tetav[adv];
  double *__restrict__ tetavf = D.tetavf;
  // Main/mod_moloch.F90:564-566, levels 2..kz
#pragma unroll
  for (int k = q.k < 2 ? 2 : q.k; k < q.k + kPtLevels && k <= g.kz; ++k) {
    const size_t o = g.at(q.j, q.i, k), om = o - g.PS;
    if constexpr (sizeof(R) == sizeof(float)) {
      // double-float theta_v; also theta_v(k-1) - theta_v(k) for the substeps'
      // solves (the scratch wz[2] is free until the advection of this round)
      const DF th(tetav, g.field3()), tf(tetavf, g.PS * (size_t)(g.kz + 1));
      const F2 lo = th.ld(om), hi = th.ld(o);
      const F2 sm = df_add(lo, hi);
      tf.st(o, F2{0.5f * sm.hi, 0.5f * sm.lo});
      D.wz[2][o] = df_diff(lo, hi);
    } else {
      tetavf[o] = 0.5 * (tetav[om] + tetav[o]);
    }
  }
}

// Main/mod_moloch.F90:582-618
template <class R>
__global__ void k_sound_div(const Dom<R> *__restrict__ doms, int uvoff, int tiles_j,
    const WorkItem *__restrict__ wl) {
  const WorkItem wi = work_item(wl, tiles_j);
  const Dom<R> &D = doms[wi.m];
  if (!D.active) return;
  const Geom g = D.g;
  const Pt q = point_at(wi, 1, 1);
  const int j = q.j, i = q.i, kz = g.kz;
  if (j > g.jx - 1 || i > g.iy - 1 || q.k > kz) return;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const int uv = (D.clk->uv_role + uvoff) & 1;
  const R *__restrict__ u = D.u[uv];
  const R *__restrict__ v = D.v[uv];
  R *__restrict__ zdiv2 = D.zdiv2;
  R *__restrict__ s = D.s;
  R *__restrict__ w = D.w;
  const R dtrdx = pick<R>(c.dtrdxs, c.dtrdxsf), dtrdy = dtrdx;
  const size_t ij = g.at2(j, i), ijE = g.at2(j + 1, i), ijN = g.at2(j, i + 1);
  const bool interior = (j >= 2 && j <= g.jx - 2 && i >= 2 && i <= g.iy - 2);
  const R rmu0 = sa.rmu[ij], rmu1 = sa.rmu[ijE], rmv0 = sa.rmv[ij], rmv1 = sa.rmv[ijN];
  const R mfac = c.lrotllr ? sa.msfx[ij] : sa.mx2[ij];
  R hx0 = 0, hx1 = 0, hy0 = 0, hy1 = 0;
  if (interior) {
    hx0 = sa.hx[ij]; hx1 = sa.hx[ijE]; hy0 = sa.hy[ij]; hy1 = sa.hy[ijN];
  }
#pragma unroll
  for (int k = q.k; k < q.k + kPtLevels && k <= kz; ++k) {
  const size_t o = (size_t)(k - 1) * g.PS;
  const R u0 = u[ij + o], u1 = u[ijE + o], v0 = v[ij + o], v1 = v[ijN + o];
  if constexpr (sizeof(R) == sizeof(double)) {
    // the constant factors formed at bind time: u*(dtrdx*rfmzu*rmu) for
    // dtrdx*u*rfmzu*rmu (one FP64 product a flux instead of three)
    const R zum = u0 * sa.dv_cu[ij + o], zup = u1 * sa.dv_cu[ijE + o];
    const R zvm = v0 * sa.dv_cv[ij + o], zvp = v1 * sa.dv_cv[ijN + o];
    zdiv2[ij + o] = sa.dv_cf[ij + o] * ((zup - zum) + (zvp - zvm));
  } else {
  R zum, zup;
  if (c.lrotllr) {
    zum = dtrdx * u0 * sa.rfmzu[ij + o];
    zup = dtrdx * u1 * sa.rfmzu[ijE + o];
  } else {
    zum = dtrdx * u0 * sa.rfmzu[ij + o] * rmu0;
    zup = dtrdx * u1 * sa.rfmzu[ijE + o] * rmu1;
  }
  const R zvm = dtrdy * v0 * sa.rfmzv[ij + o] * rmv0;
  const R zvp = dtrdy * v1 * sa.rfmzv[ijN + o] * rmv1;
  zdiv2[ij + o] = sa.fmz[ij + o] * mfac * ((zup - zum) + (zvp - zvm));
  }
  if (!interior) continue;
  if (k >= 2) {
    const size_t om = o - g.PS;  // level k-1
    const R um = u[ij + om], up = u[ijE + om], vm = v[ij + om], vp = v[ijN + om];
    const R zuh = (u0 + um) * hx0 + (u1 + up) * hx1;
    const R zvh = (v0 + vm) * hy0 + (v1 + vp) * hy1;
    s[ij + o] = -(R(0.25) * (zuh + zvh) * sa.gzitak_r[k - 1]);
  }
  if (k == kz) {
    const R zuh = u0 * hx0 + u1 * hx1;
    const R zvh = v0 * hy0 + v1 * hy1;
    const R skp1 = -(R(0.5) * (zuh + zvh));
    s[ij + (size_t)kz * g.PS] = skp1;
    w[ij + (size_t)kz * g.PS] = -skp1;
  }
  }
}

// The implicit w-Exner solve of an FP64 member (Main/mod_moloch.F90:627-671,
// s :728-734): per interior column the filtered divergence plus its vertical
// part, the Thomas elimination k = kz..2, back substitution, the Exner
// update and (after the last substep) s.  Same structure as the mixed solve
// below: a block is one 128-column row segment, one thread per column, the
// downward pass forms each level's coefficients and eliminates at once, the
// upward pass substitutes back and updates Exner a level behind; every
// level's planes arrive in shared memory as 1 KB row segments by bulk copies
// kDvStages levels ahead (the raw divergence with a 2-column halo).  Between
// the passes the eliminated w stays in w, the multipliers and the filtered
// divergence in the scratch planes wz[1] and wz[0] (free during the acoustic
// loop).  The per-level expressions are the reference's, in its order.
// (Measured on the 512x512x41 step: 3.99 ms of solves a step against 5.68
// for a column-in-shared-memory form, whose 66 KB a block left 6 warps an SM.)
// Levels read between two block barriers of the streamed column solves (a
// barrier frees the stages read since the last one for their refill).
#ifndef MLC_SOLVE_SYNC
#define MLC_SOLVE_SYNC 1
#endif
constexpr int kSolveSync = MLC_SOLVE_SYNC;
#ifndef MLC_DV_STAGES
#define MLC_DV_STAGES 3
#endif
constexpr int kDvStages = MLC_DV_STAGES;  // FP64 solve: levels in flight
constexpr int kDvW = kSolveColsD;
constexpr int kDvZW = kDvW + 4;                   // raw divergence row, 2-column halo each side
// The FP64 solve reads its metric products from bind time - (bw*dtrdz)*fmz,
// zcs2*fmz, dtrdz*fmz, the same roundings as forming them per level - (1),
// or forms them from fmz and the zone weight every level (0).
#ifndef MLC_SOLVE_PRE
#define MLC_SOLVE_PRE 1
#endif
constexpr bool kSolvePre = MLC_SOLVE_PRE != 0;
constexpr int kDvStage = 3 * kDvZW + (kSolvePre ? 8 : 7) * kDvW;   // doubles of one stage
template <class R>
__global__ void __launch_bounds__(kDvW, 4) k_sound_solve(const Dom<R> *__restrict__ doms, int advoff, int last,
    const WorkItem *__restrict__ wl) {
  static_assert(sizeof(R) == sizeof(double), "FP64 member");
  constexpr int NS = kDvStages;
  extern __shared__ __align__(16) double dv_smem[];
  __shared__ __align__(8) uint64_t mbar[NS];
  const WorkItem wi = wl ? wl[blockIdx.x]
                          : WorkItem{(int16_t)blockIdx.z, (int16_t)blockIdx.x, (int16_t)blockIdx.y, 0};
  const Dom<R> &D = doms[wi.m];
  if (!D.active) return;
  const Geom g = D.g;
  const int t = (int)threadIdx.x;
  const int x0 = (int)wi.a * kDvW;
  const int i = (int)wi.b + 2;
  if (x0 + 1 > g.jx - 2 || i > g.iy - 2) return;  // uniform over the block
  const int j = x0 + t + 1;
  const bool act = j >= 2 && j <= g.jx - 2;
  const int kz = g.kz;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const int adv = (D.clk->adv_role + advoff) & 1;
  const int PS = (int)g.PS, P = g.P;
  const size_t r0 = g.at2(1, i);
  const double *__restrict__ zraw = D.zdiv2 + r0;
  double *__restrict__ s = D.s + r0;
  double *__restrict__ w = D.w + r0;
  double *__restrict__ pai = D.pai[adv] + r0;
  const double *__restrict__ tetav = D.tetav[adv] + r0;
  double *__restrict__ tetavf = D.tetavf + r0;
  // with the products from bind time, fmz's place (down pass, up pass) holds
  // (bw*dtrdz)*fmz and dtrdz*fmz, and zcs2*fmz comes as an eighth plane
  const double *__restrict__ fmz = (kSolvePre ? sa.sv_a : sa.fmz_d) + r0;
  const double *__restrict__ fmz_up = (kSolvePre ? sa.sv_c : sa.fmz_d) + r0;
  const double *__restrict__ fmzb = (kSolvePre ? sa.sv_b : sa.fmz_d) + r0;
  const double *__restrict__ fmzf = sa.fmzf_d + r0;
  double *__restrict__ zfs = D.wz[0] + r0;   // free during the acoustic loop
  double *__restrict__ mul = D.wz[1] + r0;
  const double dts = c.dtsound;
  const double dtrdz = dts * c.rdzita;
  const double zcs2 = (dtrdz * dtrdz) * kRdrcv;
  const int ij_off = j - 1;
  const size_t ij = r0 + (size_t)ij_off;
  const bool filt = c.divfilter != 0;
  const int xe = min(x0 + kDvW, P);
  const int zs = x0 >= 2 ? x0 - 2 : 0, ze = min(x0 + kDvW + 2, P);
  const unsigned wb = (unsigned)(xe - x0) * 8u, zb = (unsigned)(ze - zs) * 8u;
  const int zc = x0 + t - zs;
  auto stage = [&](int b) { return dv_smem + (size_t)b * kDvStage; };
  auto fld = [&](double *st, int f) { return st + 3 * kDvZW + f * kDvW; };
  const int nd = kz - 1;
  // down unit u (m = kz-1-u): zraw rows, s, fmz, pai, tetav at m; w, fmzf, tetavf at m+1
  auto issue_down = [&](int u, int b) {
    const int m = kz - 1 - u;
    double *st = stage(b);
    uint64_t *bar = &mbar[b];
    fence_proxy_async();
    mbar_expect_tx(bar, (filt ? 3u : 1u) * zb + (kSolvePre ? 8u : 7u) * wb);
    const int o = (m - 1) * PS, ob = m * PS;
    bulk_load(st, zraw + o + zs, zb, bar);
    if (filt) {
      bulk_load(st + kDvZW, zraw + o - P + zs, zb, bar);
      bulk_load(st + 2 * kDvZW, zraw + o + P + zs, zb, bar);
    }
    bulk_load(fld(st, 0), s + o + x0, wb, bar);
    bulk_load(fld(st, 1), fmz + o + x0, wb, bar);
    bulk_load(fld(st, 2), pai + o + x0, wb, bar);
    bulk_load(fld(st, 3), tetav + o + x0, wb, bar);
    bulk_load(fld(st, 4), w + ob + x0, wb, bar);
    bulk_load(fld(st, 5), fmzf + ob + x0, wb, bar);
    bulk_load(fld(st, 6), tetavf + ob + x0, wb, bar);
    if constexpr (kSolvePre) bulk_load(fld(st, 7), fmzb + o + x0, wb, bar);
  };
  // up unit v (m = v + 2): w(m), mul(m) (m <= kz); pai, zfs, fmz, s, fmzf at m-1
  auto issue_up = [&](int v, int b) {
    const int m = v + 2;
    double *st = stage(b);
    uint64_t *bar = &mbar[b];
    fence_proxy_async();
    mbar_expect_tx(bar, (m <= kz ? 7u : 6u) * wb);
    const int o = (m - 1) * PS, op = (m - 2) * PS;
    bulk_load(fld(st, 0), w + o + x0, wb, bar);
    if (m <= kz) bulk_load(fld(st, 1), mul + o + x0, wb, bar);
    bulk_load(fld(st, 2), pai + op + x0, wb, bar);
    bulk_load(fld(st, 3), zfs + op + x0, wb, bar);
    bulk_load(fld(st, 4), fmz_up + op + x0, wb, bar);
    bulk_load(fld(st, 5), s + op + x0, wb, bar);
    bulk_load(fld(st, 6), fmzf + op + x0, wb, bar);
  };
  auto bail = [&](int gnext, int gend) {
    if (t == 0) {
      atomicOr(&D.clk->fault, 1);
      for (int q = gnext; q < gend && q < gnext + NS; ++q) mbar_wait_bounded(&mbar[q % NS], (unsigned)((q / NS) & 1));
    }
  };
  if (t == 0) {
    for (int q = 0; q < NS; ++q) mbar_init(&mbar[q], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (t == 0)
    for (int u = 0; u < NS && u < nd; ++u) issue_down(u, u);
  // filtered divergence plus the vertical part of level m (:531-543, :627-630)
  // fz: fmz, or (bw*dtrdz)*fmz from bind time
  auto zf_of = [&](int m, double z, double lap, double fz, double sm, double sm1) {
    if (filt) z = z + sa.xknu[m - 1] * lap;
    if constexpr (kSolvePre) return z + fz * (sm - sm1);
    const double bw = relax_weight(sa.ibnd_cr, sa.hefc, c.nspgx, ij, m);
    return z + bw * dtrdz * fz * (sm - sm1);
  };
  // fmz_k: fmz of level k, or zcs2*fmz from bind time
  double wnext = 0.0, wkp1 = 0.0, zfk = 0.0, pai_k = 0.0, tet_k = 0.0, fmz_k = 0.0, s_k = 0.0;
  if (act) {
    const int o = (kz - 1) * PS + ij_off;
    const double z = zraw[o];
    const double lap = filt ? (zraw[o - 1] + zraw[o + 1] + zraw[o - P] + zraw[o + P] - 4.0 * z) : 0.0;
    s_k = s[o];
    fmz_k = fmzb[o];
    zfk = zf_of(kz, z, lap, fmz[o], s_k, s[kz * PS + ij_off]);
    pai_k = pai[o];
    tet_k = tetav[o];
    wnext = w[kz * PS + ij_off];  // w(kz+1) = -s(kz+1)
  }
  bool ok = true;
  int synced = 0;  // first unit read since the last block barrier
  for (int u = 0; u < nd; ++u) {
    const int k = kz - u, m = k - 1;
    const int b = u % NS;
    const bool landed = mbar_wait_bounded(&mbar[b], (unsigned)((u / NS) & 1));
    const double *st = stage(b);
    if (act) {
      const int o = (k - 1) * PS + ij_off;
      const double z = st[zc];
      const double lap = filt ? (st[zc - 1] + st[zc + 1] + st[kDvZW + zc] + st[2 * kDvZW + zc] - 4.0 * z) : 0.0;
      const double *f0 = st + 3 * kDvZW + t;
      const double s_m = f0[0], fza_m = f0[kDvW], pai_m = f0[2 * kDvW], tet_m = f0[3 * kDvW];
      const double wold = f0[4 * kDvW], fmzf_k = f0[5 * kDvW], tvf0 = f0[6 * kDvW];
      const double fmz_m = kSolvePre ? f0[7 * kDvW] : fza_m;
      const double zf_m = zf_of(m, z, lap, fza_m, s_m, s_k);
      zfs[o] = zfk;
      const double tvf = tvf0 - wold * fmzf_k * dtrdz * (tet_m - tet_k);
      tetavf[o] = tvf;
      const double zrom1w = kCpd * tvf * fmzf_k;
      double zwexpl = wold - zrom1w * dtrdz * (pai_m - pai_k) - kGrav * dts;
      zwexpl = zwexpl + kRdrcv * zrom1w * dtrdz * (pai_m * zf_m - pai_k * zfk);
      const double ff = sa.ffilt[k - 1];
      double zu, zd;
      if constexpr (kSolvePre) {
        zu = fmz_m * zrom1w * pai_m + ff;  // fmz_m = zcs2*fmz
        zd = fmz_k * zrom1w * pai_k + ff;
      } else {
        zu = zcs2 * fmz_m * zrom1w * pai_m + ff;
        zd = zcs2 * fmz_k * zrom1w * pai_k + ff;
      }
      const double zrapp = 1.0 / (1.0 + zd + zu - zd * wkp1);
      wnext = zrapp * (zwexpl + zd * wnext);
      wkp1 = zrapp * zu;
      w[o] = wnext;
      mul[o] = wkp1;
      zfk = zf_m;
      pai_k = pai_m; tet_k = tet_m; fmz_k = fmz_m; s_k = s_m;
    }
    ok = ok && landed;
    if ((u + 1) % kSolveSync == 0 || u + 1 == nd) {
      if (__syncthreads_or(!ok)) {
        bail(u + 1, min(nd, synced + NS));  // the units issued and not read
        return;
      }
      // the stages read since the last barrier are free: refill them
      if (t == 0)
        for (int r = synced; r <= u; ++r)
          if (r + NS < nd) issue_down(r + NS, r % NS);
      synced = u + 1;
    }
  }
  if (act) zfs[ij_off] = zfk;  // level 1
  fence_proxy_async_global();
  __syncthreads();
  const int nu = kz;
  if (t == 0)
    for (int v = 0; v < NS && v < nu; ++v) issue_up(v, (nd + v) % NS);
  // Exner (:668-671) of level m once w(m+1) is known, and s (:728-734)
  // fz: fmz, or dtrdz*fmz from bind time
  auto exner = [&](int m, double wm, double wmp, double pk, double zf, double fz, double sm, double fzf) {
    const int o = (m - 1) * PS + ij_off;
    if constexpr (kSolvePre) pai[o] = pk * (1.0 - kRdrcv * (zf + (fz * (wm - wmp))));
    else pai[o] = pk * (1.0 - kRdrcv * (zf + (dtrdz * fz * (wm - wmp))));
    if (last && m >= 2) s[o] = (wm + sm) * fzf;
  };
  double wprev = act ? w[ij_off] : 0.0;  // w(1) = 0
  ok = true;
  synced = 0;
  for (int v = 0; v < nu; ++v) {
    const int k = v + 2, gu = nd + v;
    const int b = gu % NS;
    const bool landed = mbar_wait_bounded(&mbar[b], (unsigned)((gu / NS) & 1));
    if (act) {
      const double *f0 = stage(b) + 3 * kDvZW + t;
      const double wel = f0[0];
      const double cp = f0[2 * kDvW], czf = f0[3 * kDvW], cfz_ = f0[4 * kDvW], cs = f0[5 * kDvW],
                   cfzf = f0[6 * kDvW];
      if (k <= kz) {
        const double wk = wel + f0[kDvW] * wprev;
        w[(k - 1) * PS + ij_off] = wk;
        exner(k - 1, wprev, wk, cp, czf, cfz_, cs, cfzf);
        wprev = wk;
      } else {
        exner(kz, wprev, wel, cp, czf, cfz_, cs, cfzf);
      }
    }
    ok = ok && landed;
    if ((v + 1) % kSolveSync == 0 || v + 1 == nu) {
      if (__syncthreads_or(!ok)) {
        bail(gu + 1, nd + min(nu, synced + NS));
        return;
      }
      if (t == 0)
        for (int r = synced; r <= v; ++r)
          if (r + NS < nu) issue_up(r + NS, (nd + r) % NS);
      synced = v + 1;
    }
  }
  if (last && act) {
    s[ij_off] = 0.0;
    s[kz * PS + ij_off] = 0.0;
  }
}
#ifndef MLC_SV_STAGES
#define MLC_SV_STAGES 4
#endif
constexpr int kSvStages = MLC_SV_STAGES;  // levels in flight ahead of the one being solved
constexpr int kSvW = kSolveColsF;          // columns of a block (one row segment)
constexpr int kSvZW = kSvW + 8;      // raw divergence rows with a 4-column halo each side
constexpr int kSvStage = 3 * kSvZW + 11 * kSvW;  // floats of one stage

// The solve of a mixed member (same equations as k_sound_solve), in FP32
// only, one thread per column.  Where rounding is amplified the values are
// double-floats: theta_v at half levels, the hydrostatic balance
// -cp*theta_v*fmzf*dtrdz*(pai(k-1) - pai(k)) - g*dts of the w equation (two
// terms of ~g*dts whose difference drives w), and the Exner update
// pai - pai*increment.  The divergence filter, the elimination coefficients
// (O(1)-conditioned), the recurrence and the back substitution run in plain
// FP32.  The downward pass forms each level's coefficients and eliminates at
// once; the upward pass substitutes back and updates Exner (and, after the
// last substep, s) a level behind.  Between the passes the column's
// eliminated w stays in w, its multipliers and filtered divergence in the
// FP32 planes of wz_d[1] and wz_d[0] (free during the acoustic loop).
// wz[2] holds theta_v(k-1) - theta_v(k) from sound_prep.
//
// The inputs stream through shared memory: a block is 128 consecutive
// columns of one row, and the copy engine brings each level's planes as
// 512-byte row segments (untiled bulk copies, 16-byte aligned: the segment
// starts at a multiple of 128 columns, the raw divergence's halo of 4
// columns keeps that alignment) kSvStages levels ahead of the level being
// solved, so the per-level chain of dependent arithmetic never waits on
// memory.  The copies of one level (11 planes and 1 or 3 divergence rows)
// complete on one mbarrier; a stage is refilled after every thread has read
// it (one block barrier a level).  The upward pass reads back w, the
// multipliers and the filtered divergence the threads stored in the
// downward pass, after a proxy fence.  (Measured on the 512x512x41 step:
// 0.73 ms of solves a step against 0.95 for the same thread-per-column
// kernel with register prefetch of one level.)
template <class R, bool DFR>
__global__ void __launch_bounds__(128, 4) k_solve_mixed(const Dom<R> *__restrict__ doms, int advoff, int last,
    const WorkItem *__restrict__ wl) {
  constexpr int NS = kSvStages;
  extern __shared__ __align__(16) float sv_smem[];
  __shared__ __align__(8) uint64_t mbar[NS];
  const WorkItem wi = wl ? wl[blockIdx.x]
                          : WorkItem{(int16_t)blockIdx.z, (int16_t)blockIdx.x, (int16_t)blockIdx.y, 0};
  const Dom<R> &D = doms[wi.m];
  if (!D.active) return;
  const Geom g = D.g;
  const int t = (int)threadIdx.x;
  const int x0 = (int)wi.a * kSvW;          // first column (0-based j-1) of the block
  const int i = (int)wi.b + 2;
  if (x0 + 1 > g.jx - 2 || i > g.iy - 2) return;  // uniform over the block
  const int j = x0 + t + 1;
  const bool act = j >= 2 && j <= g.jx - 2;
  const int kz = g.kz;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const int adv = (D.clk->adv_role + advoff) & 1;
  const size_t F = g.field3(), F1 = g.PS * (size_t)(kz + 1);
  const int PS = (int)g.PS, P = g.P;
  const size_t r0 = g.at2(1, i);                  // row i, column 1
  // row bases (column 1 of row i, level 1)
  float *__restrict__ pai_h = reinterpret_cast<float *>(D.pai[adv]) + r0;
  float *__restrict__ pai_l = pai_h + F;
  float *__restrict__ tvf_h = reinterpret_cast<float *>(D.tetavf) + r0;
  float *__restrict__ tvf_l = tvf_h + F1;
  const float *__restrict__ cfz_h = reinterpret_cast<const float *>(sa.cfz) + r0;
  const float *__restrict__ cfz_l = cfz_h + F1;
  float *__restrict__ zfs = reinterpret_cast<float *>(D.wz_d[0]) + r0;
  float *__restrict__ mul = reinterpret_cast<float *>(D.wz_d[1]) + r0;
  // DFR: the low parts of the eliminated w and of the multipliers, in the
  // free lo planes of the same scratch allocations
  float *__restrict__ w_lo = zfs + F;
  float *__restrict__ mul_lo = mul + F;
  const float *__restrict__ zraw = D.zdiv2 + r0;
  const float *__restrict__ dtet = D.wz[2] + r0;
  const float *__restrict__ fmz = sa.fmz + r0;
  const float *__restrict__ fmzf = sa.fmzf + r0;
  float *__restrict__ s = D.s + r0;
  float *__restrict__ w = D.w + r0;
  const float dtrdz = c.dtsoundf * c.rdzitaf;
  const float rdrcv = float(kRdrcv);
  const float rdt = rdrcv * dtrdz;
  const F2 ngdts{-c.gdts_hi, -c.gdts_lo};
  const int ij_off = j - 1;                       // this thread's column offset in a row
  const int32_t ib = act ? sa.ibnd_cr[r0 + ij_off] : 0;
  const int nsp = c.nspgx;
  const bool filt = c.divfilter != 0;
  // copy extents: the block's columns, and the raw divergence with its halo
  const int xe = min(x0 + kSvW, P);
  const int zs = x0 >= 4 ? x0 - 4 : 0, ze = min(x0 + kSvW + 4, P);
  const unsigned wb = (unsigned)(xe - x0) * 4u, zb = (unsigned)(ze - zs) * 4u;
  const int zc = x0 + t - zs;                     // this column in a halo row
  auto stage = [&](int b) { return sv_smem + (size_t)b * kSvStage; };
  // stage layout: zraw rows i, i-1, i+1 (kSvZW each), then 11 fields of kSvW
  auto fld = [&](float *st, int f) { return st + 3 * kSvZW + f * kSvW; };
  const int nd = kz - 1;                          // down units: m = kz-1 .. 1
  // down unit u: A(m) = zraw, s, fmz, pai at level m; B(m+1) = w, fmzf,
  // dtet, tvf, cfz at interface m+1 (m = kz-1-u)
  auto issue_down = [&](int u, int b) {
    const int m = kz - 1 - u;
    float *st = stage(b);
    uint64_t *bar = &mbar[b];
    fence_proxy_async();
    mbar_expect_tx(bar, (filt ? 3u : 1u) * zb + 11u * wb);
    const int o = (m - 1) * PS, ob = m * PS;
    bulk_load(st, zraw + o + zs, zb, bar);
    if (filt) {
      bulk_load(st + kSvZW, zraw + o - P + zs, zb, bar);
      bulk_load(st + 2 * kSvZW, zraw + o + P + zs, zb, bar);
    }
    bulk_load(fld(st, 0), s + o + x0, wb, bar);
    bulk_load(fld(st, 1), fmz + o + x0, wb, bar);
    bulk_load(fld(st, 2), pai_h + o + x0, wb, bar);
    bulk_load(fld(st, 3), pai_l + o + x0, wb, bar);
    bulk_load(fld(st, 4), w + ob + x0, wb, bar);
    bulk_load(fld(st, 5), fmzf + ob + x0, wb, bar);
    bulk_load(fld(st, 6), dtet + ob + x0, wb, bar);
    bulk_load(fld(st, 7), tvf_h + ob + x0, wb, bar);
    bulk_load(fld(st, 8), tvf_l + ob + x0, wb, bar);
    bulk_load(fld(st, 9), cfz_h + ob + x0, wb, bar);
    bulk_load(fld(st, 10), cfz_l + ob + x0, wb, bar);
  };
  // up unit v (m = v + 2): w(m), mul(m) (m <= kz), and pai, zfs, fmz, s,
  // fmzf at level m-1
  auto issue_up = [&](int v, int b) {
    const int m = v + 2;
    float *st = stage(b);
    uint64_t *bar = &mbar[b];
    fence_proxy_async();
    mbar_expect_tx(bar, (m <= kz ? (DFR ? 10u : 8u) : 7u) * wb);
    const int o = (m - 1) * PS, op = (m - 2) * PS;
    bulk_load(fld(st, 0), w + o + x0, wb, bar);
    if (m <= kz) bulk_load(fld(st, 1), mul + o + x0, wb, bar);
    if (DFR && m <= kz) {
      bulk_load(fld(st, 8), w_lo + o + x0, wb, bar);
      bulk_load(fld(st, 9), mul_lo + o + x0, wb, bar);
    }
    bulk_load(fld(st, 2), pai_h + op + x0, wb, bar);
    bulk_load(fld(st, 3), pai_l + op + x0, wb, bar);
    bulk_load(fld(st, 4), zfs + op + x0, wb, bar);
    bulk_load(fld(st, 5), fmz + op + x0, wb, bar);
    bulk_load(fld(st, 6), s + op + x0, wb, bar);
    bulk_load(fld(st, 7), fmzf + op + x0, wb, bar);
  };
  // a failed wait (a copy that never landed): record it, let the copies in
  // flight land (bounded) and leave
  auto bail = [&](int gnext, int gend) {
    if (t == 0) {
      atomicOr(&D.clk->fault, 1);
      for (int q = gnext; q < gend && q < gnext + NS; ++q) mbar_wait_bounded(&mbar[q % NS], (unsigned)((q / NS) & 1));
    }
  };
  if (t == 0) {
    for (int q = 0; q < NS; ++q) mbar_init(&mbar[q], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (t == 0)
    for (int u = 0; u < NS && u < nd; ++u) issue_down(u, u);

  struct LvA {
    float z, lap, s, fmz;
    F2 pai;
  };
  auto zf_of = [&](int m, const LvA &a, float s_above) {
    float z = a.z;
    if (filt) z = z + sa.xknu_r[m - 1] * a.lap;
    const float bw = ib > 0 ? 1.f - sa.hefc_r[(size_t)(ib - 1) + (size_t)(m - 1) * nsp] : 1.f;
    return z + bw * dtrdz * a.fmz * (a.s - s_above);
  };
  // level kz and the interface below it straight from memory (once)
  LvA ak{};
  float wnext = 0.f, zfk = 0.f;
  if (act) {
    const int o = (kz - 1) * PS + ij_off;
    ak.z = zraw[o];
    ak.lap = filt ? (zraw[o - 1] + zraw[o + 1] + zraw[o - P] + zraw[o + P] - 4.f * ak.z) : 0.f;
    ak.s = s[o];
    ak.fmz = fmz[o];
    ak.pai = F2{pai_h[o], pai_l[o]};
    wnext = w[kz * PS + ij_off];
    zfk = zf_of(kz, ak, s[kz * PS + ij_off]);
  }
  float wkp1 = 0.f;
  F2 wnextd{wnext, 0.f}, wkp1d{0.f, 0.f};
  bool ok = true;
  int synced = 0;  // first unit read since the last block barrier
  for (int u = 0; u < nd; ++u) {
    const int k = kz - u, m = k - 1;
    const int b = u % NS;
    const bool landed = mbar_wait_bounded(&mbar[b], (unsigned)((u / NS) & 1));
    const float *st = stage(b);
    if (act) {
      const int o = (k - 1) * PS + ij_off;
      LvA am;
      am.z = st[zc];
      am.lap = filt ? (st[zc - 1] + st[zc + 1] + st[kSvZW + zc] + st[2 * kSvZW + zc] - 4.f * am.z) : 0.f;
      const float *f0 = st + 3 * kSvZW + t;
      am.s = f0[0];
      am.fmz = f0[kSvW];
      am.pai = F2{f0[2 * kSvW], f0[3 * kSvW]};
      const float wold = f0[4 * kSvW], bfmzf = f0[5 * kSvW], bdtet = f0[6 * kSvW];
      const F2 btvf{f0[7 * kSvW], f0[8 * kSvW]}, bcfz{f0[9 * kSvW], f0[10 * kSvW]};
      const float zf_m = zf_of(m, am, ak.s);
      zfs[o] = zfk;
      const F2 pai_m = am.pai, pai_k = ak.pai;
      const float corr = wold * bfmzf * dtrdz * bdtet;
      const F2 tvf = df_add_f(btvf, -corr);
      tvf_h[o] = tvf.hi;
      tvf_l[o] = tvf.lo;
      const F2 zrd = df_mul(tvf, bcfz);
      const F2 dp = two_sum(pai_m.hi - pai_k.hi, pai_m.lo - pai_k.lo);
      const F2 bal = df_add(ngdts, df_mul(F2{-zrd.hi, -zrd.lo}, dp));
      const float zr = df_f(zrd), pm = df_f(pai_m), pk = df_f(pai_k);
      const float ff = sa.ffilt_r[k - 1];
      const float zu = rdt * am.fmz * zr * pm + ff;
      const float zd = rdt * ak.fmz * zr * pk + ff;
      if constexpr (DFR) {
        // the recurrence in double-float: the explicit w keeps the hydrostatic
        // balance's low part, the pivots and multipliers carry theirs
        F2 zw = df_add_f(bal, wold);
        zw = df_add_f(zw, rdrcv * zr * (pm * zf_m - pk * zfk));
        const F2 den = df_add(two_sum(1.f + zd, zu), df_mul_f(F2{-wkp1d.hi, -wkp1d.lo}, zd));
        const F2 zrapp = df_recip(den);  // den >= 1: the pivot of a diagonally dominant system
        wnextd = df_mul(zrapp, df_add(zw, df_mul_f(wnextd, zd)));
        wkp1d = df_mul_f(zrapp, zu);
        w[o] = wnextd.hi;
        w_lo[o] = wnextd.lo;
        mul[o] = wkp1d.hi;
        mul_lo[o] = wkp1d.lo;
      } else {
        float zw = wold + df_f(bal);
        zw = zw + rdrcv * zr * (pm * zf_m - pk * zfk);
        const float zrapp = 1.f / (1.f + zd + zu - zd * wkp1);
        wnext = zrapp * (zw + zd * wnext);
        wkp1 = zrapp * zu;
        w[o] = wnext;
        mul[o] = wkp1;
      }
      zfk = zf_m;
      ak = am;
    }
    ok = ok && landed;
    if ((u + 1) % kSolveSync == 0 || u + 1 == nd) {
      if (__syncthreads_or(!ok)) {
        bail(u + 1, min(nd, synced + NS));  // the units issued and not read
        return;
      }
      // the stages read since the last barrier are free: refill them
      if (t == 0)
        for (int r = synced; r <= u; ++r)
          if (r + NS < nd) issue_down(r + NS, r % NS);
      synced = u + 1;
    }
  }
  if (act) zfs[ij_off] = zfk;  // level 1
  // this thread's stores of w, mul and zfs are read back by the copy engine
  fence_proxy_async_global();
  __syncthreads();
  const int nu = kz;  // up units: m = 2 .. kz+1
  if (t == 0)
    for (int v = 0; v < NS && v < nu; ++v) issue_up(v, (nd + v) % NS);
  auto exner = [&](int m, float wm, float dw, F2 pk, float zf, float fz, float sm, float fzf) {
    const int o = (m - 1) * PS + ij_off;
    const float inc = rdrcv * (zf + (dtrdz * fz * dw));
    const F2 d = df_mul_f(pk, inc);
    const F2 pn = df_add(pk, F2{-d.hi, -d.lo});
    pai_h[o] = pn.hi;
    pai_l[o] = pn.lo;
    if (last && m >= 2) s[o] = (wm + sm) * fzf;
  };
  float wprev = act ? w[ij_off] : 0.f;  // w(1) = 0
  F2 wprevd{wprev, 0.f};
  ok = true;
  synced = 0;
  for (int v = 0; v < nu; ++v) {
    const int k = v + 2, gu = nd + v;
    const int b = gu % NS;
    const bool landed = mbar_wait_bounded(&mbar[b], (unsigned)((gu / NS) & 1));
    if (act) {
      const float *f0 = stage(b) + 3 * kSvZW + t;
      const float wel = f0[0];
      const F2 cp{f0[2 * kSvW], f0[3 * kSvW]};
      const float czf = f0[4 * kSvW], cfz_ = f0[5 * kSvW], cs = f0[6 * kSvW], cfzf = f0[7 * kSvW];
      if constexpr (DFR) {
        if (k <= kz) {
          const F2 wk = df_add(F2{wel, f0[8 * kSvW]},
                               df_mul(F2{f0[kSvW], f0[9 * kSvW]}, wprevd));
          const float wkf = df_f(wk);
          w[(k - 1) * PS + ij_off] = wkf;
          exner(k - 1, df_f(wprevd), df_diff(wprevd, wk), cp, czf, cfz_, cs, cfzf);
          wprevd = wk;
        } else {
          exner(kz, df_f(wprevd), df_f(df_add_f(wprevd, -wel)), cp, czf, cfz_, cs, cfzf);
        }
      } else {
        if (k <= kz) {
          const float wk = wel + f0[kSvW] * wprev;
          w[(k - 1) * PS + ij_off] = wk;
          exner(k - 1, wprev, wprev - wk, cp, czf, cfz_, cs, cfzf);
          wprev = wk;
        } else {
          exner(kz, wprev, wprev - wel, cp, czf, cfz_, cs, cfzf);
        }
      }
    }
    ok = ok && landed;
    if ((v + 1) % kSolveSync == 0 || v + 1 == nu) {
      if (__syncthreads_or(!ok)) {
        bail(gu + 1, nd + min(nu, synced + NS));
        return;
      }
      if (t == 0)
        for (int r = synced; r <= v; ++r)
          if (r + NS < nu) issue_up(r + NS, (nd + r) % NS);
      synced = v + 1;
    }
  }
  if (last && act) {
    s[ij_off] = 0.f;
    s[kz * PS + ij_off] = 0.f;
  }
}
// Main/mod_moloch.F90:677-721 with divergence_damping :738-765 folded in
template <class R>
__global__ void k_sound_momentum(const Dom<R> *__restrict__ doms, int uvoff, int advoff,
                                 int tiles_j,
    const WorkItem *__restrict__ wl) {
  const WorkItem wi = work_item(wl, tiles_j);
  const Dom<R> &D = doms[wi.m];
  if (!D.active) return;
  const Geom g = D.g;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const int uv = (D.clk->uv_role + uvoff) & 1;
  const int adv = (D.clk->adv_role + advoff) & 1;
  const R *__restrict__ u_in = D.u[uv];
  const R *__restrict__ v_in = D.v[uv];
  R *__restrict__ u_out = D.u[uv ^ 1];
  R *__restrict__ v_out = D.v[uv ^ 1];
  const R *__restrict__ zraw = D.zdiv2;
  const double *__restrict__ pai = D.pai[adv];
  const double *__restrict__ tetav = D.tetav[adv];
  const Pt q = point_at(wi, 1, 1);
  const int j = q.j, i = q.i;
  if (j > g.jx || i > g.iy || q.k > g.kz) return;
  constexpr bool mixed = sizeof(R) == sizeof(float);
  const R dts = pick<R>(c.dtsound, c.dtsoundf);
  const R dtrdx = pick<R>(c.dtrdxs, c.dtrdxsf), dtrdy = dtrdx;
  const R dxrdt = pick<R>(c.dxrdt, c.dxrdtf);
  const size_t F = g.field3();
  // mixed member: theta_v and Exner are double-floats (hi, lo planes)
  const float *__restrict__ th_f = reinterpret_cast<const float *>(tetav);
  const float *__restrict__ pa_f = reinterpret_cast<const float *>(pai);
  // relaxation weight 1 - hefc(ib, k) (Main/mod_bdycod.F90:4033-4047)
  auto bweight = [&](const int32_t *ibnd, size_t ij0, int k) -> R {
    if constexpr (mixed) {
      const int ib = ibnd[ij0];
      return ib > 0 ? 1.f - sa.hefc_r[(size_t)(ib - 1) + (size_t)(k - 1) * c.nspgx] : 1.f;
    } else {
      return R(relax_weight(ibnd, sa.hefc, c.nspgx, ij0, k));
    }
  };
  // theta_v(a) + theta_v(b) and pai(a) - pai(b) in the field type
  auto tsum = [&](size_t a, size_t b) -> R {
    if constexpr (mixed) return (th_f[a] + th_f[b]) + (th_f[a + F] + th_f[b + F]);
    else return R(tetav[a] + tetav[b]);
  };
  auto pdif = [&](size_t a, size_t b) -> R {
    if constexpr (mixed) return (pa_f[a] - pa_f[b]) + (pa_f[a + F] - pa_f[b + F]);
    else return R(pai[a] - pai[b]);
  };
  const R zfz = R(kGrav) * dts;
  const R halfcp = R(0.5) * R(kCpd);
  const size_t ij = g.at2(j, i);
  const size_t PS = g.PS;
  const bool has_u = i <= g.iy - 1;
  const bool has_v = j <= g.jx - 1;
  const bool upd_u = has_u && j >= 2 && j <= g.jx - 1 && i >= 2 && i <= g.iy - 2;
  const bool upd_v = has_v && j >= 2 && j <= g.jx - 2 && i >= 2 && i <= g.iy - 1;
  R mu = 0, zcx = 0, hxk = 0, cor_u = 0, zcy = 0, hyk = 0, cor_v = 0, mv = 0;
  if (upd_u) {
    mu = sa.msfu[ij];
    zcx = dtrdx * mu;
    hxk = sa.hx[ij];
    cor_u = sa.coru[ij];
  }
  if (upd_v) {
    mv = sa.msfv[ij];
    zcy = c.lrotllr ? dtrdy : dtrdy * mv;
    hyk = sa.hy[ij];
    cor_v = sa.corv[ij];
  }
  const size_t W = 1, S = (size_t)g.P;
#pragma unroll
  for (int k = q.k; k < q.k + kPtLevels && k <= g.kz; ++k) {
    const size_t o = ij + (size_t)(k - 1) * PS;
    const R gk = sa.gzitakh_r[k - 1];
    if (has_u) {
      R un = u_in[o];
      if (upd_u) {
        // FP64: the constant products dxrdt*xkdamp*msfu, g*dts*hx*gzitakh and
        // coru*dts come from bind time (same operands, same order)
        if (c.divdamp) {
          R xdam;
          if constexpr (mixed) xdam = dxrdt * sa.xkdamp_r[k - 1] * mu;
          else xdam = sa.mo_du[o];
          un = un + xdam * (zraw[o] - zraw[o - W]);
        }
        const R zrom1u = halfcp * tsum(o - W, o);
        R zcor1u, zg;
        if constexpr (mixed) {
          zcor1u = cor_u * dts * v_in[o];
          zg = zfz * hxk * gk;
        } else {
          zcor1u = sa.mo_cu[ij] * v_in[o];
          zg = sa.mo_gu[o];
        }
        const R bw = bweight(sa.ibnd_ud, ij, k);
        un = un + bw * (zcor1u - zg - zcx * zrom1u * pdif(o, o - W));
      }
      u_out[o] = un;
    }
    if (has_v) {
      R vn = v_in[o];
      if (upd_v) {
        if (c.divdamp) {
          R xdam;
          if constexpr (mixed) xdam = c.lrotllr ? dxrdt * sa.xkdamp_r[k - 1] : dxrdt * sa.xkdamp_r[k - 1] * mv;
          else xdam = sa.mo_dv[o];
          vn = vn + xdam * (zraw[o] - zraw[o - S]);
        }
        const R zrom1v = halfcp * tsum(o - S, o);
        R zcor1v, zg;
        if constexpr (mixed) {
          zcor1v = cor_v * dts * u_in[o];
          zg = zfz * hyk * gk;
        } else {
          zcor1v = sa.mo_cv[ij] * u_in[o];
          zg = sa.mo_gv[o];
        }
        const R bw = bweight(sa.ibnd_vd, ij, k);
        vn = vn + bw * (-zcor1v - zg - zcy * zrom1v * pdif(o, o - S));
      }
      v_out[o] = vn;
    }
  }
}

// 16 bytes at p (16-byte aligned) as 4 floats / 4 ints
__device__ __forceinline__ void ld4(float (&x)[4], const float *p) {
  const float4 v = *reinterpret_cast<const float4 *>(p);
  x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
}
__device__ __forceinline__ void ld4i(int (&x)[4], const int32_t *p) {
  const int4 v = *reinterpret_cast<const int4 *>(p);
  x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
}
// x[q] at q = -1..3: the lane's own elements, the one west of them read singly
struct West4 {
  float w, x[4];
  __device__ __forceinline__ float at(int q) const { return q < 0 ? w : x[q]; }
};

// Blocks of 128 threads an SM the four-column point kernels are compiled for
// (the register budget follows; a few registers spill to L1).  Measured on the
// moist 512x512x41 step: 5 blocks (about 100 registers) momentum 0.37 and
// divergence 0.30 ms a step, against 0.39 and 0.35 at 4 (128 registers).
#ifndef MLC_PT4_BLOCKS
#define MLC_PT4_BLOCKS 5
#endif

// The divergence and s of a mixed member (the same equations as
// k_sound_div) with lanes of four consecutive columns: 16-byte loads at the
// lane's points and the row north of them, the east neighbour of the last
// element read singly, the level below carried from the previous level.
template <class R>
__global__ void __launch_bounds__(128, MLC_PT4_BLOCKS) k_sound_div_v4(const Dom<R> *__restrict__ doms, int uvoff,
                                                      int tiles_j,
    const WorkItem *__restrict__ wl) {
  static_assert(sizeof(R) == sizeof(float), "FP32 fields");
  const WorkItem wi = work_item(wl, tiles_j);
  const Dom<R> &D = doms[wi.m];
  if (!D.active) return;
  const Geom g = D.g;
  const int jx = g.jx, iy = g.iy, kz = g.kz;
  const int bj = wi.a, bi = wi.b;
  const int e0 = (bj * 32 + (int)threadIdx.x) * 4;
  const int i = bi * (int)blockDim.y + (int)threadIdx.y + 1;
  const int k0 = (int)wi.c * kPtLevels + 1;
  if (e0 + 1 > jx - 1 || i > iy - 1 || k0 > kz) return;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const int uv = (D.clk->uv_role + uvoff) & 1;
  const float *__restrict__ u = D.u[uv];
  const float *__restrict__ v = D.v[uv];
  float *__restrict__ zdiv2 = D.zdiv2;
  float *__restrict__ sv = D.s;
  float *__restrict__ w = D.w;
  const float dtrdx = c.dtrdxsf, dtrdy = dtrdx;
  const unsigned P = (unsigned)g.P, PS = (unsigned)g.PS;
  const unsigned ij = (unsigned)e0 + (unsigned)(i - 1) * P;
  const bool east = e0 + 4 <= jx - 1;  // element 3 has an east neighbour to read
  bool has[4], inner[4];
  bool all = true;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int j = e0 + q + 1;
    has[q] = j <= jx - 1;
    inner[q] = j >= 2 && j <= jx - 2 && i >= 2 && i <= iy - 2;
    all = all && has[q];
  }
  const bool any_inner = inner[0] || inner[1] || inner[2] || inner[3];
  auto next4 = [&](float (&e)[4], const float (&x)[4], const float *arr, unsigned o) {
    e[0] = x[1]; e[1] = x[2]; e[2] = x[3];
    e[3] = east ? arr[o + 4] : 0.f;
  };
  float rmu0[4], rmu1[4], rmv0[4], rmv1[4], mfac[4], hx0[4], hx1[4], hy0[4], hy1[4];
  ld4(rmu0, sa.rmu + ij);
  next4(rmu1, rmu0, sa.rmu, ij);
  ld4(rmv0, sa.rmv + ij);
  ld4(rmv1, sa.rmv + ij + P);
  ld4(mfac, (c.lrotllr ? sa.msfx : sa.mx2) + ij);
  ld4(hx0, sa.hx + ij);
  next4(hx1, hx0, sa.hx, ij);
  ld4(hy0, sa.hy + ij);
  ld4(hy1, sa.hy + ij + P);
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (!inner[q]) hx0[q] = hx1[q] = hy0[q] = hy1[q] = 0.f;
  // the winds of the level below (for s)
  float um[4], upm[4], vm[4], vpm[4];
  if (k0 >= 2 && any_inner) {
    const unsigned om = ij + (unsigned)(k0 - 2) * PS;
    ld4(um, u + om);
    next4(upm, um, u, om);
    ld4(vm, v + om);
    ld4(vpm, v + om + P);
  }
  for (int k = k0; k < k0 + kPtLevels && k <= kz; ++k) {
    const unsigned o = ij + (unsigned)(k - 1) * PS;
    float u0[4], u1[4], v0[4], v1[4], fu0[4], fu1[4], fv0[4], fv1[4], fz[4], zd[4];
    ld4(u0, u + o);
    next4(u1, u0, u, o);
    ld4(v0, v + o);
    ld4(v1, v + o + P);
    ld4(fu0, sa.rfmzu + o);
    next4(fu1, fu0, sa.rfmzu, o);
    ld4(fv0, sa.rfmzv + o);
    ld4(fv1, sa.rfmzv + o + P);
    ld4(fz, sa.fmz + o);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      float zum, zup;
      if (c.lrotllr) {
        zum = dtrdx * u0[q] * fu0[q];
        zup = dtrdx * u1[q] * fu1[q];
      } else {
        zum = dtrdx * u0[q] * fu0[q] * rmu0[q];
        zup = dtrdx * u1[q] * fu1[q] * rmu1[q];
      }
      const float zvm = dtrdy * v0[q] * fv0[q] * rmv0[q];
      const float zvp = dtrdy * v1[q] * fv1[q] * rmv1[q];
      zd[q] = fz[q] * mfac[q] * ((zup - zum) + (zvp - zvm));
    }
    if (all) {
      *reinterpret_cast<float4 *>(zdiv2 + o) = make_float4(zd[0], zd[1], zd[2], zd[3]);
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (has[q]) zdiv2[o + q] = zd[q];
    }
    if (any_inner) {
      if (k >= 2) {
        const float gk = sa.gzitak_r[k - 1];
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (inner[q]) {
            const float zuh = (u0[q] + um[q]) * hx0[q] + (u1[q] + upm[q]) * hx1[q];
            const float zvh = (v0[q] + vm[q]) * hy0[q] + (v1[q] + vpm[q]) * hy1[q];
            sv[o + q] = -(0.25f * (zuh + zvh) * gk);
          }
      }
      if (k == kz) {
        const unsigned ot = ij + (unsigned)kz * PS;
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (inner[q]) {
            const float zuh = u0[q] * hx0[q] + u1[q] * hx1[q];
            const float zvh = v0[q] * hy0[q] + v1[q] * hy1[q];
            const float skp1 = -(0.5f * (zuh + zvh));
            sv[ot + q] = skp1;
            w[ot + q] = -skp1;
          }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        um[q] = u0[q]; upm[q] = u1[q]; vm[q] = v0[q]; vpm[q] = v1[q];
      }
    }
  }
}

// The momentum update of a mixed member (the same equations as
// k_sound_momentum) with lanes of four consecutive columns: 16-byte loads of
// every field at the lane's points and the row south of them; the west
// neighbours are the lane's own elements but for the first, read singly.  A
// block is 32 lanes x 4 rows; grid x = 128-column tiles times row tiles, y =
// level chunks, z = member.
template <class R>
__global__ void __launch_bounds__(128, MLC_PT4_BLOCKS) k_sound_momentum_v4(const Dom<R> *__restrict__ doms,
                                                           int uvoff, int advoff, int tiles_j,
    const WorkItem *__restrict__ wl) {
  static_assert(sizeof(R) == sizeof(float), "FP32 fields");
  const WorkItem wi = work_item(wl, tiles_j);
  const Dom<R> &D = doms[wi.m];
  if (!D.active) return;
  const Geom g = D.g;
  const int jx = g.jx, iy = g.iy, kz = g.kz;
  const int bj = wi.a, bi = wi.b;
  const int e0 = (bj * 32 + (int)threadIdx.x) * 4;  // j-1 of the lane's first column
  const int i = bi * (int)blockDim.y + (int)threadIdx.y + 1;
  const int k0 = (int)wi.c * kPtLevels + 1;
  if (e0 + 1 > jx || i > iy || k0 > kz) return;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const int uv = (D.clk->uv_role + uvoff) & 1;
  const int adv = (D.clk->adv_role + advoff) & 1;
  const float *__restrict__ u_in = D.u[uv];
  const float *__restrict__ v_in = D.v[uv];
  float *__restrict__ u_out = D.u[uv ^ 1];
  float *__restrict__ v_out = D.v[uv ^ 1];
  const float *__restrict__ zraw = D.zdiv2;
  const size_t F = g.field3();
  const float *__restrict__ th_h = reinterpret_cast<const float *>(D.tetav[adv]);
  const float *__restrict__ th_l = th_h + F;
  const float *__restrict__ pa_h = reinterpret_cast<const float *>(D.pai[adv]);
  const float *__restrict__ pa_l = pa_h + F;
  const float dts = c.dtsoundf, dtrdx = c.dtrdxsf, dtrdy = dtrdx, dxrdt = c.dxrdtf;
  const float zfz = float(kGrav) * dts;
  const float halfcp = 0.5f * float(kCpd);
  const unsigned P = (unsigned)g.P;
  const unsigned ij = (unsigned)e0 + (unsigned)(i - 1) * P;
  const bool west = e0 >= 1, south = i >= 2;
  bool upd_u[4], upd_v[4], has_u[4], has_v[4];
  bool all_u = true, all_v = true;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int j = e0 + q + 1;
    has_u[q] = i <= iy - 1 && j <= jx;
    has_v[q] = j <= jx - 1;
    upd_u[q] = j >= 2 && j <= jx - 1 && i >= 2 && i <= iy - 2;
    upd_v[q] = j >= 2 && j <= jx - 2 && i >= 2 && i <= iy - 1;
    all_u = all_u && has_u[q];
    all_v = all_v && has_v[q];
  }
  // 2-D coefficients of the lane's columns (zero where nothing is updated)
  float mu[4], hx4[4], cu4[4], mv[4], hy4[4], cv4[4];
  int ibu[4], ibv[4];
  ld4(mu, sa.msfu + ij);
  ld4(hx4, sa.hx + ij);
  ld4(cu4, sa.coru + ij);
  ld4(mv, sa.msfv + ij);
  ld4(hy4, sa.hy + ij);
  ld4(cv4, sa.corv + ij);
  ld4i(ibu, sa.ibnd_ud + ij);
  ld4i(ibv, sa.ibnd_vd + ij);
  const int nsp = c.nspgx;
  for (int k = k0; k < k0 + kPtLevels && k <= kz; ++k) {
    const unsigned o = ij + (unsigned)(k - 1) * (unsigned)g.PS;
    float un[4], vn[4], uo[4], vo[4];
    ld4(uo, u_in + o);
    ld4(vo, v_in + o);
    West4 zr, th, tl, ph, pl;
    ld4(zr.x, zraw + o);
    ld4(th.x, th_h + o);
    ld4(tl.x, th_l + o);
    ld4(ph.x, pa_h + o);
    ld4(pl.x, pa_l + o);
    zr.w = th.w = tl.w = ph.w = pl.w = 0.f;
    if (west) {
      zr.w = zraw[o - 1];
      th.w = th_h[o - 1];
      tl.w = th_l[o - 1];
      ph.w = pa_h[o - 1];
      pl.w = pa_l[o - 1];
    }
    float zs[4] = {0.f, 0.f, 0.f, 0.f}, ts[4] = {0.f, 0.f, 0.f, 0.f}, tsl[4] = {0.f, 0.f, 0.f, 0.f};
    float ps[4] = {0.f, 0.f, 0.f, 0.f}, psl[4] = {0.f, 0.f, 0.f, 0.f};
    if (south) {
      ld4(zs, zraw + o - P);
      ld4(ts, th_h + o - P);
      ld4(tsl, th_l + o - P);
      ld4(ps, pa_h + o - P);
      ld4(psl, pa_l + o - P);
    }
    const float gk = sa.gzitakh_r[k - 1];
    const float xk = sa.xkdamp_r[k - 1];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      float a = uo[q];
      if (upd_u[q]) {
        if (c.divdamp) {
          const float xdam = dxrdt * xk * mu[q];
          a = a + xdam * (zr.x[q] - zr.at(q - 1));
        }
        const float zrom1u = halfcp * ((th.at(q - 1) + th.x[q]) + (tl.at(q - 1) + tl.x[q]));
        const float zcor1u = cu4[q] * dts * vo[q];
        const int ib = ibu[q];
        const float bw = ib > 0 ? 1.f - sa.hefc_r[(size_t)(ib - 1) + (size_t)(k - 1) * nsp] : 1.f;
        const float zcx = dtrdx * mu[q];
        const float pd = (ph.x[q] - ph.at(q - 1)) + (pl.x[q] - pl.at(q - 1));
        a = a + bw * (zcor1u - zfz * hx4[q] * gk - zcx * zrom1u * pd);
      }
      un[q] = a;
      float b = vo[q];
      if (upd_v[q]) {
        if (c.divdamp) {
          const float xdam = c.lrotllr ? dxrdt * xk : dxrdt * xk * mv[q];
          b = b + xdam * (zr.x[q] - zs[q]);
        }
        const float zrom1v = halfcp * ((ts[q] + th.x[q]) + (tsl[q] + tl.x[q]));
        const float zcor1v = cv4[q] * dts * uo[q];
        const int ib = ibv[q];
        const float bw = ib > 0 ? 1.f - sa.hefc_r[(size_t)(ib - 1) + (size_t)(k - 1) * nsp] : 1.f;
        const float zcy = c.lrotllr ? dtrdy : dtrdy * mv[q];
        const float pd = (ph.x[q] - ps[q]) + (pl.x[q] - psl[q]);
        b = b + bw * (-zcor1v - zfz * hy4[q] * gk - zcy * zrom1v * pd);
      }
      vn[q] = b;
    }
    if (all_u) {
      *reinterpret_cast<float4 *>(u_out + o) = make_float4(un[0], un[1], un[2], un[3]);
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (has_u[q]) u_out[o + q] = un[q];
    }
    if (all_v) {
      *reinterpret_cast<float4 *>(v_out + o) = make_float4(vn[0], vn[1], vn[2], vn[3]);
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (has_v[q]) v_out[o + q] = vn[q];
    }
  }
}

inline dim3 col_block(const LaunchGeom &L) { return dim3((unsigned)L.col_x, (unsigned)L.col_y); }
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
void Launch<R>::sound_prep(const LaunchGeom &L, const Dom<R> *d, int advoff, cudaStream_t s) {
  int tj;
  const dim3 grd = pt_grid(L, L.jx - 1, L.iy - 1, tj);
  k_sound_prep<R><<<grd, col_block(L), 0, s>>>(d, advoff, tj, L.wl_pt);
}

template <class R>
void Launch<R>::sound_div(const LaunchGeom &L, const Dom<R> *d, int uvoff, cudaStream_t s) {
  if constexpr (sizeof(R) == sizeof(float)) {
    const int tj = (L.jx - 1 + 127) / 128, ti = (L.iy - 1 + 3) / 4;
    const dim3 grd = L.wl_v4 ? dim3((unsigned)L.n_v4, 1, 1)
                             : dim3((unsigned)(tj * ti), (unsigned)((L.kz + kPtLevels - 1) / kPtLevels),
                                    (unsigned)L.nmem);
    k_sound_div_v4<R><<<grd, dim3(32, 4), 0, s>>>(d, uvoff, tj, L.wl_v4);
  } else {
    int tj;
    const dim3 grd = pt_grid(L, L.jx - 1, L.iy - 1, tj);
    k_sound_div<R><<<grd, col_block(L), 0, s>>>(d, uvoff, tj, L.wl_pt);
  }
}

template <class R>
void Launch<R>::sound_solve(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, bool last,
                            cudaStream_t s) {
  (void)uvoff;
  // one block per 128-column row segment in both precisions (the solve
  // launch shape of LaunchGeom is not used)
  if constexpr (sizeof(R) == sizeof(float)) {
    const int tj = (L.jx - 1 + kSvW - 1) / kSvW;
    const dim3 grid = L.wl_solve ? dim3((unsigned)L.n_solve, 1, 1)
                                 : dim3((unsigned)tj, (unsigned)(L.iy - 3), (unsigned)L.nmem);
    const size_t smem = (size_t)kSvStages * kSvStage * sizeof(float);
    if (L.solve_df)
      k_solve_mixed<R, true><<<grid, kSvW, smem, s>>>(d, advoff, last ? 1 : 0, L.wl_solve);
    else
      k_solve_mixed<R, false><<<grid, kSvW, smem, s>>>(d, advoff, last ? 1 : 0, L.wl_solve);
  } else {
    const int tj = (L.jx - 1 + kDvW - 1) / kDvW;
    const dim3 grid = L.wl_solve ? dim3((unsigned)L.n_solve, 1, 1)
                                 : dim3((unsigned)tj, (unsigned)(L.iy - 3), (unsigned)L.nmem);
    k_sound_solve<R><<<grid, kDvW, (size_t)kDvStages * kDvStage * sizeof(double), s>>>(
        d, advoff, last ? 1 : 0, L.wl_solve);
  }
}

template <class R>
void Launch<R>::sound_momentum(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff,
                               cudaStream_t s) {
  if constexpr (sizeof(R) == sizeof(float)) {
    // lanes of four columns: 128 columns by 4 rows a block
    const int tj = (L.jx + 127) / 128, ti = (L.iy + 3) / 4;
    const dim3 grd = L.wl_v4 ? dim3((unsigned)L.n_v4, 1, 1)
                             : dim3((unsigned)(tj * ti), (unsigned)((L.kz + kPtLevels - 1) / kPtLevels),
                                    (unsigned)L.nmem);
    k_sound_momentum_v4<R><<<grd, dim3(32, 4), 0, s>>>(d, uvoff, advoff, tj, L.wl_v4);
  } else {
    int tj;
    const dim3 grd = pt_grid(L, L.jx, L.iy, tj);
    k_sound_momentum<R><<<grd, col_block(L), 0, s>>>(d, uvoff, advoff, tj, L.wl_pt);
  }
}

template <class R>
cudaError_t Launch<R>::configure_sound() {
  if constexpr (sizeof(R) == sizeof(float))
    return cudaSuccess;  // the mixed solve uses no dynamic shared memory
  else
    return cudaFuncSetAttribute(k_sound_solve<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                200 * 1024);
}

template struct Launch<double>;
template struct Launch<float>;

}  // namespace mlc
