// mlc_end.cu -- the end of the MOLOCH step (Main/mod_moloch.F90:340-446):
// virtual temperature and temperature, lateral boundary conditions
// (boundary :448-529 with bdyval, motopnudge, morelax of Main/mod_bdycod.F90
// and the tracer ring/relaxation of Main/chemlib/mod_che_bdyco.F90),
// pressure, density and saturation diagnostics, surface pressure
// extrapolation, status_update with zero tendencies, the mass budget of
// Main/mod_massck.F90 and the NaN/Inf check on ps.
//
// The boundary clock lives on the device: bdyval blends with xbctime, then
// the reference advances it by dtsec (Main/mod_bdycod.F90:2653) before
// motopnudge and morelax blend again, so those read xbctime + dtsec; the
// final reduction kernel stores the advanced clock.
#include <algorithm>

#include "mlc_kernels.cuh"

namespace mlc {

namespace {

template <class R>
__device__ __forceinline__ R qfactor(const R *qx, size_t o, size_t F, int ipptls) {
  if (ipptls > 1) return R(1) + R(kEp1) * qx[o] - qx[o + F] - qx[o + 2 * F] - qx[o + 3 * F] - qx[o + 4 * F];
  if (ipptls == 1) return R(1) + R(kEp1) * qx[o] - qx[o + F];
  return R(1) + R(kEp1) * qx[o];
}
// The same factor for a mixed member as the exact double-float 1 + d, with
// only d = ep1*qv - condensate in FP32.  The step end divides t by qf and
// multiplies by it again after the relaxation changed qv: an FP32 qf's
// rounding (6e-8) cancels only where qv did not change, and would otherwise
// reach theta_v in the relaxation zone every step.
__device__ __forceinline__ F2 qfactor_df(const float *qx, size_t o, size_t F, int ipptls) {
  float d;
  if (ipptls > 1) d = float(kEp1) * qx[o] - qx[o + F] - qx[o + 2 * F] - qx[o + 3 * F] - qx[o + 4 * F];
  else if (ipptls == 1) d = float(kEp1) * qx[o] - qx[o + F];
  else d = float(kEp1) * qx[o];
  return fast_two_sum(1.f, d);
}

// bdyval, MOLOCH branch (Main/mod_bdycod.F90:1631-1860).  Phase 0 does the
// west/east columns (corners excluded), phase 1 the south/north rows
// (corners included), which read the corner values phase 0 left.
// Boundary blends and relaxations.  An FP64 member evaluates the reference's
// expressions x0*b0 + x1*b1 and (1 - x)*f + x*fext.  In FP32 both carry a
// rounding that repeats every step - 1 - x and x0 are rounded once and for
// all - and the relaxation turns it into a steady forcing of order
// eps*f/x (1e-5 of the field in the inner rings, with a ring-to-ring pattern
// that the divergence picks up); the increment forms b0 + x1*(b1 - b0) and
// f + x*(fext - f) round only the small correction.
template <class R>
__device__ __forceinline__ R bdy_blend(R x0, R x1, R b0, R b1) {
  if constexpr (sizeof(R) == sizeof(float)) return b0 + x1 * (b1 - b0);
  else return x0 * b0 + x1 * b1;
}
template <class R>
__device__ __forceinline__ R bdy_relax_to(R f, R x, R fext) {
  if constexpr (sizeof(R) == sizeof(float)) return f + x * (fext - f);
  else return (R(1) - x) * f + x * fext;
}

// One block per level and member runs both phases, a block barrier between
// them: everything phase 1 reads that phase 0 writes (qx, w at the level,
// TKE one interface up, written by the same level's phase 0) lies in the
// block's own level.
constexpr int kRingThreads = 1024;
template <class R>
__global__ void __launch_bounds__(kRingThreads) k_bdy_ring(const Dom<R> *__restrict__ doms, int uvoff,
                                                           int advoff) {
  const Dom<R> &D = doms[blockIdx.y];
  if (!D.active) return;
  const Geom g = D.g;
  const Scal &c = D.c;
  const Bdy<R> &bd = D.bd;
  const Clock *clk = D.clk;
  const State<R> st = state_of(D, (clk->uv_role + uvoff) & 1, (clk->adv_role + advoff) & 1);
  const int jx = g.jx, iy = g.iy;
  const int k = blockIdx.x + 1;
  if (k > g.kz) return;                                  // a member with fewer levels (whole block)
  const double xb = clk->xbctime;
  const double x1 = (xb + c.dt) * c.rtb;
  const double x0 = 1.0 - x1;
  const double cx1 = (xb + c.dt) / c.dtbdys;  // chem_bdyval_uncoupled
  const double cx0 = 1.0 - cx1;
  const R rx0 = R(x0), rx1 = R(x1);
  const size_t PS = g.PS, F = g.field3(), ko = (size_t)(k - 1) * PS;
  // Exner at a ring point: x0*b0 + x1*b1 (a mixed member: b0 + x1*(b1 - b0)
  // in double-float)
  auto set_pai_ring = [&](size_t ob) {
    if constexpr (sizeof(R) == sizeof(float)) {
      const DF b0(bd.xpaib[0], F), b1(bd.xpaib[1], F);
      const F2 a = b0.ld(ob);
      DF(st.pai, F).st(ob, df_add_f(a, float(x1) * df_diff(b1.ld(ob), a)));
    } else {
      st.pai[ob] = x0 * bd.xpaib[0][ob] + x1 * bd.xpaib[1][ob];
    }
  };
  auto blend = [&](const R *const *b, size_t o) { return bdy_blend<R>(rx0, rx1, b[0][o], b[1][o]); };
  // t at a ring point: the blend (a mixed member: double-float, lo in wz[1])
  auto set_t_ring = [&](size_t ob) {
    if constexpr (sizeof(R) == sizeof(float)) {
      const DF b0(bd.xtb[0], F), b1(bd.xtb[1], F);
      const F2 a = b0.ld(ob);
      const F2 t = df_add_f(a, float(x1) * df_diff(b1.ld(ob), a));
      st.t[ob] = t.hi;
      D.wz[1][ob] = t.lo;
    } else {
      st.t[ob] = x0 * bd.xtb[0][ob] + x1 * bd.xtb[1][ob];
    }
  };
  const int nqx = g.nqx;
  // side 0 = west/south, 1 = east/north; idx the position along the side
  auto point = [&](int phase, int side, int idx) {
  if (phase == 0) {
    const int i = idx + 2;  // i in idi = 2..iy-1 (v), ici = 2..iy-2 (others)
    if (i > iy - 1) return;
    const int jb = side == 0 ? 1 : jx - 1;   // jce1 / jce2
    const int jd = side == 0 ? 1 : jx;       // jde1 / jde2
    const int jin = side == 0 ? 2 : jx - 2;  // jci1 / jci2
    const size_t ob = g.at2(jb, i) + ko, od = g.at2(jd, i) + ko, oi = g.at2(jin, i) + ko;
    st.v[ob] = blend(bd.dvb, ob);
    if (i > iy - 2) return;
    if (k == 1) st.ps[g.at2(jb, i)] = x0 * bd.xpsb[0][g.at2(jb, i)] + x1 * bd.xpsb[1][g.at2(jb, i)];
    const R un = blend(bd.dub, od);
    st.u[od] = un;
    set_t_ring(ob);
    set_pai_ring(ob);
    st.qx[ob] = blend(bd.xqb, ob);
    if (c.present_qc) st.qx[ob + F] = blend(bd.xlb, ob);
    if (c.present_qi && c.ipptls > 1) st.qx[ob + 2 * F] = blend(bd.xib, ob);
    const bool inflow = side == 0 ? (un > R(0)) : (un < R(0));
    for (int n = 1; n < nqx; ++n) {
      if ((c.present_qc && n == 1) || (c.present_qi && n == 2)) continue;
      const size_t on = (size_t)n * F;
      st.qx[ob + on] = inflow ? R(qx_zero(n)) : st.qx[oi + on];
    }
    st.w[ob] = inflow ? R(0) : st.w[oi];
    if (c.tke) {
      // Main/mod_bdycod.F90:1684-1695 (west), 1742-1753 (east): the floor at
      // the top interface, below it inflow by u(k) + u(k-1) of the new ring
      if (k == 1) {
        st.tke[ob] = R(kTkeMin);
      } else {
        const R us = un + blend(bd.dub, od - PS);
        const bool in2 = side == 0 ? (us > R(0)) : (us < R(0));
        st.tke[ob + PS] = in2 ? R(kTkeMin) : st.tke[oi + PS];
      }
    }
    for (int n = 0; n < g.ntr; ++n) {
      const size_t on = (size_t)n * F;
      st.trac[ob + on] = bdy_blend<R>(R(cx0), R(cx1), bd.chib[0][ob + on], bd.chib[1][ob + on]);
    }
  } else {
    const int j = idx + 1;  // j in jde = 1..jx (u), jce = 1..jx-1 (others)
    if (j > jx) return;
    const int ib = side == 0 ? 1 : iy - 1;   // ice1 / ice2
    const int id = side == 0 ? 1 : iy;       // ide1 / ide2
    const int iin = side == 0 ? 2 : iy - 2;  // ici1 / ici2
    const size_t ou = g.at2(j, ib) + ko;
    st.u[ou] = blend(bd.dub, ou);
    if (j > jx - 1) return;
    const size_t ob = g.at2(j, ib) + ko, od = g.at2(j, id) + ko, oi = g.at2(j, iin) + ko;
    if (k == 1) st.ps[g.at2(j, ib)] = x0 * bd.xpsb[0][g.at2(j, ib)] + x1 * bd.xpsb[1][g.at2(j, ib)];
    const R vn = blend(bd.dvb, od);
    st.v[od] = vn;
    set_t_ring(ob);
    set_pai_ring(ob);
    st.qx[ob] = blend(bd.xqb, ob);
    if (c.present_qc) st.qx[ob + F] = blend(bd.xlb, ob);
    if (c.present_qi && c.ipptls > 1) st.qx[ob + 2 * F] = blend(bd.xib, ob);
    const bool inflow = side == 0 ? (vn > R(0)) : (vn < R(0));
    for (int n = 1; n < nqx; ++n) {
      if ((c.present_qc && n == 1) || (c.present_qi && n == 2)) continue;
      const size_t on = (size_t)n * F;
      st.qx[ob + on] = inflow ? R(qx_zero(n)) : st.qx[oi + on];
    }
    st.w[ob] = inflow ? R(0) : st.w[oi];
    if (c.tke) {
      // Main/mod_bdycod.F90:1800-1811 (south), 1858-1869 (north)
      if (k == 1) {
        st.tke[ob] = R(kTkeMin);
      } else {
        const R vs = vn + blend(bd.dvb, od - PS);
        const bool in2 = side == 0 ? (vs > R(0)) : (vs < R(0));
        st.tke[ob + PS] = in2 ? R(kTkeMin) : st.tke[oi + PS];
      }
    }
    for (int n = 0; n < g.ntr; ++n) {
      const size_t on = (size_t)n * F;
      st.trac[ob + on] = bdy_blend<R>(R(cx0), R(cx1), bd.chib[0][ob + on], bd.chib[1][ob + on]);
    }
  }
  };
  const int n0 = iy - 2, n1 = jx;  // positions a side: phase 0 i = 2..iy-1, phase 1 j = 1..jx
  for (int e = (int)threadIdx.x; e < 2 * n0; e += kRingThreads) point(0, e >= n0 ? 1 : 0, e >= n0 ? e - n0 : e);
  __syncthreads();
  for (int e = (int)threadIdx.x; e < 2 * n1; e += kRingThreads) point(1, e >= n1 ? 1 : 0, e >= n1 ? e - n1 : e);
}

// The step end's point pass, after the boundary ring: virtual temperature
// and temperature of dynamical_core :1121-1123 (tvirt_to_temp :1629-1648),
// then - with the boundary on - motopnudge (Main/mod_bdycod.F90:4049-4083)
// and morelax on every field (boundary, Main/mod_moloch.F90:478-497).  Both
// are per point, so one thread does both at its points and t goes from the
// first to the second in registers.  The ring (bdyval) runs before this pass
// although the reference's order is tvirt, bdyval, relaxation: the ring reads
// only boundary data and the interior values of qx, w and TKE, which the
// temperature pass does not write, and it writes only ring points, where
// this pass leaves t alone; tvirt at the ring points is recomputed by the
// status update.  The relaxation's clock has already moved by dtsec.
template <class R>
__global__ void k_end_relax(const Dom<R> *__restrict__ doms, int uvoff, int advoff, int tiles_j,
    const WorkItem *__restrict__ wl) {
  const WorkItem wi = work_item(wl, tiles_j);
  const Dom<R> &D = doms[wi.m];
  if (!D.active) return;
  const Geom g = D.g;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const Bdy<R> &bd = D.bd;
  const Clock *clk = D.clk;
  const State<R> st = state_of(D, (clk->uv_role + uvoff) & 1, (clk->adv_role + advoff) & 1);
  const Pt q_ = point_at(wi, 1, 1);
  const int j = q_.j, k0 = q_.k;
  if (k0 > g.kz) return;
  const int i = q_.i;
  const int jx = g.jx, iy = g.iy;
  if (j > jx - 1 || i > iy - 1) return;
  const bool inner = j >= 2 && j <= jx - 2 && i >= 2 && i <= iy - 2;
  const size_t ij = g.at2(j, i), PS = g.PS, F = g.field3();
  // the relaxation's points: jci x ici (t and the cross fields), jdi x ici
  // (u), jci x idi (v); none without the boundary
  const bool bdy = c.apply_bdy != 0 && j >= 2 && i >= 2;
  const bool cr = bdy && j <= jx - 2 && i <= iy - 2;
  const bool up = bdy && i <= iy - 2;
  const bool vp = bdy && j <= jx - 2;
  const double xb = clk->xbctime + c.dtsec;
  const double x1 = (xb + c.dt) * c.rtb;
  const double x0 = 1.0 - x1;
  const double cx1 = (xb + c.dt) / c.dtbdys;
  const double cx0 = 1.0 - cx1;
  const R rx0 = R(x0), rx1 = R(x1);
  const double trtau = 1.0 / (2.0 * 3600.0);
  const double wrtau = 1.0 / (3600.0 / 4.0);
  const int nsp = c.nspgx;
  const int ibc = cr ? sa.ibnd_cr[ij] : -1;
  const int ibu = up ? sa.ibnd_ud[ij] : -1;
  const int ibv = vp ? sa.ibnd_vd[ij] : -1;
  auto blend = [&](const R *const *b, size_t o) { return bdy_blend<R>(rx0, rx1, b[0][o], b[1][o]); };
  auto relax = [&](R f, R fext, int ib, int k) {
    const R xf = sa.hefc_r[(size_t)(ib - 1) + (size_t)(k - 1) * nsp];
    return bdy_relax_to<R>(f, xf, fext);
  };
  const R xfn0 = pick<R>(trtau * c.dtsec, float(trtau * c.dtsec));
  // The temperature part's inputs of a level, loaded one level ahead: the
  // next level's loads are issued before this level's stores (which would
  // otherwise hold them back, the arrays being reachable through one
  // descriptor), so each thread keeps two levels' loads in flight.
  const int ipp = c.ipptls;
  const int nq = ipp > 1 ? 5 : ipp == 1 ? 2 : 1;
  struct TvIn {
    R th, pa, q[5];
    float thl, pal;  // a mixed member's low parts of theta_v and Exner
  };
  auto load_in = [&](size_t o, TvIn &x) {
    if constexpr (sizeof(R) == sizeof(float)) {
      const DF th(st.tetav, F), pa(st.pai, F);
      const F2 a = th.ld(o), b = pa.ld(o);
      x.th = a.hi; x.thl = a.lo; x.pa = b.hi; x.pal = b.lo;
    } else {
      x.th = R(st.tetav[o]); x.pa = R(st.pai[o]); x.thl = x.pal = 0.f;
    }
#pragma unroll
    for (int n = 0; n < 5; ++n) x.q[n] = n < nq ? st.qx[o + (size_t)n * F] : R(0);
  };
  // qfactor of the loaded species, in its association
  auto qf_of = [&](const TvIn &x) -> R {
    if (ipp > 1) return R(1) + R(kEp1) * x.q[0] - x.q[1] - x.q[2] - x.q[3] - x.q[4];
    if (ipp == 1) return R(1) + R(kEp1) * x.q[0] - x.q[1];
    return R(1) + R(kEp1) * x.q[0];
  };
  TvIn cur, nxt;
  load_in(ij + (size_t)(k0 - 1) * PS, cur);
#pragma unroll
  for (int k = k0; k < k0 + kPtLevels && k <= g.kz; ++k) {
    const size_t o = ij + (size_t)(k - 1) * PS;
    if (k + 1 < k0 + kPtLevels && k + 1 <= g.kz) load_in(o + PS, nxt);
    // ---- tvirt and t (every cross point; t only inside the ring) ----
    F2 tdf{0.f, 0.f};  // a mixed member's double-float t
    R tr = R(0);       // an FP64 member's t
    if constexpr (sizeof(R) == sizeof(float)) {
      // t as a double-float through the step end: hi in t, lo in wz[1] (the
      // scratch is free until the next advection); status_update rebuilds
      // theta_v = t*qf/pai from it, so t's FP32 rounding never reaches theta_v
      const F2 tv = df_mul(F2{cur.th, cur.thl}, F2{cur.pa, cur.pal});
      st.tvirt[o] = df_f(tv);
      if (inner) {
        float d;  // qfactor_df of the loaded species
        if (ipp > 1) d = float(kEp1) * cur.q[0] - cur.q[1] - cur.q[2] - cur.q[3] - cur.q[4];
        else if (ipp == 1) d = float(kEp1) * cur.q[0] - cur.q[1];
        else d = float(kEp1) * cur.q[0];
        tdf = df_div(tv, fast_two_sum(1.f, d));
      } else if (!c.apply_bdy) {
        D.wz[1][o] = 0.f;  // (with the boundary on, the ring wrote it)
      }
    } else {
      const R tv = R(cur.th * cur.pa);
      st.tvirt[o] = tv;
      if (inner) tr = tv / qf_of(cur);
    }
    cur = nxt;
    // ---- motopnudge and morelax ----
    if (k == 2 && cr && c.top_nudge) {
      const size_t o2 = ij + PS;  // level 2 (w sponge, before the level's relaxation)
      const R xf = R(wrtau * c.dtsec);
      const R w2 = st.w[o2];
      const R fext = R(0) * w2;
      st.w[o2] = bdy_relax_to<R>(w2, xf, fext);
    }
    const bool nud = c.top_nudge && k <= c.nztop;
    R xfn;
    if constexpr (sizeof(R) == sizeof(float)) xfn = nud ? sa.tnudge_r[k - 1] * xfn0 : R(0);
    else xfn = nud ? R(sa.tnudge[k - 1] * trtau * c.dtsec) : R(0);
    // only nudged levels and the relaxation zone change anything
    if (up && (nud || ibu > 0)) {
      R f = st.u[o];
      if (nud) f = bdy_relax_to<R>(f, xfn, blend(bd.dub, o));
      if (ibu > 0) f = relax(f, blend(bd.dub, o), ibu, k);
      st.u[o] = f;
    }
    if (vp && (nud || ibv > 0)) {
      R f = st.v[o];
      if (nud) f = bdy_relax_to<R>(f, xfn, blend(bd.dvb, o));
      if (ibv > 0) f = relax(f, blend(bd.dvb, o), ibv, k);
      st.v[o] = f;
    }
    if (cr && (nud || ibc > 0)) {
      if constexpr (sizeof(R) == sizeof(float)) {
        // (1-x)*t + x*b as t + x*(b - t) on the double-float t
        const DF b0(bd.xtb[0], F), b1(bd.xtb[1], F);
        const F2 a = b0.ld(o);
        const F2 bt = df_add_f(a, float(x1) * df_diff(b1.ld(o), a));
        if (nud) tdf = df_add_f(tdf, xfn * df_diff(bt, tdf));
        if (ibc > 0) {
          const float xf = sa.hefc_r[(size_t)(ibc - 1) + (size_t)(k - 1) * nsp];
          tdf = df_add_f(tdf, xf * df_diff(bt, tdf));
        }
      } else {
        const double bt = x0 * bd.xtb[0][o] + x1 * bd.xtb[1][o];
        if (nud) tr = (R(1) - xfn) * tr + xfn * R(bt);
        if (ibc > 0) tr = relax(tr, R(bt), ibc, k);
      }
    }
    if (inner) {
      if constexpr (sizeof(R) == sizeof(float)) {
        st.t[o] = tdf.hi;
        D.wz[1][o] = tdf.lo;
      } else {
        st.t[o] = tr;
      }
    }
    if (!cr || ibc <= 0) continue;
    if constexpr (sizeof(R) == sizeof(float)) {
      // (1 - xf)*pai + xf*(b0 + x1*(b1 - b0)) as pai + xf*((b0 - pai) + x1*(b1 - b0))
      const float xf = sa.hefc_r[(size_t)(ibc - 1) + (size_t)(k - 1) * nsp];
      const DF pa(st.pai, F), b0(bd.xpaib[0], F), b1(bd.xpaib[1], F);
      const F2 pp = pa.ld(o), a = b0.ld(o);
      pa.st(o, df_add_f(pp, xf * (df_diff(a, pp) + float(x1) * df_diff(b1.ld(o), a))));
    } else {
      const double xf = sa.hefc[(size_t)(ibc - 1) + (size_t)(k - 1) * nsp];
      const double fext = x0 * bd.xpaib[0][o] + x1 * bd.xpaib[1][o];
      st.pai[o] = (1.0 - xf) * st.pai[o] + xf * fext;
    }
    st.qx[o] = relax(st.qx[o], blend(bd.xqb, o), ibc, k);
    {
      // morelax_fraction with frac = 0 (:3962-3993)
      const R xf = sa.hefc_r[(size_t)(ibc - 1) + (size_t)(k - 1) * nsp];
      const R f = st.w[o];
      st.w[o] = bdy_relax_to<R>(f, xf, f * R(0));
    }
    if (c.ipptls > 0 && c.present_qc) st.qx[o + F] = relax(st.qx[o + F], blend(bd.xlb, o), ibc, k);
    if (c.ipptls > 1 && c.present_qi) st.qx[o + 2 * F] = relax(st.qx[o + 2 * F], blend(bd.xib, o), ibc, k);
    for (int n = 0; n < g.ntr; ++n) {
      const size_t on = o + (size_t)n * F;
      const R xf = sa.fcx_r[ibc - 1];
      const R fext = bdy_blend<R>(R(cx0), R(cx1), bd.chib[0][on], bd.chib[1][on]);
      st.trac[on] = bdy_relax_to<R>(st.trac[on], xf, fext);
    }
  }
}

// ---- spectral nudging (Main/mod_bdycod.F90:3898-3960, called from
// Main/mod_moloch.F90:499-506 after the relaxation) ----
// The reference projects the departure d = blend(b0,b1) - f of t, u and v
// onto km2 sine modes in x (sums over the field's interior columns jj), back
// to the grid, onto lm2 modes in y (sums over its interior rows ii) and back,
// and adds cnudge(k) times the result on jj x ii.  Only d on jj x ii enters,
// and the four passes factor into
//   sx(i,m) = sum_{j in jj} d(j,i) bvx(j,m)                 (k_spec_rows)
//   C(m,l)  = sum_{i in ii} sx(i,m) bvy(i,l)                (k_spec_modes)
//   G(i,m)  = sum_l C(m,l) bvy(i,l)                          (k_spec_modes)
//   f(j,i) += cnudge(k) sum_m bvx(j,m) G(i,m)                (k_spec_apply)
// per field, level and member.  Ranges: t jj = jci1..jci1 (the reference's
// call passes jci1 as both bounds), ii = ici; u jdi x ici; v jci x idi.
// The kernels run every step and return at once unless the interval is due.

// the step's boundary update is a spectral nudging step: tspectral + dtsec
// (the reference's tspectral after its increment) is a multiple of dtrad
__device__ __forceinline__ bool spectral_due(const Scal &c, const Clock *clk) {
  return c.spectral && (int)fmod(clk->tspectral + c.dtsec, c.dtrad) == 0;
}
struct SpecRange {
  int jj1, jj2, ii1, ii2;
};
__device__ __forceinline__ SpecRange spec_range(int f, const Geom &g) {
  if (f == 0) return {2, 2, 2, g.iy - 2};
  if (f == 1) return {2, g.jx - 1, 2, g.iy - 2};
  return {2, g.jx - 2, 2, g.iy - 1};
}

// Departure of field f (0 t, 1 u, 2 v) from the blended boundary data at o.
template <class R>
__device__ __forceinline__ R spec_departure(const Dom<R> &D, const State<R> &st, int f, size_t o,
                                            double x0, double x1) {
  const Bdy<R> &bd = D.bd;
  if (f == 0) {
    if constexpr (sizeof(R) == sizeof(float)) {
      const size_t F = D.g.field3();
      const DF b0(bd.xtb[0], F), b1(bd.xtb[1], F);
      const F2 a = b0.ld(o);
      const F2 bt = df_add_f(a, float(x1) * df_diff(b1.ld(o), a));
      return df_diff(bt, F2{st.t[o], D.wz[1][o]});
    } else {
      return (x0 * bd.xtb[0][o] + x1 * bd.xtb[1][o]) - st.t[o];
    }
  }
  const R *const *b = f == 1 ? bd.dub : bd.dvb;
  const R cur = f == 1 ? st.u[o] : st.v[o];
  return bdy_blend<R>(R(x0), R(x1), b[0][o], b[1][o]) - cur;
}

// sx(i, m) of one row: a warp per row i, lanes over j; grid (rows/8,
// kz*3, members), 256 threads.
template <class R>
__global__ void __launch_bounds__(256) k_spec_rows(const Dom<R> *__restrict__ doms, int uvoff, int advoff) {
  const Dom<R> &D = doms[blockIdx.z];
  if (!D.active) return;
  const Scal &c = D.c;
  const Clock *clk = D.clk;
  if (!spectral_due(c, clk)) return;
  const Geom g = D.g;
  const int k = (int)blockIdx.y / 3 + 1, f = (int)blockIdx.y % 3;
  if (k > g.kz) return;
  const SpecRange r = spec_range(f, g);
  const int lane = (int)threadIdx.x & 31;
  const int i = r.ii1 + (int)blockIdx.x * 8 + ((int)threadIdx.x >> 5);
  if (i > r.ii2) return;
  const State<R> st = state_of(D, (clk->uv_role + uvoff) & 1, (clk->adv_role + advoff) & 1);
  const double x1 = (clk->xbctime + c.dtsec + c.dt) * c.rtb, x0 = 1.0 - x1;
  const int km2 = c.km2;
  const R *bvx = D.sa.bvx;
  R acc[kMaxModes];
#pragma unroll
  for (int m = 0; m < kMaxModes; ++m) acc[m] = R(0);
  const size_t row = g.at2(1, i) + (size_t)(k - 1) * g.PS;
  for (int j = r.jj1 + lane; j <= r.jj2; j += 32) {
    const R dv = spec_departure(D, st, f, row + (size_t)(j - 1), x0, x1);
#pragma unroll
    for (int m = 0; m < kMaxModes; ++m)
      if (m < km2) acc[m] += dv * bvx[(size_t)m * g.jx + (j - 1)];
  }
  R mine = R(0);
#pragma unroll
  for (int m = 0; m < kMaxModes; ++m) {
    if (m < km2) {
      R v = acc[m];
#pragma unroll
      for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
      if (lane == m) mine = v;
    }
  }
  if (lane < km2)
    D.spec[((size_t)(f * g.kz + k - 1) * g.iy + (size_t)(i - 1)) * km2 + lane] = mine;
}

// C(m, l) in shared memory, then G(i, m) over sx in place; one block of 256
// threads per field, level and member.
template <class R>
__global__ void __launch_bounds__(256) k_spec_modes(const Dom<R> *__restrict__ doms) {
  const Dom<R> &D = doms[blockIdx.z];
  if (!D.active) return;
  const Scal &c = D.c;
  if (!spectral_due(c, D.clk)) return;
  const Geom g = D.g;
  const int k = (int)blockIdx.y / 3 + 1, f = (int)blockIdx.y % 3;
  if (k > g.kz) return;
  const SpecRange r = spec_range(f, g);
  const int km2 = c.km2, lm2 = c.lm2, ni = r.ii2 - r.ii1 + 1;
  const R *bvy = D.sa.bvy;
  R *sx = D.spec + (size_t)(f * g.kz + k - 1) * g.iy * km2;
  __shared__ R cm[kMaxModes * kMaxModes];
  for (int p = (int)threadIdx.x; p < km2 * lm2; p += (int)blockDim.x) {
    const int m = p / lm2, l = p % lm2;
    R a = R(0);
    for (int i = r.ii1; i <= r.ii2; ++i) a += sx[(size_t)(i - 1) * km2 + m] * bvy[(size_t)l * g.iy + (i - 1)];
    cm[p] = a;
  }
  __syncthreads();
  for (int p = (int)threadIdx.x; p < ni * km2; p += (int)blockDim.x) {
    const int i = r.ii1 + p / km2, m = p % km2;
    R a = R(0);
    for (int l = 0; l < lm2; ++l) a += cm[m * lm2 + l] * bvy[(size_t)l * g.iy + (i - 1)];
    sx[(size_t)(i - 1) * km2 + m] = a;
  }
}

// f(j,i,k) += cnudge(k) sum_m bvx(j,m) G(i,m) for t, u and v at one point
// (j, i from 2), kPtLevels levels per thread.
template <class R>
__global__ void k_spec_apply(const Dom<R> *__restrict__ doms, int uvoff, int advoff, int tiles_j,
    const WorkItem *__restrict__ wl) {
  const WorkItem wi = work_item(wl, tiles_j);
  const Dom<R> &D = doms[wi.m];
  if (!D.active) return;
  const Scal &c = D.c;
  const Clock *clk = D.clk;
  if (!spectral_due(c, clk)) return;
  const Geom g = D.g;
  const Pt q_ = point_at(wi, 2, 2);
  const int j = q_.j, i = q_.i, k0 = q_.k;
  if (k0 > g.kz || j > g.jx - 1 || i > g.iy - 1) return;
  const State<R> st = state_of(D, (clk->uv_role + uvoff) & 1, (clk->adv_role + advoff) & 1);
  const int km2 = c.km2;
  const R *bvx = D.sa.bvx + (j - 1);
  const size_t ij = g.at2(j, i);
  auto proj = [&](int f, int k) {
    const R *gg = D.spec + ((size_t)(f * g.kz + k - 1) * g.iy + (size_t)(i - 1)) * km2;
    R a = R(0);
    for (int m = 0; m < km2; ++m) a += bvx[(size_t)m * g.jx] * gg[m];
    return a;
  };
  const bool tp = j == 2 && i <= g.iy - 2, up = i <= g.iy - 2, vp = j <= g.jx - 2;
#pragma unroll
  for (int k = k0; k < k0 + kPtLevels && k <= g.kz; ++k) {
    const size_t o = ij + (size_t)(k - 1) * g.PS;
    const R cn = D.sa.cnudge[k - 1];
    if (tp) {
      if constexpr (sizeof(R) == sizeof(float)) {
        const F2 t = df_add_f(F2{st.t[o], D.wz[1][o]}, cn * proj(0, k));
        st.t[o] = t.hi;
        D.wz[1][o] = t.lo;
      } else {
        st.t[o] = st.t[o] + cn * proj(0, k);
      }
    }
    if (up) st.u[o] = st.u[o] + cn * proj(1, k);
    if (vp) st.v[o] = st.v[o] + cn * proj(2, k);
  }
}

// extrapolate_surface_pressure (:1592-1606) of the interior column at ij,
// from t and q at the two lowest levels before status_update clamps q, and p
// at the lowest level (the same expression k_end_cross stores).
template <class R>
__device__ __forceinline__ void ps_column(const Dom<R> &D, const State<R> &st, size_t ij) {
  const Geom &g = D.g;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const size_t PS = g.PS, F = g.field3();
  const int ipp = c.ipptls, kz = g.kz;
  // tvirt at kz-1, kz before the clamps: from the boundary's temp_to_tvirt,
  // or tetav*pai of dynamical_core when the boundary is off
  const size_t o1 = ij + (size_t)(kz - 2) * PS, o2 = ij + (size_t)(kz - 1) * PS;
  double tv1, tv2;
  if (c.apply_bdy) {
    tv1 = (double)(st.t[o1] * qfactor(st.qx, o1, F, ipp));
    tv2 = (double)(st.t[o2] * qfactor(st.qx, o2, F, ipp));
  } else {
    tv1 = (double)st.tvirt[o1];
    tv2 = (double)st.tvirt[o2];
  }
  R p2;
  if constexpr (sizeof(R) == sizeof(float)) p2 = exner_to_pressure_f(df_f(DF(st.pai, F).ld(o2)));
  else p2 = (R)exner_to_pressure(st.pai[o2]);
  const double z1 = sa.zeta[o1], z2 = sa.zeta[o2];
  double lrt = (tv1 - tv2) / (z1 - z2);
  if (lrt < -kGovcp) lrt = -kGovcp;
  else if (lrt > -0.005) lrt = 0.65 * lrt - 0.35 * kLrate;
  const double tv = tv2 - lrt * 0.5 * z2;
  st.ps[ij] = (double)p2 * exp(kGovr * z2 / tv);
}

// ps of every interior column, for the split step (the whole step's
// k_end_cross forms it in the thread that owns the column's lowest levels)
template <class R>
__global__ void k_end_ps(const Dom<R> *__restrict__ doms, int uvoff, int advoff) {
  const Dom<R> &D = doms[blockIdx.z];
  if (!D.active) return;
  const Geom g = D.g;
  const State<R> st = state_of(D, (D.clk->uv_role + uvoff) & 1, (D.clk->adv_role + advoff) & 1);
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int i = blockIdx.y * blockDim.y + threadIdx.y + 2;
  if (j > g.jx - 2 || i > g.iy - 2) return;
  ps_column<R>(D, st, g.at2(j, i));
}

// q < c for a positive finite threshold c, exactly as the comparison (false
// for a NaN q).  FP64: on the bit patterns in the integer pipe, read through
// an opaque move (a plain reinterpretation would be turned back into an FP64
// comparison); a negative q, -0 included, has the sign bit set and compares
// below every positive pattern as a signed integer.  FP32 compares directly.
__device__ __forceinline__ long long bits_of_d(double x) {
  long long b;
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
  return b;
}
template <class R>
__device__ __forceinline__ bool below_pos(R q, double c) {
  if constexpr (sizeof(R) == sizeof(double)) {
    const long long b = bits_of_d(q);
    const bool nan = (b & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
    return !nan && b < __double_as_longlong(c);
  } else {
    return q < R(c);
  }
}

// Cross-point work after the boundary, per point: uvstagtouvx and
// temp_to_tvirt of boundary (:520-523), p (:348-352), the edits mkslice
// makes to the state (Main/mod_slice.F90:136-147: qx and tracer floors),
// then status_update (:1403-1443): tendencies, q clamps, tvirt, tetav, rho,
// qsat.  The surface pressure is extrapolated before the clamps: in the
// whole step by the thread holding the column's two lowest levels (chunks
// of levels are counted from the top), in the split step by k_end_ps.
//   kEndAll   the whole sequence with zero tendencies (mlc_step).  rho and
//             qsat of :348-352, and tvirt and tetav of the boundary, are
//             recomputed from the same inputs by status_update, so they are
//             computed once, after it.
//   kEndPre   up to mkslice: the state the physics reads.
//   kEndPost  status_update with the member's tendencies (Dom::tend).
constexpr int kEndAll = 0, kEndPre = 1, kEndPost = 2;
constexpr double kTracFloor = 1.0e-50;  // mkslice's tracer floor (Main/mod_slice.F90:141-147)
template <class R, int PH>
__global__ void k_end_cross(const Dom<R> *__restrict__ doms, int uvoff, int advoff, int tiles_j,
    const WorkItem *__restrict__ wl) {
  const WorkItem wi = work_item(wl, tiles_j);
  const Dom<R> &D = doms[wi.m];
  if (!D.active) return;
  const Geom g = D.g;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const State<R> st = state_of(D, (D.clk->uv_role + uvoff) & 1, (D.clk->adv_role + advoff) & 1);
  const Pt q_ = point_at(wi, 1, 1);
  const int j = q_.j, i = q_.i;
  const int jx = g.jx, iy = g.iy, kz = g.kz;
  // level chunks counted from the top, so the chunk holding kz also holds
  // kz-1 (the levels ps is extrapolated from)
  const int khi = kz - (int)wi.c * kPtLevels, klo = max(1, khi - kPtLevels + 1);
  if (j > jx - 1 || i > iy - 1 || khi < 1) return;
  const size_t ij = g.at2(j, i), PS = g.PS, F = g.field3(), S = (size_t)g.P;
  const bool inner = j >= 2 && j <= jx - 2 && i >= 2 && i <= iy - 2;
  const int ipp = c.ipptls;
  // the whole step: ps before this thread clamps q at kz-1, kz
  if (PH == kEndAll && khi == kz && inner) ps_column<R>(D, st, ij);
#pragma unroll
  for (int k = klo; k <= khi; ++k) {
  const size_t o = ij + (size_t)(k - 1) * PS;
  if (PH != kEndPost && c.apply_bdy) {
    {
      const R *u = st.u, *v = st.v;
      R a;
      if (j == 1) a = R(0.5) * (u[o] + u[o + 1]);
      else if (j == jx - 1) a = R(0.5) * (u[o + 1] + u[o]);
      else a = R(0.5625) * (u[o + 1] + u[o]) - R(0.0625) * (u[o + 2] + u[o - 1]);
      st.ux[o] = a;
      if (i == 1) a = R(0.5) * (v[o] + v[o + S]);
      else if (i == iy - 1) a = R(0.5) * (v[o + S] + v[o]);
      else a = R(0.5625) * (v[o + S] + v[o]) - R(0.0625) * (v[o + 2 * S] + v[o - S]);
      st.vx[o] = a;
    }
  }
  // pressure (FP64 Exner reconstruction; FP32 for the FP32 field of a mixed member)
  if (PH != kEndPost) {
    if constexpr (sizeof(R) == sizeof(float)) st.p[o] = exner_to_pressure_f(df_f(DF(st.pai, F).ld(o)));
    else st.p[o] = (R)exner_to_pressure(st.pai[o]);
  }
  if (PH == kEndPre) {
    // the state at mkslice: tvirt and theta_v of the boundary (before the
    // floors), rho and qsat of :348-352, then mkslice's floors
    const R tk = st.t[o], pk = st.p[o];
    if (c.apply_bdy) {
      st.tvirt[o] = tk * qfactor(st.qx, o, F, ipp);
      if constexpr (sizeof(R) == sizeof(float)) {
        const F2 t2{tk, D.wz[1][o]};
        DF(st.tetav, F).st(o, df_div(df_mul(t2, qfactor_df(st.qx, o, F, ipp)), DF(st.pai, F).ld(o)));
      } else {
        st.tetav[o] = (double)st.tvirt[o] / st.pai[o];
      }
    }
    st.rho[o] = pk / (R(kRgas) * tk);
    if constexpr (sizeof(R) == sizeof(float)) st.qsat[o] = pfwsat_f(tk, pk);
    else st.qsat[o] = (R)pfwsat((double)tk, (double)pk);
    if (inner) {
      for (int n = 0; n < g.nqx; ++n) {
        const size_t on = o + (size_t)n * F;
        if (below_pos<R>(st.qx[on], qx_check(n))) st.qx[on] = R(qx_zero(n));
      }
      for (int n = 0; n < g.ntr; ++n) {
        const size_t on = o + (size_t)n * F;
        if (below_pos<double>((double)st.trac[on], kTracFloor)) st.trac[on] = R(0);
      }
    }
    continue;
  }
  // status_update
  {
    const R *ten = PH == kEndPost ? D.tend : nullptr;
    if (inner) {
      if (ten) {
        // t, ux, vx += dtsec * tendency (a mixed member's t is a double-float)
        if constexpr (sizeof(R) == sizeof(float)) {
          const F2 t2 = df_add_f(F2{st.t[o], D.wz[1][o]}, c.dtsecf * ten[o]);
          st.t[o] = t2.hi;
          D.wz[1][o] = t2.lo;
          st.ux[o] = st.ux[o] + c.dtsecf * ten[o + F];
          st.vx[o] = st.vx[o] + c.dtsecf * ten[o + 2 * F];
        } else {
          st.t[o] = st.t[o] + c.dtsec * ten[o];
          st.ux[o] = st.ux[o] + c.dtsec * ten[o + F];
          st.vx[o] = st.vx[o] + c.dtsec * ten[o + 2 * F];
        }
      }
      const R dts = pick<R>(c.dtsec, c.dtsecf);
      // The whole step's mkslice floor and status_update clamp with zero
      // tendencies are one clamp: after the floor q >= check or q = zero, and
      // zero < check or zero = check, so the second clamp changes nothing (for
      // the tracers, the floor leaves no negative value)
      for (int n = 0; n < g.nqx; ++n) {
        const size_t on = o + (size_t)n * F;
        R q = st.qx[on];
        if (ten) q = q + dts * ten[o + (size_t)(3 + n) * F];
        if (below_pos<R>(q, qx_check(n))) q = R(qx_zero(n));
        st.qx[on] = q;
      }
      for (int n = 0; n < g.ntr; ++n) {
        const size_t on = o + (size_t)n * F;
        R q = st.trac[on];
        if (PH == kEndAll) {
          if (below_pos<double>((double)q, kTracFloor)) q = R(0);  // mkslice
        } else {
          if (ten) q = q + dts * ten[o + (size_t)(3 + g.nqx + n) * F];
          if (q < R(0)) q = R(0);
        }
        st.trac[on] = q;
      }
    }
    const R tk = st.t[o];
    const R qf = qfactor(st.qx, o, F, ipp);
    const R tv = tk * qf;
    st.tvirt[o] = tv;
    const R pk = st.p[o];
    st.rho[o] = pk / (R(kRgas) * tk);
    if constexpr (sizeof(R) == sizeof(float)) {
      // theta_v = tvirt/pai from the double-float t (Main/mod_moloch.F90:1403-1443):
      // where nothing relaxed t, t*qf/pai gives back theta_v to ~1e-14
      const F2 t2{tk, D.wz[1][o]};
      DF(st.tetav, F).st(o, df_div(df_mul(t2, qfactor_df(st.qx, o, F, ipp)), DF(st.pai, F).ld(o)));
      st.qsat[o] = pfwsat_f(tk, pk);
    } else {
      st.tetav[o] = (double)tv / st.pai[o];
      st.qsat[o] = (R)pfwsat((double)tk, (double)pk);
    }
  }
  }
}

// 16 bytes at p (16-byte aligned) as 4 floats; a float4 store
__device__ __forceinline__ void ld4f(float (&x)[4], const float *p) {
  const float4 v = *reinterpret_cast<const float4 *>(p);
  x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
}
__device__ __forceinline__ void st4f(float *p, const float (&x)[4]) {
  *reinterpret_cast<float4 *>(p) = make_float4(x[0], x[1], x[2], x[3]);
}

// k_end_cross of a mixed member with lanes of four consecutive columns
// (16-byte loads and stores; the same expressions): ux, vx, p, the
// status_update clamps, tvirt, rho, theta_v (double-float) and qsat.  A block
// is 32 lanes x 4 rows; grid x = 128-column tiles times row tiles, y = level
// chunks, z = member.
template <class R>
__global__ void __launch_bounds__(128) k_end_cross_v4(const Dom<R> *__restrict__ doms, int uvoff,
                                                      int advoff, int tiles_j,
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
  // level chunks counted from the top (the chunk holding kz holds kz-1)
  const int khi = kz - (int)wi.c * kPtLevels, klo = max(1, khi - kPtLevels + 1);
  if (e0 + 1 > jx - 1 || i > iy - 1 || khi < 1) return;
  const Scal &c = D.c;
  const State<R> st = state_of(D, (D.clk->uv_role + uvoff) & 1, (D.clk->adv_role + advoff) & 1);
  const float *__restrict__ u = st.u;
  const float *__restrict__ v = st.v;
  float *__restrict__ ux = st.ux;
  float *__restrict__ vx = st.vx;
  float *__restrict__ pp = st.p;
  float *__restrict__ tt = st.t;
  float *__restrict__ tvir = st.tvirt;
  float *__restrict__ rho = st.rho;
  float *__restrict__ qsat = st.qsat;
  float *__restrict__ qx = st.qx;
  float *__restrict__ trac = st.trac;
  const float *__restrict__ tlo = D.wz[1];
  const size_t F = g.field3();
  float *__restrict__ pa_h = reinterpret_cast<float *>(st.pai);
  float *__restrict__ th_h = reinterpret_cast<float *>(st.tetav);
  const unsigned P = (unsigned)g.P, PS = (unsigned)g.PS;
  const unsigned ij = (unsigned)e0 + (unsigned)(i - 1) * P;
  const int ipp = c.ipptls;
  bool has[4], inner[4];
  bool all = true;
  int nvalid = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int j = e0 + q + 1;
    has[q] = j <= jx - 1;
    inner[q] = j >= 2 && j <= jx - 2 && i >= 2 && i <= iy - 2;
    all = all && has[q];
    nvalid += has[q] ? 1 : 0;
  }
  const bool any_inner = inner[0] || inner[1] || inner[2] || inner[3];
  auto store = [&](float *dst, const float (&x)[4]) {
    if (all) {
      st4f(dst, x);
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (has[q]) dst[q] = x[q];
    }
  };
  // ps of the lane's interior columns before this thread clamps q at kz-1, kz
  if (khi == kz)
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (inner[q]) ps_column<R>(D, st, (size_t)ij + (size_t)q);
  for (int k = klo; k <= khi; ++k) {
    const unsigned o = ij + (unsigned)(k - 1) * PS;
    if (c.apply_bdy) {
      // u at j-1 .. j+2 and v at rows i-1 .. i+2 (:1535-1566)
      float uc[4], ue1 = 0.f, ue2 = 0.f, uw = 0.f;
      ld4f(uc, u + o);
      if (e0 >= 1) uw = u[o - 1];
      if (nvalid == 4) ue1 = u[o + 4];          // j+1 of the last column (<= jx)
      if (e0 + 4 <= jx - 2) ue2 = u[o + 5];     // j+2 of the last column
      const float un[6] = {uw, uc[0], uc[1], uc[2], uc[3], ue1};  // u at j-1 .. j+4 of column 0
      float a[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = e0 + q + 1;
        const float u0 = un[q + 1], u1 = un[q + 2], um = un[q];
        const float u2 = q < 3 ? un[q + 3] : ue2;
        if (j == 1) a[q] = 0.5f * (u0 + u1);
        else if (j == jx - 1) a[q] = 0.5f * (u1 + u0);
        else a[q] = 0.5625f * (u1 + u0) - 0.0625f * (u2 + um);
      }
      store(ux + o, a);
      float vc[4], vn[4], vs[4] = {0.f, 0.f, 0.f, 0.f}, vnn[4] = {0.f, 0.f, 0.f, 0.f};
      ld4f(vc, v + o);
      ld4f(vn, v + o + P);
      if (i >= 2 && i <= iy - 2) {
        ld4f(vs, v + o - P);
        ld4f(vnn, v + o + 2 * P);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (i == 1) a[q] = 0.5f * (vc[q] + vn[q]);
        else if (i == iy - 1) a[q] = 0.5f * (vn[q] + vc[q]);
        else a[q] = 0.5625f * (vn[q] + vc[q]) - 0.0625f * (vnn[q] + vs[q]);
      }
      store(vx + o, a);
    }
    // pressure (FP32 of the double-float Exner)
    float ph[4], pl[4], pk[4];
    ld4f(ph, pa_h + o);
    ld4f(pl, pa_h + F + o);
#pragma unroll
    for (int q = 0; q < 4; ++q) pk[q] = exner_to_pressure_f(ph[q] + pl[q]);
    store(pp + o, pk);
    // mkslice's floors, then status_update's (zero tendencies): at inner
    // points qx below its check value becomes its zero value, and a tracer
    // below 1e-50 becomes 0 (in FP32 every value below 1e-50 is <= 0)
    if (any_inner) {
      for (int n = 0; n < g.nqx; ++n) {
        float x[4];
        ld4f(x, qx + o + (size_t)n * F);
        bool ch = false;
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (inner[q] && x[q] < float(qx_check(n))) {
            x[q] = float(qx_zero(n));
            ch = true;
          }
        if (ch) store(qx + o + (size_t)n * F, x);
      }
      for (int n = 0; n < g.ntr; ++n) {
        float x[4];
        ld4f(x, trac + o + (size_t)n * F);
        bool ch = false;
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (inner[q] && x[q] <= 0.f) {
            x[q] = 0.f;
            ch = true;
          }
        if (ch) store(trac + o + (size_t)n * F, x);
      }
    }
    float tk[4], tl[4], tv[4], rh[4], th_o[4], tl_o[4], qs[4];
    ld4f(tk, tt + o);
    ld4f(tl, tlo + o);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const size_t oq = o + q;
      const float qf = qfactor(qx, oq, F, ipp);
      tv[q] = tk[q] * qf;
      rh[q] = pk[q] / (float(kRgas) * tk[q]);
      // theta_v = tvirt/pai from the double-float t (Main/mod_moloch.F90:1403-1443)
      const F2 th2 = df_div(df_mul(F2{tk[q], tl[q]}, qfactor_df(qx, oq, F, ipp)), F2{ph[q], pl[q]});
      th_o[q] = th2.hi;
      tl_o[q] = th2.lo;
      qs[q] = pfwsat_f(tk[q], pk[q]);
    }
    store(tvir + o, tv);
    store(rho + o, rh);
    store(th_h + o, th_o);
    store(th_h + F + o, tl_o);
    store(qsat + o, qs);
  }
}

// uvxtouvstag at the end of status_update (:1440)
template <class R>
__global__ void k_end_uvstag(const Dom<R> *__restrict__ doms, int uvoff, int advoff, int tiles_j,
    const WorkItem *__restrict__ wl) {
  const WorkItem wi = work_item(wl, tiles_j);
  const Dom<R> &D = doms[wi.m];
  if (!D.active) return;
  const Geom g = D.g;
  const int uv = (D.clk->uv_role + uvoff) & 1, adv = (D.clk->adv_role + advoff) & 1;
  const R *__restrict__ ux = D.ux[adv];
  const R *__restrict__ vx = D.vx[adv];
  R *__restrict__ u = D.u[uv];
  R *__restrict__ v = D.v[uv];
  const Pt q_ = point_at(wi, 1, 1);
  const int j = q_.j, k0 = q_.k;
  if (k0 > g.kz) return;
  const int i = q_.i;
  const int jx = g.jx, iy = g.iy;
  if (j > jx || i > iy) return;
  const size_t ij = g.at2(j, i), PS = g.PS, S = (size_t)g.P;
  const bool do_u = (j >= 2 && j <= jx - 1 && i >= 2 && i <= iy - 2);
  const bool do_v = (j >= 2 && j <= jx - 2 && i >= 2 && i <= iy - 1);
  if (!do_u && !do_v) return;
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
  }
}

// Mass budget (Main/mod_massck.F90:77-170) and ps extrema.  Block b sums the
// rows (i,k) it owns in a fixed order and writes seven partials; the single-
// block pass then adds the partials in block order, so the result does not
// depend on scheduling and a domain gives the same bits alone or in a batch.
constexpr int kRedThreads = 256;
constexpr int kRedWarps = kRedThreads / 32;
constexpr int kNPart = 7;  // dry, dryadv, qmass, qadv, ps max, ps min, non-finite flag

// dz of the member's field type (the FP32 copy for a mixed member)
template <class R>
__device__ __forceinline__ const R *pick_dz(const Stat<R> &sa) {
  if constexpr (sizeof(R) == sizeof(float)) return sa.dz_r;
  else return sa.dz;
}
// 16 bytes at p (16-byte aligned) as V elements
template <class R, int V>
__device__ __forceinline__ void ld_vec16(R (&x)[V], const R *p) {
  const uint4 w = *reinterpret_cast<const uint4 *>(p);
  memcpy(x, &w, 16);
}

// Partial sums of the mass budget (Main/mod_massck.F90:57-369) and the ps
// extrema of one member, per block.  The interior sums run over the member's
// 3-D arrays as flat vectors of 16 bytes (every row starts on 128 bytes, so a
// vector never straddles a row); a grid-stride loop over the vectors keeps
// many loads in flight.  The species of a point are summed before they are
// weighted by its dry mass dx^2*dz*rho.  FP32 members form the point products
// in FP32, add each vector's in FP32 and accumulate them as double-floats;
// dx^2 is applied once per thread.  The lateral fluxes and the ps extrema
// are grid-stride loops over their own items.  Sums are in a fixed order for
// a given member, whatever else the launch holds.
// Per member, by one warp of the reduction's last block: add the partials
// (lanes stride over the blocks in block order, then a fixed shuffle tree,
// so the result does not depend on which block finished last), store the
// diagnostics, then advance the boundary clock and the buffer roles to the
// next step's and re-arm the block count.
template <class R>
__device__ void reduce_finish(const Dom<R> &D, int uvoff, int advoff, int lane) {
  const double *part = D.partials;
  const int nblocks = D.red_blocks;
  double a[4] = {0, 0, 0, 0}, pmax = -INFINITY, pmin = INFINITY, bad = 0;
  for (int b = lane; b < nblocks; b += 32) {
    const double *p = part + (size_t)b * kNPart;
    for (int q = 0; q < 4; ++q) a[q] += __ldcg(p + q);
    pmax = fmax(pmax, __ldcg(p + 4));
    pmin = fmin(pmin, __ldcg(p + 5));
    bad += __ldcg(p + 6);
  }
  const unsigned full = 0xffffffffu;
  for (int off = 16; off > 0; off >>= 1) {
    for (int q = 0; q < 4; ++q) a[q] += __shfl_down_sync(full, a[q], off);
    pmax = fmax(pmax, __shfl_down_sync(full, pmax, off));
    pmin = fmin(pmin, __shfl_down_sync(full, pmin, off));
    bad += __shfl_down_sync(full, bad, off);
  }
  if (lane != 0) return;
  DiagDev *diag = D.diag;
  Clock *clk = D.clk;
  const bool isbad = bad != 0.0;
  diag->drymass = a[0]; diag->dryadv = a[1]; diag->qmass = a[2]; diag->qadv = a[3];
  diag->ps_max = isbad ? NAN : pmax;
  diag->ps_min = isbad ? NAN : pmin;
  diag->nonfinite = isbad ? 1 : 0;
  if (isbad && !clk->nonfinite) { clk->nonfinite = 1; clk->bad_step = clk->step; }
  if (D.c.apply_bdy) clk->xbctime = clk->xbctime + D.c.dtsec;
  if (D.c.apply_bdy && D.c.spectral) clk->tspectral = clk->tspectral + D.c.dtsec;
  clk->step = clk->step + 1;
  clk->uv_role = (clk->uv_role + uvoff) & 1;
  clk->adv_role = (clk->adv_role + advoff) & 1;
  clk->red_done = 0u;
}

template <class R>
__global__ void __launch_bounds__(kRedThreads) k_reduce_partial(const Dom<R> *__restrict__ doms,
                                                                int uvoff, int advoff) {
  __shared__ double sh[kRedWarps][kNPart];
  const Dom<R> &D = doms[blockIdx.y];
  if (!D.active) return;
  const int nb = D.red_blocks;
  if ((int)blockIdx.x >= nb) return;
  const Geom g = D.g;
  const Scal &c = D.c;
  const Stat<R> &sa = D.sa;
  const State<R> st = state_of(D, (D.clk->uv_role + uvoff) & 1, (D.clk->adv_role + advoff) & 1);
  const int jx = g.jx, iy = g.iy, kz = g.kz, nqx = g.nqx;
  const double dx = c.dx, dt = c.dt, dxsq = dx * dx;
  const size_t F = g.field3();
  const unsigned gt = blockIdx.x * kRedThreads + threadIdx.x;  // this thread's first item
  const unsigned gs = (unsigned)nb * kRedThreads;              // stride
  double dry = 0, dadv = 0, qm = 0, qadv = 0, pmax = -INFINITY, pmin = INFINITY, bad = 0;
  const bool budget = c.debug_level > 0;
  if (budget) {
    constexpr int V = 16 / (int)sizeof(R);
    const unsigned nvec = (unsigned)(g.PS * (size_t)kz) / V;  // below 2^31 / V
    const unsigned P = (unsigned)g.P;
    const R *__restrict__ dzp = pick_dz<R>(sa);
    F2 dry2{0.f, 0.f}, qm2{0.f, 0.f};
    for (unsigned v = gt; v < nvec; v += gs) {
      const unsigned base = v * V;
      const unsigned r = base / P;               // (i-1) + (k-1)*iy
      const int c0 = (int)(base - r * P);        // j-1 of the vector's first element
      const int i = (int)(r % (unsigned)iy) + 1;
      if (i < 2 || i > iy - 2 || c0 + 1 > jx - 2) continue;
      R dz[V], rh[V], qs[V], q1[V];
      ld_vec16<R, V>(dz, dzp + base);
      ld_vec16<R, V>(rh, st.rho + base);
      if constexpr (sizeof(R) == sizeof(float)) {
        // FP32 state, FP64-accurate sums: dz as the double-float {dz_r,
        // dz_lo}, dz*rho and each species' share as double-float products,
        // double-float running sums (about 1e-14 relative against the FP64
        // sums of the same FP32 state)
        R dzl[V];
        ld_vec16<R, V>(dzl, sa.dz_lo + base);
        F2 dr[V];
#pragma unroll
        for (int q = 0; q < V; ++q) {
          const int j = c0 + q + 1;
          dr[q] = (j >= 2 && j <= jx - 2) ? df_mul_f(F2{dz[q], dzl[q]}, rh[q]) : F2{0.f, 0.f};
          dry2 = df_add(dry2, dr[q]);
        }
        for (int n = 0; n < nqx; ++n) {
          ld_vec16<R, V>(q1, st.qx + base + (size_t)n * F);
#pragma unroll
          for (int q = 0; q < V; ++q) qm2 = df_add(qm2, df_mul_f(dr[q], q1[q]));
        }
      } else {
        ld_vec16<R, V>(qs, st.qx + base);
        for (int n = 1; n < nqx; ++n) {
          ld_vec16<R, V>(q1, st.qx + base + (size_t)n * F);
#pragma unroll
          for (int q = 0; q < V; ++q) qs[q] += q1[q];
        }
#pragma unroll
        for (int q = 0; q < V; ++q) {
          const int j = c0 + q + 1;
          if (j >= 2 && j <= jx - 2) {
            const double wpt = dxsq * (double)dz[q] * (double)rh[q];
            dry += wpt;
            qm += (double)qs[q] * wpt;
          }
        }
      }
    }
    if constexpr (sizeof(R) == sizeof(float)) {
      dry = ((double)dry2.hi + (double)dry2.lo) * dxsq;
      qm = ((double)qm2.hi + (double)qm2.lo) * dxsq;
    }
    // west and east columns over i in ice = 1 .. iy-1 (:85-100)
    const unsigned nwe = (unsigned)((iy - 1) * kz);
    for (unsigned e = gt; e < nwe; e += gs) {
      const int i = (int)(e % (unsigned)(iy - 1)) + 1, k = (int)(e / (unsigned)(iy - 1)) + 1;
      const size_t ko = (size_t)(k - 1) * g.PS;
      const size_t ow = g.at2(1, i) + ko, oe = g.at2(jx - 1, i) + ko;
      {
        // FP64 products of the state's values in both precisions (a few
        // thousand terms: the budget stays FP64-accurate for a mixed member)
        const double uw = (double)st.u[g.at2(1, i) + ko], ue = (double)st.u[g.at2(jx, i) + ko];
        const double dzw = (double)sa.dz[ow], rw = (double)st.rho[ow];
        const double dze = (double)sa.dz[oe], re = (double)st.rho[oe];
        dadv += uw * dt * dx * dzw * rw;
        dadv -= ue * dt * dx * dze * re;
        for (int n = 0; n < nqx; ++n) {
          qadv += (double)st.qx[ow + (size_t)n * F] * uw * dt * dx * dzw * rw;
          qadv -= (double)st.qx[oe + (size_t)n * F] * ue * dt * dx * dze * re;
        }
      }
    }
    // south (v at ide1) and north (v at ide2) rows, j in jci (:101-116)
    const unsigned nsn = (unsigned)(2 * kz * (jx - 3));
    for (unsigned e = gt; e < nsn; e += gs) {
      const int j = (int)(e % (unsigned)(jx - 3)) + 2;
      const unsigned rest = e / (unsigned)(jx - 3);
      const bool south = (rest & 1u) == 0;
      const int k = (int)(rest >> 1) + 1;
      const int i = south ? 1 : iy - 1, iv = south ? 1 : iy;
      const size_t ko = (size_t)(k - 1) * g.PS;
      const size_t o = g.at2(j, i) + ko;
      const double vv = (double)st.v[g.at2(j, iv) + ko];
      const double dzr = (double)sa.dz[o], rh = (double)st.rho[o];
      const double fl = vv * dt * dx * dzr * rh;
      dadv = south ? dadv + fl : dadv - fl;
      for (int n = 0; n < nqx; ++n) {
        const double q = (double)st.qx[o + (size_t)n * F] * vv * dt * dx * dzr * rh;
        qadv = south ? qadv + q : qadv - q;
      }
    }
  }
  // ps extrema over the interior
  const unsigned nps = (unsigned)((iy - 3) * (jx - 3));
  for (unsigned e = gt; e < nps; e += gs) {
    const int j = (int)(e % (unsigned)(jx - 3)) + 2, i = (int)(e / (unsigned)(jx - 3)) + 2;
    const double x = st.ps[g.at2(j, i)];
    if (!isfinite(x)) bad = 1;
    else { pmax = fmax(pmax, x); pmin = fmin(pmin, x); }
  }
  const unsigned full = 0xffffffffu;
  for (int off = 16; off > 0; off >>= 1) {
    dry += __shfl_down_sync(full, dry, off);
    qm += __shfl_down_sync(full, qm, off);
    dadv += __shfl_down_sync(full, dadv, off);
    qadv += __shfl_down_sync(full, qadv, off);
    bad += __shfl_down_sync(full, bad, off);
    pmax = fmax(pmax, __shfl_down_sync(full, pmax, off));
    pmin = fmin(pmin, __shfl_down_sync(full, pmin, off));
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    sh[warp][0] = dry; sh[warp][1] = dadv; sh[warp][2] = qm; sh[warp][3] = qadv;
    sh[warp][4] = pmax; sh[warp][5] = pmin; sh[warp][6] = bad;
  }
  __syncthreads();
  __shared__ bool last;
  if (threadIdx.x == 0) {
    double a[kNPart] = {0, 0, 0, 0, -INFINITY, INFINITY, 0};
    for (int w = 0; w < kRedWarps; ++w) {
      a[0] += sh[w][0]; a[1] += sh[w][1]; a[2] += sh[w][2]; a[3] += sh[w][3];
      a[4] = fmax(a[4], sh[w][4]); a[5] = fmin(a[5], sh[w][5]); a[6] += sh[w][6];
    }
    double *p = D.partials + (size_t)blockIdx.x * kNPart;
    for (int q = 0; q < kNPart; ++q) p[q] = a[q];
    // the member's last block to finish adds the partials: its partials are
    // visible before its ticket, and every other block's before theirs
    __threadfence();
    last = atomicAdd(&D.clk->red_done, 1u) == (unsigned)nb - 1u;
  }
  __syncthreads();
  if (!last || threadIdx.x >= 32) return;
  __threadfence();
  reduce_finish<R>(D, uvoff, advoff, (int)threadIdx.x);
}

template <class R>
__global__ void k_unpack3(const double *__restrict__ src, R *__restrict__ dst, Geom g, int nj, int ni, int nk) {
  const size_t n = (size_t)nj * ni * nk;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e % nj);
    const size_t r = e / nj;
    const int i = (int)(r % ni);
    const int k = (int)(r / ni);
    dst[(size_t)j + (size_t)i * g.P + (size_t)k * g.PS] = (R)src[e];
  }
}

template <class R>
__global__ void k_pack3(const R *__restrict__ src, double *__restrict__ dst, Geom g, int nj, int ni, int nk) {
  const size_t n = (size_t)nj * ni * nk;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e % nj);
    const size_t r = e / nj;
    const int i = (int)(r % ni);
    const int k = (int)(r / ni);
    dst[e] = (double)src[(size_t)j + (size_t)i * g.P + (size_t)k * g.PS];
  }
}

// hi = fl(x), lo = fl(x - hi): x to ~48 bits as two floats
__global__ void k_unpack3_df(const double *__restrict__ src, float *__restrict__ dst, Geom g, int nj,
                             int ni, int nk, size_t nplane) {
  const size_t n = (size_t)nj * ni * nk;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e % nj);
    const size_t r = e / nj;
    const int i = (int)(r % ni);
    const int k = (int)(r / ni);
    const size_t o = (size_t)j + (size_t)i * g.P + (size_t)k * g.PS;
    const double x = src[e];
    const float hi = (float)x;
    dst[o] = hi;
    dst[o + nplane] = (float)(x - (double)hi);
  }
}

__global__ void k_pack3_df(const float *__restrict__ src, double *__restrict__ dst, Geom g, int nj,
                           int ni, int nk, size_t nplane) {
  const size_t n = (size_t)nj * ni * nk;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e % nj);
    const size_t r = e / nj;
    const int i = (int)(r % ni);
    const int k = (int)(r / ni);
    const size_t o = (size_t)j + (size_t)i * g.P + (size_t)k * g.PS;
    dst[e] = (double)src[o] + (double)src[o + nplane];
  }
}

inline dim3 grid2(int nj, int ni, dim3 b, int nmem) {
  return dim3((unsigned)((nj + b.x - 1) / b.x), (unsigned)((ni + b.y - 1) / b.y), (unsigned)nmem);
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

// some 16 elements per thread, at most 4 blocks per SM
int reduce_blocks(const Geom &g) {
  const size_t n = g.PS * (size_t)g.kz;
  const size_t per_block = (size_t)kRedThreads * 16;
  const size_t nb = (n + per_block - 1) / per_block;
  return (int)std::min<size_t>(std::max<size_t>(nb, 1), 152 * 4);
}

// status_update of the turbulent kinetic energy (Main/mod_moloch.F90:
// 1419-1424): on jci x ici at the kz+1 interfaces, tke + dtsec * tketen (the
// physics' tendency; none in a whole step), then the floor tkemin.
template <class R>
__global__ void k_end_tke(const Dom<R> *__restrict__ doms, int whole, int tiles_j,
    const WorkItem *__restrict__ wl) {
  const WorkItem wi = work_item(wl, tiles_j);
  const Dom<R> &D = doms[wi.m];
  if (!D.active || !D.c.tke) return;
  const Geom g = D.g;
  const Pt q = point_at(wi, 1, 1);
  if (q.j < 2 || q.j > g.jx - 2 || q.i < 2 || q.i > g.iy - 2 || q.k > g.kz) return;
  const R *ten = whole ? nullptr : D.tend;
  // tketen follows the kz-plane tendencies (t, u, v, the species, tracers)
  const R *tt = ten ? ten + (size_t)(3 + g.nqx + g.ntr) * g.field3() : nullptr;
  const R dts = pick<R>(D.c.dtsec, D.c.dtsecf);
  const int klast = q.k + kPtLevels - 1 >= g.kz ? g.kz + 1 : q.k + kPtLevels - 1;
  for (int k = q.k; k <= klast; ++k) {
    const size_t o = g.at(q.j, q.i, k);
    R v = D.tke[o];
    if (tt) v = v + dts * tt[o];
    if (v < R(kTkeMin)) v = R(kTkeMin);
    D.tke[o] = v;
  }
}

template <class R>
void Launch<R>::bdy_ring(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s) {
  k_bdy_ring<R><<<dim3((unsigned)L.kz, (unsigned)L.nmem), kRingThreads, 0, s>>>(d, uvoff, advoff);
}

template <class R>
void Launch<R>::end_relax(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s) {
  const dim3 b((unsigned)L.col_x, (unsigned)L.col_y);
  int tj;
  const dim3 grd = pt_grid(L, L.jx - 1, L.iy - 1, tj);
  k_end_relax<R><<<grd, b, 0, s>>>(d, uvoff, advoff, tj, L.wl_pt);
}

template <class R>
void Launch<R>::bdy_spectral(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff,
                             cudaStream_t s) {
  const unsigned fk = (unsigned)(L.kz * 3);
  k_spec_rows<R><<<dim3((unsigned)((L.iy + 7) / 8), fk, (unsigned)L.nmem), 256, 0, s>>>(d, uvoff, advoff);
  k_spec_modes<R><<<dim3(1, fk, (unsigned)L.nmem), 256, 0, s>>>(d);
  const dim3 b((unsigned)L.col_x, (unsigned)L.col_y);
  int tj;
  const dim3 grd = pt_grid(L, L.jx - 2, L.iy - 2, tj);
  k_spec_apply<R><<<grd, b, 0, s>>>(d, uvoff, advoff, tj, L.wl_pt);
}

template <class R>
void Launch<R>::end_cross(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s) {
  const dim3 b((unsigned)L.col_x, (unsigned)L.col_y);
  if constexpr (sizeof(R) == sizeof(float)) {
    const int tj = (L.jx - 1 + 127) / 128, ti = (L.iy - 1 + 3) / 4;
    const dim3 grd = L.wl_v4 ? dim3((unsigned)L.n_v4, 1, 1)
                             : dim3((unsigned)(tj * ti), (unsigned)((L.kz + kPtLevels - 1) / kPtLevels),
                                    (unsigned)L.nmem);
    k_end_cross_v4<R><<<grd, dim3(32, 4), 0, s>>>(d, uvoff, advoff, tj, L.wl_v4);
  } else {
    int tj;
    const dim3 grd = pt_grid(L, L.jx - 1, L.iy - 1, tj);
    k_end_cross<R, kEndAll><<<grd, b, 0, s>>>(d, uvoff, advoff, tj, L.wl_pt);
  }
}

template <class R>
void Launch<R>::end_cross_split(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, bool post,
                                cudaStream_t s) {
  const dim3 b((unsigned)L.col_x, (unsigned)L.col_y);
  int tj;
  const dim3 grd = pt_grid(L, L.jx - 1, L.iy - 1, tj);
  if (post) {
    k_end_cross<R, kEndPost><<<grd, b, 0, s>>>(d, uvoff, advoff, tj, L.wl_pt);
  } else {
    k_end_ps<R><<<grid2(L.jx - 3, L.iy - 3, b, L.nmem), b, 0, s>>>(d, uvoff, advoff);
    k_end_cross<R, kEndPre><<<grd, b, 0, s>>>(d, uvoff, advoff, tj, L.wl_pt);
  }
}

template <class R>
void Launch<R>::end_uvstag(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff, cudaStream_t s) {
  const dim3 b((unsigned)L.col_x, (unsigned)L.col_y);
  int tj;
  const dim3 grd = pt_grid(L, L.jx, L.iy, tj);
  k_end_uvstag<R><<<grd, b, 0, s>>>(d, uvoff, advoff, tj, L.wl_pt);
}

template <class R>
void Launch<R>::end_tke(const LaunchGeom &L, const Dom<R> *d, bool whole_step, cudaStream_t s) {
  const dim3 b((unsigned)L.col_x, (unsigned)L.col_y);
  int tj;
  const dim3 grd = pt_grid(L, L.jx, L.iy, tj);
  k_end_tke<R><<<grd, b, 0, s>>>(d, whole_step ? 1 : 0, tj, L.wl_pt);
}

template <class R>
void Launch<R>::end_reduce(const LaunchGeom &L, const Dom<R> *d, int uvoff, int advoff,
                           cudaStream_t s) {
  k_reduce_partial<R><<<dim3((unsigned)L.red_blocks, (unsigned)L.nmem), kRedThreads, 0, s>>>(
      d, uvoff, advoff);
}

template <class R>
void Launch<R>::unpack3(const double *src, R *dst, const Geom &g, int nj, int ni, int nk, cudaStream_t s) {
  k_unpack3<R><<<152 * 8, 256, 0, s>>>(src, dst, g, nj, ni, nk);
}

template <class R>
void Launch<R>::pack3(const R *src, double *dst, const Geom &g, int nj, int ni, int nk, cudaStream_t s) {
  k_pack3<R><<<152 * 8, 256, 0, s>>>(src, dst, g, nj, ni, nk);
}

template <class R>
void Launch<R>::unpack3_df(const double *src, double *dst, const Geom &g, int nj, int ni, int nk,
                           size_t nplane, cudaStream_t s) {
  k_unpack3_df<<<152 * 8, 256, 0, s>>>(src, reinterpret_cast<float *>(dst), g, nj, ni, nk, nplane);
}

template <class R>
void Launch<R>::pack3_df(const double *src, double *dst, const Geom &g, int nj, int ni, int nk,
                         size_t nplane, cudaStream_t s) {
  k_pack3_df<<<152 * 8, 256, 0, s>>>(reinterpret_cast<const float *>(src), dst, g, nj, ni, nk, nplane);
}

template struct Launch<double>;
template struct Launch<float>;

}  // namespace mlc
