// moloch_oracle.cpp -- TEST INFRASTRUCTURE ONLY: the CPU oracle.
//
// A plain C++ FP64 restatement of RegCM's MOLOCH timestep, loop by loop and
// in the reference's order of operations, for checking the GPU library.  It
// follows (all paths relative to the RegCM source tree):
//   Main/mod_moloch.F90:201-308   init_moloch
//   Main/mod_moloch.F90:312-446   moloch (physics and zenitm left out; of mkslice,
//                                 Main/mod_slice.F90:110-147, its edits of the state)
//   Main/mod_moloch.F90:448-529   boundary
//   Main/mod_moloch.F90:531-765   divergence_diffusion, sound, divergence_damping
//   Main/mod_moloch.F90:767-1042  advection, wafone
//   Main/mod_moloch.F90:1044-1141 reset_tendencies, dynamical_core
//   Main/mod_moloch.F90:1403-1648 status_update, interpolations,
//                                 local_flow_param, surface pressure, tvirt
//   Main/mod_bdycod.F90:1618-1875,2653  bdyval (MOLOCH branch) and its clock
//   Main/mod_bdycod.F90:3962-4083 morelax_*, setup_bdywt, motopnudge
//   Main/chemlib/mod_che_bdyco.F90:391-535,965-1026 tracer ring and relaxation
//   Main/mod_massck.F90:57-200    MOLOCH mass budget sums
//   Share/pfwsat.inc:1-43         saturation mixing ratio
//
// Parity is unpinned by the reference's own tests: RegCM ships no golden
// vectors or unit tests for this path and its Fortran cannot be compiled in
// this environment (no Fortran compiler, MPI or netCDF).  The oracle is
// pinned by physical invariants and known-answer checks in tests/.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
// this file's library, as the checker.  Elementwise loops may run under
// OpenMP (results do not depend on the thread count); reductions are serial.
#include "oracle_common.h"
#include "../include/moloch_gb300.h"
#include "../include/moloch_gb300_restart.h"

#include <algorithm>
#include <cstdio>
#include <memory>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

struct Oracle {
  // ---- extents (Main/mod_atm_interface.F90:182-382, serial non-band) ----
  int jx, iy, kz, kzp1, kzm1, nqx, ntr;
  int jde1, jde2, jdi1, jdi2, jdii1, jdii2, jce1, jce2, jci1, jci2;
  int ide1, ide2, idi1, idi2, idii1, idii2, ice1, ice2, ici1, ici2;
  int jmin, jmax, imin, imax;
  mlc_params prm;
  double dx, rdx, dt, dtsec;
  bool have_static = false, have_state = false, have_bdy = false;

  // ---- static ----
  F2<double> msfu, msfv, msfx, mx2, rmx, rmu, rmv, coru, corv, hx, hy;
  std::vector<double> rlat;  // 1-based
  F3 fmz, fmzf, rfmzu, rfmzv, zeta, dz;
  std::vector<double> zita, zitah, ffilt, tnudge, gzitak, gzitakh, xkdamp, xknu;
  F2<double> hefc;  // (1:nspgx, 1:kz)
  std::vector<double> fcx;
  F2<int32_t> ibnd_cr, ibnd_ud, ibnd_vd;
  bool hb_cr = false, hb_ud = false, hb_vd = false;
  F3 bdywtu, bdywtv, bdywtw;
  double mo_dzita = 0, rdzita = 0, dtstepa = 0, dtsound = 0;
  // spectral nudging (Main/mod_bdycod.F90:3844-3960)
  int km = 0, lm = 0;
  F2<double> bvx, bvy, sx, sy, zn1;
  std::vector<double> cnudge;  // 1-based
  double tspectral = 0;

  // ---- state ----
  F3 u, v, w, pai, tetav, t, tvirt, ux, vx, p, rho, qsat;
  std::vector<F3> qx, trac;
  F2<double> ps;
  bool use_tke = false;   // ibltyp = 2
  F3 tke, tkex;           // (jce, ice, 1:kzp1) and its copy at the levels

  // ---- boundary ----
  F3 xtb[2], xqb[2], xpaib[2], xlb[2], xib[2], dub[2], dvb[2];
  F2<double> xpsb[2];
  std::vector<F3> chib[2];
  double xbctime = 0, dtbdys = 1, rtb = 1;

  // ---- physics tendencies (jci x ici, Main/mod_atm_interface.F90:606-617) ----
  F3 tten, uten, vten, tketen;
  std::vector<F3> qxten, chiten;
  bool step_open = false;

  // ---- work ----
  F3 s, wwkw, tetavf, zdiv2, laplacian, wz, p0, wfw, wx, zpby, zpbw, ud, vd;

  int create(const mlc_dims *d, const mlc_params *pp);
  int bind_static(const mlc_static_ptrs *st);
  void init_moloch();
  void moloch(mlc_diag *dg);
  void moloch_dynamics();
  void moloch_finish(mlc_diag *dg);
  void mkslice();
  void reset_tendencies();
  void dynamical_core(double dta, double dts);
  void sound(double dts);
  void divergence_damping(double dts);
  void divergence_diffusion();
  void advection(double dta);
  void wafone(F3 &pp, double dta);
  void boundary();
  void bdyval();
  void motopnudge(double wfac, double dta);
  void morelax_external(int j1, int j2, int i1, int i2, const F2<int32_t> &ibnd, bool hb,
                        F3 &f, const F3 *bnd);
  void morelax_fraction(int j1, int j2, int i1, int i2, const F2<int32_t> &ibnd, bool hb,
                        F3 &f, double frac);
  void morelax_chiten();
  void lowpass_init();
  void lowpass_filter(int j1, int j2, int i1, int i2, int jj1, int jj2, int ii1, int ii2, F2<double> &f);
  void mospectral_nudge(int j1, int j2, int i1, int i2, int jj1, int jj2, int ii1, int ii2, F3 &f,
                        const F3 *bnd);
  void status_update(double dtinc);
  void massck(mlc_diag *dg);
  void uvstagtouvx();
  void uvxtouvstag();
  void zstagtoh(const F3 &fl, F3 &hl);
  void htozstag(const F3 &hl, F3 &fl);
  void temp_to_tvirt();
  void tvirt_to_temp();
  void extrapolate_surface_pressure();
};

// Share/pfwsat.inc:1-43
static inline double pfwsat(double t, double p) {
  const double a0 = 0.611213476e+03, a1 = 0.444007856e+02, a2 = 0.143064234e+01,
               a3 = 0.264461437e-01, a4 = 0.305903558e-03, a5 = 0.196237241e-05,
               a6 = 0.892344772e-08, a7 = -0.373208410e-10, a8 = 0.209339997e-13;
  const double c0 = 0.611123516e+03, c1 = 0.503109514e+02, c2 = 0.188369801e+01,
               c3 = 0.420547422e-01, c4 = 0.614396778e-03, c5 = 0.602780717e-05,
               c6 = 0.387940929e-07, c7 = 0.149436277e-09, c8 = 0.262655803e-12;
  double t_limit = t - tzero;
  double td = std::min(std::max(t_limit, -75.0), 100.0);
  double es;
  if (td >= 0.0) {
    es = std::min(a0 + td * (a1 + td * (a2 + td * (a3 + td * (a4 + td * (a5 + td * (a6 + td * (a7 + td * a8))))))),
                  0.15 * p);
  } else {
    es = std::min(c0 + td * (c1 + td * (c2 + td * (c3 + td * (c4 + td * (c5 + td * (c6 + td * (c7 + td * c8))))))),
                  0.15 * p);
  }
  return ep2 * (es / (p - es));
}

// Main/mod_moloch.F90:1571-1590 (double-precision build: minden 1e-30,
// minnum is the same literal held as a 4-byte real).
static inline double local_flow_param(double num, double den) {
  const double minden = 1.0e-30;
  const double minnum = (double)(float)1.0e-30;
  if (std::fabs(den) < minden) {
    return (std::fabs(num) < minnum) ? 1.0 : 0.0;
  }
  return num / den;
}

// Fortran min/max on doubles (no NaN inputs reach them on this path).
static inline double fmin2(double a, double b) { return (b < a) ? b : a; }
static inline double fmax2(double a, double b) { return (b > a) ? b : a; }

// Share/mod_zita.F90:105-115 gzita
static inline double gzita(double zita, double ztop, double a0) {
  double ratio = zita / ztop;
  return ((0.0 - 1.0 * a0) * ratio - (3.0 - 2.0 * a0) * (ratio * ratio) +
          (2.0 - 1.0 * a0) * (ratio * ratio * ratio)) + 1.0;
}

int Oracle::create(const mlc_dims *d, const mlc_params *pp) {
  jx = d->jx; iy = d->iy; kz = d->kz; nqx = d->nqx; ntr = d->ntr;
  if (jx < 8 || iy < 8 || kz < 4 || nqx < 1 || ntr < 0) return MLC_ERR_INVALID;
  prm = *pp;
  kzp1 = kz + 1; kzm1 = kz - 1;
  // Main/mod_atm_interface.F90:236-290 with all four boundaries present
  jde1 = 1; jde2 = jx; jdi1 = 2; jdi2 = jx - 1; jdii1 = 3; jdii2 = jx - 2;
  ide1 = 1; ide2 = iy; idi1 = 2; idi2 = iy - 1; idii1 = 3; idii2 = iy - 2;
  jce1 = 1; jce2 = jx - 1; jci1 = 2; jci2 = jx - 2;
  ice1 = 1; ice2 = iy - 1; ici1 = 2; ici2 = iy - 2;
  // Main/mod_moloch.F90:266-280 with jcross/icross of mod_mppparam.F90:1734-1758
  jmin = 1; jmax = jx - 1; imin = 1; imax = iy - 1;
  dx = prm.dx; rdx = 1.0 / dx; dtsec = prm.dtsec; dt = prm.dtsec;

  msfu.init(jde1, jde2, ide1, ide2); msfv.init(jde1, jde2, ide1, ide2);
  msfx.init(jde1, jde2, ide1, ide2);
  mx2.init(jde1, jde2, ide1, ide2); rmx.init(jde1, jde2, ide1, ide2);
  rmu.init(jde1, jde2, ide1, ide2); rmv.init(jde1, jde2, ide1, ide2);
  coru.init(jde1, jde2, ice1, ice2); corv.init(jce1, jce2, ide1, ide2);
  hx.init(jde1, jde2, ice1, ice2); hy.init(jce1, jce2, ide1, ide2);
  rlat.assign(iy + 1, 0.0);
  fmz.init(jce1, jce2, ice1, ice2, 1, kz); fmzf.init(jce1, jce2, ice1, ice2, 1, kzp1);
  rfmzu.init(jde1, jde2, ice1, ice2, 1, kz); rfmzv.init(jce1, jce2, ide1, ide2, 1, kz);
  zeta.init(jce1, jce2, ice1, ice2, 1, kz); dz.init(jce1, jce2, ice1, ice2, 1, kz);
  zita.assign(kzp1 + 1, 0.0); zitah.assign(kz + 1, 0.0); ffilt.assign(kz + 1, 0.0);
  tnudge.assign(kz + 1, 0.0); gzitak.assign(kzp1 + 1, 0.0); gzitakh.assign(kz + 1, 0.0);
  xkdamp.assign(kz + 1, 0.0); xknu.assign(kz + 1, 0.0);
  hefc.init(1, prm.nspgx, 1, kz); fcx.assign(prm.nspgx + 1, 0.0);
  ibnd_cr.init(jde1, jde2, ide1, ide2); ibnd_ud.init(jde1, jde2, ide1, ide2);
  ibnd_vd.init(jde1, jde2, ide1, ide2);
  bdywtu.init(jdi1, jdi2, ici1, ici2, 1, kz); bdywtv.init(jci1, jci2, idi1, idi2, 1, kz);
  bdywtw.init(jci1, jci2, ici1, ici2, 1, kz);

  u.init(jde1, jde2, ice1, ice2, 1, kz); v.init(jce1, jce2, ide1, ide2, 1, kz);
  w.init(jce1, jce2, ice1, ice2, 1, kzp1);
  for (F3 *f : {&pai, &tetav, &t, &tvirt, &ux, &vx, &p, &rho, &qsat})
    f->init(jce1, jce2, ice1, ice2, 1, kz);
  qx.assign(nqx, F3()); for (auto &f : qx) f.init(jce1, jce2, ice1, ice2, 1, kz);
  trac.assign(ntr, F3()); for (auto &f : trac) f.init(jce1, jce2, ice1, ice2, 1, kz);
  ps.init(jce1, jce2, ice1, ice2);
  tten.init(jci1, jci2, ici1, ici2, 1, kz);
  uten.init(jci1, jci2, ici1, ici2, 1, kz);
  vten.init(jci1, jci2, ici1, ici2, 1, kz);
  qxten.assign(nqx, F3()); for (auto &f : qxten) f.init(jci1, jci2, ici1, ici2, 1, kz);
  chiten.assign(ntr, F3()); for (auto &f : chiten) f.init(jci1, jci2, ici1, ici2, 1, kz);
  // Main/mod_atm_interface.F90:611-612, Main/mod_moloch.F90:184
  use_tke = prm.ibltyp == 2;
  if (use_tke) {
    tke.init(jce1, jce2, ice1, ice2, 1, kzp1);
    tketen.init(jci1, jci2, ici1, ici2, 1, kzp1);
    tkex.init(jce1, jce2, ice1, ice2, 1, kz);
  }

  for (int b = 0; b < 2; ++b) {
    for (F3 *f : {&xtb[b], &xqb[b], &xpaib[b], &xlb[b], &xib[b]})
      f->init(jce1, jce2, ice1, ice2, 1, kz);
    dub[b].init(jde1, jde2, ice1, ice2, 1, kz);
    dvb[b].init(jce1, jce2, ide1, ide2, 1, kz);
    xpsb[b].init(jce1, jce2, ice1, ice2);
    chib[b].assign(ntr, F3());
    for (auto &f : chib[b]) f.init(jce1, jce2, ice1, ice2, 1, kz);
  }

  // allocate_moloch (Main/mod_moloch.F90:159-199), serial extents
  s.init(jce1, jce2, ice1, ice2, 1, kzp1);
  wwkw.init(jce1, jce2, ice1, ice2, 2, kzp1);
  tetavf.init(jce1, jce2, ice1, ice2, 2, kz);
  zdiv2.init(jce1, jce2, ice1, ice2, 1, kz);
  laplacian.init(jci1, jci2, ici1, ici2, 1, kz);
  wz.init(jce1, jce2, ice1, ice2, 1, kz);
  p0.init(jce1, jce2, ice1, ice2, 1, kz);
  wfw.init(jce1, jce2, ice1, ice2, 1, kzp1);
  wx.init(jce1, jce2, ice1, ice2, 1, kz);
  zpby.init(jce1, jce2, ici1, ice2, 1, kz);
  zpbw.init(jci1, jce2, ici1, ici2, 1, kz);
  ud.init(jde1, jde2, ice1, ice2, 1, kz);
  vd.init(jce1, jce2, ide1, ide2, 1, kz);
  return MLC_OK;
}

int Oracle::bind_static(const mlc_static_ptrs *st) {
  auto ld2 = [](F2<double> &a, const double *src) {
    if (src) std::memcpy(a.d.data(), src, a.d.size() * sizeof(double));
  };
  ld2(msfu, st->msfu); ld2(msfv, st->msfv); ld2(msfx, st->msfx);
  ld2(hx, st->hx); ld2(hy, st->hy);
  if (st->rlat) for (int i = 1; i <= iy; ++i) rlat[i] = st->rlat[i - 1];
  fmz.load(st->fmz); fmzf.load(st->fmzf); rfmzu.load(st->rfmzu); rfmzv.load(st->rfmzv);
  zeta.load(st->zeta); dz.load(st->dz);
  for (int k = 1; k <= kzp1; ++k) zita[k] = st->zita[k - 1];
  for (int k = 1; k <= kz; ++k) {
    zitah[k] = st->zitah[k - 1];
    ffilt[k] = st->ffilt[k - 1];
    tnudge[k] = st->tnudge ? st->tnudge[k - 1] : 0.0;
  }
  cnudge.assign(kz + 1, 0.0);
  if (prm.mo_spectral_nudge) {
    if (!st->cnudge) return MLC_ERR_INVALID;
    for (int k = 1; k <= kz; ++k) cnudge[k] = st->cnudge[k - 1];
    lowpass_init();
  }
  std::memcpy(hefc.d.data(), st->hefc, hefc.d.size() * sizeof(double));
  for (int n = 1; n <= prm.nspgx; ++n) fcx[n] = st->fcx ? st->fcx[n - 1] : 0.0;
  std::memcpy(ibnd_cr.d.data(), st->ibnd_cr, ibnd_cr.d.size() * sizeof(int32_t));
  std::memcpy(ibnd_ud.d.data(), st->ibnd_ud, ibnd_ud.d.size() * sizeof(int32_t));
  std::memcpy(ibnd_vd.d.data(), st->ibnd_vd, ibnd_vd.d.size() * sizeof(int32_t));
  hb_cr = hb_ud = hb_vd = false;
  for (auto x : ibnd_cr.d) hb_cr |= (x > 0);
  for (auto x : ibnd_ud.d) hb_ud |= (x > 0);
  for (auto x : ibnd_vd.d) hb_vd |= (x > 0);
  // coriolis from the u/v latitudes, Main/mod_moloch.F90:258-259
  for (int i = ice1; i <= ice2; ++i)
    for (int j = jde1; j <= jde2; ++j)
      coru(j, i) = eomeg2 * std::sin(st->ulat[(j - 1) + (size_t)(i - 1) * jx] * degrad);
  for (int i = ide1; i <= ide2; ++i)
    for (int j = jce1; j <= jce2; ++j)
      corv(j, i) = eomeg2 * std::sin(st->vlat[(j - 1) + (size_t)(i - 1) * (jx - 1)] * degrad);
  init_moloch();
  have_static = true;
  return MLC_OK;
}

// Main/mod_moloch.F90:261-307 (the parts that do not read the state)
void Oracle::init_moloch() {
  for (int i = ide1; i <= ide2; ++i)
    for (int j = jde1; j <= jde2; ++j) {
      mx2(j, i) = msfx(j, i) * msfx(j, i);
      rmx(j, i) = d_one / msfx(j, i);
      rmu(j, i) = d_one / msfu(j, i);
      rmv(j, i) = d_one / msfv(j, i);
    }
  for (int k = 1; k <= kzp1; ++k) gzitak[k] = gzita(zita[k], prm.mo_ztop, prm.mo_a0);
  for (int k = 1; k <= kz; ++k) gzitakh[k] = gzita(zitah[k], prm.mo_ztop, prm.mo_a0);
  mo_dzita = zita[kz];  // Main/mod_params.F90:2462
  rdzita = 1.0 / mo_dzita;
  const double numax = 0.125, ddamp = 0.850;
  for (int k = 1; k <= kz; ++k) {
    xkdamp[k] = numax * ddamp * (1.0 / (k + 1.0) - 1.0 / (kz + 2.0));
    xknu[k] = numax * (0.55 + 0.45 * ((double)(kz - k + 1) - 1.0) / ((double)kz - 1.0));
  }
  // setup_bdywt, Main/mod_bdycod.F90:4033-4047
  auto bdywt = [&](int j1, int j2, int i1, int i2, F3 &mask, const F2<int32_t> &ib) {
    for (int k = 1; k <= kz; ++k)
      for (int i = i1; i <= i2; ++i)
        for (int j = j1; j <= j2; ++j) {
          int b = ib(j, i);
          mask(j, i, k) = (b > 0) ? 1.0 - hefc(b, k) : 1.0;
        }
  };
  bdywt(jdi1, jdi2, ici1, ici2, bdywtu, ibnd_ud);
  bdywt(jci1, jci2, idi1, idi2, bdywtv, ibnd_vd);
  bdywt(jci1, jci2, ici1, ici2, bdywtw, ibnd_cr);
  dtstepa = dtsec / (double)prm.mo_nadv;
  dtsound = dtstepa / (double)prm.mo_nsound;
}

// ---------------------------------------------------------------- step ----
// Main/mod_moloch.F90:312-446, as its two halves around the physics: the
// dynamics through mkslice's edits of the state (:312-357), then
// status_update with the tendencies the physics left, the mass check and
// the ps check (:376-422).
void Oracle::moloch(mlc_diag *dg) {
  moloch_dynamics();
  moloch_finish(dg);
}

void Oracle::moloch_dynamics() {
  reset_tendencies();
  dynamical_core(dtstepa, dtsound);
  if (prm.do_apply_bdy) boundary();
  // :348-352
#pragma omp parallel for
  for (int k = 1; k <= kz; ++k)
    for (int i = ice1; i <= ice2; ++i)
      for (int j = jce1; j <= jce2; ++j) {
        p(j, i, k) = std::pow(pai(j, i, k), cpovr) * p00;
        rho(j, i, k) = p(j, i, k) / (rgas * t(j, i, k));
        qsat(j, i, k) = pfwsat(t(j, i, k), p(j, i, k));
      }
  extrapolate_surface_pressure();
  mkslice();
}

void Oracle::moloch_finish(mlc_diag *dg) {
  status_update(dtsec);
  if (prm.debug_level > 0) massck(dg);
  // :407-422 -- any non-finite ps is reported (the reference tests max/min)
  double mx = -INFINITY, mn = INFINITY;
  int bad = 0;
  for (int i = ici1; i <= ici2; ++i)
    for (int j = jci1; j <= jci2; ++j) {
      double x = ps(j, i);
      if (!std::isfinite(x)) bad = 1;
      if (x > mx) mx = x;
      if (x < mn) mn = x;
    }
  if (dg) { dg->ps_max = mx; dg->ps_min = mn; dg->nonfinite = bad; dg->xbctime = xbctime; }
}

// Main/mod_moloch.F90:1044-1083
void Oracle::reset_tendencies() {
  std::fill(tten.d.begin(), tten.d.end(), 0.0);
  std::fill(uten.d.begin(), uten.d.end(), 0.0);
  std::fill(vten.d.begin(), vten.d.end(), 0.0);
  for (auto &f : qxten) std::fill(f.d.begin(), f.d.end(), 0.0);
  for (auto &f : chiten) std::fill(f.d.begin(), f.d.end(), 0.0);
  if (use_tke) std::fill(tketen.d.begin(), tketen.d.end(), 0.0);
  std::fill(s.d.begin(), s.d.end(), 0.0);
  for (int k = 1; k <= kz; ++k)
    for (int i = ici1; i <= ici2; ++i)
      for (int j = jci1; j <= jci2; ++j) zdiv2(j, i, k) = 0.0;
  std::fill(wwkw.d.begin(), wwkw.d.end(), 0.0);
}

// Main/mod_moloch.F90:1085-1141
void Oracle::dynamical_core(double dta, double dts) {
  for (int nadv = 1; nadv <= prm.mo_nadv; ++nadv) {
    sound(dts);
    advection(dta);
  }
#pragma omp parallel for
  for (int k = 1; k <= kz; ++k)
    for (int i = ice1; i <= ice2; ++i)
      for (int j = jce1; j <= jce2; ++j) tvirt(j, i, k) = tetav(j, i, k) * pai(j, i, k);
  tvirt_to_temp();
}

// Main/mod_moloch.F90:531-543
void Oracle::divergence_diffusion() {
#pragma omp parallel for
  for (int k = 1; k <= kz; ++k)
    for (int i = ici1; i <= ici2; ++i)
      for (int j = jci1; j <= jci2; ++j)
        laplacian(j, i, k) = (zdiv2(j - 1, i, k) + zdiv2(j + 1, i, k) + zdiv2(j, i - 1, k) +
                              zdiv2(j, i + 1, k) - 4.0 * zdiv2(j, i, k));
#pragma omp parallel for
  for (int k = 1; k <= kz; ++k)
    for (int i = ici1; i <= ici2; ++i)
      for (int j = jci1; j <= jci2; ++j)
        zdiv2(j, i, k) = zdiv2(j, i, k) + xknu[k] * laplacian(j, i, k);
}

// Main/mod_moloch.F90:545-736
void Oracle::sound(double dts) {
  const bool lrot = prm.lrotllr != 0;
  const double dtrdx = dts * rdx, dtrdy = dts * rdx, dtrdz = dts * rdzita;
  const double zcs2 = (dtrdz * dtrdz) * rdrcv;

#pragma omp parallel for
  for (int k = 2; k <= kz; ++k)
    for (int i = ice1; i <= ice2; ++i)
      for (int j = jce1; j <= jce2; ++j)
        tetavf(j, i, k) = 0.5 * (tetav(j, i, k - 1) + tetav(j, i, k));

  for (int nsound = 1; nsound <= prm.mo_nsound; ++nsound) {
    ud.d = u.d;  // :573-575
    vd.d = v.d;  // :576-578

    // :582-587
    for (int i = ici1; i <= ici2; ++i)
      for (int j = jci1; j <= jci2; ++j) {
        double zuh = u(j, i, kz) * hx(j, i) + u(j + 1, i, kz) * hx(j + 1, i);
        double zvh = v(j, i, kz) * hy(j, i) + v(j, i + 1, kz) * hy(j, i + 1);
        s(j, i, kzp1) = -0.5 * (zuh + zvh);
        w(j, i, kzp1) = -s(j, i, kzp1);
      }
    // :591-597
#pragma omp parallel for
    for (int k = 2; k <= kz; ++k)
      for (int i = ici1; i <= ici2; ++i)
        for (int j = jci1; j <= jci2; ++j) {
          double zuh = (u(j, i, k) + u(j, i, k - 1)) * hx(j, i) +
                       (u(j + 1, i, k) + u(j + 1, i, k - 1)) * hx(j + 1, i);
          double zvh = (v(j, i, k) + v(j, i, k - 1)) * hy(j, i) +
                       (v(j, i + 1, k) + v(j, i + 1, k - 1)) * hy(j, i + 1);
          s(j, i, k) = -0.25 * (zuh + zvh) * gzitak[k];
        }
    // :602-618
#pragma omp parallel for
    for (int k = 1; k <= kz; ++k)
      for (int i = ice1; i <= ice2; ++i)
        for (int j = jce1; j <= jce2; ++j) {
          if (lrot) {
            double zum = dtrdx * u(j, i, k) * rfmzu(j, i, k);
            double zup = dtrdx * u(j + 1, i, k) * rfmzu(j + 1, i, k);
            double zvm = dtrdy * v(j, i, k) * rfmzv(j, i, k) * rmv(j, i);
            double zvp = dtrdy * v(j, i + 1, k) * rfmzv(j, i + 1, k) * rmv(j, i + 1);
            zdiv2(j, i, k) = fmz(j, i, k) * msfx(j, i) * ((zup - zum) + (zvp - zvm));
          } else {
            double zum = dtrdx * u(j, i, k) * rfmzu(j, i, k) * rmu(j, i);
            double zup = dtrdx * u(j + 1, i, k) * rfmzu(j + 1, i, k) * rmu(j + 1, i);
            double zvm = dtrdy * v(j, i, k) * rfmzv(j, i, k) * rmv(j, i);
            double zvp = dtrdy * v(j, i + 1, k) * rfmzv(j, i + 1, k) * rmv(j, i + 1);
            zdiv2(j, i, k) = fmz(j, i, k) * mx2(j, i) * ((zup - zum) + (zvp - zvm));
          }
        }
    if (prm.mo_divdamp) divergence_damping(dts);
    if (prm.mo_divfilter) divergence_diffusion();
    // :627-630
#pragma omp parallel for
    for (int k = 1; k <= kz; ++k)
      for (int i = ici1; i <= ici2; ++i)
        for (int j = jci1; j <= jci2; ++j)
          zdiv2(j, i, k) = zdiv2(j, i, k) +
                           bdywtw(j, i, k) * dtrdz * fmz(j, i, k) * (s(j, i, k) - s(j, i, k + 1));
    // :634-656 downward elimination
#pragma omp parallel for
    for (int i = ici1; i <= ici2; ++i)
      for (int j = jci1; j <= jci2; ++j)
        for (int k = kz; k >= 2; --k) {
          tetavf(j, i, k) = tetavf(j, i, k) -
                            w(j, i, k) * fmzf(j, i, k) * dtrdz * (tetav(j, i, k - 1) - tetav(j, i, k));
          double zrom1w = cpd * tetavf(j, i, k) * fmzf(j, i, k);
          double zwexpl = w(j, i, k) - zrom1w * dtrdz * (pai(j, i, k - 1) - pai(j, i, k)) - egrav * dts;
          zwexpl = zwexpl + rdrcv * zrom1w * dtrdz *
                                (pai(j, i, k - 1) * zdiv2(j, i, k - 1) - pai(j, i, k) * zdiv2(j, i, k));
          double zu = zcs2 * fmz(j, i, k - 1) * zrom1w * pai(j, i, k - 1) + ffilt[k];
          double zd = zcs2 * fmz(j, i, k) * zrom1w * pai(j, i, k) + ffilt[k];
          double zrapp = d_one / (d_one + zd + zu - zd * wwkw(j, i, k + 1));
          w(j, i, k) = zrapp * (zwexpl + zd * w(j, i, k + 1));
          wwkw(j, i, k) = zrapp * zu;
        }
    // :660-664 back substitution
#pragma omp parallel for
    for (int i = ici1; i <= ici2; ++i)
      for (int j = jci1; j <= jci2; ++j)
        for (int k = 2; k <= kz; ++k) w(j, i, k) = w(j, i, k) + wwkw(j, i, k) * w(j, i, k - 1);
    // :668-671
#pragma omp parallel for
    for (int k = 1; k <= kz; ++k)
      for (int i = ici1; i <= ici2; ++i)
        for (int j = jci1; j <= jci2; ++j)
          pai(j, i, k) = pai(j, i, k) *
                         (d_one - rdrcv * (zdiv2(j, i, k) +
                                           (dtrdz * fmz(j, i, k) * (w(j, i, k) - w(j, i, k + 1)))));
    // :677-721
    const double zfz = egrav * dts;
#pragma omp parallel for
    for (int k = 1; k <= kz; ++k)
      for (int i = ici1; i <= ici2; ++i)
        for (int j = jdi1; j <= jdi2; ++j) {
          double zcx = dtrdx * msfu(j, i);
          double zrom1u = 0.5 * cpd * (tetav(j - 1, i, k) + tetav(j, i, k));
          double zcor1u = coru(j, i) * dts * vd(j, i, k);
          u(j, i, k) = u(j, i, k) + bdywtu(j, i, k) * (zcor1u - zfz * hx(j, i) * gzitakh[k] -
                                                       zcx * zrom1u * (pai(j, i, k) - pai(j - 1, i, k)));
        }
#pragma omp parallel for
    for (int k = 1; k <= kz; ++k)
      for (int i = idi1; i <= idi2; ++i)
        for (int j = jci1; j <= jci2; ++j) {
          double zcy = lrot ? dtrdy : dtrdy * msfv(j, i);
          double zrom1v = 0.5 * cpd * (tetav(j, i - 1, k) + tetav(j, i, k));
          double zcor1v = corv(j, i) * dts * ud(j, i, k);
          v(j, i, k) = v(j, i, k) + bdywtv(j, i, k) * (-zcor1v - zfz * hy(j, i) * gzitakh[k] -
                                                       zcy * zrom1v * (pai(j, i, k) - pai(j, i - 1, k)));
        }
  }
  // :728-734
#pragma omp parallel for
  for (int k = 2; k <= kz; ++k)
    for (int i = ici1; i <= ici2; ++i)
      for (int j = jci1; j <= jci2; ++j) s(j, i, k) = (w(j, i, k) + s(j, i, k)) * fmzf(j, i, k);
  for (int i = ici1; i <= ici2; ++i)
    for (int j = jci1; j <= jci2; ++j) {
      s(j, i, 1) = 0.0;
      s(j, i, kzp1) = 0.0;
    }
}

// Main/mod_moloch.F90:738-765
void Oracle::divergence_damping(double dts) {
  const double dxrdt = dx / dts;
  const bool lrot = prm.lrotllr != 0;
#pragma omp parallel for
  for (int k = 1; k <= kz; ++k)
    for (int i = ici1; i <= ici2; ++i)
      for (int j = jdi1; j <= jdi2; ++j) {
        double xdam = dxrdt * xkdamp[k] * msfu(j, i);
        u(j, i, k) = u(j, i, k) + xdam * (zdiv2(j, i, k) - zdiv2(j - 1, i, k));
      }
#pragma omp parallel for
  for (int k = 1; k <= kz; ++k)
    for (int i = idi1; i <= idi2; ++i)
      for (int j = jci1; j <= jci2; ++j) {
        double xdam = lrot ? dxrdt * xkdamp[k] : dxrdt * xkdamp[k] * msfv(j, i);
        v(j, i, k) = v(j, i, k) + xdam * (zdiv2(j, i, k) - zdiv2(j, i - 1, k));
      }
}

// Main/mod_moloch.F90:767-836
void Oracle::advection(double dta) {
  uvstagtouvx();
  zstagtoh(w, wx);
  if (use_tke) zstagtoh(tke, tkex);
  wafone(tetav, dta);
  wafone(pai, dta);
  wafone(ux, dta);
  wafone(vx, dta);
  wafone(wx, dta);
  wafone(qx[0], dta);
  if (prm.ipptls > 0)
    for (int n = 1; n < nqx; ++n) wafone(qx[n], dta);  // iqfrst = iqc
  if (use_tke) wafone(tkex, dta);
  for (int n = 0; n < ntr; ++n) wafone(trac[n], dta);   // ichem = 1
  // curvature terms :809-825
  if (prm.lrotllr) {
    for (int k = 1; k <= kz; ++k)
      for (int i = ici1; i <= ici2; ++i)
        for (int j = jci1; j <= jci2; ++j) {
          double dlat = degrad * 0.5 * (rlat[i] + rlat[i + 1]);
          double tanx = std::sin(dlat) * msfx(j, i) * rearthrad;
          ux(j, i, k) = ux(j, i, k) + ux(j, i, k) * vx(j, i, k) * tanx * dta;
          vx(j, i, k) = vx(j, i, k) - ux(j, i, k) * ux(j, i, k) * tanx * dta;
        }
  } else {
#pragma omp parallel for
    for (int k = 1; k <= kz; ++k)
      for (int i = ici1; i <= ici2; ++i)
        for (int j = jci1; j <= jci2; ++j) {
          double tanx = (msfu(j - 1, i) - msfu(j, i)) * rdx;
          double tany = (msfv(j, i - 1) - msfv(j, i)) * rdx;
          ux(j, i, k) = ux(j, i, k) + ux(j, i, k) * vx(j, i, k) * tanx * dta;
          vx(j, i, k) = vx(j, i, k) - ux(j, i, k) * ux(j, i, k) * tany * dta;
        }
  }
  uvxtouvstag();
  htozstag(wx, w);
  if (use_tke) htozstag(tkex, tke);
}

// Main/mod_moloch.F90:838-1042 (do_vadvtwice = .true.)
void Oracle::wafone(F3 &pp, double dta) {
  const double wlow = 0.0, whigh = 2.0;
  const bool lrot = prm.lrotllr != 0;
  const double dtrdx = dta * rdx, dtrdy = dta * rdx;
  const double dtrdz = 0.5 * (dta * rdzita);

  auto vertical_pass = [&](const F3 &src, F3 &dst) {
    for (int i = ice1; i <= ice2; ++i)
      for (int j = jce1; j <= jce2; ++j) {
        wfw(j, i, 1) = 0.0;
        wfw(j, i, kzp1) = 0.0;
      }
#pragma omp parallel for
    for (int k = 1; k <= kzm1; ++k)
      for (int i = ice1; i <= ice2; ++i)
        for (int j = jce1; j <= jce2; ++j) {
          double zamu = s(j, i, k + 1) * dtrdz;
          double is;
          int k1, k1p1;
          if (zamu >= 0.0) {
            is = 1.0; k1 = k + 1; k1p1 = k1 + 1;
            if (k1p1 > kz) k1p1 = kz;
          } else {
            is = -1.0; k1 = k - 1; k1p1 = k;
            if (k1 < 1) k1 = 1;
          }
          double r = local_flow_param(src(j, i, k1) - src(j, i, k1p1), src(j, i, k) - src(j, i, k + 1));
          double b = fmax2(wlow, fmin2(whigh, fmax2(r, fmin2(2.0 * r, 1.0))));
          double zphi = is + zamu * b - is * b;
          wfw(j, i, k + 1) = 0.5 * s(j, i, k + 1) *
                             ((d_one + zphi) * src(j, i, k + 1) + (d_one - zphi) * src(j, i, k));
        }
#pragma omp parallel for
    for (int k = 1; k <= kz; ++k)
      for (int i = ice1; i <= ice2; ++i)
        for (int j = jce1; j <= jce2; ++j) {
          double zrfmu = dtrdz * fmz(j, i, k) / fmzf(j, i, k);
          double zrfmd = dtrdz * fmz(j, i, k) / fmzf(j, i, k + 1);
          double zdv = (s(j, i, k) * zrfmu - s(j, i, k + 1) * zrfmd) * src(j, i, k);
          dst(j, i, k) = src(j, i, k) - wfw(j, i, k) * zrfmu + wfw(j, i, k + 1) * zrfmd + zdv;
        }
  };
  vertical_pass(pp, wz);
  vertical_pass(wz, wz);  // :894-922 reads and writes wz (pointwise per level)

  // meridional flux :984-998 (or :926-940 for ROTLLR)
#pragma omp parallel for
  for (int k = 1; k <= kz; ++k)
    for (int i = ici1; i <= ice2; ++i)
      for (int j = jce1; j <= jce2; ++j) {
        double zamu = lrot ? v(j, i, k) * dtrdy : v(j, i, k) * msfv(j, i) * dtrdy;
        double is;
        int ih;
        if (zamu > 0.0) { is = 1.0; ih = i - 1; }
        else { is = -1.0; ih = std::min(i + 1, imax); }
        int ihm1 = std::max(ih - 1, imin);
        double r = local_flow_param(wz(j, ih, k) - wz(j, ihm1, k), wz(j, i, k) - wz(j, i - 1, k));
        double b = fmax2(wlow, fmin2(whigh, fmax2(r, fmin2(2.0 * r, 1.0))));
        double zphi = is + zamu * b - is * b;
        zpby(j, i, k) = 0.5 * v(j, i, k) * ((d_one + zphi) * wz(j, i - 1, k) + (d_one - zphi) * wz(j, i, k));
      }
#pragma omp parallel for
  for (int k = 1; k <= kz; ++k)
    for (int i = ici1; i <= ici2; ++i)
      for (int j = jce1; j <= jce2; ++j) {
        if (lrot) {
          double zhxvtn = dtrdy * rmv(j, i + 1) * msfx(j, i);
          double zhxvts = dtrdy * rmv(j, i) * msfx(j, i);
          double zrfmn = zhxvtn * fmz(j, i, k) * rfmzv(j, i + 1, k);
          double zrfms = zhxvts * fmz(j, i, k) * rfmzv(j, i, k);
          double zdv = (v(j, i + 1, k) * zrfmn - v(j, i, k) * zrfms) * pp(j, i, k);
          p0(j, i, k) = wz(j, i, k) + (zpby(j, i, k) * zrfms - zpby(j, i + 1, k) * zrfmn + zdv);
        } else {
          // the reference uses rfmzu here (Main/mod_moloch.F90:1000-1001)
          double zrfmn = dtrdy * fmz(j, i, k) * rfmzu(j, i + 1, k);
          double zrfms = dtrdy * fmz(j, i, k) * rfmzu(j, i, k);
          double zdv = (v(j, i + 1, k) * rmv(j, i + 1) * zrfmn - v(j, i, k) * rmv(j, i) * zrfms) * pp(j, i, k);
          p0(j, i, k) = wz(j, i, k) + mx2(j, i) * (zpby(j, i, k) * zrfms - zpby(j, i + 1, k) * zrfmn + zdv);
        }
      }
  // zonal flux :1015-1029 (or :957-971)
#pragma omp parallel for
  for (int k = 1; k <= kz; ++k)
    for (int i = ici1; i <= ici2; ++i)
      for (int j = jci1; j <= jce2; ++j) {
        double zamu = u(j, i, k) * msfu(j, i) * dtrdx;
        double is;
        int jh;
        if (zamu > 0.0) { is = 1.0; jh = j - 1; }
        else { is = -1.0; jh = std::min(j + 1, jmax); }
        int jhm1 = std::max(jh - 1, jmin);
        double r = local_flow_param(p0(jh, i, k) - p0(jhm1, i, k), p0(j, i, k) - p0(j - 1, i, k));
        double b = fmax2(wlow, fmin2(whigh, fmax2(r, fmin2(2.0 * r, 1.0))));
        double zphi = is + zamu * b - is * b;
        zpbw(j, i, k) = 0.5 * u(j, i, k) * ((d_one + zphi) * p0(j - 1, i, k) + (d_one - zphi) * p0(j, i, k));
      }
#pragma omp parallel for
  for (int k = 1; k <= kz; ++k)
    for (int i = ici1; i <= ici2; ++i)
      for (int j = jci1; j <= jci2; ++j) {
        if (lrot) {
          double zcostx = dtrdx * msfx(j, i);
          double zrfmw = zcostx * fmz(j, i, k) * rfmzu(j, i, k);
          double zrfme = zcostx * fmz(j, i, k) * rfmzu(j + 1, i, k);
          double zdv = (u(j + 1, i, k) * zrfme - u(j, i, k) * zrfmw) * pp(j, i, k);
          pp(j, i, k) = p0(j, i, k) + zpbw(j, i, k) * zrfmw - zpbw(j + 1, i, k) * zrfme + zdv;
        } else {
          double zrfmw = dtrdx * fmz(j, i, k) * rfmzu(j, i, k);
          double zrfme = dtrdx * fmz(j, i, k) * rfmzu(j + 1, i, k);
          double zdv = (u(j + 1, i, k) * rmu(j + 1, i) * zrfme - u(j, i, k) * rmu(j, i) * zrfmw) * pp(j, i, k);
          pp(j, i, k) = p0(j, i, k) + mx2(j, i) * (zpbw(j, i, k) * zrfmw - zpbw(j + 1, i, k) * zrfme + zdv);
        }
      }
}

// Main/mod_moloch.F90:1445-1459
void Oracle::zstagtoh(const F3 &fl, F3 &hl) {
  for (int k = 2; k <= kzm1; ++k)
    for (int i = ice1; i <= ice2; ++i)
      for (int j = jce1; j <= jce2; ++j)
        hl(j, i, k) = 0.5625 * (fl(j, i, k + 1) + fl(j, i, k)) - 0.0625 * (fl(j, i, k + 2) + fl(j, i, k - 1));
  for (int i = ice1; i <= ice2; ++i)
    for (int j = jce1; j <= jce2; ++j) {
      hl(j, i, 1) = 0.5 * (fl(j, i, 2) + fl(j, i, 1));
      hl(j, i, kz) = 0.5 * (fl(j, i, kzp1) + fl(j, i, kz));
    }
}

// Main/mod_moloch.F90:1461-1475
void Oracle::htozstag(const F3 &hl, F3 &fl) {
  for (int k = 3; k <= kzm1; ++k)
    for (int i = ice1; i <= ice2; ++i)
      for (int j = jce1; j <= jce2; ++j)
        fl(j, i, k) = 0.5625 * (hl(j, i, k) + hl(j, i, k - 1)) - 0.0625 * (hl(j, i, k + 1) + hl(j, i, k - 2));
  for (int i = ice1; i <= ice2; ++i)
    for (int j = jce1; j <= jce2; ++j) {
      fl(j, i, 2) = 0.5 * (hl(j, i, 2) + hl(j, i, 1));
      fl(j, i, kz) = 0.5 * (hl(j, i, kz) + hl(j, i, kzm1));
    }
}

// Main/mod_moloch.F90:1477-1522
void Oracle::uvxtouvstag() {
#pragma omp parallel for
  for (int k = 1; k <= kz; ++k)
    for (int i = ici1; i <= ici2; ++i)
      for (int j = jdii1; j <= jdii2; ++j)
        u(j, i, k) = 0.5625 * (ux(j, i, k) + ux(j - 1, i, k)) - 0.0625 * (ux(j + 1, i, k) + ux(j - 2, i, k));
  for (int k = 1; k <= kz; ++k)
    for (int i = ici1; i <= ici2; ++i) {
      u(jdi2, i, k) = 0.5 * (ux(jci2, i, k) + ux(jce2, i, k));
      u(jdi1, i, k) = 0.5 * (ux(jci1, i, k) + ux(jce1, i, k));
    }
#pragma omp parallel for
  for (int k = 1; k <= kz; ++k)
    for (int i = idii1; i <= idii2; ++i)
      for (int j = jci1; j <= jci2; ++j)
        v(j, i, k) = 0.5625 * (vx(j, i, k) + vx(j, i - 1, k)) - 0.0625 * (vx(j, i + 1, k) + vx(j, i - 2, k));
  for (int k = 1; k <= kz; ++k)
    for (int j = jci1; j <= jci2; ++j) {
      v(j, idi2, k) = 0.5 * (vx(j, ici2, k) + vx(j, ice2, k));
      v(j, idi1, k) = 0.5 * (vx(j, ici1, k) + vx(j, ice1, k));
    }
}

// Main/mod_moloch.F90:1524-1569
void Oracle::uvstagtouvx() {
#pragma omp parallel for
  for (int k = 1; k <= kz; ++k)
    for (int i = ice1; i <= ice2; ++i)
      for (int j = jci1; j <= jci2; ++j)
        ux(j, i, k) = 0.5625 * (u(j + 1, i, k) + u(j, i, k)) - 0.0625 * (u(j + 2, i, k) + u(j - 1, i, k));
  for (int k = 1; k <= kz; ++k)
    for (int i = ice1; i <= ice2; ++i) {
      ux(jce1, i, k) = 0.5 * (u(jde1, i, k) + u(jdi1, i, k));
      ux(jce2, i, k) = 0.5 * (u(jde2, i, k) + u(jdi2, i, k));
    }
#pragma omp parallel for
  for (int k = 1; k <= kz; ++k)
    for (int i = ici1; i <= ici2; ++i)
      for (int j = jce1; j <= jce2; ++j)
        vx(j, i, k) = 0.5625 * (v(j, i + 1, k) + v(j, i, k)) - 0.0625 * (v(j, i + 2, k) + v(j, i - 1, k));
  for (int k = 1; k <= kz; ++k)
    for (int j = jce1; j <= jce2; ++j) {
      vx(j, ice1, k) = 0.5 * (v(j, ide1, k) + v(j, idi1, k));
      vx(j, ice2, k) = 0.5 * (v(j, ide2, k) + v(j, idi2, k));
    }
}

// Main/mod_moloch.F90:1592-1606
void Oracle::extrapolate_surface_pressure() {
  for (int i = ici1; i <= ici2; ++i)
    for (int j = jci1; j <= jci2; ++j) {
      double lrt = (tvirt(j, i, kzm1) - tvirt(j, i, kz)) / (zeta(j, i, kzm1) - zeta(j, i, kz));
      if (lrt < -govcp) {
        lrt = -govcp;
      } else if (lrt > -0.005) {
        lrt = 0.65 * lrt - 0.35 * lrate;
      }
      double tv = tvirt(j, i, kz) - lrt * 0.5 * zeta(j, i, kz);
      ps(j, i) = p(j, i, kz) * std::exp(govr * zeta(j, i, kz) / tv);
    }
}

static inline double qfac(const std::vector<F3> &qx, int ipptls, int j, int i, int k) {
  if (ipptls > 1)
    return d_one + ep1 * qx[0](j, i, k) - qx[1](j, i, k) - qx[2](j, i, k) - qx[3](j, i, k) - qx[4](j, i, k);
  if (ipptls == 1) return d_one + ep1 * qx[0](j, i, k) - qx[1](j, i, k);
  return d_one + ep1 * qx[0](j, i, k);
}

// Main/mod_moloch.F90:1608-1627
void Oracle::temp_to_tvirt() {
#pragma omp parallel for
  for (int k = 1; k <= kz; ++k)
    for (int i = ice1; i <= ice2; ++i)
      for (int j = jce1; j <= jce2; ++j) tvirt(j, i, k) = t(j, i, k) * qfac(qx, prm.ipptls, j, i, k);
}

// Main/mod_moloch.F90:1629-1648
void Oracle::tvirt_to_temp() {
#pragma omp parallel for
  for (int k = 1; k <= kz; ++k)
    for (int i = ici1; i <= ici2; ++i)
      for (int j = jci1; j <= jci2; ++j) t(j, i, k) = tvirt(j, i, k) / qfac(qx, prm.ipptls, j, i, k);
}

// Main/mod_bdycod.F90:3844-3896 (serial: njcross = jx-1, nicross = iy-1,
// ds in km); cnudge comes with the static fields.
void Oracle::lowpass_init() {
  const double ds = dx / 1000.0;
  const int njcross = jx - 1, nicross = iy - 1;
  km = std::max((int)std::lround((njcross * ds) / 1500.0), 1);
  lm = std::max((int)std::lround((nicross * ds) / 750.0), 1);
  const double dxa = mathpi / (double)(njcross - 1);
  const double dya = mathpi / (double)(nicross - 1);
  std::vector<double> px(2 * km + 1), py(2 * lm + 1);
  for (int k = 1; k <= 2 * km; ++k) px[k] = std::exp(-std::pow((double)k / (double)km, 2));
  for (int l = 1; l <= 2 * lm; ++l) py[l] = std::exp(-std::pow((double)l / (double)lm, 2));
  bvx.init(jde1, jde2, 1, 2 * km);
  bvy.init(ide1, ide2, 1, 2 * lm);
  sx.init(ide1, ide2, 1, 2 * km);
  sy.init(jde1, jde2, 1, 2 * lm);
  zn1.init(jde1, jde2, ide1, ide2);
  const int jxm1 = jx - 1, iym1 = iy - 1;
  for (int k = 1; k <= 2 * km; ++k)
    for (int j = jde1; j <= jde2; ++j)
      bvx(j, k) = std::sqrt(2.0 / (double)jxm1 * px[k]) * std::sin(k * (j - 2) * dxa);
  for (int l = 1; l <= 2 * lm; ++l)
    for (int i = ide1; i <= ide2; ++i)
      bvy(i, l) = std::sqrt(2.0 / (double)iym1 * py[l]) * std::sin(l * (i - 2) * dya);
}

// Main/mod_bdycod.F90:3898-3938 (row_reduce/column_reduce: one process)
void Oracle::lowpass_filter(int j1, int j2, int i1, int i2, int jj1, int jj2, int ii1, int ii2,
                            F2<double> &f) {
  for (int k = 1; k <= 2 * km; ++k)
    for (int i = i1; i <= i2; ++i) {
      sx(i, k) = 0.0;
      for (int j = jj1; j <= jj2; ++j) sx(i, k) = sx(i, k) + f(j, i) * bvx(j, k);
    }
  std::fill(f.d.begin(), f.d.end(), 0.0);
  for (int k = 1; k <= 2 * km; ++k)
    for (int i = i1; i <= i2; ++i)
      for (int j = j1; j <= j2; ++j) f(j, i) = f(j, i) + sx(i, k) * bvx(j, k);
  for (int l = 1; l <= 2 * lm; ++l)
    for (int j = j1; j <= j2; ++j) {
      sy(j, l) = 0.0;
      for (int i = ii1; i <= ii2; ++i) sy(j, l) = sy(j, l) + f(j, i) * bvy(i, l);
    }
  std::fill(f.d.begin(), f.d.end(), 0.0);
  for (int l = 1; l <= 2 * lm; ++l)
    for (int i = i1; i <= i2; ++i)
      for (int j = j1; j <= j2; ++j) f(j, i) = f(j, i) + sy(j, l) * bvy(i, l);
}

// Main/mod_bdycod.F90:3940-3960
void Oracle::mospectral_nudge(int j1, int j2, int i1, int i2, int jj1, int jj2, int ii1, int ii2,
                              F3 &f, const F3 *bnd) {
  const double x1 = (xbctime + dt) * rtb;
  const double x0 = 1.0 - x1;
  for (int k = 1; k <= kz; ++k) {
    for (int i = i1; i <= i2; ++i)
      for (int j = j1; j <= j2; ++j)
        zn1(j, i) = (x0 * bnd[0](j, i, k) + x1 * bnd[1](j, i, k)) - f(j, i, k);
    lowpass_filter(j1, j2, i1, i2, jj1, jj2, ii1, ii2, zn1);
    for (int i = ii1; i <= ii2; ++i)
      for (int j = jj1; j <= jj2; ++j) f(j, i, k) = f(j, i, k) + cnudge[k] * zn1(j, i);
  }
}

// Main/mod_moloch.F90:448-529 (diagnostics left out)
void Oracle::boundary() {
  bdyval();
  if (prm.mo_top_nudge) motopnudge(0.0, dtsec);
  morelax_external(jdi1, jdi2, ici1, ici2, ibnd_ud, hb_ud, u, dub);
  morelax_external(jci1, jci2, idi1, idi2, ibnd_vd, hb_vd, v, dvb);
  morelax_external(jci1, jci2, ici1, ici2, ibnd_cr, hb_cr, t, xtb);
  morelax_external(jci1, jci2, ici1, ici2, ibnd_cr, hb_cr, pai, xpaib);
  morelax_external(jci1, jci2, ici1, ici2, ibnd_cr, hb_cr, qx[0], xqb);
  morelax_fraction(jci1, jci2, ici1, ici2, ibnd_cr, hb_cr, w, 0.0);
  if (prm.ipptls > 0) {
    if (prm.present_qc) morelax_external(jci1, jci2, ici1, ici2, ibnd_cr, hb_cr, qx[1], xlb);
    if (prm.ipptls > 1 && prm.present_qi)
      morelax_external(jci1, jci2, ici1, ici2, ibnd_cr, hb_cr, qx[2], xib);
  }
  if (ntr > 0) morelax_chiten();
  if (prm.mo_spectral_nudge) {
    // Main/mod_moloch.F90:499-506; the temperature call sums its x
    // projection over jci1..jci1 only, as the reference passes it
    tspectral = tspectral + dtsec;
    if ((int)std::fmod(tspectral, prm.dtrad) == 0) {
      mospectral_nudge(jce1, jce2, ice1, ice2, jci1, jci1, ici1, ici2, t, xtb);
      mospectral_nudge(jde1, jde2, ice1, ice2, jdi1, jdi2, ici1, ici2, u, dub);
      mospectral_nudge(jce1, jce2, ide1, ide2, jci1, jci2, idi1, idi2, v, dvb);
    }
  }
  uvstagtouvx();
  temp_to_tvirt();
  for (int k = 1; k <= kz; ++k)
    for (int i = ice1; i <= ice2; ++i)
      for (int j = jce1; j <= jce2; ++j) tetav(j, i, k) = tvirt(j, i, k) / pai(j, i, k);
}

// Main/mod_bdycod.F90:1618-1875 (MOLOCH branch), 2653 (clock);
// tracer ring: Main/chemlib/mod_che_bdyco.F90:487-532 (time-dependent data)
void Oracle::bdyval() {
  const double x1 = (xbctime + dt) * rtb;
  const double x0 = 1.0 - x1;
  const int iqc = 1, iqi = 2;  // 0-based species
  auto skip = [&](int n) {
    return (prm.present_qc && n == iqc) || (prm.present_qi && n == iqi);
  };
  auto blend = [&](const F3 *b, int j, int i, int k) { return x0 * b[0](j, i, k) + x1 * b[1](j, i, k); };
  // west and east: corners excluded
  for (int side = 0; side < 2; ++side) {
    const int jb = side == 0 ? jce1 : jce2;      // cross column
    const int jd = side == 0 ? jde1 : jde2;      // dot column
    const int jin = side == 0 ? jci1 : jci2;     // interior neighbour
    for (int i = ici1; i <= ici2; ++i) ps(jb, i) = x0 * xpsb[0](jb, i) + x1 * xpsb[1](jb, i);
    for (int k = 1; k <= kz; ++k)
      for (int i = ici1; i <= ici2; ++i) u(jd, i, k) = blend(dub, jd, i, k);
    for (int k = 1; k <= kz; ++k)
      for (int i = idi1; i <= idi2; ++i) v(jb, i, k) = blend(dvb, jb, i, k);
    for (int k = 1; k <= kz; ++k)
      for (int i = ici1; i <= ici2; ++i) {
        t(jb, i, k) = blend(xtb, jb, i, k);
        pai(jb, i, k) = blend(xpaib, jb, i, k);
        qx[0](jb, i, k) = blend(xqb, jb, i, k);
      }
    if (prm.present_qc)
      for (int k = 1; k <= kz; ++k)
        for (int i = ici1; i <= ici2; ++i) qx[iqc](jb, i, k) = blend(xlb, jb, i, k);
    if (prm.present_qi && prm.ipptls > 1)
      for (int k = 1; k <= kz; ++k)
        for (int i = ici1; i <= ici2; ++i) qx[iqi](jb, i, k) = blend(xib, jb, i, k);
    for (int n = 1; n < nqx; ++n) {
      if (skip(n)) continue;
      for (int k = 1; k <= kz; ++k)
        for (int i = ici1; i <= ici2; ++i) {
          double qxint = qx[n](jin, i, k);
          bool inflow = side == 0 ? (u(jd, i, k) > 0.0) : (u(jd, i, k) < 0.0);
          qx[n](jb, i, k) = inflow ? qxzeroval[n] : qxint;
        }
    }
    for (int k = 1; k <= kz; ++k)
      for (int i = ici1; i <= ici2; ++i) {
        bool inflow = side == 0 ? (u(jd, i, k) > 0.0) : (u(jd, i, k) < 0.0);
        w(jb, i, k) = inflow ? 0.0 : w(jin, i, k);
      }
    if (use_tke) {  // :1684-1695, :1742-1753
      for (int i = ici1; i <= ici2; ++i) tke(jb, i, 1) = tkemin;
      for (int k = 2; k <= kz; ++k)
        for (int i = ici1; i <= ici2; ++i) {
          double us = u(jd, i, k) + u(jd, i, k - 1);
          bool inflow = side == 0 ? (us > 0.0) : (us < 0.0);
          tke(jb, i, k + 1) = inflow ? tkemin : tke(jin, i, k + 1);
        }
    }
  }
  // south and north: corners included
  for (int side = 0; side < 2; ++side) {
    const int ib = side == 0 ? ice1 : ice2;
    const int id = side == 0 ? ide1 : ide2;
    const int iin = side == 0 ? ici1 : ici2;
    for (int j = jce1; j <= jce2; ++j) ps(j, ib) = x0 * xpsb[0](j, ib) + x1 * xpsb[1](j, ib);
    for (int k = 1; k <= kz; ++k)
      for (int j = jde1; j <= jde2; ++j) u(j, ib, k) = blend(dub, j, ib, k);
    for (int k = 1; k <= kz; ++k)
      for (int j = jce1; j <= jce2; ++j) v(j, id, k) = blend(dvb, j, id, k);
    for (int k = 1; k <= kz; ++k)
      for (int j = jce1; j <= jce2; ++j) {
        t(j, ib, k) = blend(xtb, j, ib, k);
        pai(j, ib, k) = blend(xpaib, j, ib, k);
        qx[0](j, ib, k) = blend(xqb, j, ib, k);
      }
    if (prm.present_qc)
      for (int k = 1; k <= kz; ++k)
        for (int j = jce1; j <= jce2; ++j) qx[iqc](j, ib, k) = blend(xlb, j, ib, k);
    if (prm.present_qi && prm.ipptls > 1)
      for (int k = 1; k <= kz; ++k)
        for (int j = jce1; j <= jce2; ++j) qx[iqi](j, ib, k) = blend(xib, j, ib, k);
    for (int n = 1; n < nqx; ++n) {
      if (skip(n)) continue;
      for (int k = 1; k <= kz; ++k)
        for (int j = jce1; j <= jce2; ++j) {
          double qxint = qx[n](j, iin, k);
          bool inflow = side == 0 ? (v(j, id, k) > 0.0) : (v(j, id, k) < 0.0);
          qx[n](j, ib, k) = inflow ? qxzeroval[n] : qxint;
        }
    }
    for (int k = 1; k <= kz; ++k)
      for (int j = jce1; j <= jce2; ++j) {
        bool inflow = side == 0 ? (v(j, id, k) > 0.0) : (v(j, id, k) < 0.0);
        w(j, ib, k) = inflow ? 0.0 : w(j, iin, k);
      }
    if (use_tke) {  // :1800-1811, :1858-1869
      for (int j = jce1; j <= jce2; ++j) tke(j, ib, 1) = tkemin;
      for (int k = 2; k <= kz; ++k)
        for (int j = jce1; j <= jce2; ++j) {
          double vs = v(j, id, k) + v(j, id, k - 1);
          bool inflow = side == 0 ? (vs > 0.0) : (vs < 0.0);
          tke(j, ib, k + 1) = inflow ? tkemin : tke(j, iin, k + 1);
        }
    }
  }
  if (ntr > 0) {
    // chem_bdyval_uncoupled, time-dependent data: x1 = (xbctime + dt)/dtbdys
    const double cx1 = (xbctime + dt) / dtbdys;
    const double cx0 = 1.0 - cx1;
    for (int n = 0; n < ntr; ++n) {
      for (int k = 1; k <= kz; ++k)
        for (int i = ici1; i <= ici2; ++i) {
          trac[n](jce1, i, k) = cx0 * chib[0][n](jce1, i, k) + cx1 * chib[1][n](jce1, i, k);
          trac[n](jce2, i, k) = cx0 * chib[0][n](jce2, i, k) + cx1 * chib[1][n](jce2, i, k);
        }
      for (int k = 1; k <= kz; ++k)
        for (int j = jce1; j <= jce2; ++j) {
          trac[n](j, ice1, k) = cx0 * chib[0][n](j, ice1, k) + cx1 * chib[1][n](j, ice1, k);
          trac[n](j, ice2, k) = cx0 * chib[0][n](j, ice2, k) + cx1 * chib[1][n](j, ice2, k);
        }
    }
  }
  xbctime = xbctime + dtsec;
}

// Main/mod_bdycod.F90:4049-4083
void Oracle::motopnudge(double wfac, double dta) {
  const double trtau = 1.0 / (2.0 * 3600.0);
  const double wrtau = 1.0 / (3600.0 / 4.0);
  const double x1 = (xbctime + dt) * rtb;
  const double x0 = 1.0 - x1;
  const int nztop = prm.nztop;
  for (int i = ici1; i <= ici2; ++i)
    for (int j = jci1; j <= jci2; ++j) {
      double fext = wfac * w(j, i, 2);
      double xf = wrtau * dta;
      w(j, i, 2) = (1.0 - xf) * w(j, i, 2) + xf * fext;
    }
  for (int k = 1; k <= nztop; ++k)
    for (int i = ici1; i <= ici2; ++i)
      for (int j = jci1; j <= jci2; ++j) {
        double fext = x0 * xtb[0](j, i, k) + x1 * xtb[1](j, i, k);
        double xf = tnudge[k] * trtau * dta;
        t(j, i, k) = (1.0 - xf) * t(j, i, k) + xf * fext;
      }
  for (int k = 1; k <= nztop; ++k)
    for (int i = ici1; i <= ici2; ++i)
      for (int j = jdi1; j <= jdi2; ++j) {
        double fext = x0 * dub[0](j, i, k) + x1 * dub[1](j, i, k);
        double xf = tnudge[k] * trtau * dta;
        u(j, i, k) = (1.0 - xf) * u(j, i, k) + xf * fext;
      }
  for (int k = 1; k <= nztop; ++k)
    for (int i = idi1; i <= idi2; ++i)
      for (int j = jci1; j <= jci2; ++j) {
        double fext = x0 * dvb[0](j, i, k) + x1 * dvb[1](j, i, k);
        double xf = tnudge[k] * trtau * dta;
        v(j, i, k) = (1.0 - xf) * v(j, i, k) + xf * fext;
      }
}

// Main/mod_bdycod.F90:3995-4031
void Oracle::morelax_external(int j1, int j2, int i1, int i2, const F2<int32_t> &ibnd, bool hb,
                              F3 &f, const F3 *bnd) {
  if (!hb) return;
  const double x1 = (xbctime + dt) * rtb;
  const double x0 = 1.0 - x1;
  for (int k = 1; k <= kz; ++k)
    for (int i = i1; i <= i2; ++i)
      for (int j = j1; j <= j2; ++j) {
        int ib = ibnd(j, i);
        if (ib > 0) {
          double xf = hefc(ib, k);
          double fext = (x0 * bnd[0](j, i, k) + x1 * bnd[1](j, i, k));
          f(j, i, k) = (1.0 - xf) * f(j, i, k) + xf * fext;
        }
      }
}

// Main/mod_bdycod.F90:3962-3993
void Oracle::morelax_fraction(int j1, int j2, int i1, int i2, const F2<int32_t> &ibnd, bool hb,
                              F3 &f, double frac) {
  if (!hb) return;
  for (int k = 1; k <= kz; ++k)
    for (int i = i1; i <= i2; ++i)
      for (int j = j1; j <= j2; ++j) {
        int ib = ibnd(j, i);
        if (ib > 0) {
          double xf = hefc(ib, k);
          f(j, i, k) = (1.0 - xf) * f(j, i, k) + xf * f(j, i, k) * frac;
        }
      }
}

// Main/chemlib/mod_che_bdyco.F90:965-1026 with cba = ba_cr
// (Main/mod_che_interface.F90:162-173); the south/north/west/east masks are
// disjoint on the domains this library accepts, so one pass suffices.
void Oracle::morelax_chiten() {
  if (!hb_cr) return;
  const double x1 = (xbctime + dt) / dtbdys;
  const double x0 = 1.0 - x1;
  for (int n = 0; n < ntr; ++n)
    for (int k = 1; k <= kz; ++k)
      for (int i = ici1; i <= ici2; ++i)
        for (int j = jci1; j <= jci2; ++j) {
          int ib = ibnd_cr(j, i);
          if (ib > 0) {
            double xf = fcx[ib];
            double fext = (x0 * chib[0][n](j, i, k) + x1 * chib[1][n](j, i, k));
            trac[n](j, i, k) = (1.0 - xf) * trac[n](j, i, k) + xf * fext;
          }
        }
}

// Main/mod_slice.F90:110-147 (idynamic = 3): the edits mkslice makes to the
// MOLOCH state through its atms pointers (qxb3d => qx, chib3d => trac).  The
// fields it derives for the physics (pf3d, th3d, rhb3d, ...) are not state.
void Oracle::mkslice() {
  for (int n = 0; n < nqx; ++n)
    for (int k = 1; k <= kz; ++k)
      for (int i = ici1; i <= ici2; ++i)
        for (int j = jci1; j <= jci2; ++j)
          if (qx[n](j, i, k) < qxcheckval[n]) qx[n](j, i, k) = qxzeroval[n];
  for (int n = 0; n < ntr; ++n)
    for (int k = 1; k <= kz; ++k)
      for (int i = ici1; i <= ici2; ++i)
        for (int j = jci1; j <= jci2; ++j)
          if (trac[n](j, i, k) < 1.0e-50) trac[n](j, i, k) = 0.0;
}

// Main/mod_moloch.F90:1403-1443
void Oracle::status_update(double dtinc) {
  for (int k = 1; k <= kz; ++k)
    for (int i = ici1; i <= ici2; ++i)
      for (int j = jci1; j <= jci2; ++j) {
        t(j, i, k) = t(j, i, k) + dtinc * tten(j, i, k);
        ux(j, i, k) = ux(j, i, k) + dtinc * uten(j, i, k);
        vx(j, i, k) = vx(j, i, k) + dtinc * vten(j, i, k);
      }
  for (int n = 0; n < nqx; ++n)
    for (int k = 1; k <= kz; ++k)
      for (int i = ici1; i <= ici2; ++i)
        for (int j = jci1; j <= jci2; ++j) {
          qx[n](j, i, k) = qx[n](j, i, k) + dtinc * qxten[n](j, i, k);
          if (qx[n](j, i, k) < qxcheckval[n]) qx[n](j, i, k) = qxzeroval[n];
        }
  if (use_tke)
    for (int k = 1; k <= kzp1; ++k)
      for (int i = ici1; i <= ici2; ++i)
        for (int j = jci1; j <= jci2; ++j) {
          tke(j, i, k) = tke(j, i, k) + dtinc * tketen(j, i, k);
          if (tke(j, i, k) < tkemin) tke(j, i, k) = tkemin;
        }
  for (int n = 0; n < ntr; ++n)
    for (int k = 1; k <= kz; ++k)
      for (int i = ici1; i <= ici2; ++i)
        for (int j = jci1; j <= jci2; ++j) {
          trac[n](j, i, k) = trac[n](j, i, k) + dtinc * chiten[n](j, i, k);
          if (trac[n](j, i, k) < 0.0) trac[n](j, i, k) = 0.0;
        }
  temp_to_tvirt();
#pragma omp parallel for
  for (int k = 1; k <= kz; ++k)
    for (int i = ice1; i <= ice2; ++i)
      for (int j = jce1; j <= jce2; ++j) {
        tetav(j, i, k) = tvirt(j, i, k) / pai(j, i, k);
        rho(j, i, k) = p(j, i, k) / (rgas * t(j, i, k));
        qsat(j, i, k) = pfwsat(t(j, i, k), p(j, i, k));
      }
  uvxtouvstag();
}

// Main/mod_massck.F90:57-200 (MOLOCH branch; precipitation and evaporation
// are zero without physics)
void Oracle::massck(mlc_diag *dg) {
  const double dxsq = dx * dx;
  double tdrym = 0.0, tdadv = 0.0, tqmass = 0.0, tqadv = 0.0;
  for (int k = 1; k <= kz; ++k)
    for (int i = ici1; i <= ici2; ++i)
      for (int j = jci1; j <= jci2; ++j) tdrym = tdrym + dxsq * dz(j, i, k) * rho(j, i, k);
  for (int k = 1; k <= kz; ++k)
    for (int i = ice1; i <= ice2; ++i)
      tdadv = tdadv + u(jde1, i, k) * dt * dx * dz(jce1, i, k) * rho(jce1, i, k);
  for (int k = 1; k <= kz; ++k)
    for (int i = ice1; i <= ice2; ++i)
      tdadv = tdadv - u(jde2, i, k) * dt * dx * dz(jce2, i, k) * rho(jce2, i, k);
  for (int k = 1; k <= kz; ++k)
    for (int j = jci1; j <= jci2; ++j)
      tdadv = tdadv + v(j, ide1, k) * dt * dx * dz(j, ice1, k) * rho(j, ice1, k);
  for (int k = 1; k <= kz; ++k)
    for (int j = jci1; j <= jci2; ++j)
      tdadv = tdadv - v(j, ide2, k) * dt * dx * dz(j, ice2, k) * rho(j, ice2, k);
  for (int n = 0; n < nqx; ++n) {
    for (int k = 1; k <= kz; ++k)
      for (int i = ici1; i <= ici2; ++i)
        for (int j = jci1; j <= jci2; ++j)
          tqmass = tqmass + qx[n](j, i, k) * dxsq * dz(j, i, k) * rho(j, i, k);
    for (int k = 1; k <= kz; ++k)
      for (int i = ice1; i <= ice2; ++i)
        tqadv = tqadv + qx[n](jce1, i, k) * u(jde1, i, k) * dt * dx * dz(jce1, i, k) * rho(jce1, i, k);
    for (int k = 1; k <= kz; ++k)
      for (int i = ice1; i <= ice2; ++i)
        tqadv = tqadv - qx[n](jce2, i, k) * u(jde2, i, k) * dt * dx * dz(jce2, i, k) * rho(jce2, i, k);
    for (int k = 1; k <= kz; ++k)
      for (int j = jci1; j <= jci2; ++j)
        tqadv = tqadv + qx[n](j, ice1, k) * v(j, ide1, k) * dt * dx * dz(j, ice1, k) * rho(j, ice1, k);
    for (int k = 1; k <= kz; ++k)
      for (int j = jci1; j <= jci2; ++j)
        tqadv = tqadv - qx[n](j, ice2, k) * v(j, ide2, k) * dt * dx * dz(j, ice2, k) * rho(j, ice2, k);
  }
  if (dg) { dg->drymass = tdrym; dg->dryadv = tdadv; dg->qmass = tqmass; dg->qadv = tqadv; }
}

}  // namespace orc

// ------------------------------------------------------------- C API ----
using orc::Oracle;

extern "C" {

void *orc_create(const mlc_dims *d, const mlc_params *p) {
  auto o = std::make_unique<Oracle>();
  if (o->create(d, p) != MLC_OK) return nullptr;
  return o.release();
}

void orc_destroy(void *h) { delete static_cast<Oracle *>(h); }

int orc_bind_static(void *h, const mlc_static_ptrs *s) {
  return static_cast<Oracle *>(h)->bind_static(s);
}

int orc_set_state(void *h, const mlc_state_ptrs *st) {
  Oracle &o = *static_cast<Oracle *>(h);
  o.u.load(st->u); o.v.load(st->v); o.w.load(st->w); o.pai.load(st->pai);
  o.tetav.load(st->tetav); o.t.load(st->t); o.tvirt.load(st->tvirt);
  o.ux.load(st->ux); o.vx.load(st->vx); o.p.load(st->p); o.rho.load(st->rho);
  o.qsat.load(st->qsat);
  size_t n3 = o.pai.d.size();
  for (int n = 0; n < o.nqx; ++n) o.qx[n].load(st->qx + n * n3);
  for (int n = 0; n < o.ntr; ++n) o.trac[n].load(st->trac + n * n3);
  std::memcpy(o.ps.d.data(), st->ps, o.ps.d.size() * sizeof(double));
  if (o.use_tke && st->tke) o.tke.load(st->tke);
  // init_moloch: w(:,:,1) = 0 (Main/mod_moloch.F90:264-266)
  for (int i = o.ice1; i <= o.ice2; ++i)
    for (int j = o.jce1; j <= o.jce2; ++j) o.w(j, i, 1) = 0.0;
  o.have_state = true;
  return MLC_OK;
}

int orc_get_state(void *h, const mlc_state_ptrs *st) {
  Oracle &o = *static_cast<Oracle *>(h);
  auto put = [](const orc::F3 &f, double *dst) { if (dst) f.store(dst); };
  put(o.u, st->u); put(o.v, st->v); put(o.w, st->w); put(o.pai, st->pai);
  put(o.tetav, st->tetav); put(o.t, st->t); put(o.tvirt, st->tvirt);
  put(o.ux, st->ux); put(o.vx, st->vx); put(o.p, st->p); put(o.rho, st->rho);
  put(o.qsat, st->qsat);
  size_t n3 = o.pai.d.size();
  if (st->qx) for (int n = 0; n < o.nqx; ++n) o.qx[n].store(st->qx + n * n3);
  if (st->trac) for (int n = 0; n < o.ntr; ++n) o.trac[n].store(st->trac + n * n3);
  if (st->ps) std::memcpy(st->ps, o.ps.d.data(), o.ps.d.size() * sizeof(double));
  if (o.use_tke && st->tke) o.tke.store(st->tke);
  return MLC_OK;
}

int orc_set_boundary(void *h, const mlc_bdy_ptrs *b, double xbctime, double dtbdys) {
  Oracle &o = *static_cast<Oracle *>(h);
  size_t n3 = o.pai.d.size();
  for (int s = 0; s < 2; ++s) {
    o.xtb[s].load(b->xtb[s]); o.xqb[s].load(b->xqb[s]); o.xpaib[s].load(b->xpaib[s]);
    if (b->xlb[s]) o.xlb[s].load(b->xlb[s]);
    if (b->xib[s]) o.xib[s].load(b->xib[s]);
    o.dub[s].load(b->dub[s]); o.dvb[s].load(b->dvb[s]);
    std::memcpy(o.xpsb[s].d.data(), b->xpsb[s], o.xpsb[s].d.size() * sizeof(double));
    for (int n = 0; n < o.ntr; ++n) o.chib[s][n].load(b->chib[s] + n * n3);
  }
  o.xbctime = xbctime;
  o.dtbdys = dtbdys;
  o.rtb = 1.0 / dtbdys;  // setup_bdycon, Main/mod_bdycod.F90:505
  o.have_bdy = true;
  return MLC_OK;
}

int orc_step(void *h, int nsteps, mlc_diag *dg) {
  Oracle &o = *static_cast<Oracle *>(h);
  if (!o.have_static || !o.have_state || (o.prm.do_apply_bdy && !o.have_bdy) || o.step_open)
    return MLC_ERR_STATE;
  mlc_diag tmp{};
  for (int n = 0; n < nsteps; ++n) {
    o.moloch(&tmp);
    tmp.steps_done = n + 1;
    if (tmp.nonfinite) break;
  }
  tmp.xbctime = o.xbctime;
  if (dg) *dg = tmp;
  return tmp.nonfinite ? MLC_ERR_NONFINITE : MLC_OK;
}

// The step split around the physics: the dynamics through mkslice, then
// (after orc_set_tendencies) status_update, mass check and ps check.
int orc_step_dynamics(void *h) {
  Oracle &o = *static_cast<Oracle *>(h);
  if (!o.have_static || !o.have_state || (o.prm.do_apply_bdy && !o.have_bdy) || o.step_open)
    return MLC_ERR_STATE;
  o.moloch_dynamics();
  o.step_open = true;
  return MLC_OK;
}

int orc_set_tendencies(void *h, const mlc_tend_ptrs *tp) {
  Oracle &o = *static_cast<Oracle *>(h);
  if (!o.step_open || !tp) return MLC_ERR_STATE;
  const size_t n3 = o.tten.d.size();
  if (tp->tten) o.tten.load(tp->tten);
  if (tp->uten) o.uten.load(tp->uten);
  if (tp->vten) o.vten.load(tp->vten);
  if (tp->qxten) for (int n = 0; n < o.nqx; ++n) o.qxten[n].load(tp->qxten + n * n3);
  if (tp->chiten) for (int n = 0; n < o.ntr; ++n) o.chiten[n].load(tp->chiten + n * n3);
  if (o.use_tke && tp->tketen) o.tketen.load(tp->tketen);
  return MLC_OK;
}

int orc_step_finish(void *h, mlc_diag *dg) {
  Oracle &o = *static_cast<Oracle *>(h);
  if (!o.step_open) return MLC_ERR_STATE;
  mlc_diag tmp{};
  o.moloch_finish(&tmp);
  o.step_open = false;
  tmp.steps_done = 1;
  tmp.xbctime = o.xbctime;
  if (dg) *dg = tmp;
  return tmp.nonfinite ? MLC_ERR_NONFINITE : MLC_OK;
}

// The restart state of Main/mod_init.F90:421-450 (copies from the SAV
// fields) and :941-960 (p, qs, rho, tvirt with qv only, tetav), loop by loop
// over jce x ice; ux and vx stay zero as getmem leaves them.
int orc_restart_state(const mlc_dims *d, const mlc_sav_fields *f, const mlc_state_ptrs *st) {
  const size_t jx = d->jx, iy = d->iy, kz = d->kz;
  const size_t nj = jx - 1, ni = iy - 1;
  std::memcpy(st->u, f->u, jx * ni * kz * sizeof(double));
  std::memcpy(st->v, f->v, nj * iy * kz * sizeof(double));
  std::memcpy(st->w, f->w, nj * ni * (kz + 1) * sizeof(double));
  std::memcpy(st->t, f->t, nj * ni * kz * sizeof(double));
  std::memcpy(st->pai, f->pai, nj * ni * kz * sizeof(double));
  std::memcpy(st->qx, f->qx, nj * ni * kz * d->nqx * sizeof(double));
  if (d->ntr > 0) std::memcpy(st->trac, f->trac, nj * ni * kz * d->ntr * sizeof(double));
  if (f->tke && st->tke) std::memcpy(st->tke, f->tke, nj * ni * (kz + 1) * sizeof(double));
  std::memcpy(st->ps, f->ps, nj * ni * sizeof(double));
  for (size_t k = 0; k < kz; ++k)
    for (size_t i = 0; i < ni; ++i)
      for (size_t j = 0; j < nj; ++j) {
        const size_t e = j + nj * (i + ni * k);
        st->p[e] = std::pow(st->pai[e], orc::cpovr) * orc::p00;
      }
  for (size_t k = 0; k < kz; ++k)
    for (size_t i = 0; i < ni; ++i)
      for (size_t j = 0; j < nj; ++j) {
        const size_t e = j + nj * (i + ni * k);
        st->qsat[e] = orc::pfwsat(st->t[e], st->p[e]);
        st->rho[e] = st->p[e] / (orc::rgas * st->t[e]);
      }
  for (size_t k = 0; k < kz; ++k)
    for (size_t i = 0; i < ni; ++i)
      for (size_t j = 0; j < nj; ++j) {
        const size_t e = j + nj * (i + ni * k);
        st->tvirt[e] = st->t[e] * (1.0 + orc::ep1 * st->qx[e]);
        st->tetav[e] = st->tvirt[e] / st->pai[e];
      }
  std::memset(st->ux, 0, nj * ni * kz * sizeof(double));
  std::memset(st->vx, 0, nj * ni * kz * sizeof(double));
  return MLC_OK;
}

// One call of sound(dtsound) alone, for substep-level parity tests.
int orc_sound_only(void *h) {
  Oracle &o = *static_cast<Oracle *>(h);
  o.reset_tendencies();
  o.sound(o.dtsound);
  return MLC_OK;
}

// pfwsat elementwise over n points (Share/pfwsat.inc:1-43), for building
// synthetic inputs without the library.
int orc_pfwsat(size_t n, const double *t, const double *p, double *qs) {
  for (size_t m = 0; m < n; ++m) qs[m] = orc::pfwsat(t[m], p[m]);
  return MLC_OK;
}

// Threads of the OpenMP loops (the 1-core and all-cores CPU baselines).
int orc_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : 1);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

// Copy a work array out: 0 = s, 1 = zdiv2, 2 = tetavf.
int orc_get_work(void *h, int which, double *dst) {
  Oracle &o = *static_cast<Oracle *>(h);
  const orc::F3 *f = which == 0 ? &o.s : which == 1 ? &o.zdiv2 : which == 2 ? &o.tetavf : nullptr;
  if (!f) return MLC_ERR_INVALID;
  f->store(dst);
  return MLC_OK;
}

}  // extern "C"
