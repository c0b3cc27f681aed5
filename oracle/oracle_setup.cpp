// oracle_setup.cpp -- TEST INFRASTRUCTURE ONLY.
//
// The oracle's own restatement of RegCM's MOLOCH setup routines, written
// against Fortran-bounded arrays, to check the library's host setup helpers
// bit for bit:
//   Share/mod_zita.F90:54-150           levels, G, b, metric factors
//   Main/mod_params.F90:3316-3395        compute_moloch_static
//   Main/mpplib/mod_runparams.F90:648-702 relax_coefficients
//   Main/mod_bdycod.F90:478-560          setup_bdycon (MOLOCH, Lehmann)
//   Main/mod_init.F90:1008-1025          sponge ffilt
//   Main/mod_atm_interface.F90:384-545   setup_boundaries
//   Main/mod_bdycod.F90:3762-3796        paicompute
#include "oracle_common.h"
#include "../include/moloch_gb300.h"

namespace orc {

// model_zitaf / model_zitah (Share/mod_zita.F90:54-86), as orc_setup_levels
static void orc_setup_levels_(int kz, double ztop, double *zitaf_out, double *zitah_out) {
  std::vector<double> zitaf(kz + 2), zitah(kz + 1);
  double dz = ztop / (double)kz;
  zitaf[kz + 1] = 0.0;
  zitaf[1] = ztop;
  for (int k = kz; k >= 2; --k) zitaf[k] = zitaf[k + 1] + dz;
  zitah[kz] = dz * 0.5;
  zitah[1] = ztop - dz * 0.5;
  for (int k = kz - 1; k >= 2; --k) zitah[k] = zitah[k + 1] + dz;
  for (int k = 1; k <= kz + 1; ++k) zitaf_out[k - 1] = zitaf[k];
  for (int k = 1; k <= kz; ++k) zitah_out[k - 1] = zitah[k];
}

static double zfz(double ztop, double zh) { return ztop / (std::exp(ztop / zh) - 1.0); }
static double bzita(double zita, double ztop, double zh) { return zfz(ztop, zh) * (std::exp(zita / zh) - 1.0); }
static double bzitap(double zita, double ztop, double zh) { return zfz(ztop, zh) * std::exp(zita / zh) / zh; }
static double gzita_(double zita, double ztop, double a0) {
  double ratio = zita / ztop;
  return ((0.0 - 1.0 * a0) * ratio - (3.0 - 2.0 * a0) * (ratio * ratio) +
          (2.0 - 1.0 * a0) * (ratio * ratio * ratio)) + 1.0;
}
static double gzitap(double zita, double ztop, double a0) {
  double ratio = zita / ztop;
  return ((0.0 - 1.0 * a0) * 1.0 - (6.0 - 4.0 * a0) * ratio + (6.0 - 3.0 * a0) * (ratio * ratio)) / ztop;
}
static double md_fmz(double zita, double geopot, double ztop, double zh, double a0) {
  double orog = geopot * regrav;
  return 1.0 / (gzitap(zita, ztop, a0) * orog + bzitap(zita, ztop, zh));
}
static double md_zeta(double zita, double geopot, double ztop, double zh, double a0) {
  double orog = geopot * regrav;
  return orog * (gzita_(zita, ztop, a0) - 1.0) + bzita(zita, ztop, zh);
}

// spline1d (Share/mod_spline.F90:387-459), 1-based arrays, y2 updated in
// place as the Fortran does.
static void spline1d(int nold, const std::vector<double> &xold, const std::vector<double> &yold,
                     std::vector<double> &y2, int nnew, const std::vector<double> &xnew,
                     std::vector<double> &ynew) {
  const double afac = 6.0, bfac = d_one / afac;
  std::vector<double> p(nold), q(nold);
  int noldm1 = nold - 1;
  double dxl = xold[2] - xold[1];
  double dxr = xold[3] - xold[2];
  double dydxl = (yold[2] - yold[1]) / dxl;
  double dydxr = (yold[3] - yold[2]) / dxr;
  double rtdxc = 0.5 / (dxl + dxr);
  p[1] = rtdxc * (bfac * (dydxr - dydxl) - dxl * y2[1]);
  q[1] = -rtdxc * dxr;
  if (nold > 3) {
    for (int k = 3; k <= nold; ++k) {
      dxl = dxr;
      dydxl = dydxr;
      dxr = xold[k + 1] - xold[k];
      dydxr = (yold[k + 1] - yold[k]) / dxr;
      double dxc = dxl + dxr;
      double den = d_one / (dxl * q[k - 2] + dxc + dxc);
      p[k - 1] = den * (bfac * (dydxr - dydxl) - dxl * p[k - 2]);
      q[k - 1] = -den * dxr;
    }
  }
  for (int k = noldm1; k >= 2; --k) y2[k] = p[k - 1] + q[k - 1] * y2[k + 1];
  int k = -1, kold = 0;
  double ak = 0, bk = 0, ck = 0;
  for (int k1 = 1; k1 <= nnew; ++k1) {
    double xk = xnew[k1];
    if (xk < xold[1]) { ynew[k1] = yold[1]; continue; }
    if (xk >= xold[nold]) { ynew[k1] = yold[nold]; continue; }
    for (int k2 = 2; k2 <= nold; ++k2) {
      if (xold[k2] <= xk) continue;
      kold = k2 - 1;
      break;
    }
    if (k == kold) {
      double x = xk - xold[k];
      double xsq = x * x;
      ynew[k1] = ak * xsq * x + bk * xsq + ck * x + yold[k];
      continue;
    }
    k = kold;
    double y2k = y2[k], y2kp1 = y2[k + 1];
    double dx = xold[k + 1] - xold[k];
    double rdx = d_one / dx;
    ak = bfac * rdx * (y2kp1 - y2k);
    bk = 0.5 * y2k;
    ck = rdx * (yold[k + 1] - yold[k]) - bfac * dx * (y2kp1 + y2k + y2k);
    double x = xk - xold[k];
    double xsq = x * x;
    ynew[k1] = ak * xsq * x + bk * xsq + ck * x + yold[k];
  }
}

// exponential_nudging (Main/mpplib/mod_runparams.F90:611-637) with
// sigma = sigmazita(zita), hsigma = sigmazita(zitah) (Main/mod_params.F90:
// 2464-2465, Share/mod_zita.F90:40-45).
static void exponential_nudging(int kz, double ztop, double high, double medium, double low,
                                std::vector<double> &nudge) {
  std::vector<double> zf(kz + 1), zh(kz);
  orc_setup_levels_(kz, ztop, zf.data(), zh.data());
  std::vector<double> sigma(kz + 2), hsigma(kz + 1);
  for (int k = 1; k <= kz + 1; ++k) sigma[k] = 1.0 - zf[k - 1] / ztop;
  for (int k = 1; k <= kz; ++k) hsigma[k] = 1.0 - zh[k - 1] / ztop;
  int kw;
  for (kw = 2; kw <= kz; ++kw)
    if (sigma[kw] > 0.40) break;
  std::vector<double> zcin = {0.0, sigma[1], sigma[kw], sigma[kz + 1]};
  std::vector<double> ncin = {0.0, high, medium, low};
  std::vector<double> ycin = {0.0, 0.0, 0.0, 0.0};
  nudge.assign(kz + 1, 0.0);
  spline1d(3, zcin, ncin, ycin, kz, hsigma, nudge);
}

}  // namespace orc

using namespace orc;

extern "C" {

int orc_setup_levels(int kz, double ztop, double *zitaf_out, double *zitah_out) {
  orc_setup_levels_(kz, ztop, zitaf_out, zitah_out);
  return 0;
}

int orc_exponential_nudging(int kz, double ztop, double high, double medium, double low,
                            double *anudge) {
  std::vector<double> nudge;
  exponential_nudging(kz, ztop, high, medium, low, nudge);
  for (int k = 1; k <= kz; ++k) anudge[k - 1] = nudge[k];
  return 0;
}

// compute_moloch_static on serial extents; ht/htu/htv/msfu/msfv are (jx,iy).
int orc_setup_metric(const mlc_dims *d, const mlc_params *p, const double *ht_, const double *htu_,
                     const double *htv_, const double *msfu_, const double *msfv_,
                     const double *zita, const double *zitah, double *hx_o, double *hy_o,
                     double *zeta_o, double *fmz_o, double *rfmzu_o, double *rfmzv_o,
                     double *fmzf_o, double *zetaf_o, double *dz_o) {
  const int jx = d->jx, iy = d->iy, kz = d->kz;
  F2<double> ht(1, jx, 1, iy), htu(1, jx, 1, iy), htv(1, jx, 1, iy), msfu(1, jx, 1, iy), msfv(1, jx, 1, iy);
  std::memcpy(ht.d.data(), ht_, ht.d.size() * 8);
  std::memcpy(htu.d.data(), htu_, htu.d.size() * 8);
  std::memcpy(htv.d.data(), htv_, htv.d.size() * 8);
  std::memcpy(msfu.d.data(), msfu_, msfu.d.size() * 8);
  std::memcpy(msfv.d.data(), msfv_, msfv.d.size() * 8);
  const double rdx = 1.0 / p->dx;
  const double ztop = p->mo_ztop, zh = p->mo_h, a0 = p->mo_a0;
  F2<double> hx(1, jx, 1, iy - 1), hy(1, jx - 1, 1, iy);
  for (int i = 1; i <= iy - 1; ++i)
    for (int j = 1; j <= jx; ++j) {
      if (j == 1)
        hx(j, i) = 2.0 * rdx * regrav * msfu(j, i) * (ht(j, i) - htu(j, i));
      else
        hx(j, i) = rdx * regrav * msfu(j, i) * (ht(j, i) - ht(j - 1, i));
    }
  for (int i = 1; i <= iy; ++i)
    for (int j = 1; j <= jx - 1; ++j) {
      if (p->lrotllr) {
        if (i == 1) hy(j, i) = 2.0 * rdx * regrav * (ht(j, i) - htv(j, i));
        else hy(j, i) = rdx * regrav * (ht(j, i) - ht(j, i - 1));
      } else {
        if (i == 1) hy(j, i) = 2.0 * rdx * regrav * msfv(j, i) * (ht(j, i) - htv(j, i));
        else hy(j, i) = rdx * regrav * msfv(j, i) * (ht(j, i) - ht(j, i - 1));
      }
    }
  F3 zeta(1, jx - 1, 1, iy - 1, 1, kz), fmz(1, jx - 1, 1, iy - 1, 1, kz);
  F3 rfmzu(1, jx, 1, iy - 1, 1, kz), rfmzv(1, jx - 1, 1, iy, 1, kz);
  F3 fmzf(1, jx - 1, 1, iy - 1, 1, kz + 1), zetaf(1, jx - 1, 1, iy - 1, 1, kz + 1), dz(1, jx - 1, 1, iy - 1, 1, kz);
  for (int k = 1; k <= kz; ++k)
    for (int i = 1; i <= iy - 1; ++i)
      for (int j = 1; j <= jx - 1; ++j) {
        zeta(j, i, k) = md_zeta(zitah[k - 1], ht(j, i), ztop, zh, a0);
        fmz(j, i, k) = md_fmz(zitah[k - 1], ht(j, i), ztop, zh, a0);
      }
  for (int k = 1; k <= kz; ++k)
    for (int i = 1; i <= iy - 1; ++i)
      for (int j = 1; j <= jx; ++j) rfmzu(j, i, k) = 1.0 / md_fmz(zitah[k - 1], htu(j, i), ztop, zh, a0);
  for (int k = 1; k <= kz; ++k)
    for (int i = 1; i <= iy; ++i)
      for (int j = 1; j <= jx - 1; ++j) rfmzv(j, i, k) = 1.0 / md_fmz(zitah[k - 1], htv(j, i), ztop, zh, a0);
  for (int k = 1; k <= kz + 1; ++k)
    for (int i = 1; i <= iy - 1; ++i)
      for (int j = 1; j <= jx - 1; ++j) {
        fmzf(j, i, k) = md_fmz(zita[k - 1], ht(j, i), ztop, zh, a0);
        zetaf(j, i, k) = md_zeta(zita[k - 1], ht(j, i), ztop, zh, a0);
      }
  for (int k = 1; k <= kz; ++k)
    for (int i = 1; i <= iy - 1; ++i)
      for (int j = 1; j <= jx - 1; ++j) dz(j, i, k) = zetaf(j, i, k) - zetaf(j, i, k + 1);
  std::memcpy(hx_o, hx.d.data(), hx.d.size() * 8);
  std::memcpy(hy_o, hy.d.data(), hy.d.size() * 8);
  zeta.store(zeta_o); fmz.store(fmz_o); rfmzu.store(rfmzu_o); rfmzv.store(rfmzv_o);
  fmzf.store(fmzf_o); zetaf.store(zetaf_o); dz.store(dz_o);
  return 0;
}

// relax_coefficients, Main/mpplib/mod_runparams.F90:648-702
int orc_relax_coefficients(int np, double gmmin, double gmmax, double *coeff) {
  const int npmax = 32;
  double p[npmax + 1], q[npmax + 1], pp[npmax + 1], qq[npmax + 1];
  int n = 1;
  p[0] = 0.0; p[1] = 1.0; q[0] = 1.0; q[1] = 0.0;
  double my = std::sqrt(gmmax / gmmin);
  while (n < np) {
    my = std::sqrt((my + 1.0 / my) / 2.0);
    for (int i = 0; i <= n + n; ++i) { pp[i] = 0.0; qq[i] = 0.0; }
    for (int i = 0; i <= n; ++i)
      for (int j = 0; j <= n; ++j) {
        pp[i + j] = pp[i + j] + p[i] * p[j] + q[i] * q[j];
        qq[i + j] = qq[i + j] + 2.0 * my * p[i] * q[j];
      }
    for (int i = 0; i <= n + n; ++i) { p[i] = pp[i]; q[i] = qq[i]; }
    n = 2 * n;
  }
  if (n != np && np != 1) return -1;
  for (int i = n; i >= 1; --i) {
    double kk = p[i] / q[i - 1];
    for (int j = i; j >= 1; --j) {
      double xxx = q[j];
      q[j] = p[j] - kk * q[j - 1];
      p[j] = xxx;
    }
    double xxx = q[0];
    q[0] = p[0];
    p[0] = xxx;
    double kdt2 = kk * std::sqrt(gmmin * gmmax);
    coeff[i - 1] = kdt2 / (1.0 + kdt2);
  }
  return 0;
}

// setup_bdycon (Lehmann) + mod_init sponge; zeta is (jx-1,iy-1,kz).
int orc_setup_relaxation(const mlc_dims *d, const mlc_params *p, const double *zeta_,
                         double *hefc_o, double *fcx_o, double *tnudge_o, double *ffilt_o,
                         int *nztop_o) {
  const int jx = d->jx, iy = d->iy, kz = d->kz, nspgx = p->nspgx;
  F3 zeta(1, jx - 1, 1, iy - 1, 1, kz);
  zeta.load(zeta_);
  std::vector<double> gmeanz(kz + 1);
  const double np = (double)((jx - 1) * (iy - 1));
  int nztop = 0;
  for (int k = 1; k <= kz; ++k) {
    double meanz = 0.0;
    for (int j = 1; j <= jx - 1; ++j)
      for (int i = 1; i <= iy - 1; ++i) meanz = meanz + zeta(j, i, k) / np;
    gmeanz[k] = meanz;
    if (gmeanz[k] > 18000.0) nztop = nztop + 1;
  }
  F2<double> hefc(1, nspgx, 1, kz);
  for (int k = 1; k <= kz; ++k) { hefc(1, k) = 1.0; hefc(nspgx, k) = 0.0; }
  if (p->bdy_use_lehmann) {
    double cflmax = std::min(0.999, (300.0 * (p->dtsec / (double)p->mo_nadv)) / (2.0 * p->dx));
    double cflmin = std::max(0.001, (10.0 * (p->dtsec / (double)p->mo_nadv)) / (2.0 * p->dx));
    std::vector<double> c(nspgx);
    for (int k = 1; k <= kz; ++k) {
      orc_relax_coefficients(nspgx - 2, cflmin, cflmax, c.data());
      for (int n = 2; n <= nspgx - 1; ++n) hefc(n, k) = c[n - 2];
    }
  } else {
    // Main/mod_bdycod.F90:538-544
    std::vector<double> anudge;
    exponential_nudging(kz, p->mo_ztop, p->high_nudge, p->medium_nudge, p->low_nudge, anudge);
    for (int k = 1; k <= kz; ++k)
      for (int n = 2; n <= nspgx - 1; ++n) hefc(n, k) = std::exp(-(double)(n - 1) / anudge[k]);
  }
  std::memcpy(hefc_o, hefc.d.data(), hefc.d.size() * 8);
  if (d->ntr > 0) {  // setup_che_bdycon (ichem = 1)
    fcx_o[0] = 1.0;
    fcx_o[nspgx - 1] = 0.0;
    orc_relax_coefficients(nspgx - 2, 0.1, 1.0, fcx_o + 1);
  } else {
    for (int n = 0; n < nspgx; ++n) fcx_o[n] = 0.0;
  }
  for (int k = 1; k <= kz; ++k) {
    if (p->mo_top_nudge && k <= nztop)
      tnudge_o[k - 1] = std::pow(std::sin(0.5 * mathpi * (gmeanz[k] - 18000.0) / (p->mo_h - 18000.0)), 2);
    else
      tnudge_o[k - 1] = 0.0;
    if (gmeanz[k] < 18000.0) {
      ffilt_o[k - 1] = 0.0;
    } else {
      double zzi = (gmeanz[k] - 18000.0) / (p->mo_ztop - 18000.0);
      double sn = std::sin(0.5 * mathpi * zzi);
      ffilt_o[k - 1] = 0.8 * (sn * sn);
    }
  }
  *nztop_o = p->mo_top_nudge ? nztop : 0;
  return 0;
}

// The domain-mean level heights of setup_bdycon (gmeanz, same sum order
// as orc_setup_relaxation), for the spectral nudging weights.
int orc_gmeanz(const mlc_dims *d, const double *zeta_, double *gmeanz_o) {
  const int jx = d->jx, iy = d->iy, kz = d->kz;
  F3 zeta(1, jx - 1, 1, iy - 1, 1, kz);
  zeta.load(zeta_);
  const double np = (double)((jx - 1) * (iy - 1));
  for (int k = 1; k <= kz; ++k) {
    double meanz = 0.0;
    for (int j = 1; j <= jx - 1; ++j)
      for (int i = 1; i <= iy - 1; ++i) meanz = meanz + zeta(j, i, k) / np;
    gmeanz_o[k - 1] = meanz;
  }
  return 0;
}

// lowpass_init's level weights (Main/mod_bdycod.F90:3890-3894).
int orc_setup_spectral(const mlc_params *p, int kz, const double *gmeanz, double *cnudge) {
  const double rtb = 1.0 / p->dtbdys;
  const double cn0 = p->dtrad * rtb;
  for (int k = 1; k <= kz; ++k) {
    const double r = gmeanz[k - 1] / p->mo_h;  // x**2 is x*x in Fortran
    cnudge[k - 1] = cn0 * std::min(r * r, 1.0);
  }
  return 0;
}

// setup_boundaries, one process, non-band: ibnd (jx, iy).
int orc_setup_boundaries(int jx, int iy, int ldotx, int ldoty, int nspgx, int nspgd, int32_t *out) {
  F2<int32_t> ibnd(1, jx, 1, iy, -1);
  F2<uint8_t> bs(1, jx, 1, iy, 0), bn(1, jx, 1, iy, 0);
  int jcx = ldotx ? 0 : 1, icy = ldoty ? 0 : 1;
  int nspx = ldotx ? nspgd : nspgx, nspy = ldoty ? nspgd : nspgx;
  int igbb1 = 2, igbb2 = nspy - 1, jgbl1 = 2, jgbl2 = nspx - 1;
  int igbt1 = iy - icy - nspy + 2, igbt2 = iy - 1 - icy;
  int jgbr1 = jx - jcx - nspx + 2, jgbr2 = jx - 1 - jcx;
  for (int i = 1; i <= iy; ++i)
    if (i >= igbb1 && i <= igbb2)
      for (int j = 1; j <= jx; ++j)
        if (j >= jgbl1 && j <= jgbr2) {
          if (j <= jgbl2 && i >= j) continue;
          if (j >= jgbr1 && i >= (jgbr2 - j + 2)) continue;
          ibnd(j, i) = i - igbb1 + 2;
          bs(j, i) = 1;
        }
  for (int i = 1; i <= iy; ++i)
    if (i >= igbt1 && i <= igbt2)
      for (int j = 1; j <= jx; ++j)
        if (j >= jgbl1 && j <= jgbr2) {
          if (j <= jgbl2 && j <= (igbt2 - i + 2)) continue;
          if (j >= jgbr1 && (igbt2 - i) >= (jgbr2 - j)) continue;
          ibnd(j, i) = igbt2 - i + 2;
          bn(j, i) = 1;
        }
  for (int i = 1; i <= iy; ++i)
    for (int j = 1; j <= jx; ++j) {
      if (bn(j, i) || bs(j, i)) continue;
      if (i < igbb1 || i > igbt2) continue;
      if (j >= jgbl1 && j <= jgbl2) ibnd(j, i) = j - jgbl1 + 2;
    }
  for (int i = 1; i <= iy; ++i)
    for (int j = 1; j <= jx; ++j) {
      if (bn(j, i) || bs(j, i)) continue;
      if (i < igbb1 || i > igbt2) continue;
      if (j >= jgbr1 && j <= jgbr2) ibnd(j, i) = jgbr2 - j + 2;
    }
  std::memcpy(out, ibnd.d.data(), ibnd.d.size() * sizeof(int32_t));
  return 0;
}

// nspgx/nspgd as initparam derives them (Share/mod_dynparam.F90:762-786):
// the default 6 points scaled to the resolution ds (km), at most a quarter
// of the smaller extent, at least 6; a namelist value (> 0) replaces the
// default; with Lehmann weights for MOLOCH a power of two plus 2 points.
int orc_setup_nspg(int jx, int iy, double ds, int lehmann, int nspgx_nl, int nspgd_nl,
                   int *nspgx_o, int *nspgd_o) {
  int nspgx = 6, nspgd = 6;
  const int quarter = std::min(jx, iy) / 4;
  nspgx = std::max(std::min(std::max((int)((double)(nspgx * 50) / ds), nspgx), quarter), 6);
  nspgd = std::max(std::min(std::max((int)((double)(nspgd * 50) / ds), nspgd), quarter), 6);
  if (nspgx_nl > 0) nspgx = nspgx_nl;
  if (nspgd_nl > 0) nspgd = nspgd_nl;
  nspgx = std::max(nspgx, 6);
  nspgd = std::max(nspgd, 6);
  if (lehmann) {
    nspgx = std::min(std::max(6, (int)std::lround(20.0 * std::pow(ds, -0.35)) + 1), 34);
    int isp = 1;
    while (isp < nspgx - 2) isp *= 2;
    nspgx = isp + 2;
    nspgd = nspgx;
  }
  *nspgx_o = nspgx;
  *nspgd_o = nspgd;
  return 0;
}

// paicompute on cross extents.
int orc_paicompute(const mlc_dims *d, const double *ps_, const double *z_, const double *t_,
                   const double *q_, const double *fmzf_, double mo_dzita, double *pai_o) {
  const int jx = d->jx, iy = d->iy, kz = d->kz;
  F2<double> ps(1, jx - 1, 1, iy - 1);
  std::memcpy(ps.d.data(), ps_, ps.d.size() * 8);
  F3 z(1, jx - 1, 1, iy - 1, 1, kz), t(1, jx - 1, 1, iy - 1, 1, kz), q(1, jx - 1, 1, iy - 1, 1, kz);
  F3 fmzf(1, jx - 1, 1, iy - 1, 1, kz + 1), pai(1, jx - 1, 1, iy - 1, 1, kz);
  z.load(z_); t.load(t_); q.load(q_); fmzf.load(fmzf_);
  for (int j = 1; j <= jx - 1; ++j)
    for (int i = 1; i <= iy - 1; ++i) {
      double zdelta = z(j, i, kz) * egrav;
      double tv1 = t(j, i, kz) * (d_one + ep1 * q(j, i, kz));
      double tv2 = t(j, i, kz - 1) * (d_one + ep1 * q(j, i, kz - 1));
      double lrt = (tv2 - tv1) / (z(j, i, kz - 1) - z(j, i, kz));
      if (lrt > govcp) lrt = govcp;
      else if (lrt < -0.005) lrt = 0.5 * lrt - 0.5 * lrate;
      double tv = tv1 - 0.5 * z(j, i, kz) * lrt;
      double zz = d_one / (rgas * tv);
      double pp = ps(j, i) * std::exp(-zdelta * zz);
      double paikp1 = std::pow(pp / p00, rovcp);
      pai(j, i, kz) = paikp1;
      for (int k = kz - 1; k >= 1; --k) {
        tv1 = t(j, i, k) * (d_one + ep1 * q(j, i, k));
        tv2 = t(j, i, k + 1) * (d_one + ep1 * q(j, i, k + 1));
        double zb = 2.0 * egrav * mo_dzita / (fmzf(j, i, k + 1) * cpd) + tv1 - tv2;
        double zd = std::sqrt(zb * zb + 4.0 * tv2 * tv1);
        paikp1 = -paikp1 / (2.0 * tv2) * (zb - zd);
        pai(j, i, k) = paikp1;
      }
    }
  pai.store(pai_o);
  return 0;
}

}  // extern "C"
