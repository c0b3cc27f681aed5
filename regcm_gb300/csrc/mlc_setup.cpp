// mlc_setup.cpp -- host-side FP64 setup of the MOLOCH static inputs.
//
// Everything here runs once per domain on the host, in IEEE double, with the
// operation order of the Fortran it replaces (file:line in each comment), so
// a domain built here is bit-identical to the one RegCM's own setup builds on
// the same machine.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/moloch_gb300_setup.h"
#include "mlc_constants.h"

using namespace mlc;

namespace {

// Column-major index helpers for the extents of moloch_gb300.h.
struct Grid {
  int jx, iy, kz;
  size_t dot(int j, int i) const { return (size_t)(j - 1) + (size_t)(i - 1) * jx; }
  size_t cross2(int j, int i) const { return (size_t)(j - 1) + (size_t)(i - 1) * (jx - 1); }
  size_t cross3(int j, int i, int k) const {
    return (size_t)(j - 1) + (size_t)(jx - 1) * ((size_t)(i - 1) + (size_t)(iy - 1) * (k - 1));
  }
  size_t upt3(int j, int i, int k) const {  // (jx, iy-1, k)
    return (size_t)(j - 1) + (size_t)jx * ((size_t)(i - 1) + (size_t)(iy - 1) * (k - 1));
  }
  size_t vpt3(int j, int i, int k) const {  // (jx-1, iy, k)
    return (size_t)(j - 1) + (size_t)(jx - 1) * ((size_t)(i - 1) + (size_t)iy * (k - 1));
  }
};

// Share/mod_zita.F90:88-150: decay function b(zeta), its derivative, and the
// derivative of G(zeta); md_fmz_h (Eq. 9) and md_zeta_h.
struct Coord {
  double ztop, zh, a0, zfz;
  Coord(double ztop_, double zh_, double a0_) : ztop(ztop_), zh(zh_), a0(a0_) {
    zfz = ztop / (std::exp(ztop / zh) - 1.0);
  }
  double b(double z) const { return zfz * (std::exp(z / zh) - 1.0); }
  double bp(double z) const { return zfz * std::exp(z / zh) / zh; }
  double gp(double z) const {
    double r = z / ztop;
    return ((0.0 - 1.0 * a0) * 1.0 - (6.0 - 4.0 * a0) * r + (6.0 - 3.0 * a0) * (r * r)) / ztop;
  }
  // geopotential -> orography height happens inside (md_fmz, md_zeta)
  double fmz(double z, double geopot) const {
    double orog = geopot * kRegrav;
    return 1.0 / (gp(z) * orog + bp(z));
  }
  double zeta(double z, double geopot) const {
    double orog = geopot * kRegrav;
    return orog * (gzita(z, ztop, a0) - 1.0) + b(z);
  }
};

// The factors of md_fmz/md_zeta that depend only on the level (the
// exponentials of b(zeta)), formed once per level; the per-point results
// are the same expressions on the same values.
struct Level {
  double gp, bp, gm1, b;
  Level(const Coord &c, double z) : gp(c.gp(z)), bp(c.bp(z)), gm1(gzita(z, c.ztop, c.a0) - 1.0), b(c.b(z)) {}
  double fmz(double geopot) const {
    double orog = geopot * kRegrav;
    return 1.0 / (gp * orog + bp);
  }
  double zeta(double geopot) const {
    double orog = geopot * kRegrav;
    return orog * gm1 + b;
  }
};

}  // namespace

extern "C" {

int mlc_setup_levels(int kz, double ztop, double *zita, double *zitah) {
  if (kz < 2 || !(ztop > 0.0) || !zita || !zitah) return MLC_ERR_INVALID;
  // model_zitaf: accumulate dz upward from the surface
  double dz = ztop / (double)kz;
  zita[kz] = 0.0;            // zitaf(kzp1)
  zita[0] = ztop;            // zitaf(1)
  for (int k = kz; k >= 2; --k) zita[k - 1] = zita[k] + dz;
  // model_zitah
  zitah[kz - 1] = dz * 0.5;
  zitah[0] = ztop - dz * 0.5;
  for (int k = kz - 1; k >= 2; --k) zitah[k - 1] = zitah[k] + dz;
  return MLC_OK;
}

int mlc_setup_nspg(int jx, int iy, double ds_km, int lehmann, int nspgx_nl, int nspgd_nl,
                   int *nspgx, int *nspgd) {
  if (!nspgx || !nspgd || !(ds_km > 0.0)) return MLC_ERR_INVALID;
  int mn4 = (jx < iy ? jx : iy) / 4;
  auto scale = [&](int n) {
    int a = (int)((double)(n * 50) / ds_km);
    a = a > n ? a : n;
    a = a < mn4 ? a : mn4;
    return a > 6 ? a : 6;
  };
  // defaults 6, rescaled by ds; a namelist value (> 0) replaces them
  int gx = scale(6), gd = scale(6);
  if (nspgx_nl > 0) gx = nspgx_nl;
  if (nspgd_nl > 0) gd = nspgd_nl;
  gx = gx > 6 ? gx : 6;
  gd = gd > 6 ? gd : 6;
  if (lehmann) {
    // a power of two plus the two end points (weights 1 and 0)
    long v = std::lround(20.0 * std::pow(ds_km, -0.35)) + 1;
    v = v > 6 ? v : 6;
    v = v < 34 ? v : 34;
    int isp = 1;
    while (isp < v - 2) isp *= 2;
    gx = isp + 2;
    gd = gx;
  }
  *nspgx = gx;
  *nspgd = gd;
  return MLC_OK;
}

int mlc_setup_metric(const mlc_dims *d, const mlc_params *p, const double *ht, const double *htu,
                     const double *htv, const double *msfu, const double *msfv, const double *zita,
                     const double *zitah, double *hx, double *hy, double *zeta, double *fmz,
                     double *rfmzu, double *rfmzv, double *fmzf, double *zetaf, double *dz) {
  if (!d || !p || !ht || !htu || !htv || !msfu || !msfv || !zita || !zitah) return MLC_ERR_INVALID;
  const Grid g{d->jx, d->iy, d->kz};
  const int jx = g.jx, iy = g.iy, kz = g.kz;
  const double rdx = 1.0 / p->dx;
  const Coord c(p->mo_ztop, p->mo_h, p->mo_a0);
  // terrain slopes, Main/mod_params.F90:3325-3355
  if (hx)
    for (int i = 1; i <= iy - 1; ++i)
      for (int j = 1; j <= jx; ++j) {
        double v = (j == 1) ? 2.0 * rdx * kRegrav * msfu[g.dot(j, i)] * (ht[g.dot(j, i)] - htu[g.dot(j, i)])
                            : rdx * kRegrav * msfu[g.dot(j, i)] * (ht[g.dot(j, i)] - ht[g.dot(j - 1, i)]);
        hx[g.dot(j, i)] = v;  // (jx, iy-1) shares the dot stride
      }
  if (hy)
    for (int i = 1; i <= iy; ++i)
      for (int j = 1; j <= jx - 1; ++j) {
        double m = p->lrotllr ? 1.0 : msfv[g.dot(j, i)];
        double v;
        if (p->lrotllr) {
          v = (i == 1) ? 2.0 * rdx * kRegrav * (ht[g.dot(j, i)] - htv[g.dot(j, i)])
                       : rdx * kRegrav * (ht[g.dot(j, i)] - ht[g.dot(j, i - 1)]);
        } else {
          v = (i == 1) ? 2.0 * rdx * kRegrav * m * (ht[g.dot(j, i)] - htv[g.dot(j, i)])
                       : rdx * kRegrav * m * (ht[g.dot(j, i)] - ht[g.dot(j, i - 1)]);
        }
        hy[g.cross2(j, i)] = v;  // (jx-1, iy)
      }
  // vertical metric, Main/mod_params.F90:3358-3390
  for (int k = 1; k <= kz; ++k) {
    const Level lv(c, zitah[k - 1]);
    for (int i = 1; i <= iy - 1; ++i)
      for (int j = 1; j <= jx - 1; ++j) {
        double h = ht[g.dot(j, i)];
        if (zeta) zeta[g.cross3(j, i, k)] = lv.zeta(h);
        if (fmz) fmz[g.cross3(j, i, k)] = lv.fmz(h);
      }
    if (rfmzu)
      for (int i = 1; i <= iy - 1; ++i)
        for (int j = 1; j <= jx; ++j) rfmzu[g.upt3(j, i, k)] = 1.0 / lv.fmz(htu[g.dot(j, i)]);
    if (rfmzv)
      for (int i = 1; i <= iy; ++i)
        for (int j = 1; j <= jx - 1; ++j) rfmzv[g.vpt3(j, i, k)] = 1.0 / lv.fmz(htv[g.dot(j, i)]);
  }
  std::vector<double> zf;
  const bool need_zf = (zetaf != nullptr) || (dz != nullptr);
  if (need_zf) zf.assign((size_t)(jx - 1) * (iy - 1) * (kz + 1), 0.0);
  for (int k = 1; k <= kz + 1; ++k) {
    const Level lv(c, zita[k - 1]);
    for (int i = 1; i <= iy - 1; ++i)
      for (int j = 1; j <= jx - 1; ++j) {
        double h = ht[g.dot(j, i)];
        if (fmzf) fmzf[g.cross3(j, i, k)] = lv.fmz(h);
        if (need_zf) zf[g.cross3(j, i, k)] = lv.zeta(h);
      }
  }
  if (zetaf) std::memcpy(zetaf, zf.data(), zf.size() * sizeof(double));
  if (dz)
    for (int k = 1; k <= kz; ++k)
      for (int i = 1; i <= iy - 1; ++i)
        for (int j = 1; j <= jx - 1; ++j)
          dz[g.cross3(j, i, k)] = zf[g.cross3(j, i, k)] - zf[g.cross3(j, i, k + 1)];
  return MLC_OK;
}

int mlc_relax_coefficients(int np, double gmmin, double gmmax, double *coeff) {
  // Lehmann (1993): continued-fraction recursion on the polynomial pair
  // (p, q), then the coefficients from its back-expansion.
  const int npmax = 32;
  if (np < 1 || np > npmax || !coeff || !(gmmin > 0.0) || !(gmmax > 0.0)) return MLC_ERR_INVALID;
  double pc[npmax + 1] = {0}, qc[npmax + 1] = {0}, pn[npmax + 1], qn[npmax + 1];
  int n = 1;
  pc[0] = 0.0; pc[1] = 1.0;
  qc[0] = 1.0; qc[1] = 0.0;
  double my = std::sqrt(gmmax / gmmin);
  while (n < np) {
    my = std::sqrt((my + 1.0 / my) / 2.0);
    for (int i = 0; i <= 2 * n; ++i) { pn[i] = 0.0; qn[i] = 0.0; }
    for (int i = 0; i <= n; ++i)
      for (int j = 0; j <= n; ++j) {
        pn[i + j] = pn[i + j] + pc[i] * pc[j] + qc[i] * qc[j];
        qn[i + j] = qn[i + j] + 2.0 * my * pc[i] * qc[j];
      }
    for (int i = 0; i <= 2 * n; ++i) { pc[i] = pn[i]; qc[i] = qn[i]; }
    n = 2 * n;
  }
  if (n != np && np != 1) return MLC_ERR_INVALID;  // not a power of two
  for (int i = n; i >= 1; --i) {
    double kk = pc[i] / qc[i - 1];
    for (int j = i; j >= 1; --j) {
      double keep = qc[j];
      qc[j] = pc[j] - kk * qc[j - 1];
      pc[j] = keep;
    }
    double keep = qc[0];
    qc[0] = pc[0];
    pc[0] = keep;
    double kdt2 = kk * std::sqrt(gmmin * gmmax);
    coeff[i - 1] = kdt2 / (1.0 + kdt2);
  }
  return MLC_OK;
}

int mlc_setup_spectral(const mlc_params *p, int kz, const double *gmeanz, double *cnudge) {
  if (!p || !gmeanz || !cnudge || kz < 1 || p->dtbdys <= 0.0 || p->mo_h <= 0.0)
    return MLC_ERR_INVALID;
  const double cn0 = p->dtrad * (1.0 / p->dtbdys);
  for (int k = 0; k < kz; ++k) {
    const double r = gmeanz[k] / p->mo_h;
    const double r2 = r * r;
    cnudge[k] = cn0 * (r2 < 1.0 ? r2 : 1.0);
  }
  return MLC_OK;
}

int mlc_exponential_nudging(int kz, double ztop, double high, double medium, double low,
                            double *anudge) {
  if (kz < 2 || !(ztop > 0.0) || !anudge) return MLC_ERR_INVALID;
  if (!(high > 0.0) || !(medium > 0.0) || !(low > 0.0)) return MLC_ERR_INVALID;
  std::vector<double> zita(kz + 1), zitah(kz);
  mlc_setup_levels(kz, ztop, zita.data(), zitah.data());
  // sigmazita (Share/mod_zita.F90:40-45) at full and half levels
  auto sig = [&](double z) { return 1.0 - z / ztop; };
  // the first full level k in 2..kz with sigma(k) > 0.4, else kz+1
  int kmid = kz + 1;
  for (int k = 2; k <= kz; ++k)
    if (sig(zita[k - 1]) > 0.40) {
      kmid = k;
      break;
    }
  const double xo[3] = {sig(zita[0]), sig(zita[kmid - 1]), sig(zita[kz])};
  const double yo[3] = {high, medium, low};
  // spline1d with three knots and y2 = 0 at both ends: one interior value
  // y2(2) = p(1), in the routine's own arithmetic (bfac = 1/6)
  const double bfac = 1.0 / 6.0;
  const double dxl = xo[1] - xo[0], dxr = xo[2] - xo[1];
  const double dydxl = (yo[1] - yo[0]) / dxl, dydxr = (yo[2] - yo[1]) / dxr;
  const double rtdxc = 0.5 / (dxl + dxr);
  const double y2[3] = {0.0, rtdxc * (bfac * (dydxr - dydxl) - dxl * 0.0) + (-rtdxc * dxr) * 0.0, 0.0};
  for (int k = 0; k < kz; ++k) {
    const double xk = sig(zitah[k]);
    if (xk < xo[0]) {
      anudge[k] = yo[0];
      continue;
    }
    if (xk >= xo[2]) {
      anudge[k] = yo[2];
      continue;
    }
    const int q = xo[1] > xk ? 0 : 1;  // interval [xo[q], xo[q+1])
    const double dx = xo[q + 1] - xo[q];
    const double rdx = 1.0 / dx;
    const double ak = bfac * rdx * (y2[q + 1] - y2[q]);
    const double bk = 0.5 * y2[q];
    const double ck = rdx * (yo[q + 1] - yo[q]) - bfac * dx * (y2[q + 1] + y2[q] + y2[q]);
    const double x = xk - xo[q];
    const double xsq = x * x;
    anudge[k] = ak * xsq * x + bk * xsq + ck * x + yo[q];
  }
  return MLC_OK;
}

int mlc_setup_relaxation(const mlc_dims *d, mlc_params *p, const double *zeta, double *hefc,
                         double *fcx, double *tnudge, double *ffilt, double *gmeanz_out) {
  if (!d || !p || !zeta || !hefc) return MLC_ERR_INVALID;
  const int jx = d->jx, iy = d->iy, kz = d->kz, nsp = p->nspgx;
  if (nsp < 3) return MLC_ERR_INVALID;
  // domain-mean level height (Main/mod_bdycod.F90:507-520, mod_init.F90:1008-1015)
  std::vector<double> gmeanz(kz);
  const double np = (double)(jx - 1) * (double)(iy - 1);
  for (int k = 0; k < kz; ++k) {
    double acc = 0.0;
    const double *lev = zeta + (size_t)k * (jx - 1) * (iy - 1);
    for (int j = 0; j < jx - 1; ++j)
      for (int i = 0; i < iy - 1; ++i) acc = acc + lev[(size_t)j + (size_t)i * (jx - 1)] / np;
    gmeanz[k] = acc;
  }
  int nztop = 0;
  for (int k = 0; k < kz; ++k)
    if (gmeanz[k] > kZzTop) ++nztop;
  p->nztop = (p->mo_top_nudge) ? nztop : 0;
  if (!p->bdy_use_lehmann) {
    // exponential nudging (Main/mod_bdycod.F90:538-544)
    std::vector<double> anudge(kz);
    int st = mlc_exponential_nudging(kz, p->mo_ztop, p->high_nudge, p->medium_nudge,
                                     p->low_nudge, anudge.data());
    if (st != MLC_OK) return st;
    for (int k = 0; k < kz; ++k) {
      double *col = hefc + (size_t)k * nsp;
      col[0] = 1.0;
      col[nsp - 1] = 0.0;
      for (int n = 2; n <= nsp - 1; ++n) col[n - 1] = std::exp(-(double)(n - 1) / anudge[k]);
    }
  } else {
  // Lehmann weights (Main/mod_bdycod.F90:522-537)
  const double dta = p->dtsec / (double)p->mo_nadv;
  double cflmax = (300.0 * dta) / (2.0 * p->dx);
  cflmax = cflmax < 0.999 ? cflmax : 0.999;
  double cflmin = (10.0 * dta) / (2.0 * p->dx);
  cflmin = cflmin > 0.001 ? cflmin : 0.001;
  std::vector<double> w(nsp, 0.0);
  if (nsp > 2) {
    int st = mlc_relax_coefficients(nsp - 2, cflmin, cflmax, w.data());
    if (st != MLC_OK) return st;
  }
  for (int k = 0; k < kz; ++k) {
    double *col = hefc + (size_t)k * nsp;
    col[0] = 1.0;
    col[nsp - 1] = 0.0;
    for (int n = 0; n < nsp - 2; ++n) col[n + 1] = w[n];
  }
  }
  if (fcx && d->ntr > 0) {
    // setup_che_bdycon runs with chemistry only (ichem = 1: tracers)
    fcx[0] = 1.0;
    fcx[nsp - 1] = 0.0;
    int st = mlc_relax_coefficients(nsp - 2, 0.1, 1.0, fcx + 1);
    if (st != MLC_OK) return st;
  } else if (fcx) {
    for (int n = 0; n < nsp; ++n) fcx[n] = 0.0;
  }
  if (tnudge)
    for (int k = 0; k < kz; ++k) {
      if (p->mo_top_nudge && k + 1 <= nztop) {
        double s = std::sin(0.5 * kPi * (gmeanz[k] - kZzTop) / (p->mo_h - kZzTop));
        tnudge[k] = s * s;
      } else {
        tnudge[k] = 0.0;
      }
    }
  if (ffilt)
    for (int k = 0; k < kz; ++k) {
      if (gmeanz[k] < kZzTop) {
        ffilt[k] = 0.0;
      } else {
        double zzi = (gmeanz[k] - kZzTop) / (p->mo_ztop - kZzTop);
        double s = std::sin(0.5 * kPi * zzi);
        ffilt[k] = kZfiltFac * (s * s);
      }
    }
  if (gmeanz_out) std::memcpy(gmeanz_out, gmeanz.data(), kz * sizeof(double));
  return MLC_OK;
}

int mlc_setup_boundaries(int jx, int iy, int ldotx, int ldoty, int nspgx, int nspgd, int32_t *ibnd) {
  if (!ibnd || jx < 4 || iy < 4) return MLC_ERR_INVALID;
  const int jcx = ldotx ? 0 : 1, icy = ldoty ? 0 : 1;
  const int nspx = ldotx ? nspgd : nspgx, nspy = ldoty ? nspgd : nspgx;
  const int igbb1 = 2, igbb2 = nspy - 1, jgbl1 = 2, jgbl2 = nspx - 1;
  const int igbt1 = iy - icy - nspy + 2, igbt2 = iy - 1 - icy;
  const int jgbr1 = jx - jcx - nspx + 2, jgbr2 = jx - 1 - jcx;
  auto at = [&](int j, int i) -> int32_t & { return ibnd[(size_t)(j - 1) + (size_t)(i - 1) * jx]; };
  std::vector<uint8_t> ns((size_t)jx * iy, 0);  // 1 = south, 2 = north
  auto tag = [&](int j, int i) -> uint8_t & { return ns[(size_t)(j - 1) + (size_t)(i - 1) * jx]; };
  for (int i = 1; i <= iy; ++i)
    for (int j = 1; j <= jx; ++j) at(j, i) = -1;
  // south band, corner triangles left to the west/east bands
  for (int i = 1; i <= iy; ++i) {
    if (i < igbb1 || i > igbb2) continue;
    for (int j = 1; j <= jx; ++j) {
      if (j < jgbl1 || j > jgbr2) continue;
      if (j <= jgbl2 && i >= j) continue;
      if (j >= jgbr1 && i >= (jgbr2 - j + 2)) continue;
      at(j, i) = i - igbb1 + 2;
      tag(j, i) |= 1;
    }
  }
  // north band
  for (int i = 1; i <= iy; ++i) {
    if (i < igbt1 || i > igbt2) continue;
    for (int j = 1; j <= jx; ++j) {
      if (j < jgbl1 || j > jgbr2) continue;
      if (j <= jgbl2 && j <= (igbt2 - i + 2)) continue;
      if (j >= jgbr1 && (igbt2 - i) >= (jgbr2 - j)) continue;
      at(j, i) = igbt2 - i + 2;
      tag(j, i) |= 2;
    }
  }
  // west and east bands, outside the north/south bands
  for (int i = 1; i <= iy; ++i)
    for (int j = 1; j <= jx; ++j) {
      if (tag(j, i)) continue;
      if (i < igbb1 || i > igbt2) continue;
      if (j >= jgbl1 && j <= jgbl2) at(j, i) = j - jgbl1 + 2;
    }
  for (int i = 1; i <= iy; ++i)
    for (int j = 1; j <= jx; ++j) {
      if (tag(j, i)) continue;
      if (i < igbb1 || i > igbt2) continue;
      if (j >= jgbr1 && j <= jgbr2) at(j, i) = jgbr2 - j + 2;
    }
  return MLC_OK;
}

int mlc_paicompute(const mlc_dims *d, const mlc_params *p, const double *ps, const double *zeta,
                   const double *t, const double *qv, const double *fmzf, const double *zita,
                   double *pai) {
  if (!d || !p || !ps || !zeta || !t || !qv || !fmzf || !zita || !pai) return MLC_ERR_INVALID;
  const Grid g{d->jx, d->iy, d->kz};
  const int kz = g.kz;
  const double mo_dzita = zita[kz - 1];  // zita(kz), Main/mod_params.F90:2462
  for (int i = 1; i <= g.iy - 1; ++i)
    for (int j = 1; j <= g.jx - 1; ++j) {
      auto tv = [&](int k) { return t[g.cross3(j, i, k)] * (1.0 + kEp1 * qv[g.cross3(j, i, k)]); };
      const double zkz = zeta[g.cross3(j, i, kz)];
      double zdelta = zkz * kGrav;
      double tv1 = tv(kz), tv2 = tv(kz - 1);
      double lrt = (tv2 - tv1) / (zeta[g.cross3(j, i, kz - 1)] - zkz);
      if (lrt > kGovcp) {
        lrt = kGovcp;
      } else if (lrt < -0.005) {
        lrt = 0.5 * lrt - 0.5 * kLrate;
      }
      double tvs = tv1 - 0.5 * zkz * lrt;
      double zz = 1.0 / (kRgas * tvs);
      double pp = ps[g.cross2(j, i)] * std::exp(-zdelta * zz);
      double paik = std::pow(pp / kP00, kRovcp);
      pai[g.cross3(j, i, kz)] = paik;
      for (int k = kz - 1; k >= 1; --k) {
        tv1 = tv(k);
        tv2 = tv(k + 1);
        double zb = 2.0 * kGrav * mo_dzita / (fmzf[g.cross3(j, i, k + 1)] * kCpd) + tv1 - tv2;
        double zd = std::sqrt(zb * zb + 4.0 * tv2 * tv1);
        paik = -paik / (2.0 * tv2) * (zb - zd);
        pai[g.cross3(j, i, k)] = paik;
      }
    }
  return MLC_OK;
}

int mlc_pfwsat(size_t n, const double *t, const double *p, double *qs) {
  if (!t || !p || !qs) return MLC_ERR_INVALID;
  for (size_t m = 0; m < n; ++m) qs[m] = pfwsat(t[m], p[m]);
  return MLC_OK;
}

}  // extern "C"
