// mlc_constants.h -- physical constants of the MOLOCH path.
//
// Values and derivations of Share/mod_constants.F90 (non-RCEMIP build):
// egrav :107, boltzk :115, navgdr :117, amd :130, amw :132, rgasmol :153,
// rgas :161, cpd :181, cvd :185, derived ratios :225-233, tzero :241,
// p00 :273, lrate :282, pi :301, degrad :307, earth radius :350-355,
// rotation :358-360, ep1/ep2 :383-386.  Each derived value is the same IEEE
// double operation the Fortran parameter expression performs, so host and
// device code see bit-identical constants.
#pragma once
#include <cmath>

#ifdef __CUDACC__
#define MLC_HD __host__ __device__
#else
#define MLC_HD
#endif

namespace mlc {

constexpr double kGrav = 9.80665;
constexpr double kBoltz = 1.3806490e-23;
constexpr double kAvogadro = 6.02214076e23;
constexpr double kAmd = 28.96454;
constexpr double kAmw = 18.01528;
constexpr double kRgasMol = kAvogadro * kBoltz;
constexpr double kRgas = (kRgasMol / kAmd) * 1000.0;
constexpr double kCpd = 3.5 * kRgas;
constexpr double kCvd = 2.5 * kRgas;
constexpr double kRegrav = 1.0 / kGrav;
constexpr double kRcpd = 1.0 / kCpd;
constexpr double kRovcp = kRgas * kRcpd;
constexpr double kRdrcv = kRgas / kCvd;
constexpr double kCpovr = kCpd / kRgas;
constexpr double kGovr = kGrav / kRgas;
constexpr double kGovcp = kGrav / kCpd;
constexpr double kTzero = 273.15;
constexpr double kP00 = 1.000000e5;
constexpr double kLrate = 0.00649;
constexpr double kPi = 3.14159265358979323846;
constexpr double kDegrad = kPi / 180.0;
constexpr double kEarthRad = 6.371229e6;
constexpr double kRearthRad = 1.0 / kEarthRad;
constexpr double kOmega2 = 2.0 * 7.2921159e-5;
constexpr double kEp1 = kAmd / kAmw - 1.0;
constexpr double kEp2 = kAmw / kAmd;

// Main/mpplib/mod_runparams.F90:184-192 (qv, qc, qi, qr, qs, qg, qh, ...):
// values below qxcheckval(n) are reset to qxzeroval(n) (0-based n here).
MLC_HD inline double qx_check(int n) {
  switch (n) {
    case 0: return 1.0e-8;
    case 7: return 1.0e10;
    case 8: return 100.0;
    case 9: return 0.01;
    default: return 1.0e-16;
  }
}
MLC_HD inline double qx_zero(int n) {
  switch (n) {
    case 0: return 1.0e-8;
    case 7: return 1.0e10;
    case 8: return 100.0;
    case 9: return 0.01;
    default: return 0.0;
  }
}

// Floor of the turbulent kinetic energy with the UW PBL (ibltyp = 2):
// tkemin = uwtkemin (Main/mod_pbl_interface.F90:68, Main/pbllib/mod_pbl_uwtcm.F90:81).
constexpr double kTkeMin = 1.0e-3;

// Height above which top nudging and the w sponge act (Main/mod_bdycod.F90:121).
constexpr double kZzTop = 18000.0;
// Sponge amplitude (Main/mod_init.F90:62).
constexpr double kZfiltFac = 0.8;
// Base damping coefficients (Main/mod_moloch.F90:147-148).
constexpr double kNuMax = 0.125;
constexpr double kDdamp = 0.850;

// Flatau saturation mixing ratio in kg/kg, Share/pfwsat.inc:1-43.  The
// polynomial is evaluated in Horner form from the highest coefficient, the
// same nesting as the reference.
MLC_HD inline double pfwsat(double t, double p) {
  double td = t - kTzero;
  td = td < -75.0 ? -75.0 : td;
  td = td > 100.0 ? 100.0 : td;
  double es;
  if (td >= 0.0) {
    es = 0.611213476e+03 + td * (0.444007856e+02 + td * (0.143064234e+01 +
         td * (0.264461437e-01 + td * (0.305903558e-03 + td * (0.196237241e-05 +
         td * (0.892344772e-08 + td * (-0.373208410e-10 + td * 0.209339997e-13)))))));
  } else {
    es = 0.611123516e+03 + td * (0.503109514e+02 + td * (0.188369801e+01 +
         td * (0.420547422e-01 + td * (0.614396778e-03 + td * (0.602780717e-05 +
         td * (0.387940929e-07 + td * (0.149436277e-09 + td * 0.262655803e-12)))))));
  }
  double cap = 0.15 * p;
  es = cap < es ? cap : es;
  return kEp2 * (es / (p - es));
}

// pfwsat in FP32 for the diagnostics of a mixed member (stored in FP32).
MLC_HD inline float pfwsat_f(float t, float p) {
  float td = t - float(kTzero);
  td = td < -75.f ? -75.f : td;
  td = td > 100.f ? 100.f : td;
  float es;
  if (td >= 0.f) {
    es = 0.611213476e+03f + td * (0.444007856e+02f + td * (0.143064234e+01f +
         td * (0.264461437e-01f + td * (0.305903558e-03f + td * (0.196237241e-05f +
         td * (0.892344772e-08f + td * (-0.373208410e-10f + td * 0.209339997e-13f)))))));
  } else {
    es = 0.611123516e+03f + td * (0.503109514e+02f + td * (0.188369801e+01f +
         td * (0.420547422e-01f + td * (0.614396778e-03f + td * (0.602780717e-05f +
         td * (0.387940929e-07f + td * (0.149436277e-09f + td * 0.262655803e-12f)))))));
  }
  float cap = 0.15f * p;
  es = cap < es ? cap : es;
  return float(kEp2) * (es / (p - es));
}

// p = pai**(cp/R) * p00 (Main/mod_moloch.F90:349).  cp/R evaluates to 3.5
// exactly in IEEE double (cpd = 3.5*rgas), so pai**3.5 = pai^3 * sqrt(pai):
// three multiplies and a square root instead of pow, equal to a few ulp.
static_assert(kCpovr == 3.5, "cp/R must be 3.5 for the pai^3*sqrt(pai) form");
MLC_HD inline double exner_to_pressure(double pai) {
  return pai * pai * pai * sqrt(pai) * kP00;
}
MLC_HD inline float exner_to_pressure_f(float pai) {
  return pai * pai * pai * sqrtf(pai) * float(kP00);
}

// G(zeta) of Share/mod_zita.F90:105-115.
MLC_HD inline double gzita(double zita, double ztop, double a0) {
  double r = zita / ztop;
  double r2 = r * r;
  double r3 = r2 * r;
  return ((0.0 - 1.0 * a0) * r - (3.0 - 2.0 * a0) * r2 + (2.0 - 1.0 * a0) * r3) + 1.0;
}

}  // namespace mlc
