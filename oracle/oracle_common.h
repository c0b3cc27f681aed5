// oracle_common.h -- TEST INFRASTRUCTURE ONLY.
//
// Shared pieces of the CPU oracle: Fortran-style arrays with explicit lower
// bounds (so every loop range reads like the reference's), and the physical
// constants of Share/mod_constants.F90 (non-RCEMIP branch), each evaluated in
// IEEE double exactly as the Fortran parameter expressions are.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use the
// oracle, as the checker.  The product library never links it.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace orc {

// Share/mod_constants.F90 (non-RCEMIP)
constexpr double egrav = 9.80665;                         // :107
constexpr double boltzk = 1.3806490e-23;                  // :115
constexpr double navgdr = 6.02214076e23;                  // :117
constexpr double amd = 28.96454;                          // :130
constexpr double amw = 18.01528;                          // :132
constexpr double rgasmol = navgdr * boltzk;               // :153
constexpr double rgas = (rgasmol / amd) * 1000.0;         // :161
constexpr double cpd = 3.5 * rgas;                        // :181
constexpr double cvd = 2.5 * rgas;                        // :185
constexpr double d_one = 1.0;
constexpr double regrav = d_one / egrav;                  // :225-233
constexpr double rcpd = d_one / cpd;
constexpr double rovcp = rgas * rcpd;
constexpr double rdrcv = rgas / cvd;
constexpr double cpovr = cpd / rgas;
constexpr double govr = egrav / rgas;
constexpr double govcp = egrav / cpd;
constexpr double tzero = 273.15;                          // :241
constexpr double p00 = 1.000000e5;                        // :273
constexpr double stdp = 1.013250e5;
constexpr double stdt = 288.15;
constexpr double lrate = 0.00649;                         // :282
constexpr double mathpi = 3.14159265358979323846;         // :301,307
constexpr double degrad = mathpi / 180.0;
constexpr double earthrad = 6.371229e6;                   // :350,355
constexpr double rearthrad = 1.0 / earthrad;
constexpr double eomeg = 7.2921159e-5;                    // :358-360
constexpr double eomeg2 = 2.0 * eomeg;
constexpr double ep1 = amd / amw - d_one;                 // :383-386
constexpr double ep2 = amw / amd;

// Main/mpplib/mod_runparams.F90:184-192
// tkemin of the UW PBL (ibltyp = 2): Main/mod_pbl_interface.F90:68 takes
// uwtkemin, Main/pbllib/mod_pbl_uwtcm.F90:81
constexpr double tkemin = 1.0e-3;
constexpr double qxcheckval[10] = {1.0e-8, 1.0e-16, 1.0e-16, 1.0e-16, 1.0e-16,
                                   1.0e-16, 1.0e-16, 1.0e10, 100.0, 0.01};
constexpr double qxzeroval[10] = {1.0e-8, 0.0, 0.0, 0.0, 0.0,
                                  0.0, 0.0, 1.0e10, 100.0, 0.01};

// 2-D array with Fortran lower bounds, j fastest.
template <class T>
struct F2 {
  int j1 = 1, j2 = 0, i1 = 1, i2 = 0, nj = 0;
  std::vector<T> d;
  F2() = default;
  F2(int j1_, int j2_, int i1_, int i2_, T v = T(0)) { init(j1_, j2_, i1_, i2_, v); }
  void init(int j1_, int j2_, int i1_, int i2_, T v = T(0)) {
    j1 = j1_; j2 = j2_; i1 = i1_; i2 = i2_; nj = j2 - j1 + 1;
    d.assign((size_t)nj * (i2 - i1 + 1), v);
  }
  T &operator()(int j, int i) { return d[(size_t)(j - j1) + (size_t)(i - i1) * nj]; }
  const T &operator()(int j, int i) const { return d[(size_t)(j - j1) + (size_t)(i - i1) * nj]; }
};

// 3-D array with Fortran lower bounds, j fastest then i then k.
struct F3 {
  int j1 = 1, j2 = 0, i1 = 1, i2 = 0, k1 = 1, k2 = 0, nj = 0, ni = 0;
  std::vector<double> d;
  F3() = default;
  F3(int j1_, int j2_, int i1_, int i2_, int k1_, int k2_) { init(j1_, j2_, i1_, i2_, k1_, k2_); }
  void init(int j1_, int j2_, int i1_, int i2_, int k1_, int k2_, double v = 0.0) {
    j1 = j1_; j2 = j2_; i1 = i1_; i2 = i2_; k1 = k1_; k2 = k2_;
    nj = j2 - j1 + 1; ni = i2 - i1 + 1;
    d.assign((size_t)nj * ni * (k2 - k1 + 1), v);
  }
  double &operator()(int j, int i, int k) {
    return d[(size_t)(j - j1) + (size_t)nj * ((size_t)(i - i1) + (size_t)ni * (size_t)(k - k1))];
  }
  const double &operator()(int j, int i, int k) const {
    return d[(size_t)(j - j1) + (size_t)nj * ((size_t)(i - i1) + (size_t)ni * (size_t)(k - k1))];
  }
  void load(const double *src) { std::memcpy(d.data(), src, d.size() * sizeof(double)); }
  void store(double *dst) const { std::memcpy(dst, d.data(), d.size() * sizeof(double)); }
};

}  // namespace orc
