/*
 * moloch_gb300_setup.h -- host-side FP64 setup helpers of the MOLOCH step.
 *
 * These compute, on the host and once per domain, the time-invariant inputs
 * that RegCM's Fortran setup leaves in module globals before the first call
 * of moloch.  A Fortran caller keeps using its own setup and passes the
 * arrays to mlc_bind_static; a C, C++ or Python caller that has no RegCM
 * setup (the benchmark, the serving loop) builds them here.  All arrays use
 * the extents documented in moloch_gb300.h; no function touches the GPU.
 */
#ifndef MOLOCH_GB300_SETUP_H
#define MOLOCH_GB300_SETUP_H

#include "moloch_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* model_zitaf / model_zitah (Share/mod_zita.F90:54-86): zita (kz+1) from the
 * top (k=1, = ztop) to the surface (k=kz+1, = 0); zitah (kz) at mid-levels. */
int mlc_setup_levels(int kz, double ztop, double *zita, double *zitah);

/* nspgx/nspgd as initparam derives them for MOLOCH
 * (Share/mod_dynparam.F90:767-786).  ds in km. */
int mlc_setup_nspg(int jx, int iy, double ds_km, int bdy_use_lehmann,
                   int nspgx_namelist, int nspgd_namelist,
                   int *nspgx, int *nspgd);

/* compute_moloch_static (Main/mod_params.F90:3316-3395).  ht, htu, htv are
 * surface geopotential (m^2/s^2) at cross, u and v points on (jx, iy);
 * msfu/msfv (jx, iy).  Outputs: hx (jx,iy-1), hy (jx-1,iy), zeta, fmz, dz
 * (jx-1,iy-1,kz), rfmzu (jx,iy-1,kz), rfmzv (jx-1,iy,kz), fmzf and zetaf
 * (jx-1,iy-1,kz+1).  Any output pointer may be NULL. */
int mlc_setup_metric(const mlc_dims *d, const mlc_params *p,
                     const double *ht, const double *htu, const double *htv,
                     const double *msfu, const double *msfv,
                     const double *zita, const double *zitah,
                     double *hx, double *hy, double *zeta, double *fmz,
                     double *rfmzu, double *rfmzv, double *fmzf,
                     double *zetaf, double *dz);

/* exponential_nudging (Main/mpplib/mod_runparams.F90:611-637): the nudging
 * profile anudge (kz) at the half levels, from the three strengths at the
 * top, at the first full level with sigma > 0.4 and at the surface, through
 * RegCM's spline1d (Share/mod_spline.F90:387-459). */
int mlc_exponential_nudging(int kz, double ztop, double high, double medium, double low,
                            double *anudge);

/* relax_coefficients (Main/mpplib/mod_runparams.F90:648-702): Lehmann's
 * optimal relaxation weights; np must be 1 or a power of two (<= 32). */
int mlc_relax_coefficients(int np, double gmmin, double gmmax, double *coeff);

/* The MOLOCH half of setup_bdycon (Main/mod_bdycod.F90:478-560) and the
 * sponge of init (Main/mod_init.F90:1008-1025): hefc (nspgx,kz) with
 * Lehmann's weights when p->bdy_use_lehmann is set, else the exponential
 * nudging profile (exponential_nudging, Main/mpplib/mod_runparams.F90:
 * 611-637, from p->high_nudge, medium_nudge, low_nudge); fcx (nspgx) for
 * tracers (Main/chemlib/mod_che_bdyco.F90:1036-1039), the domain-mean level
 * height, nztop and tnudge (kz), ffilt (kz).  zeta is (jx-1,iy-1,kz).
 * Writes p->nztop. */
int mlc_setup_relaxation(const mlc_dims *d, mlc_params *p, const double *zeta,
                         double *hefc, double *fcx, double *tnudge,
                         double *ffilt, double *gmeanz);

/* The level weights of spectral nudging (lowpass_init, Main/mod_bdycod.F90:
 * 3890-3894): cnudge(k) = dtrad/dtbdys * min((gmeanz(k)/mo_h)^2, 1), from the
 * domain-mean level heights gmeanz (kz) of mlc_setup_relaxation. */
int mlc_setup_spectral(const mlc_params *p, int kz, const double *gmeanz, double *cnudge);

/* setup_boundaries (Main/mod_atm_interface.F90:384-545), one-process,
 * non-band domain: ibnd (jx, iy) = relaxation-zone index (>= 2) or -1.
 * ldotx/ldoty select dot (1) or cross (0) staggering in x and y:
 * ba_cr = (0,0), ba_ud = (1,0), ba_vd = (0,1). */
int mlc_setup_boundaries(int jx, int iy, int ldotx, int ldoty, int nspgx,
                         int nspgd, int32_t *ibnd);

/* paicompute (Main/mod_bdycod.F90:3762-3796): hydrostatic Exner function
 * from surface pressure ps (jx-1,iy-1) [Pa], height above ground zeta,
 * temperature t and qv (jx-1,iy-1,kz) and fmzf (jx-1,iy-1,kz+1). */
int mlc_paicompute(const mlc_dims *d, const mlc_params *p, const double *ps,
                   const double *zeta, const double *t, const double *qv,
                   const double *fmzf, const double *zita, double *pai);

/* pfwsat (Share/pfwsat.inc:1-43), elementwise over n points. */
int mlc_pfwsat(size_t n, const double *t, const double *p, double *qs);

#ifdef __cplusplus
}
#endif

#endif /* MOLOCH_GB300_SETUP_H */
