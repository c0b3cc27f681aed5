/*
 * moloch_gb300_restart.h -- SAV restart files of a MOLOCH domain.
 *
 * RegCM checkpoints the MOLOCH state in its SAV file (write_savefile,
 * Main/mod_savefile.F90:802-1324; the MOLOCH part :867-883 and :1128-1139,
 * tracers :1042-1046 and :1258-1260) and restarts from it (read_savefile
 * :594-800, the MOLOCH part :618-630; Main/mod_init.F90:421-450 copies the
 * fields into mo_atm and :941-966 derives the diagnostics).  These calls
 * write and read the MOLOCH variables of that file: the same variable and
 * dimension names, shapes and attributes, as a netCDF classic file
 * (64-bit offset format; CDF-5 when a variable exceeds 4 GiB) in FP64, which
 * the netCDF library RegCM links reads like its own.  The reader also takes
 * CDF-1 and CDF-5 files and FP32 variables (a single-precision RegCM build);
 * netCDF-4/HDF5 files are refused with MLC_ERR_UNSUPPORTED.  The surface,
 * radiation and physics variables of a full SAV file are outside this path
 * and are neither written nor needed.
 */
#ifndef MOLOCH_GB300_RESTART_H
#define MOLOCH_GB300_RESTART_H

#include <stddef.h>

#include "moloch_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The MOLOCH fields of a SAV file, Fortran arrays with the extents of a
 * one-process run.  Read by mlc_sav_write, filled by mlc_sav_read. */
typedef struct mlc_sav_fields {
  double *u;     /* atm_u   (jx,iy-1,kz)        dims (jdot,icross,khalf)        */
  double *v;     /* atm_v   (jx-1,iy,kz)        dims (jcross,idot,khalf)        */
  double *w;     /* atm_w   (jx-1,iy-1,kz+1)    dims (jcross,icross,kfull)      */
  double *t;     /* atm_t   (jx-1,iy-1,kz)                                      */
  double *pai;   /* atm_pai (jx-1,iy-1,kz)                                      */
  double *qx;    /* atm_qx  (jx-1,iy-1,kz,nqx)  dims (jcross,icross,khalf,nqx)  */
  double *ps;    /* ps      (jx-1,iy-1)                                         */
  double *trac;  /* trac    (jx-1,iy-1,kz,ntr)  only when ntr > 0 (ichem = 1)   */
  double *tke;   /* atm_tke (jx-1,iy-1,kz+1)    dims (jcross,icross,kfull);
                    written and read when not NULL (ibltyp = 2)               */
} mlc_sav_fields;

/* Write the fields to `path` with the global attributes idatex and
 * calendar (saveready, Main/mod_savefile.F90:2099-2169; NULL: omitted). */
int mlc_sav_write(const char *path, const mlc_dims *d, const mlc_sav_fields *f,
                  const char *idatex, const char *calendar);

/* Read the fields of `path` into f (every pointer but trac required; trac
 * when d->ntr > 0).  The file's dimensions must equal d: MLC_ERR_INVALID
 * otherwise, or when a variable is missing.  idatex (optional, idatex_len
 * bytes) receives the file's idatex attribute. */
int mlc_sav_read(const char *path, const mlc_dims *d, const mlc_sav_fields *f, char *idatex,
                 size_t idatex_len);

/* The restart state of Main/mod_init.F90:421-450,941-966 from the SAV fields:
 * u, v, w, t, pai, qx, trac and ps copied; p = pai^(cp/R)*p00,
 * qsat = pfwsat(t,p), rho = p/(R t), tvirt = t*(1 + ep1*qv),
 * tetav = tvirt/pai; ux and vx zero (advection rebuilds them from u and v
 * before it reads them). */
int mlc_sav_restart_state(const mlc_dims *d, const mlc_sav_fields *f, const mlc_state_ptrs *st);

/* Snapshot member m of a context (its state on the device) into a SAV file;
 * MLC_ERR_STATE inside a step split at the physics. */
int mlc_member_write_sav(mlc_ctx *ctx, int m, const char *path, const char *idatex,
                         const char *calendar);

/* Restart member m from a SAV file: mlc_sav_read, mlc_sav_restart_state and
 * mlc_member_upload_state.  The boundary data and clock come with
 * mlc_member_set_boundary, as bdyin restores them from the restart date. */
int mlc_member_read_sav(mlc_ctx *ctx, int m, const char *path);

#ifdef __cplusplus
}
#endif

#endif
