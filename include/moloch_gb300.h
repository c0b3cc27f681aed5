/*
 * moloch_gb300.h -- C ABI of the GB300 (sm_103a) MOLOCH dynamical-core step.
 *
 * This library replaces the three public procedures of RegCM's MOLOCH module
 *   public :: allocate_moloch, init_moloch, moloch      (Main/mod_moloch.F90:127)
 * which take no arguments and work on module globals.  Here the same state is
 * passed explicitly, as plain host pointers in the reference's own layout:
 * Fortran column-major (j fastest, then i, then k, then species n), with the
 * extents a one-process, non-periodic RegCM run gives them (every ga/gb halo
 * collapses to zero, Main/mod_atm_interface.F90:204-233,286-309):
 *
 *   dot 2-D   (jx, iy)            msfu, msfv, msfx, ibnd_*
 *   u points  (jx, iy-1[, kz])    u, hx, rfmzu, dub, ulat     (jde, ice)
 *   v points  (jx-1, iy[, kz])    v, hy, rfmzv, dvb, vlat     (jce, ide)
 *   cross     (jx-1, iy-1[, kz])  pai, tetav, t, tvirt, ux, vx, p, rho, qsat,
 *                                 fmz, zeta, dz, xtb, xqb, xpaib, xlb, xib, ps
 *   w levels  (jx-1, iy-1, kz+1)  w, fmzf
 *   species   (jx-1, iy-1, kz, n) qx (n = nqx), trac and chib (n = ntr)
 *
 * jx and iy are the reference's dot-point extents (namelist dimparam); the
 * cross-point grid is (jx-1) x (iy-1).  k = 1 is the model top.
 *
 * Status codes: 0 = OK, negative = error (mlc_strerror gives the text).  The
 * Fortran shim maps a negative status to RegCM's fatal() the way the reference
 * aborts (Share/mod_message.F90:86-99).  The library never frees caller memory.
 * One context owns one CUDA stream and its device arena; a context is not
 * thread-safe, distinct contexts may be driven from distinct host threads.
 */
#ifndef MOLOCH_GB300_H
#define MOLOCH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define MLC_OK                 0
#define MLC_ERR_INVALID       -1  /* bad argument, extent or parameter      */
#define MLC_ERR_UNSUPPORTED   -2  /* option outside the built path          */
#define MLC_ERR_CUDA          -3  /* CUDA runtime error                     */
#define MLC_ERR_NOMEM         -4  /* device allocation failed               */
#define MLC_ERR_STATE         -5  /* call order violated (e.g. no static)   */
#define MLC_ERR_NONFINITE     -6  /* NaN/Inf in ps: "CFL VIOLATION"         */
#define MLC_ERR_NODEVICE      -7  /* no CUDA device visible                 */
#define MLC_ERR_BUDGET        -8  /* request exceeds the device budget      */
#define MLC_ERR_TOO_LARGE     -9  /* size beyond a fixed maximum            */

/* ---- precision modes --------------------------------------------------- */
#define MLC_PREC_FP64   0  /* every field and operation in FP64            */
#define MLC_PREC_MIXED  1  /* FP32 fields and horizontal stencils; FP64
                              vertical implicit solve, Exner/pressure and
                              mass budget sums                             */

/* Domain extents.  Reference names in brackets. */
typedef struct mlc_dims {
  int32_t jx;    /* dot points west->east            [jx, dimparam]       */
  int32_t iy;    /* dot points south->north          [iy, dimparam]       */
  int32_t kz;    /* full levels, k=1 at the top      [kz]                 */
  int32_t nqx;   /* water species in qx, qv first    [nqx, mod_params]    */
  int32_t ntr;   /* passive tracers in trac (ichem=1 when > 0) [ntr]      */
} mlc_dims;

/* Run parameters (Share/mod_dynparam.F90:141-152,203-211,
 * Main/mpplib/mod_runparams.F90).  Defaults: mlc_default_params(). */
typedef struct mlc_params {
  double  dtsec;          /* model step [s]                      [dtsec]   */
  double  dx;             /* grid spacing [m]                    [dx]      */
  double  mo_ztop;        /* model top [m]                       [mo_ztop] */
  double  mo_h;           /* decay height of b(zeta) [m]         [mo_h]    */
  double  mo_a0;          /* G(zeta) shape parameter             [mo_a0]   */
  double  dtbdys;         /* boundary data interval [s]          [dtbdys]  */
  int32_t mo_nadv;        /* advection steps per dt              [mo_nadv] */
  int32_t mo_nsound;      /* acoustic substeps per advection step          */
  int32_t mo_divdamp;     /* divergence damping on/off           [mo_divdamp]   */
  int32_t mo_divfilter;   /* divergence filter on/off            [mo_divfilter] */
  int32_t mo_top_nudge;   /* top nudging on/off                  [mo_top_nudge] */
  int32_t mo_spectral_nudge; /* spectral nudging on/off          [mo_spectral_nudge] */
  int32_t do_apply_bdy;   /* lateral boundary relaxation on/off [do_apply_bdy] */
  int32_t lrotllr;        /* ROTLLR projection branch            [iproj]   */
  int32_t ipptls;         /* microphysics class 0-5: nqx 2 (0, 1), 5 (2, 3),
                             7 (4), 10 (5)                      [ipptls]  */
  int32_t present_qc;     /* boundary data carries qc            [present_qc] */
  int32_t present_qi;     /* boundary data carries qi            [present_qi] */
  int32_t nspgx;          /* relaxation zone width, cross points [nspgx]   */
  int32_t nspgd;          /* relaxation zone width, dot points   [nspgd]   */
  int32_t nztop;          /* levels nudged at the top            [nztop]   */
  int32_t debug_level;    /* > 0: mass budget every step         [debug_level] */
  int32_t precision;      /* MLC_PREC_FP64 or MLC_PREC_MIXED               */
  double  dtrad;          /* spectral nudging interval [s] (radiation step) [dtrad] */
  int32_t bdy_use_lehmann; /* relaxation weights: Lehmann's (1) or exponential
                              nudging (0)                     [bdy_use_lehmann] */
  int32_t ibltyp;         /* PBL scheme; 2 (UW) carries TKE, advected with
                             the step                         [ibltyp]  */
  double  high_nudge;     /* exponential nudging strength at the top,   */
  double  medium_nudge;   /* near sigma 0.4 and at the surface          */
  double  low_nudge;      /*          [high_nudge, medium_nudge, low_nudge] */
} mlc_params;

/* Time-invariant fields (host pointers, read once by mlc_bind_static).
 * Reference: mddom%*, mo_atm%fmz/fmzf/rfmzu/rfmzv/zeta/dz, hefc, tnudge,
 * ffilt, zita/zitah and ba_cr/ba_ud/ba_vd%ibnd. */
typedef struct mlc_static_ptrs {
  const double  *msfu, *msfv, *msfx;  /* (jx,iy) map factors               */
  const double  *ulat;                /* (jx,iy-1) latitude of u points    */
  const double  *vlat;                /* (jx-1,iy) latitude of v points    */
  const double  *rlat;                /* (iy) row latitude (ROTLLR only)   */
  const double  *hx;                  /* (jx,iy-1)  terrain slope at u     */
  const double  *hy;                  /* (jx-1,iy)  terrain slope at v     */
  const double  *fmz;                 /* (jx-1,iy-1,kz)                     */
  const double  *fmzf;                /* (jx-1,iy-1,kz+1)                   */
  const double  *rfmzu;               /* (jx,iy-1,kz)                       */
  const double  *rfmzv;               /* (jx-1,iy,kz)                       */
  const double  *zeta;                /* (jx-1,iy-1,kz) height above ground */
  const double  *dz;                  /* (jx-1,iy-1,kz) layer depth         */
  const double  *zita;                /* (kz+1) full-level zita             */
  const double  *zitah;               /* (kz)   half-level zita             */
  const double  *ffilt;               /* (kz) implicit-w sponge             */
  const double  *hefc;                /* (nspgx,kz) relaxation weights      */
  const double  *fcx;                 /* (nspgx) tracer relaxation weights  */
  const double  *tnudge;              /* (kz) top-nudging profile           */
  const int32_t *ibnd_cr;             /* (jx,iy) zone index, cross points   */
  const int32_t *ibnd_ud;             /* (jx,iy) zone index, u points       */
  const int32_t *ibnd_vd;             /* (jx,iy) zone index, v points       */
  const double  *cnudge;              /* (kz) spectral nudging weights (read
                                         only when mo_spectral_nudge)       */
} mlc_static_ptrs;

/* Prognostic and diagnostic state (mo_atm fields, sfs%psa). */
typedef struct mlc_state_ptrs {
  double *u;      /* (jx,iy-1,kz)     */
  double *v;      /* (jx-1,iy,kz)     */
  double *w;      /* (jx-1,iy-1,kz+1) */
  double *pai;    /* Exner function   */
  double *tetav;  /* virtual potential temperature */
  double *t;      /* temperature      */
  double *tvirt;  /* virtual temperature */
  double *ux;     /* u at cross points */
  double *vx;     /* v at cross points */
  double *p;      /* pressure         */
  double *rho;    /* density          */
  double *qsat;   /* saturation mixing ratio */
  double *qx;     /* (jx-1,iy-1,kz,nqx) */
  double *trac;   /* (jx-1,iy-1,kz,ntr), may be NULL when ntr = 0 */
  double *ps;     /* (jx-1,iy-1) surface pressure */
  double *tke;    /* (jx-1,iy-1,kz+1) turbulent kinetic energy [m2/s2] at
                     the interfaces; used when ibltyp = 2, else may be NULL */
} mlc_state_ptrs;

/* Lateral boundary data: index 0 = b0, 1 = b1 (v3dbound%b0/%b1). */
typedef struct mlc_bdy_ptrs {
  const double *xtb[2];   /* (jx-1,iy-1,kz) temperature        */
  const double *xqb[2];   /* (jx-1,iy-1,kz) qv                 */
  const double *xpaib[2]; /* (jx-1,iy-1,kz) Exner              */
  const double *xlb[2];   /* (jx-1,iy-1,kz) qc (present_qc)    */
  const double *xib[2];   /* (jx-1,iy-1,kz) qi (present_qi)    */
  const double *dub[2];   /* (jx,iy-1,kz)   u                  */
  const double *dvb[2];   /* (jx-1,iy,kz)   v                  */
  const double *xpsb[2];  /* (jx-1,iy-1)    surface pressure   */
  const double *chib[2];  /* (jx-1,iy-1,kz,ntr) tracers        */
} mlc_bdy_ptrs;

/* Per-step diagnostics (Main/mod_moloch.F90:407-422, Main/mod_massck.F90). */
typedef struct mlc_diag {
  double  ps_max, ps_min;   /* over interior cross points [Pa]          */
  int32_t nonfinite;        /* 1 when ps max/min is NaN or Inf          */
  int32_t steps_done;       /* steps completed by this call             */
  double  drymass;          /* sum dx^2 dz rho, interior [kg]           */
  double  dryadv;           /* dry-air boundary flux over dt [kg]       */
  double  qmass;            /* sum of qx dx^2 dz rho, interior [kg]     */
  double  qadv;             /* water boundary flux over dt [kg]         */
  double  xbctime;          /* boundary clock after the call [s]        */
} mlc_diag;

typedef struct mlc_ctx mlc_ctx;

/* Fill p with the reference defaults (mod_dynparam / mod_runparams). */
void mlc_default_params(mlc_params *p);

/* allocate_moloch (Main/mod_moloch.F90:159-199): validate extents and
 * parameters, pick device 0 (or the current device), allocate the device
 * arena.  No state is valid until mlc_bind_static + mlc_upload_state. */
int mlc_create(const mlc_dims *dims, const mlc_params *params, mlc_ctx **out);

/* The static half of init_moloch (Main/mod_moloch.F90:201-308) plus the
 * fields compute_moloch_static leaves in mddom/mo_atm
 * (Main/mod_params.F90:3316-3395): copied to the device once; the library
 * derives coriolis, 1/m, m^2, G(zeta), xkdamp, xknu and bdywt{u,v,w}. */
int mlc_bind_static(mlc_ctx *ctx, const mlc_static_ptrs *s);

/* Copy the host state into the device arena (init from b0 or restart,
 * Main/mod_init.F90:155-219).  Sets w(:,:,1) = 0 as init_moloch does. */
int mlc_upload_state(mlc_ctx *ctx, const mlc_state_ptrs *st);

/* Copy the device state back into the host arrays (NULL members skipped). */
int mlc_download_state(mlc_ctx *ctx, const mlc_state_ptrs *st);

/* Boundary arrays b0/b1 and the boundary clock (xbctime, dtbdys), the data
 * bdyin (Main/mod_bdycod.F90:1079-1200) leaves for bdyval and morelax.  Each
 * step advances xbctime by dtsec, as bdyval does (mod_bdycod.F90:2653). */
int mlc_set_boundary(mlc_ctx *ctx, const mlc_bdy_ptrs *b, double xbctime,
                     double dtbdys);

/* moloch (Main/mod_moloch.F90:312-446) nsteps times: dynamical core,
 * boundary relaxation, diagnostics, mkslice's edits of the state, status
 * update, mass budget (when debug_level > 0) and the NaN/Inf check on ps.
 * Physics is not part of this path: tendencies are zero (the split step
 * below takes them).  out (optional) receives the diagnostics
 * of the last step.  Returns MLC_ERR_NONFINITE when ps is not finite. */
int mlc_step(mlc_ctx *ctx, int nsteps, mlc_diag *out);

/* Release the device arena and stream. */
void mlc_destroy(mlc_ctx *ctx);

/* Text for a status code. */
const char *mlc_strerror(int status);

/* Text of the CUDA error behind the last MLC_ERR_CUDA / MLC_ERR_NOMEM
 * returned on the calling thread. */
const char *mlc_last_error(void);

/* ---- ensembles, uneven batches and a serving pool: several domains (the
 * members) advanced by the same kernel launches.  Each member owns its
 * arena and is described to the kernels by one entry of a device table;
 * every kernel stage is one launch whose grid covers the largest member, so
 * one recorded graph replays the step of all members.  Members share the
 * parameters (dt, substeps, options, precision) and may differ in anything
 * else: extents, levels, terrain, state, boundary data and boundary clock.
 * A member's result does not depend on the other members (bit for bit).
 * mlc_create is mlc_create_batch with nmem = 1 and the single-domain calls
 * address member 0.  No counterpart in the reference, where an ensemble is
 * a set of separate runs (Share/mod_ensemble.F90). */
int mlc_create_batch(const mlc_dims *dims, const mlc_params *params, int nmem, mlc_ctx **out);
/* nmem members with extents dims[0..nmem-1]. */
int mlc_create_multi(const mlc_dims *dims, const mlc_params *params, int nmem, mlc_ctx **out);
/* Member slots of the context (the size of the diagnostics array). */
int mlc_members(const mlc_ctx *ctx);
int mlc_member_bind_static(mlc_ctx *ctx, int m, const mlc_static_ptrs *s);
int mlc_member_upload_state(mlc_ctx *ctx, int m, const mlc_state_ptrs *st);
int mlc_member_download_state(mlc_ctx *ctx, int m, const mlc_state_ptrs *st);
int mlc_member_set_boundary(mlc_ctx *ctx, int m, const mlc_bdy_ptrs *b, double xbctime,
                            double dtbdys);
/* nsteps steps of every active member; out (optional) receives one entry per
 * slot (steps_done = 0 for empty slots). */
int mlc_step_batch(mlc_ctx *ctx, int nsteps, mlc_diag *out);

/* ---- physics coupling: the step split at the physics
 * (Main/mod_moloch.F90:354-376).  mlc_step_dynamics runs every active
 * member through the dynamical core, the boundary, p/rho/qsat, the surface
 * pressure and the edits mkslice makes to the state (Main/mod_slice.F90:
 * 110-147: the qx and tracer floors); the state is then the one the physics
 * reads (mlc_member_download_state returns it).  The physics' tendencies go
 * in with mlc_member_set_tendencies; mlc_step_finish applies status_update
 * (:1403-1443) with them, the mass budget and the ps check, and ends the
 * step (out, optional: one entry per slot).  Tendencies are zero at every
 * step's start (reset_tendencies :1044-1083): a member without
 * set_tendencies gets zero, NULL arrays are zero, and mlc_step equals
 * mlc_step_dynamics + mlc_step_finish with no tendencies.  While a step is
 * open, calls that step, upload, bind, add or remove members or change
 * launch shapes return MLC_ERR_STATE; download_state and set_tendencies are
 * accepted.  Split steps launch their kernels one by one (no graph). */
typedef struct mlc_tend_ptrs {
  const double *tten;    /* (jx-3,iy-3,kz) temperature tendency on jci x ici [K/s]  */
  const double *uten;    /* (jx-3,iy-3,kz) zonal wind (cross points) [m/s^2]        */
  const double *vten;    /* (jx-3,iy-3,kz) meridional wind (cross points) [m/s^2]   */
  const double *qxten;   /* (jx-3,iy-3,kz,nqx) water species [kg/kg/s]              */
  const double *chiten;  /* (jx-3,iy-3,kz,ntr) tracers                              */
  const double *tketen;  /* (jx-3,iy-3,kz+1) TKE (ibltyp = 2) [m2/s3]                */
} mlc_tend_ptrs;
int mlc_step_dynamics(mlc_ctx *ctx);
int mlc_member_set_tendencies(mlc_ctx *ctx, int m, const mlc_tend_ptrs *t);
int mlc_step_finish(mlc_ctx *ctx, mlc_diag *out);

/* Serving pool: a context of `capacity` empty slots whose members join and
 * leave between steps (continuous batching).  A join allocates the member's
 * arena from the context's stream-ordered pool; it is refused with
 * MLC_ERR_BUDGET when the bytes held by all members would exceed
 * budget_bytes (0: no bound) and with MLC_ERR_BUDGET when no slot is free.
 * A joined member needs bind_static, upload_state and (with boundaries)
 * set_boundary before the next step. */
int mlc_create_pool(const mlc_params *params, int capacity, size_t budget_bytes, mlc_ctx **out);
int mlc_pool_add(mlc_ctx *ctx, const mlc_dims *dims, int *slot);
int mlc_pool_remove(mlc_ctx *ctx, int slot);
/* Device bytes held by the members' arenas. */
size_t mlc_pool_bytes(const mlc_ctx *ctx);
/* Exact arena bytes of one member with these extents and parameters. */
size_t mlc_member_footprint(const mlc_dims *dims, const mlc_params *params);

/* Launch shapes picked by mlc_autotune, and the per-step device time of the
 * tuned kernels against the fixed 32x8 configuration (column kernels and
 * horizontal WAF tiles 32x8; vertical WAF blocks of 32 x 8 columns, one
 * thread per column; solve 32x2). */
typedef struct mlc_tune_report {
  int32_t col_x, col_y;      /* column kernels                        */
  int32_t solve_x, solve_y;  /* accepted for compatibility and reported;
                                the solves run on 128-column row
                                segments whatever these say            */
  int32_t vert_x, vert_y;    /* vertical WAF passes                   */
  int32_t htile;             /* horizontal WAF tile, columns x rows:
                                0 32x8, 1 64x8, 2 64x4, 3 32x4        */
  double  ms_fixed;          /* tuned kernel groups, fixed shapes [ms/step] */
  double  ms_tuned;          /* the same groups, picked shapes [ms/step]    */
} mlc_tune_report;

/* Try candidate launch shapes on this context's own state (snapshotted and
 * restored, so the state is unchanged afterwards), keep the fastest per
 * kernel group, and re-record the step graphs.  No counterpart in the
 * reference. */
int mlc_autotune(mlc_ctx *ctx, int steps_per_trial, mlc_tune_report *rep);

/* Apply launch shapes, e.g. a report saved from mlc_autotune on the same
 * workload (its ms fields are ignored).  Each shape must be one of the
 * autotuner's candidates, else MLC_ERR_INVALID and nothing changes.  Results
 * do not depend on the shapes. */
int mlc_set_launch_shapes(mlc_ctx *ctx, const mlc_tune_report *shapes);

/* Device bytes one domain of these extents holds (for admission control). */
size_t mlc_footprint_bytes(const mlc_dims *dims, int precision);

/* ---- measurement and tracing (no counterpart in the reference, which
 * times moloch with system_clock timers, Main/mpplib/mod_service.F90) ---- */

/* mlc_step plus the device time of the steps, from CUDA events recorded on
 * the context stream around the step launches. */
int mlc_step_timed(mlc_ctx *ctx, int nsteps, mlc_diag *out, float *ms);

typedef struct mlc_kernel_time {
  char    name[32];
  int32_t launches;
  double  ms;
} mlc_kernel_time;

/* Run nsteps steps without graph replay, with events around every kernel
 * group; returns the per-group launch count and total device time. */
int mlc_profile_steps(mlc_ctx *ctx, int nsteps, mlc_kernel_time *out, int max_out,
                      int *n_out);

/* Kernels one step launches (known after the first step). */
int mlc_launches_per_step(const mlc_ctx *ctx);

/* Record steps into CUDA graphs (default 1) or launch them one by one (0). */
int mlc_set_graphs(mlc_ctx *ctx, int on);

/* Test hook of the bounded device waits (no counterpart in the reference).
 * With polls > 0, every block of the member's horizontal WAF waits, before
 * it issues any copy, on an mbarrier that nothing completes, gives up after
 * `polls` polls and records the fault the way a tile copy that never lands
 * does: the step then returns MLC_ERR_CUDA ("a bounded device wait gave
 * up") and the member's state is not valid.  Nothing faults or hangs on the
 * GPU.  0 (the default) turns the hook off. */
int mlc_member_test_stall(mlc_ctx *ctx, int member, int polls);

/* Mixed precision only (no counterpart in the reference): the implicit
 * w-Exner solve's Thomas recurrence and back substitution in double-float
 * arithmetic, about 48 significant bits (1, the default), or in FP32 (0).
 * The solve's right-hand side (hydrostatic balance) and the Exner update
 * are double-float either way.  Takes effect at the next step. */
int mlc_set_solve_precision(mlc_ctx *ctx, int df_recurrence);

/* FP64 throughput of the current device (no counterpart in the reference):
 * independent FP64 multiply-add chains on every SM, the best of `repeats`
 * timed launches, in FLOP/s (a multiply-add counts two).  The plain FP64
 * step is bound by this pipe on GB300; benchmarks report against it. */
int mlc_fp64_peak(int repeats, double *flops);

/* ---- mass budget without allocation (no counterpart in the reference) --
 * For callers that own their device memory and cannot let the library call
 * cudaMalloc (a host model whose memory manager owns the device heap, code
 * in callbacks or inside graph capture): the mass budget of
 * Main/mod_massck.F90:77-170 from caller-owned DEVICE arrays in the packed
 * layout above (rho, dz: cross 3-D; qx: cross 3-D x nqx; u, v: staggered
 * 3-D; ps: cross 2-D).  out (device) receives 7 doubles: drymass, dryadv,
 * qmass, qadv, ps max, ps min, non-finite flag.  dt is the model step.
 * Partial sums live in a fixed 256 KiB file-scope device array, so domains
 * with more than 32768 rows ((iy-1)*kz) get MLC_ERR_TOO_LARGE.  The first
 * call on each device looks up that array's address: make it before any
 * stream capture.  The address is kept with the id of the CUDA context it
 * was taken in and looked up again when the current context differs (after
 * cudaDeviceReset the module loads at a new address); a call that does the
 * lookup again must also come outside a capture.  Kernels are enqueued on
 * `stream` (a cudaStream_t, NULL = default stream) and the call returns
 * without waiting; calls that overlap on the GPU share the array and race,
 * so serialise them. */
int mlc_mass_budget_noalloc(const mlc_dims *d, double dx, double dt, const double *rho,
                            const double *dz, const double *qx, const double *u,
                            const double *v, const double *ps, double *out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MOLOCH_GB300_H */
