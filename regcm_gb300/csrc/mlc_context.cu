// mlc_context.cu -- the C ABI of moloch_gb300.h: one context per domain.
//
// A context owns one CUDA stream and one device arena (a single cudaMalloc
// carved into 256-byte aligned arrays), holds the domain's static fields,
// state, boundary data and scratch in the padded layout of mlc_device.cuh,
// and steps it with the kernels of mlc_sound.cu, mlc_advect.cu and
// mlc_end.cu.  A step is recorded once into a CUDA graph per buffer
// arrangement (the acoustic and advection ping-pong pairs alternate between
// at most two arrangements) and replayed; the boundary clock and the
// diagnostics stay on the device so replays need no host work.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include "../../include/moloch_gb300.h"
#include "mlc_kernels.cuh"

using namespace mlc;

namespace {

constexpr size_t kAlign = 256;
constexpr int kMaxLevels = 128;

size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// Assigns arena offsets; with base == nullptr it only measures.
struct Carver {
  char *base = nullptr;
  size_t off = 0;
  template <class T>
  T *take(size_t count) {
    size_t o = off;
    off = align_up(off + count * sizeof(T));
    return base ? reinterpret_cast<T *>(base + o) : nullptr;
  }
};

template <class R>
struct Arrays {
  State<R> st{};
  // second halves of the ping-pong pairs
  R *u2, *v2, *ux2, *vx2, *qx2, *trac2, *wx2;
  double *pai2, *tetav2;
  R *wz[kMaxAdv];
  double *wz_pai, *wz_tet;  // wz of the FP64 fields of a mixed domain
  Work<R> wk{};
  Stat<R> sa{};
  Bdy<R> bd{};
  // writable views of the static arrays
  R *fmz, *fmzf, *rfmzu, *rfmzv, *zrfmu, *zrfmd, *hx, *hy, *msfu, *msfv, *msfx, *mx2, *rmu, *rmv,
      *coru, *corv;
  double *fmz_d, *fmzf_d;
  double *zeta, *dz, *hefc, *fcx, *tnudge, *ffilt, *gzitakh, *xkdamp, *xknu, *gzitak, *rlat;
  int32_t *ibnd_cr, *ibnd_ud, *ibnd_vd;
  R *bfield[2][8];  // xtb, xqb, (unused), xlb, xib, dub, dvb, chib
  double *xpaib[2], *xpsb[2];
  double *staging;
  size_t staging_elems;
  double *partials;
  Clock *clk;
  DiagDev *diag;
};

int n_advected(const mlc_dims &d, const mlc_params &p) {
  // tetav, pai, ux, vx, wx, qv, qx(iqfrst:nqx) when ipptls > 0, trac
  return 6 + (p.ipptls > 0 ? d.nqx - 1 : 0) + d.ntr;
}

size_t state_elems(const mlc_dims &d) {
  const size_t c2 = (size_t)(d.jx - 1) * (d.iy - 1);
  const size_t u3 = (size_t)d.jx * (d.iy - 1) * d.kz, v3 = (size_t)(d.jx - 1) * d.iy * d.kz;
  const size_t c3 = c2 * d.kz;
  return u3 + v3 + c2 * (d.kz + 1) + c3 * (9 + d.nqx + d.ntr) + c2;
}

template <class R>
void carve(Carver &cv, Arrays<R> &a, const Geom &g, const mlc_dims &d, const mlc_params &p) {
  const size_t F = g.field3(), F1 = g.PS * (size_t)(g.kz + 1), P2 = g.PS;
  State<R> &st = a.st;
  st.u = cv.take<R>(F); st.v = cv.take<R>(F); st.w = cv.take<R>(F1);
  st.pai = cv.take<double>(F); st.tetav = cv.take<double>(F); st.t = cv.take<R>(F);
  st.tvirt = cv.take<R>(F); st.ux = cv.take<R>(F); st.vx = cv.take<R>(F);
  st.p = cv.take<R>(F); st.rho = cv.take<R>(F); st.qsat = cv.take<R>(F);
  st.qx = cv.take<R>(F * d.nqx);
  st.trac = d.ntr ? cv.take<R>(F * d.ntr) : nullptr;
  st.ps = cv.take<double>(P2);
  a.u2 = cv.take<R>(F); a.v2 = cv.take<R>(F); a.tetav2 = cv.take<double>(F); a.pai2 = cv.take<double>(F);
  a.ux2 = cv.take<R>(F); a.vx2 = cv.take<R>(F); a.qx2 = cv.take<R>(F * d.nqx);
  a.trac2 = d.ntr ? cv.take<R>(F * d.ntr) : nullptr;
  a.wx2 = cv.take<R>(F);
  const int nadv = n_advected(d, p);
  for (int f = 0; f < kMaxAdv; ++f) a.wz[f] = f < nadv ? cv.take<R>(F) : nullptr;
  a.wz_pai = sizeof(R) == sizeof(double) ? nullptr : cv.take<double>(F);
  a.wz_tet = sizeof(R) == sizeof(double) ? nullptr : cv.take<double>(F);
  a.wk.s = cv.take<R>(F1); a.wk.zdiv2 = cv.take<R>(F); a.wk.tetavf = cv.take<double>(F1);
  a.wk.wx = cv.take<R>(F);
  a.fmz = cv.take<R>(F); a.fmzf = cv.take<R>(F1); a.rfmzu = cv.take<R>(F); a.rfmzv = cv.take<R>(F);
  if (sizeof(R) == sizeof(double)) {
    a.fmz_d = reinterpret_cast<double *>(a.fmz);
    a.fmzf_d = reinterpret_cast<double *>(a.fmzf);
  } else {
    a.fmz_d = cv.take<double>(F);
    a.fmzf_d = cv.take<double>(F1);
  }
  a.zrfmu = cv.take<R>(F); a.zrfmd = cv.take<R>(F);
  a.zeta = cv.take<double>(F); a.dz = cv.take<double>(F);
  a.hx = cv.take<R>(P2); a.hy = cv.take<R>(P2); a.msfu = cv.take<R>(P2); a.msfv = cv.take<R>(P2);
  a.msfx = cv.take<R>(P2); a.mx2 = cv.take<R>(P2); a.rmu = cv.take<R>(P2); a.rmv = cv.take<R>(P2);
  a.coru = cv.take<R>(P2); a.corv = cv.take<R>(P2);
  a.ibnd_cr = cv.take<int32_t>(P2); a.ibnd_ud = cv.take<int32_t>(P2); a.ibnd_vd = cv.take<int32_t>(P2);
  a.hefc = cv.take<double>((size_t)p.nspgx * d.kz); a.fcx = cv.take<double>(p.nspgx);
  a.tnudge = cv.take<double>(d.kz); a.ffilt = cv.take<double>(d.kz); a.gzitakh = cv.take<double>(d.kz);
  a.xkdamp = cv.take<double>(d.kz); a.xknu = cv.take<double>(d.kz); a.gzitak = cv.take<double>(d.kz + 1);
  a.rlat = cv.take<double>(d.iy);
  const bool moist_b = p.present_qc || p.present_qi;
  for (int b = 0; b < 2; ++b) {
    a.bfield[b][0] = cv.take<R>(F);                                   // xtb
    a.bfield[b][1] = cv.take<R>(F);                                   // xqb
    a.bfield[b][2] = nullptr;
    a.xpaib[b] = cv.take<double>(F);
    a.bfield[b][3] = (moist_b && p.present_qc) ? cv.take<R>(F) : nullptr;  // xlb
    a.bfield[b][4] = (moist_b && p.present_qi) ? cv.take<R>(F) : nullptr;  // xib
    a.bfield[b][5] = cv.take<R>(F);                                   // dub
    a.bfield[b][6] = cv.take<R>(F);                                   // dvb
    a.bfield[b][7] = d.ntr ? cv.take<R>(F * d.ntr) : nullptr;         // chib
    a.xpsb[b] = cv.take<double>(P2);
  }
  a.staging = nullptr;  // one staging buffer per context, outside the member arenas
  a.staging_elems = state_elems(d);
  a.partials = cv.take<double>((size_t)reduce_blocks(g) * 8);
  a.clk = cv.take<Clock>(1);
  a.diag = cv.take<DiagDev>(1);
}

template <class R>
void bind_views(Arrays<R> &a) {
  Stat<R> &s = a.sa;
  s.fmz = a.fmz; s.fmzf = a.fmzf; s.rfmzu = a.rfmzu; s.rfmzv = a.rfmzv;
  s.fmz_d = a.fmz_d; s.fmzf_d = a.fmzf_d;
  s.zrfmu = a.zrfmu; s.zrfmd = a.zrfmd; s.zeta = a.zeta; s.dz = a.dz;
  s.hx = a.hx; s.hy = a.hy; s.msfu = a.msfu; s.msfv = a.msfv; s.msfx = a.msfx; s.mx2 = a.mx2;
  s.rmu = a.rmu; s.rmv = a.rmv; s.coru = a.coru; s.corv = a.corv;
  s.ibnd_cr = a.ibnd_cr; s.ibnd_ud = a.ibnd_ud; s.ibnd_vd = a.ibnd_vd;
  s.hefc = a.hefc; s.fcx = a.fcx; s.tnudge = a.tnudge; s.ffilt = a.ffilt; s.gzitakh = a.gzitakh;
  s.xkdamp = a.xkdamp; s.xknu = a.xknu; s.gzitak = a.gzitak; s.rlat = a.rlat;
  for (int b = 0; b < 2; ++b) {
    a.bd.xtb[b] = a.bfield[b][0]; a.bd.xqb[b] = a.bfield[b][1]; a.bd.xpaib[b] = a.xpaib[b];
    a.bd.xlb[b] = a.bfield[b][3]; a.bd.xib[b] = a.bfield[b][4]; a.bd.dub[b] = a.bfield[b][5];
    a.bd.dvb[b] = a.bfield[b][6]; a.bd.chib[b] = a.bfield[b][7]; a.bd.xpsb[b] = a.xpsb[b];
  }
}

Geom make_geom(const mlc_dims &d, int elem_bytes) {
  Geom g{};
  g.jx = d.jx; g.iy = d.iy; g.kz = d.kz; g.nqx = d.nqx; g.ntr = d.ntr;
  g.nmem = 1;
  g.col_x = 32; g.col_y = 4;
  g.solve_x = 32; g.solve_y = 2;
  g.vert_x = 32; g.vert_y = 2;
  g.htile = 0;
  const int per_line = 128 / elem_bytes;
  g.P = (d.jx + per_line - 1) / per_line * per_line;
  g.PS = (size_t)g.P * d.iy;
  return g;
}

int validate(const mlc_dims *d, const mlc_params *p) {
  if (!d || !p) return MLC_ERR_INVALID;
  if (d->jx < 10 || d->iy < 10 || d->kz < 4 || d->kz > kMaxLevels) return MLC_ERR_INVALID;
  if (d->nqx < 2 || d->nqx > 10 || d->ntr < 0 || d->ntr > 8) return MLC_ERR_INVALID;
  if (!(p->dtsec > 0) || !(p->dx > 0) || !(p->mo_ztop > 0) || p->mo_nadv < 1 || p->mo_nsound < 1)
    return MLC_ERR_INVALID;
  if (!(p->dtbdys > 0) || p->nspgx < 3 || p->nspgd < 3) return MLC_ERR_INVALID;
  if (p->ipptls < 0 || p->ipptls > 2) return MLC_ERR_UNSUPPORTED;
  if (p->ipptls == 2 && d->nqx < 5) return MLC_ERR_INVALID;
  if (p->mo_spectral_nudge) return MLC_ERR_UNSUPPORTED;
  if (p->precision != MLC_PREC_FP64 && p->precision != MLC_PREC_MIXED) return MLC_ERR_INVALID;
  if (n_advected(*d, *p) > kMaxAdv) return MLC_ERR_UNSUPPORTED;
  // the tracer relaxation assumes disjoint south/north and west/east bands
  if (d->ntr > 0 && (d->jx - 1 < 2 * p->nspgx || d->iy - 1 < 2 * p->nspgx)) return MLC_ERR_UNSUPPORTED;
  return MLC_OK;
}

}  // namespace

struct mlc_ctx {
  mlc_dims dims{};
  mlc_params prm{};
  int device = 0;
  cudaStream_t stream = nullptr;
  Geom g{};
  Scal c{};
  void *arena = nullptr;
  double *staging = nullptr;  // layout conversion buffer shared by all members
  size_t arena_bytes = 0;   // all members
  size_t member_bytes = 0;  // one member's arena (the member stride)
  int nmem = 1;
  Arrays<double> ad{};      // member 0's views (kernels rebase by member)
  Arrays<float> af{};
  std::vector<char> m_static, m_state, m_bdy;
  bool have_static = false, have_state = false, have_bdy = false;
  double rdzita_set = 0.0, dtbdys_set = 0.0;
  int uv_role = 0;   // which buffer of the u/v pair is current
  int adv_role = 0;  // which buffer of the advected pairs is current
  cudaGraphExec_t graph[4] = {nullptr, nullptr, nullptr, nullptr};
  bool use_graphs = true;
  int launches_per_step = 0;
  double xbctime_host = 0.0;
};

namespace {

// Views of member m's arrays (member 0's layout, m * member_bytes further).
template <class R>
Arrays<R> member_arrays(const mlc_ctx *x, int m) {
  Arrays<R> a{};
  Carver cv{static_cast<char *>(x->arena) + (size_t)m * x->member_bytes, 0};
  carve<R>(cv, a, x->g, x->dims, x->prm);
  bind_views<R>(a);
  a.staging = x->staging;
  return a;
}

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return MLC_OK;
  if (e == cudaErrorMemoryAllocation) return MLC_ERR_NOMEM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return MLC_ERR_NODEVICE;
  return MLC_ERR_CUDA;
}

#define MLC_TRY(x)                              \
  do {                                          \
    cudaError_t e_ = (x);                       \
    if (e_ != cudaSuccess) return cuda_status(e_); \
  } while (0)

// Pointers of the current buffer arrangement.
template <class R>
struct Roles {
  State<R> st;      // canonical state (current buffers)
  R *u_alt, *v_alt;
  R *ux_alt, *vx_alt, *qx_alt, *trac_alt, *wx_alt;
  double *pai_alt, *tetav_alt;
};

template <class R>
Roles<R> roles_of(const Arrays<R> &a, int uv_role, int adv_role) {
  Roles<R> r{};
  r.st = a.st;
  if (uv_role) { r.st.u = a.u2; r.st.v = a.v2; r.u_alt = a.st.u; r.v_alt = a.st.v; }
  else { r.u_alt = a.u2; r.v_alt = a.v2; }
  if (adv_role) {
    r.st.tetav = a.tetav2; r.st.pai = a.pai2; r.st.ux = a.ux2; r.st.vx = a.vx2; r.st.qx = a.qx2;
    r.st.trac = a.trac2;
    r.tetav_alt = a.st.tetav; r.pai_alt = a.st.pai; r.ux_alt = a.st.ux; r.vx_alt = a.st.vx;
    r.qx_alt = a.st.qx; r.trac_alt = a.st.trac;
  } else {
    r.tetav_alt = a.tetav2; r.pai_alt = a.pai2; r.ux_alt = a.ux2; r.vx_alt = a.vx2;
    r.qx_alt = a.qx2; r.trac_alt = a.trac2;
  }
  return r;
}

// Optional per-launch event recorder (eager steps only, never captured).
struct Recorder {
  struct Mark {
    const char *name;
    cudaEvent_t a, b;
  };
  std::vector<Mark> marks;
  cudaStream_t s = nullptr;
  const char *cur = nullptr;
  cudaEvent_t open = nullptr;
  void begin(const char *name) {
    if (!s) return;
    cur = name;
    cudaEventCreate(&open);
    cudaEventRecord(open, s);
  }
  void end() {
    if (!s) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, s);
    marks.push_back({cur, open, e});
  }
  ~Recorder() {
    for (auto &m : marks) { cudaEventDestroy(m.a); cudaEventDestroy(m.b); }
  }
};

#define REC(name, call) \
  do {                  \
    if (rec) rec->begin(name); \
    call;               \
    if (rec) rec->end(); \
  } while (0)

// Enqueue one model step (Main/mod_moloch.F90:312-446) on the context stream.
// Returns the number of kernels launched; updates the roles it leaves.
template <class R>
int enqueue_step(mlc_ctx *x, Arrays<R> &a, Recorder *rec = nullptr) {
  using L = Launch<R>;
  const Geom &g = x->g;
  const Scal &c = x->c;
  cudaStream_t s = x->stream;
  int nl = 0;
  const mlc_dims &d = x->dims;
  const mlc_params &p = x->prm;
  const size_t F = g.field3();
  for (int nadv = 0; nadv < c.nadv; ++nadv) {
    Roles<R> r = roles_of(a, x->uv_role, x->adv_role);
    Work<R> wk = a.wk;
    // ---- sound ----
    REC("sound_prep", L::sound_prep(g, r.st, wk, s)); ++nl;
    R *ucur = r.st.u, *vcur = r.st.v, *ualt = r.u_alt, *valt = r.v_alt;
    for (int ns = 0; ns < c.nsound; ++ns) {
      SoundBufs<R> b{ucur, vcur, ualt, valt};
      State<R> st = r.st;
      st.u = ucur; st.v = vcur;
      REC("sound_div", L::sound_div(g, c, a.sa, st, wk, b, s)); ++nl;
      REC("sound_solve", L::sound_solve(g, c, a.sa, st, wk, ns == c.nsound - 1, s)); ++nl;
      REC("sound_momentum", L::sound_momentum(g, c, a.sa, st, wk, b, s)); ++nl;
      std::swap(ucur, ualt);
      std::swap(vcur, valt);
    }
    if (c.nsound & 1) x->uv_role ^= 1;
    r.st.u = ucur; r.st.v = vcur;
    // ---- advection ----
    REC("adv_prep", L::adv_prep(g, r.st, wk, s)); ++nl;
    AdvTable<R> t{};
    AdvTable<double> tp{};  // the FP64 fields (theta_v, Exner) of a mixed domain
    int n = 0;
    auto add = [&](const R *cur, R *out) { t.cur[n] = cur; t.wz[n] = a.wz[n]; t.out[n] = out; ++n; };
    if constexpr (sizeof(R) == sizeof(double)) {
      add(reinterpret_cast<const R *>(r.st.tetav), reinterpret_cast<R *>(r.tetav_alt));
      add(reinterpret_cast<const R *>(r.st.pai), reinterpret_cast<R *>(r.pai_alt));
    } else {
      tp.cur[0] = r.st.tetav; tp.wz[0] = a.wz_tet; tp.out[0] = r.tetav_alt;
      tp.cur[1] = r.st.pai; tp.wz[1] = a.wz_pai; tp.out[1] = r.pai_alt;
      tp.n = 2;
    }
    add(r.st.ux, r.ux_alt);
    add(r.st.vx, r.vx_alt);
    add(wk.wx, a.wx2);
    add(r.st.qx, r.qx_alt);
    if (p.ipptls > 0)
      for (int q = 1; q < d.nqx; ++q) add(r.st.qx + q * F, r.qx_alt + q * F);
    for (int q = 0; q < d.ntr; ++q) add(r.st.trac + q * F, r.trac_alt + q * F);
    t.n = n;
    REC("adv_vertical", L::adv_vertical(g, c, a.sa, wk, t, s)); ++nl;
    REC("adv_horizontal", L::adv_horizontal(g, c, a.sa, r.st, t, s)); ++nl;
    if (tp.n) {
      REC("adv_vertical_f64", L::adv_vertical_f64(g, c, a.sa, wk, tp, s)); ++nl;
      REC("adv_horizontal_f64", L::adv_horizontal_f64(g, c, a.sa, r.st, tp, s)); ++nl;
    }
    if (p.ipptls == 0 && d.nqx > 1) {
      // species that are not advected keep their values in the other buffer
      cudaMemcpy2DAsync(r.qx_alt + F, x->member_bytes, r.st.qx + F, x->member_bytes,
                        (size_t)(d.nqx - 1) * F * sizeof(R), (size_t)x->nmem,
                        cudaMemcpyDeviceToDevice, s);
    }
    x->adv_role ^= 1;
    Roles<R> r2 = roles_of(a, x->uv_role, x->adv_role);
    Work<R> wk2 = wk;
    wk2.wx = a.wx2;
    if (c.curvature) { REC("adv_curvature", L::adv_curvature(g, c, a.sa, r2.st, s)); ++nl; }
    REC("adv_back", L::adv_back(g, r2.st, wk2, s)); ++nl;
    // wx is scratch: its advected copy lives in wx2 and both roles of the
    // pair are rebuilt from w each advection step, so no swap is kept.
  }
  Roles<R> r = roles_of(a, x->uv_role, x->adv_role);
  // ---- step end ----
  REC("end_tvirt", L::end_tvirt(g, c, r.st, s)); ++nl;
  if (c.apply_bdy) {
    REC("bdy_ring", L::bdy_ring(g, c, r.st, a.bd, a.clk, s)); nl += 2;
    REC("bdy_relax", L::bdy_relax(g, c, a.sa, r.st, a.bd, a.clk, s)); ++nl;
  }
  REC("end_cross", L::end_cross(g, c, a.sa, r.st, s)); ++nl;
  REC("end_uvstag", L::end_uvstag(g, r.st, s)); ++nl;
  REC("end_reduce", L::end_reduce(g, c, a.sa, r.st, a.partials, reduce_blocks(g), a.diag, a.clk, s)); nl += 2;
  return nl;
}

template <class R>
int step_impl(mlc_ctx *x, Arrays<R> &a, int nsteps) {
  for (int n = 0; n < nsteps; ++n) {
    const int key = x->uv_role * 2 + x->adv_role;
    if (x->use_graphs) {
      if (!x->graph[key]) {
        const int uv0 = x->uv_role, adv0 = x->adv_role;
        cudaGraph_t gr = nullptr;
        MLC_TRY(cudaStreamBeginCapture(x->stream, cudaStreamCaptureModeThreadLocal));
        x->launches_per_step = enqueue_step<R>(x, a);
        cudaError_t e = cudaStreamEndCapture(x->stream, &gr);
        if (e != cudaSuccess) return cuda_status(e);
        cudaGraphExec_t ex = nullptr;
        e = cudaGraphInstantiate(&ex, gr, 0);
        cudaGraphDestroy(gr);
        if (e != cudaSuccess) return cuda_status(e);
        x->graph[key] = ex;
        x->uv_role = uv0;  // replay below moves the roles
        x->adv_role = adv0;
      }
      MLC_TRY(cudaGraphLaunch(x->graph[key], x->stream));
      // the roles a step leaves are fixed: replay the bookkeeping only
      for (int m = 0; m < x->c.nadv; ++m) {
        if (x->c.nsound & 1) x->uv_role ^= 1;
        x->adv_role ^= 1;
      }
    } else {
      x->launches_per_step = enqueue_step<R>(x, a);
    }
  }
  return cuda_status(cudaGetLastError());
}

// ---- host <-> device transfers -------------------------------------------

// Copy a packed (Fortran extents nj x ni x nk) host array into the padded
// device layout through the staging buffer at element offset `soff`.  One
// stream orders every copy and (un)pack, so consecutive fields may reuse the
// same staging slice.
struct Staging {
  double *p;
  size_t n;
};

template <class R>
int put3(mlc_ctx *x, Staging sg, const double *h, R *dst, int nj, int ni, int nk, size_t soff) {
  if (!h) return MLC_OK;
  const size_t n = (size_t)nj * ni * nk;
  if (soff + n > sg.n) return MLC_ERR_INVALID;
  MLC_TRY(cudaMemcpyAsync(sg.p + soff, h, n * sizeof(double), cudaMemcpyHostToDevice, x->stream));
  Launch<R>::unpack3(sg.p + soff, dst, x->g, nj, ni, nk, x->stream);
  return MLC_OK;
}

template <class R>
int get3(mlc_ctx *x, Staging sg, const R *src, double *h, int nj, int ni, int nk, size_t soff) {
  if (!h) return MLC_OK;
  const size_t n = (size_t)nj * ni * nk;
  if (soff + n > sg.n) return MLC_ERR_INVALID;
  Launch<R>::pack3(src, sg.p + soff, x->g, nj, ni, nk, x->stream);
  MLC_TRY(cudaMemcpyAsync(h, sg.p + soff, n * sizeof(double), cudaMemcpyDeviceToHost, x->stream));
  return MLC_OK;
}

// 2-D padded copy of a small host array (built on the host, then one copy).
template <class T>
int put2_host(mlc_ctx *x, const T *h, T *dst, int nj, int ni) {
  std::vector<T> tmp((size_t)x->g.PS, T(0));
  for (int i = 0; i < ni; ++i)
    for (int j = 0; j < nj; ++j) tmp[(size_t)j + (size_t)i * x->g.P] = h[(size_t)j + (size_t)i * nj];
  MLC_TRY(cudaMemcpyAsync(dst, tmp.data(), tmp.size() * sizeof(T), cudaMemcpyHostToDevice, x->stream));
  return cuda_status(cudaStreamSynchronize(x->stream));
}

template <class R>
int put2r(mlc_ctx *x, const std::vector<double> &h, R *dst, int nj, int ni) {
  std::vector<R> tmp((size_t)nj * ni);
  for (size_t e = 0; e < tmp.size(); ++e) tmp[e] = (R)h[e];
  return put2_host<R>(x, tmp.data(), dst, nj, ni);
}

int put1(mlc_ctx *x, const double *h, double *dst, size_t n) {
  MLC_TRY(cudaMemcpyAsync(dst, h, n * sizeof(double), cudaMemcpyHostToDevice, x->stream));
  return cuda_status(cudaStreamSynchronize(x->stream));
}

#define MLC_CHK(x)              \
  do {                          \
    int s_ = (x);               \
    if (s_ != MLC_OK) return s_; \
  } while (0)

template <class R>
int bind_static_impl(mlc_ctx *x, Arrays<R> &a, const mlc_static_ptrs *s) {
  const Staging SG{a.staging, a.staging_elems};
  const mlc_dims &d = x->dims;
  const mlc_params &p = x->prm;
  const int jx = d.jx, iy = d.iy, kz = d.kz;
  if (!s->msfu || !s->msfv || !s->msfx || !s->ulat || !s->vlat || !s->hx || !s->hy || !s->fmz ||
      !s->fmzf || !s->rfmzu || !s->rfmzv || !s->zeta || !s->dz || !s->zita || !s->zitah ||
      !s->ffilt || !s->hefc || !s->ibnd_cr || !s->ibnd_ud || !s->ibnd_vd)
    return MLC_ERR_INVALID;
  if (d.ntr > 0 && !s->fcx) return MLC_ERR_INVALID;
  if (p.lrotllr && !s->rlat) return MLC_ERR_INVALID;
  // 3-D metric: one field at a time through the staging buffer
  MLC_CHK(put3<R>(x, SG, s->fmz, a.fmz, jx - 1, iy - 1, kz, 0));
  MLC_CHK(put3<R>(x, SG, s->fmzf, a.fmzf, jx - 1, iy - 1, kz + 1, 0));
  if (sizeof(R) != sizeof(double)) {
    MLC_CHK(put3<double>(x, SG, s->fmz, a.fmz_d, jx - 1, iy - 1, kz, 0));
    MLC_CHK(put3<double>(x, SG, s->fmzf, a.fmzf_d, jx - 1, iy - 1, kz + 1, 0));
  }
  MLC_CHK(put3<R>(x, SG, s->rfmzu, a.rfmzu, jx, iy - 1, kz, 0));
  MLC_CHK(put3<R>(x, SG, s->rfmzv, a.rfmzv, jx - 1, iy, kz, 0));
  MLC_CHK(put3<double>(x, SG, s->zeta, a.zeta, jx - 1, iy - 1, kz, 0));
  MLC_CHK(put3<double>(x, SG, s->dz, a.dz, jx - 1, iy - 1, kz, 0));
  // vertical WAF ratios (dtrdz*fmz)/fmzf, Main/mod_moloch.F90:888-889
  {
    const double mo_dzita = s->zita[kz - 1];
    const double dtrdz = 0.5 * (x->c.dtstepa * (1.0 / mo_dzita));
    const size_t c2 = (size_t)(jx - 1) * (iy - 1);
    std::vector<double> zu(c2 * kz), zd(c2 * kz);
    for (int k = 0; k < kz; ++k)
      for (size_t e = 0; e < c2; ++e) {
        const double fz = s->fmz[e + c2 * k];
        zu[e + c2 * k] = dtrdz * fz / s->fmzf[e + c2 * k];
        zd[e + c2 * k] = dtrdz * fz / s->fmzf[e + c2 * (k + 1)];
      }
    MLC_CHK(put3<R>(x, SG, zu.data(), a.zrfmu, jx - 1, iy - 1, kz, 0));
    MLC_CHK(put3<R>(x, SG, zd.data(), a.zrfmd, jx - 1, iy - 1, kz, 0));
    MLC_TRY(cudaStreamSynchronize(x->stream));
  }
  // 2-D fields and init_moloch derivations (Main/mod_moloch.F90:258-271)
  const size_t nd = (size_t)jx * iy;
  std::vector<double> t2(nd);
  auto copy2 = [&](const double *h, size_t n) { t2.assign(h, h + n); };
  copy2(s->msfu, nd); MLC_CHK(put2r<R>(x, t2, a.msfu, jx, iy));
  copy2(s->msfv, nd); MLC_CHK(put2r<R>(x, t2, a.msfv, jx, iy));
  copy2(s->msfx, nd); MLC_CHK(put2r<R>(x, t2, a.msfx, jx, iy));
  for (size_t e = 0; e < nd; ++e) t2[e] = s->msfx[e] * s->msfx[e];
  MLC_CHK(put2r<R>(x, t2, a.mx2, jx, iy));
  for (size_t e = 0; e < nd; ++e) t2[e] = 1.0 / s->msfu[e];
  MLC_CHK(put2r<R>(x, t2, a.rmu, jx, iy));
  for (size_t e = 0; e < nd; ++e) t2[e] = 1.0 / s->msfv[e];
  MLC_CHK(put2r<R>(x, t2, a.rmv, jx, iy));
  copy2(s->hx, (size_t)jx * (iy - 1)); MLC_CHK(put2r<R>(x, t2, a.hx, jx, iy - 1));
  copy2(s->hy, (size_t)(jx - 1) * iy); MLC_CHK(put2r<R>(x, t2, a.hy, jx - 1, iy));
  t2.resize((size_t)jx * (iy - 1));
  for (size_t e = 0; e < t2.size(); ++e) t2[e] = kOmega2 * std::sin(s->ulat[e] * kDegrad);
  MLC_CHK(put2r<R>(x, t2, a.coru, jx, iy - 1));
  t2.resize((size_t)(jx - 1) * iy);
  for (size_t e = 0; e < t2.size(); ++e) t2[e] = kOmega2 * std::sin(s->vlat[e] * kDegrad);
  MLC_CHK(put2r<R>(x, t2, a.corv, jx - 1, iy));
  MLC_CHK(put2_host<int32_t>(x, s->ibnd_cr, a.ibnd_cr, jx, iy));
  MLC_CHK(put2_host<int32_t>(x, s->ibnd_ud, a.ibnd_ud, jx, iy));
  MLC_CHK(put2_host<int32_t>(x, s->ibnd_vd, a.ibnd_vd, jx, iy));
  // zone indices address rows 1..nspgx of hefc/fcx: reject anything else
  for (const int32_t *b : {s->ibnd_cr, s->ibnd_ud, s->ibnd_vd})
    for (size_t e = 0; e < nd; ++e)
      if (b[e] > p.nspgx || b[e] == 0 || b[e] < -1) return MLC_ERR_INVALID;
  // the relaxation zones are non-empty (ba%havebound)
  auto any_pos = [&](const int32_t *b) {
    for (size_t e = 0; e < nd; ++e) if (b[e] > 0) return 1;
    return 0;
  };
  x->c.hb_cr |= any_pos(s->ibnd_cr); x->c.hb_ud |= any_pos(s->ibnd_ud); x->c.hb_vd |= any_pos(s->ibnd_vd);
  // the curvature terms vanish identically with uniform map factors
  {
    bool curv = p.lrotllr != 0;
    for (int i = 2; i <= iy - 2 && !curv; ++i)
      for (int j = 2; j <= jx - 2 && !curv; ++j) {
        const size_t e = (size_t)(j - 1) + (size_t)(i - 1) * jx;
        if ((s->msfu[e - 1] - s->msfu[e]) != 0.0 || (s->msfv[e - jx] - s->msfv[e]) != 0.0) curv = true;
      }
    x->c.curvature |= curv ? 1 : 0;
  }
  // 1-D vertical arrays, Main/mod_moloch.F90:262-300
  std::vector<double> v1(kz + 1);
  for (int k = 1; k <= kz + 1; ++k) v1[k - 1] = gzita(s->zita[k - 1], p.mo_ztop, p.mo_a0);
  MLC_CHK(put1(x, v1.data(), a.gzitak, kz + 1));
  for (int k = 1; k <= kz; ++k) v1[k - 1] = gzita(s->zitah[k - 1], p.mo_ztop, p.mo_a0);
  MLC_CHK(put1(x, v1.data(), a.gzitakh, kz));
  for (int k = 1; k <= kz; ++k)
    v1[k - 1] = kNuMax * kDdamp * (1.0 / (k + 1.0) - 1.0 / (kz + 2.0));
  MLC_CHK(put1(x, v1.data(), a.xkdamp, kz));
  for (int k = 1; k <= kz; ++k)
    v1[k - 1] = kNuMax * (0.55 + 0.45 * ((double)(kz - k + 1) - 1.0) / ((double)kz - 1.0));
  MLC_CHK(put1(x, v1.data(), a.xknu, kz));
  MLC_CHK(put1(x, s->ffilt, a.ffilt, kz));
  if (s->tnudge) MLC_CHK(put1(x, s->tnudge, a.tnudge, kz));
  else MLC_TRY(cudaMemsetAsync(a.tnudge, 0, kz * sizeof(double), x->stream));
  MLC_CHK(put1(x, s->hefc, a.hefc, (size_t)p.nspgx * kz));
  if (s->fcx) MLC_CHK(put1(x, s->fcx, a.fcx, p.nspgx));
  if (s->rlat) MLC_CHK(put1(x, s->rlat, a.rlat, iy));
  MLC_TRY(cudaStreamSynchronize(x->stream));
  return MLC_OK;
}

template <class R>
int upload_state_impl(mlc_ctx *x, Arrays<R> &a, const mlc_state_ptrs *h) {
  const Staging SG{a.staging, a.staging_elems};
  const mlc_dims &d = x->dims;
  const int jx = d.jx, iy = d.iy, kz = d.kz;
  Roles<R> r = roles_of(a, x->uv_role, x->adv_role);
  State<R> &st = r.st;
  size_t off = 0;
  const size_t c3 = (size_t)(jx - 1) * (iy - 1) * kz;
  auto adv = [&](size_t n) { size_t o = off; off += n; return o; };
  MLC_CHK(put3<R>(x, SG, h->u, st.u, jx, iy - 1, kz, adv((size_t)jx * (iy - 1) * kz)));
  MLC_CHK(put3<R>(x, SG, h->v, st.v, jx - 1, iy, kz, adv((size_t)(jx - 1) * iy * kz)));
  MLC_CHK(put3<R>(x, SG, h->w, st.w, jx - 1, iy - 1, kz + 1, adv((size_t)(jx - 1) * (iy - 1) * (kz + 1))));
  MLC_CHK(put3<double>(x, SG, h->pai, st.pai, jx - 1, iy - 1, kz, adv(c3)));
  MLC_CHK(put3<double>(x, SG, h->tetav, st.tetav, jx - 1, iy - 1, kz, adv(c3)));
  R *f3[] = {st.t, st.tvirt, st.ux, st.vx, st.p, st.rho, st.qsat};
  const double *h3[] = {h->t, h->tvirt, h->ux, h->vx, h->p, h->rho, h->qsat};
  for (int q = 0; q < 7; ++q) MLC_CHK(put3<R>(x, SG, h3[q], f3[q], jx - 1, iy - 1, kz, adv(c3)));
  const size_t F = x->g.field3();
  for (int n = 0; n < d.nqx && h->qx; ++n)
    MLC_CHK(put3<R>(x, SG, h->qx + n * c3, st.qx + n * F, jx - 1, iy - 1, kz, adv(c3)));
  for (int n = 0; n < d.ntr && h->trac; ++n)
    MLC_CHK(put3<R>(x, SG, h->trac + n * c3, st.trac + n * F, jx - 1, iy - 1, kz, adv(c3)));
  if (h->ps) {
    const size_t c2 = (size_t)(jx - 1) * (iy - 1);
    MLC_CHK(put3<double>(x, SG, h->ps, st.ps, jx - 1, iy - 1, 1, adv(c2)));
  }
  // init_moloch: w(:,:,1) = 0 (Main/mod_moloch.F90:264-266)
  if (h->w) MLC_TRY(cudaMemsetAsync(st.w, 0, x->g.PS * sizeof(R), x->stream));
  return cuda_status(cudaStreamSynchronize(x->stream));
}

template <class R>
int download_state_impl(mlc_ctx *x, Arrays<R> &a, const mlc_state_ptrs *h) {
  const Staging SG{a.staging, a.staging_elems};
  const mlc_dims &d = x->dims;
  const int jx = d.jx, iy = d.iy, kz = d.kz;
  Roles<R> r = roles_of(a, x->uv_role, x->adv_role);
  const State<R> &st = r.st;
  size_t off = 0;
  const size_t c3 = (size_t)(jx - 1) * (iy - 1) * kz;
  auto adv = [&](size_t n) { size_t o = off; off += n; return o; };
  MLC_CHK(get3<R>(x, SG, st.u, h->u, jx, iy - 1, kz, adv((size_t)jx * (iy - 1) * kz)));
  MLC_CHK(get3<R>(x, SG, st.v, h->v, jx - 1, iy, kz, adv((size_t)(jx - 1) * iy * kz)));
  MLC_CHK(get3<R>(x, SG, st.w, h->w, jx - 1, iy - 1, kz + 1, adv((size_t)(jx - 1) * (iy - 1) * (kz + 1))));
  MLC_CHK(get3<double>(x, SG, st.pai, h->pai, jx - 1, iy - 1, kz, adv(c3)));
  MLC_CHK(get3<double>(x, SG, st.tetav, h->tetav, jx - 1, iy - 1, kz, adv(c3)));
  const R *f3[] = {st.t, st.tvirt, st.ux, st.vx, st.p, st.rho, st.qsat};
  double *h3[] = {h->t, h->tvirt, h->ux, h->vx, h->p, h->rho, h->qsat};
  for (int q = 0; q < 7; ++q) MLC_CHK(get3<R>(x, SG, f3[q], h3[q], jx - 1, iy - 1, kz, adv(c3)));
  const size_t F = x->g.field3();
  for (int n = 0; n < d.nqx && h->qx; ++n)
    MLC_CHK(get3<R>(x, SG, st.qx + n * F, h->qx + n * c3, jx - 1, iy - 1, kz, adv(c3)));
  for (int n = 0; n < d.ntr && h->trac; ++n)
    MLC_CHK(get3<R>(x, SG, st.trac + n * F, h->trac + n * c3, jx - 1, iy - 1, kz, adv(c3)));
  if (h->ps) {
    const size_t c2 = (size_t)(jx - 1) * (iy - 1);
    MLC_CHK(get3<double>(x, SG, st.ps, h->ps, jx - 1, iy - 1, 1, adv(c2)));
  }
  return cuda_status(cudaStreamSynchronize(x->stream));
}

template <class R>
int set_boundary_impl(mlc_ctx *x, Arrays<R> &a, const mlc_bdy_ptrs *b) {
  const Staging SG{a.staging, a.staging_elems};
  const mlc_dims &d = x->dims;
  const mlc_params &p = x->prm;
  const int jx = d.jx, iy = d.iy, kz = d.kz;
  const size_t c3 = (size_t)(jx - 1) * (iy - 1) * kz;
  const size_t F = x->g.field3();
  for (int s = 0; s < 2; ++s) {
    if (!b->xtb[s] || !b->xqb[s] || !b->xpaib[s] || !b->dub[s] || !b->dvb[s] || !b->xpsb[s])
      return MLC_ERR_INVALID;
    if (p.present_qc && !b->xlb[s]) return MLC_ERR_INVALID;
    if (p.present_qi && !b->xib[s]) return MLC_ERR_INVALID;
    if (d.ntr > 0 && !b->chib[s]) return MLC_ERR_INVALID;
    MLC_CHK(put3<R>(x, SG, b->xtb[s], a.bfield[s][0], jx - 1, iy - 1, kz, 0));
    MLC_CHK(put3<R>(x, SG, b->xqb[s], a.bfield[s][1], jx - 1, iy - 1, kz, 0));
    MLC_CHK(put3<double>(x, SG, b->xpaib[s], a.xpaib[s], jx - 1, iy - 1, kz, 0));
    if (p.present_qc) MLC_CHK(put3<R>(x, SG, b->xlb[s], a.bfield[s][3], jx - 1, iy - 1, kz, 0));
    if (p.present_qi) MLC_CHK(put3<R>(x, SG, b->xib[s], a.bfield[s][4], jx - 1, iy - 1, kz, 0));
    MLC_CHK(put3<R>(x, SG, b->dub[s], a.bfield[s][5], jx, iy - 1, kz, 0));
    MLC_CHK(put3<R>(x, SG, b->dvb[s], a.bfield[s][6], jx - 1, iy, kz, 0));
    for (int n = 0; n < d.ntr; ++n)
      MLC_CHK(put3<R>(x, SG, b->chib[s] + n * c3, a.bfield[s][7] + n * F, jx - 1, iy - 1, kz, 0));
    MLC_CHK(put3<double>(x, SG, b->xpsb[s], a.xpsb[s], jx - 1,
                         iy - 1, 1, 0));
    MLC_TRY(cudaStreamSynchronize(x->stream));
  }
  return MLC_OK;
}

template <class R>
size_t footprint(const mlc_dims &d, const mlc_params &p, int elem) {
  Geom g = make_geom(d, elem);
  Arrays<R> a{};
  Carver cv;
  carve<R>(cv, a, g, d, p);
  return cv.off + state_elems(d) * sizeof(double);
}

}  // namespace

extern "C" {

void mlc_default_params(mlc_params *p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  // Share/mod_dynparam.F90:141-152,203-211 and Main/mod_params.F90:237
  p->dtsec = 100.0;
  p->dx = 50000.0;
  p->mo_ztop = 30000.0;
  p->mo_h = 8000.0;
  p->mo_a0 = 0.0;
  p->dtbdys = 6.0 * 3600.0;
  p->mo_nadv = 2;
  p->mo_nsound = 5;
  p->mo_divdamp = 1;
  p->mo_divfilter = 1;
  p->mo_top_nudge = 1;
  p->mo_spectral_nudge = 0;  // built path: spectral nudging off
  p->do_apply_bdy = 1;
  p->lrotllr = 0;
  p->ipptls = 1;
  p->present_qc = 0;
  p->present_qi = 0;
  p->nspgx = 6;
  p->nspgd = 6;
  p->nztop = 0;
  p->debug_level = 0;
  p->precision = MLC_PREC_FP64;
}

const char *mlc_strerror(int st) {
  switch (st) {
    case MLC_OK: return "ok";
    case MLC_ERR_INVALID: return "invalid argument, extent or parameter";
    case MLC_ERR_UNSUPPORTED: return "option outside the built path";
    case MLC_ERR_CUDA: return "CUDA runtime error";
    case MLC_ERR_NOMEM: return "device allocation failed";
    case MLC_ERR_STATE: return "call order violated (static fields, state or boundary missing)";
    case MLC_ERR_NONFINITE: return "CFL VIOLATION: non-finite surface pressure";
    case MLC_ERR_NODEVICE: return "no CUDA device";
    case MLC_ERR_BUDGET: return "request exceeds the device memory budget";
    case MLC_ERR_TOO_LARGE: return "size beyond the fixed maximum";
    default: return "unknown status";
  }
}

size_t mlc_footprint_bytes(const mlc_dims *d, int precision) {
  mlc_params p;
  mlc_default_params(&p);
  p.ipptls = d->nqx >= 5 ? 2 : 1;
  p.present_qc = p.present_qi = 1;
  p.nspgx = 34;
  if (precision == MLC_PREC_MIXED) return footprint<float>(*d, p, 4);
  return footprint<double>(*d, p, 8);
}

int mlc_create_batch(const mlc_dims *dims, const mlc_params *params, int nmem, mlc_ctx **out) {
  if (!out) return MLC_ERR_INVALID;
  *out = nullptr;
  int st = validate(dims, params);
  if (st != MLC_OK) return st;
  if (nmem < 1 || nmem > 4096) return MLC_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return MLC_ERR_NODEVICE;
  std::unique_ptr<mlc_ctx> x(new (std::nothrow) mlc_ctx());
  if (!x) return MLC_ERR_NOMEM;
  x->dims = *dims;
  x->prm = *params;
  x->nmem = nmem;
  x->m_static.assign(nmem, 0);
  x->m_state.assign(nmem, 0);
  x->m_bdy.assign(nmem, 0);
  MLC_TRY(cudaGetDevice(&x->device));
  const bool mixed = params->precision == MLC_PREC_MIXED;
  x->g = make_geom(*dims, mixed ? 4 : 8);
  Scal &c = x->c;
  c.dx = params->dx;
  c.rdx = 1.0 / params->dx;
  c.dtsec = params->dtsec;
  c.dt = params->dtsec;
  c.dtstepa = params->dtsec / (double)params->mo_nadv;
  c.dtsound = c.dtstepa / (double)params->mo_nsound;
  c.dtbdys = params->dtbdys;
  c.rtb = 1.0 / params->dtbdys;
  c.nadv = params->mo_nadv;
  c.nsound = params->mo_nsound;
  c.divdamp = params->mo_divdamp;
  c.divfilter = params->mo_divfilter;
  c.top_nudge = params->mo_top_nudge;
  c.apply_bdy = params->do_apply_bdy;
  c.lrotllr = params->lrotllr;
  c.ipptls = params->ipptls;
  c.present_qc = params->present_qc;
  c.present_qi = params->present_qi;
  c.nspgx = params->nspgx;
  c.nztop = params->mo_top_nudge ? params->nztop : 0;
  c.debug_level = params->debug_level;
  MLC_TRY(cudaStreamCreateWithFlags(&x->stream, cudaStreamNonBlocking));
  Carver cv;
  if (mixed) carve<float>(cv, x->af, x->g, *dims, *params);
  else carve<double>(cv, x->ad, x->g, *dims, *params);
  x->member_bytes = cv.off;
  x->arena_bytes = cv.off * (size_t)nmem;
  x->g.nmem = nmem;
  x->g.mstride = x->member_bytes;
  cudaError_t e = cudaMalloc(&x->arena, x->arena_bytes);
  if (e == cudaSuccess) e = cudaMalloc(&x->staging, state_elems(*dims) * sizeof(double));
  if (e != cudaSuccess) {
    cudaGetLastError();
    if (x->arena) cudaFree(x->arena);
  if (x->staging) cudaFree(x->staging);
    cudaStreamDestroy(x->stream);
    return MLC_ERR_NOMEM;
  }
  if (mixed) x->af = member_arrays<float>(x.get(), 0);
  else x->ad = member_arrays<double>(x.get(), 0);
  // every array starts at zero: s and w at the ring stay zero as the
  // reference's reset_tendencies and init_moloch leave them
  e = cudaMemsetAsync(x->arena, 0, x->arena_bytes, x->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(x->stream);
  if (e == cudaSuccess) e = mixed ? Launch<float>::configure_sound() : Launch<double>::configure_sound();
  if (e == cudaSuccess) e = mixed ? Launch<float>::configure_advect() : Launch<double>::configure_advect();
  if (e != cudaSuccess) {
    cudaFree(x->arena);
    cudaFree(x->staging);
    cudaStreamDestroy(x->stream);
    return cuda_status(e);
  }
  *out = x.release();
  return MLC_OK;
}

int mlc_create(const mlc_dims *dims, const mlc_params *params, mlc_ctx **out) {
  return mlc_create_batch(dims, params, 1, out);
}

static void drop_graphs(mlc_ctx *x) {
  for (auto &gx : x->graph)
    if (gx) { cudaGraphExecDestroy(gx); gx = nullptr; }
}

static bool all_set(const std::vector<char> &v) {
  for (char c : v)
    if (!c) return false;
  return true;
}

int mlc_member_bind_static(mlc_ctx *x, int m, const mlc_static_ptrs *s) {
  if (!x || !s || m < 0 || m >= x->nmem) return MLC_ERR_INVALID;
  if (!s->zita) return MLC_ERR_INVALID;
  const double rdz = 1.0 / s->zita[x->dims.kz - 1];
  if (x->rdzita_set != 0.0 && rdz != x->rdzita_set) return MLC_ERR_INVALID;  // members share levels
  drop_graphs(x);
  x->c.rdzita = rdz;
  x->rdzita_set = rdz;
  int st;
  if (x->prm.precision == MLC_PREC_MIXED) {
    Arrays<float> a = member_arrays<float>(x, m);
    st = bind_static_impl<float>(x, a, s);
  } else {
    Arrays<double> a = member_arrays<double>(x, m);
    st = bind_static_impl<double>(x, a, s);
  }
  if (st == MLC_OK) x->m_static[m] = 1;
  x->have_static = all_set(x->m_static);
  return st;
}

int mlc_bind_static(mlc_ctx *x, const mlc_static_ptrs *s) { return mlc_member_bind_static(x, 0, s); }

int mlc_member_upload_state(mlc_ctx *x, int m, const mlc_state_ptrs *h) {
  if (!x || !h || m < 0 || m >= x->nmem) return MLC_ERR_INVALID;
  int st;
  if (x->prm.precision == MLC_PREC_MIXED) {
    Arrays<float> a = member_arrays<float>(x, m);
    st = upload_state_impl<float>(x, a, h);
  } else {
    Arrays<double> a = member_arrays<double>(x, m);
    st = upload_state_impl<double>(x, a, h);
  }
  if (st == MLC_OK) x->m_state[m] = 1;
  x->have_state = all_set(x->m_state);
  return st;
}

int mlc_upload_state(mlc_ctx *x, const mlc_state_ptrs *h) { return mlc_member_upload_state(x, 0, h); }

int mlc_member_download_state(mlc_ctx *x, int m, const mlc_state_ptrs *h) {
  if (!x || !h || m < 0 || m >= x->nmem) return MLC_ERR_INVALID;
  if (x->prm.precision == MLC_PREC_MIXED) {
    Arrays<float> a = member_arrays<float>(x, m);
    return download_state_impl<float>(x, a, h);
  }
  Arrays<double> a = member_arrays<double>(x, m);
  return download_state_impl<double>(x, a, h);
}

int mlc_download_state(mlc_ctx *x, const mlc_state_ptrs *h) {
  return mlc_member_download_state(x, 0, h);
}

int mlc_member_set_boundary(mlc_ctx *x, int m, const mlc_bdy_ptrs *b, double xbctime,
                            double dtbdys) {
  if (!x || !b || !(dtbdys > 0) || m < 0 || m >= x->nmem) return MLC_ERR_INVALID;
  if (x->nmem > 1 && x->dtbdys_set != 0.0 && dtbdys != x->dtbdys_set) return MLC_ERR_INVALID;
  x->dtbdys_set = dtbdys;
  x->prm.dtbdys = dtbdys;
  x->c.dtbdys = dtbdys;
  x->c.rtb = 1.0 / dtbdys;
  drop_graphs(x);  // rtb/dtbdys are baked into recorded graphs
  int st;
  Clock *dclk;
  if (x->prm.precision == MLC_PREC_MIXED) {
    Arrays<float> a = member_arrays<float>(x, m);
    st = set_boundary_impl<float>(x, a, b);
    dclk = a.clk;
  } else {
    Arrays<double> a = member_arrays<double>(x, m);
    st = set_boundary_impl<double>(x, a, b);
    dclk = a.clk;
  }
  if (st != MLC_OK) return st;
  Clock clk{};
  clk.xbctime = xbctime;
  MLC_TRY(cudaMemcpyAsync(dclk, &clk, sizeof(Clock), cudaMemcpyHostToDevice, x->stream));
  MLC_TRY(cudaStreamSynchronize(x->stream));
  x->m_bdy[m] = 1;
  x->have_bdy = all_set(x->m_bdy);
  return MLC_OK;
}

int mlc_set_boundary(mlc_ctx *x, const mlc_bdy_ptrs *b, double xbctime, double dtbdys) {
  return mlc_member_set_boundary(x, 0, b, xbctime, dtbdys);
}

// Diagnostics of every member after the last step (out has nmem entries).
static int fetch_diags(mlc_ctx *x, int nsteps, mlc_diag *out) {
  const bool mixed = x->prm.precision == MLC_PREC_MIXED;
  const char *diag0 = reinterpret_cast<const char *>(mixed ? (void *)x->af.diag : (void *)x->ad.diag);
  const char *clk0 = reinterpret_cast<const char *>(mixed ? (void *)x->af.clk : (void *)x->ad.clk);
  std::vector<DiagDev> dd(x->nmem);
  std::vector<Clock> ck(x->nmem);
  MLC_TRY(cudaMemcpy2DAsync(dd.data(), sizeof(DiagDev), diag0, x->member_bytes, sizeof(DiagDev),
                            x->nmem, cudaMemcpyDeviceToHost, x->stream));
  MLC_TRY(cudaMemcpy2DAsync(ck.data(), sizeof(Clock), clk0, x->member_bytes, sizeof(Clock),
                            x->nmem, cudaMemcpyDeviceToHost, x->stream));
  MLC_TRY(cudaStreamSynchronize(x->stream));
  bool bad = false;
  for (int m = 0; m < x->nmem; ++m) {
    if (ck[m].nonfinite) bad = true;
    if (!out) continue;
    out[m].ps_max = dd[m].ps_max;
    out[m].ps_min = dd[m].ps_min;
    out[m].nonfinite = ck[m].nonfinite;
    out[m].steps_done = nsteps;
    out[m].drymass = dd[m].drymass;
    out[m].dryadv = dd[m].dryadv;
    out[m].qmass = dd[m].qmass;
    out[m].qadv = dd[m].qadv;
    out[m].xbctime = ck[m].xbctime;
  }
  return bad ? MLC_ERR_NONFINITE : MLC_OK;
}

int mlc_step_batch(mlc_ctx *x, int nsteps, mlc_diag *out) {
  if (!x || nsteps < 0) return MLC_ERR_INVALID;
  if (!x->have_static || !x->have_state || (x->c.apply_bdy && !x->have_bdy)) return MLC_ERR_STATE;
  const bool mixed = x->prm.precision == MLC_PREC_MIXED;
  int st = mixed ? step_impl<float>(x, x->af, nsteps) : step_impl<double>(x, x->ad, nsteps);
  if (st != MLC_OK) return st;
  return fetch_diags(x, nsteps, out);
}

int mlc_step(mlc_ctx *x, int nsteps, mlc_diag *out) {
  if (!x) return MLC_ERR_INVALID;
  if (x->nmem == 1) return mlc_step_batch(x, nsteps, out);
  std::vector<mlc_diag> all(x->nmem);
  int st = mlc_step_batch(x, nsteps, all.data());
  if (out && st != MLC_ERR_INVALID && st != MLC_ERR_STATE) *out = all[0];
  return st;
}

int mlc_members(const mlc_ctx *x) { return x ? x->nmem : 0; }

void mlc_destroy(mlc_ctx *x) {
  if (!x) return;
  for (auto &gx : x->graph)
    if (gx) cudaGraphExecDestroy(gx);
  if (x->stream) cudaStreamSynchronize(x->stream);
  if (x->arena) cudaFree(x->arena);
  if (x->staging) cudaFree(x->staging);
  if (x->stream) cudaStreamDestroy(x->stream);
  delete x;
}

// mlc_step with the device time of the steps measured by CUDA events on the
// context stream (bracketing exactly the step launches).
int mlc_step_timed(mlc_ctx *x, int nsteps, mlc_diag *out, float *ms) {
  if (!x || !ms) return MLC_ERR_INVALID;
  if (!x->have_static || !x->have_state || (x->c.apply_bdy && !x->have_bdy)) return MLC_ERR_STATE;
  cudaEvent_t e0, e1;
  MLC_TRY(cudaEventCreate(&e0));
  MLC_TRY(cudaEventCreate(&e1));
  MLC_TRY(cudaEventRecord(e0, x->stream));
  const bool mixed = x->prm.precision == MLC_PREC_MIXED;
  int st = mixed ? step_impl<float>(x, x->af, nsteps) : step_impl<double>(x, x->ad, nsteps);
  if (st == MLC_OK) {
    cudaEventRecord(e1, x->stream);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(ms, e0, e1);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != MLC_OK) return st;
  st = mlc_step(x, 0, out);
  if (out) out->steps_done = nsteps;
  return st;
}

// Per-kernel device times of `nsteps` eager steps (events around every
// launch group on the context stream).  Fills up to max_out entries.
int mlc_profile_steps(mlc_ctx *x, int nsteps, mlc_kernel_time *out, int max_out, int *n_out) {
  if (!x || !out || !n_out) return MLC_ERR_INVALID;
  if (!x->have_static || !x->have_state || (x->c.apply_bdy && !x->have_bdy)) return MLC_ERR_STATE;
  Recorder rec;
  rec.s = x->stream;
  const bool mixed = x->prm.precision == MLC_PREC_MIXED;
  for (int n = 0; n < nsteps; ++n) {
    if (mixed) enqueue_step<float>(x, x->af, &rec);
    else enqueue_step<double>(x, x->ad, &rec);
  }
  MLC_TRY(cudaStreamSynchronize(x->stream));
  int n = 0;
  for (auto &m : rec.marks) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, m.a, m.b);
    int slot = -1;
    for (int q = 0; q < n; ++q)
      if (std::strcmp(out[q].name, m.name) == 0) slot = q;
    if (slot < 0) {
      if (n >= max_out) continue;
      slot = n++;
      std::memset(&out[slot], 0, sizeof(out[slot]));
      std::strncpy(out[slot].name, m.name, sizeof(out[slot].name) - 1);
    }
    out[slot].launches += 1;
    out[slot].ms += ms;
  }
  *n_out = n;
  return cuda_status(cudaGetLastError());
}

}  // extern "C"

// ---- autotuner ------------------------------------------------------------
namespace {

const int kColCand[][2] = {{32, 4}, {32, 8}, {64, 2}, {64, 4}, {128, 1}, {16, 8}};
const int kSolveCand[][2] = {{32, 2}, {32, 1}, {64, 1}, {32, 4}, {16, 4}};
const int kVertCand[][2] = {{32, 2}, {32, 1}, {64, 1}, {32, 4}, {16, 4}};
constexpr int kNCol = 6, kNSolve = 5, kNVert = 5, kNTile = 4;

int group_of(const char *name) {
  if (!std::strcmp(name, "sound_solve")) return 1;
  if (!std::strncmp(name, "adv_vertical", 12)) return 2;
  if (!std::strncmp(name, "adv_horizontal", 14)) return 3;
  if (!std::strcmp(name, "bdy_ring") || !std::strcmp(name, "end_reduce")) return -1;
  return 0;  // column kernels
}

bool shapes_fit(const Geom &g, int elem) {
  const size_t col3 = (size_t)3 * (g.kz + 2) * sizeof(double);
  if (col3 * g.solve_x * g.solve_y > 200 * 1024) return false;
  if ((size_t)3 * (g.kz + 2) * elem * g.vert_x * g.vert_y > 200 * 1024) return false;
  return g.col_x * g.col_y <= 1024;
}

// Per-group device time (ms) of `steps` eager steps with the shapes in x->g.
template <class R>
int time_groups(mlc_ctx *x, Arrays<R> &a, int steps, double ms[4]) {
  Recorder rec;
  rec.s = x->stream;
  for (int n = 0; n < steps; ++n) enqueue_step<R>(x, a, &rec);
  MLC_TRY(cudaStreamSynchronize(x->stream));
  for (int q = 0; q < 4; ++q) ms[q] = 0.0;
  for (auto &m : rec.marks) {
    float t = 0.f;
    cudaEventElapsedTime(&t, m.a, m.b);
    const int gq = group_of(m.name);
    if (gq >= 0) ms[gq] += t;
  }
  for (int q = 0; q < 4; ++q) ms[q] /= steps;
  return cuda_status(cudaGetLastError());
}

template <class R>
int autotune_impl(mlc_ctx *x, Arrays<R> &a, int steps, mlc_tune_report *rep) {
  void *snap = nullptr;
  if (cudaMalloc(&snap, x->arena_bytes) != cudaSuccess) {
    cudaGetLastError();
    return MLC_ERR_NOMEM;
  }
  const int uv0 = x->uv_role, adv0 = x->adv_role;
  MLC_TRY(cudaMemcpyAsync(snap, x->arena, x->arena_bytes, cudaMemcpyDeviceToDevice, x->stream));
  auto restore = [&]() {
    cudaMemcpyAsync(x->arena, snap, x->arena_bytes, cudaMemcpyDeviceToDevice, x->stream);
    x->uv_role = uv0;
    x->adv_role = adv0;
  };
  const Geom base = x->g;
  double best[4] = {1e30, 1e30, 1e30, 1e30};
  int pick[4] = {0, 0, 0, 0};
  int st = MLC_OK;
  const int ntrial = 6;
  for (int tr = 0; tr < ntrial && st == MLC_OK; ++tr) {
    Geom g = base;
    g.col_x = kColCand[tr % kNCol][0]; g.col_y = kColCand[tr % kNCol][1];
    g.solve_x = kSolveCand[tr % kNSolve][0]; g.solve_y = kSolveCand[tr % kNSolve][1];
    g.vert_x = kVertCand[tr % kNVert][0]; g.vert_y = kVertCand[tr % kNVert][1];
    g.htile = tr % kNTile;
    const bool fit = shapes_fit(g, (int)sizeof(R));
    if (!fit) {  // fall back to the base solve/vertical shapes for this trial
      g.solve_x = base.solve_x; g.solve_y = base.solve_y;
      g.vert_x = base.vert_x; g.vert_y = base.vert_y;
    }
    x->g = g;
    double ms[4];
    restore();
    st = time_groups<R>(x, a, 1, ms);  // first use of the shapes
    if (st != MLC_OK) break;
    restore();
    st = time_groups<R>(x, a, steps, ms);
    if (st != MLC_OK) break;
    const int idx[4] = {tr % kNCol, fit ? tr % kNSolve : 0, fit ? tr % kNVert : 0, tr % kNTile};
    for (int q = 0; q < 4; ++q)
      if (ms[q] < best[q]) { best[q] = ms[q]; pick[q] = idx[q]; }
  }
  // the fixed reference configuration: 32 x 8 columns and tiles
  Geom fixed = base;
  fixed.col_x = 32; fixed.col_y = 8; fixed.htile = 0;
  fixed.solve_x = 32; fixed.solve_y = 2; fixed.vert_x = 32; fixed.vert_y = 2;
  double msf[4] = {0, 0, 0, 0}, mst[4] = {0, 0, 0, 0};
  if (st == MLC_OK) {
    x->g = fixed;
    restore();
    st = time_groups<R>(x, a, steps, msf);
  }
  Geom tuned = base;
  tuned.col_x = kColCand[pick[0]][0]; tuned.col_y = kColCand[pick[0]][1];
  tuned.solve_x = kSolveCand[pick[1]][0]; tuned.solve_y = kSolveCand[pick[1]][1];
  tuned.vert_x = kVertCand[pick[2]][0]; tuned.vert_y = kVertCand[pick[2]][1];
  tuned.htile = pick[3];
  if (!shapes_fit(tuned, (int)sizeof(R))) tuned = base;
  if (st == MLC_OK) {
    x->g = tuned;
    restore();
    st = time_groups<R>(x, a, steps, mst);
  }
  restore();
  cudaStreamSynchronize(x->stream);
  cudaFree(snap);
  if (st != MLC_OK) {
    x->g = base;
    return st;
  }
  x->g = tuned;
  for (auto &gx : x->graph)
    if (gx) { cudaGraphExecDestroy(gx); gx = nullptr; }
  if (rep) {
    rep->col_x = tuned.col_x; rep->col_y = tuned.col_y;
    rep->solve_x = tuned.solve_x; rep->solve_y = tuned.solve_y;
    rep->vert_x = tuned.vert_x; rep->vert_y = tuned.vert_y;
    rep->htile = tuned.htile;
    rep->ms_fixed = msf[0] + msf[1] + msf[2] + msf[3];
    rep->ms_tuned = mst[0] + mst[1] + mst[2] + mst[3];
  }
  return MLC_OK;
}

}  // namespace

extern "C" {

int mlc_autotune(mlc_ctx *x, int steps, mlc_tune_report *rep) {
  if (!x || steps < 1) return MLC_ERR_INVALID;
  if (!x->have_static || !x->have_state || (x->c.apply_bdy && !x->have_bdy)) return MLC_ERR_STATE;
  return x->prm.precision == MLC_PREC_MIXED ? autotune_impl<float>(x, x->af, steps, rep)
                                            : autotune_impl<double>(x, x->ad, steps, rep);
}

// Kernels one mlc_step(ctx, 1) launches (for launch accounting).
int mlc_launches_per_step(const mlc_ctx *x) { return x ? x->launches_per_step : 0; }

// Run steps without graph capture (for tests of the capture path).
int mlc_set_graphs(mlc_ctx *x, int on) {
  if (!x) return MLC_ERR_INVALID;
  x->use_graphs = on != 0;
  return MLC_OK;
}

}  // extern "C"
