// mlc_context.cu -- the C ABI of moloch_gb300.h.
//
// A context owns one CUDA stream, a stream-ordered memory pool and a table of
// member slots.  A member is one domain: one allocation (its arena) carved
// into 256-byte aligned arrays that hold its static fields, state, boundary
// data and scratch in the padded layout of mlc_device.cuh.  The kernels of
// mlc_sound.cu, mlc_advect.cu and mlc_end.cu read a device table with one
// descriptor Dom<R> per active member, so each kernel stage is one launch for
// all members whatever their extents.  The boundary clocks, diagnostics and
// ping-pong buffer roles stay on the device (the last kernel of a step
// advances them), so one recorded CUDA graph replays every step; it is
// recorded again only when the launch geometry changes (members joining or
// leaving, new launch shapes).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include <cuda.h>          // CUtensorMap and its enums (the encoder is fetched at run time)
#include <cudaTypedefs.h>

#include "../../include/moloch_gb300.h"
#include "../../include/moloch_gb300_restart.h"
#include "mlc_kernels.cuh"

using namespace mlc;

namespace {

constexpr size_t kAlign = 256;
constexpr int kMaxLevels = 128;
constexpr int kMaxSlots = 4096;
constexpr int kMaxExtent = 32768;

// Text of the last failing CUDA call on this thread (mlc_last_error).
thread_local const char *g_last_error = "no error";

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

template <class T>
T *W(const T *p) { return const_cast<T *>(p); }

// Advected fields of type R per member (the table order of mlc_advect.cu).
int n_table_r(const mlc_dims &d, const mlc_params &p, bool f64) {
  return (f64 ? 2 : 0) + 4 + (p.ipptls > 0 ? d.nqx - 1 : 0) + (p.ibltyp == 2 ? 1 : 0) + d.ntr;
}

// Doubles of the packed state of one domain (the staging buffer's size).
size_t state_elems(const mlc_dims &d) {
  const size_t c2 = (size_t)(d.jx - 1) * (d.iy - 1);
  const size_t u3 = (size_t)d.jx * (d.iy - 1) * d.kz, v3 = (size_t)(d.jx - 1) * d.iy * d.kz;
  const size_t c3 = c2 * d.kz;
  // w and tke (kz+1 levels), the cross-point fields, species and ps
  return u3 + v3 + 2 * c2 * (d.kz + 1) + c3 * (9 + d.nqx + d.ntr) + c2;
}

Geom make_geom(const mlc_dims &d, int elem_bytes) {
  Geom g{};
  g.jx = d.jx; g.iy = d.iy; g.kz = d.kz; g.nqx = d.nqx; g.ntr = d.ntr;
  const int per_line = 128 / elem_bytes;
  g.P = (d.jx + per_line - 1) / per_line * per_line;
  g.PS = (size_t)g.P * d.iy;
  return g;
}

// Sine modes of spectral nudging (lowpass_init, Main/mod_bdycod.F90:3852-3853;
// one process: njcross = jx-1, nicross = iy-1, ds in km): 2*km in x, 2*lm in y.
void spectral_modes(const mlc_dims &d, const mlc_params &p, int &km2, int &lm2) {
  const double ds = p.dx / 1000.0;
  const long km = std::lround(((double)(d.jx - 1) * ds) / 1500.0);
  const long lm = std::lround(((double)(d.iy - 1) * ds) / 750.0);
  km2 = 2 * (int)std::max(km, 1L);
  lm2 = 2 * (int)std::max(lm, 1L);
}

Scal make_scal(const mlc_params &p) {
  Scal c{};
  c.dx = p.dx;
  c.rdx = 1.0 / p.dx;
  c.dtsec = p.dtsec;
  c.dt = p.dtsec;
  c.dtstepa = p.dtsec / (double)p.mo_nadv;
  c.dtsound = c.dtstepa / (double)p.mo_nsound;
  c.dtbdys = p.dtbdys;
  c.rtb = 1.0 / p.dtbdys;
  c.nadv = p.mo_nadv;
  c.nsound = p.mo_nsound;
  c.divdamp = p.mo_divdamp;
  c.divfilter = p.mo_divfilter;
  c.top_nudge = p.mo_top_nudge;
  c.apply_bdy = p.do_apply_bdy;
  c.lrotllr = p.lrotllr;
  c.ipptls = p.ipptls;
  c.present_qc = p.present_qc;
  c.present_qi = p.present_qi;
  c.nspgx = p.nspgx;
  c.nztop = p.mo_top_nudge ? p.nztop : 0;
  c.debug_level = p.debug_level;
  c.dxf = float(c.dx); c.rdxf = float(c.rdx); c.dtsecf = float(c.dtsec);
  c.dtstepaf = float(c.dtstepa); c.dtsoundf = float(c.dtsound);
  const double gdts = kGrav * c.dtsound;
  c.gdts_hi = float(gdts);
  c.gdts_lo = float(gdts - (double)c.gdts_hi);
  c.dtrdxs = c.dtsound * c.rdx;
  c.dxrdt = c.dx / c.dtsound;
  c.dtrdxsf = c.dtsoundf * c.rdxf;
  c.dxrdtf = c.dxf / c.dtsoundf;
  c.spectral = p.mo_spectral_nudge;
  c.dtrad = p.dtrad;
  c.tke = p.ibltyp == 2 ? 1 : 0;
  return c;
}

// Lay out one member's arrays.  Both halves of every ping-pong pair, one wz
// scratch field per advected field, the FP64 copies of the vertical metric
// for the solve of a mixed member, boundary pairs b0/b1 and the reduction
// partials.
template <class R>
void carve_dom(Carver &cv, Dom<R> &D, const Geom &g, const mlc_dims &d, const mlc_params &p) {
  const bool f64 = sizeof(R) == sizeof(double);
  const size_t F = g.field3(), F1 = g.PS * (size_t)(g.kz + 1), P2 = g.PS;
  for (int h = 0; h < 2; ++h) {
    D.u[h] = cv.take<R>(F); D.v[h] = cv.take<R>(F);
    D.ux[h] = cv.take<R>(F); D.vx[h] = cv.take<R>(F); D.wx[h] = cv.take<R>(F);
    D.qx[h] = cv.take<R>(F * d.nqx);
    D.trac[h] = d.ntr ? cv.take<R>(F * d.ntr) : nullptr;
    D.pai[h] = cv.take<double>(F); D.tetav[h] = cv.take<double>(F);
    D.tkex[h] = p.ibltyp == 2 ? cv.take<R>(F) : nullptr;
  }
  D.tke = p.ibltyp == 2 ? cv.take<R>(F1) : nullptr;
  D.w = cv.take<R>(F1); D.t = cv.take<R>(F); D.tvirt = cv.take<R>(F); D.p = cv.take<R>(F);
  D.rho = cv.take<R>(F); D.qsat = cv.take<R>(F); D.ps = cv.take<double>(P2);
  D.s = cv.take<R>(F1); D.zdiv2 = cv.take<R>(F); D.tetavf = cv.take<double>(F1);
  const int nr = n_table_r(d, p, f64);
  for (int f = 0; f < kMaxFields; ++f) D.wz[f] = f < nr ? cv.take<R>(F) : nullptr;
  for (int f = 0; f < 2; ++f) D.wz_d[f] = f64 ? nullptr : cv.take<double>(F);
  D.vdiv = f64 ? cv.take<double>(F) : nullptr;
  D.vzamu = f64 ? cv.take<double>(F) : nullptr;
  D.vzmih = f64 ? cv.take<double>(F) : nullptr;
  D.vzmi = f64 ? cv.take<double>(F) : nullptr;
  Stat<R> &s = D.sa;
  s.fmz = cv.take<R>(F); s.fmzf = cv.take<R>(F1); s.rfmzu = cv.take<R>(F); s.rfmzv = cv.take<R>(F);
  if (f64) {
    s.fmz_d = reinterpret_cast<const double *>(s.fmz);
    s.fmzf_d = reinterpret_cast<const double *>(s.fmzf);
    s.cfz = nullptr;
  } else {
    s.fmz_d = s.fmzf_d = nullptr;
    s.cfz = cv.take<double>(F1);
  }
  s.zrfmu = cv.take<R>(F); s.zrfmd = cv.take<R>(F);
  s.zeta = cv.take<double>(F); s.dz = cv.take<double>(F);
  s.hx = cv.take<R>(P2); s.hy = cv.take<R>(P2); s.msfu = cv.take<R>(P2); s.msfv = cv.take<R>(P2);
  s.msfx = cv.take<R>(P2); s.mx2 = cv.take<R>(P2); s.rmu = cv.take<R>(P2); s.rmv = cv.take<R>(P2);
  s.coru = cv.take<R>(P2); s.corv = cv.take<R>(P2);
  s.ibnd_cr = cv.take<int32_t>(P2); s.ibnd_ud = cv.take<int32_t>(P2); s.ibnd_vd = cv.take<int32_t>(P2);
  s.hefc = cv.take<double>((size_t)p.nspgx * d.kz); s.fcx = cv.take<double>(p.nspgx);
  s.tnudge = cv.take<double>(d.kz); s.ffilt = cv.take<double>(d.kz); s.gzitakh = cv.take<double>(d.kz);
  s.xkdamp = cv.take<double>(d.kz); s.xknu = cv.take<double>(d.kz); s.gzitak = cv.take<double>(d.kz + 1);
  s.rlat = cv.take<double>(d.iy);
  if (f64) {
    s.dv_cu = cv.take<double>(F); s.dv_cv = cv.take<double>(F); s.dv_cf = cv.take<double>(F);
    s.mo_du = cv.take<double>(F); s.mo_dv = cv.take<double>(F);
    s.mo_gu = cv.take<double>(F); s.mo_gv = cv.take<double>(F);
    s.mo_cu = cv.take<double>(P2); s.mo_cv = cv.take<double>(P2);
    s.sv_a = cv.take<double>(F); s.sv_b = cv.take<double>(F); s.sv_c = cv.take<double>(F);
  } else {
    s.dv_cu = s.dv_cv = s.dv_cf = s.mo_du = s.mo_dv = s.mo_gu = s.mo_gv = s.mo_cu = s.mo_cv = nullptr;
    s.sv_a = s.sv_b = s.sv_c = nullptr;
  }
  if (f64) {
    s.gzitak_r = reinterpret_cast<const R *>(s.gzitak);
    s.gzitakh_r = reinterpret_cast<const R *>(s.gzitakh);
    s.xkdamp_r = reinterpret_cast<const R *>(s.xkdamp);
    s.xknu_r = reinterpret_cast<const R *>(s.xknu);
    s.ffilt_r = reinterpret_cast<const R *>(s.ffilt);
    s.tnudge_r = reinterpret_cast<const R *>(s.tnudge);
    s.hefc_r = reinterpret_cast<const R *>(s.hefc);
    s.fcx_r = reinterpret_cast<const R *>(s.fcx);
    s.dz_r = reinterpret_cast<const R *>(s.dz);
    s.dz_lo = nullptr;
  } else {
    s.gzitak_r = cv.take<R>(d.kz + 1); s.gzitakh_r = cv.take<R>(d.kz);
    s.xkdamp_r = cv.take<R>(d.kz); s.xknu_r = cv.take<R>(d.kz); s.ffilt_r = cv.take<R>(d.kz);
    s.tnudge_r = cv.take<R>(d.kz); s.hefc_r = cv.take<R>((size_t)p.nspgx * d.kz);
    s.fcx_r = cv.take<R>(p.nspgx); s.dz_r = cv.take<R>(F); s.dz_lo = cv.take<R>(F);
  }
  Bdy<R> &b = D.bd;
  for (int h = 0; h < 2; ++h) {
    b.xtb[h] = cv.take<double>(F); b.xqb[h] = cv.take<R>(F); b.xpaib[h] = cv.take<double>(F);
    b.xlb[h] = p.present_qc ? cv.take<R>(F) : nullptr;
    b.xib[h] = p.present_qi ? cv.take<R>(F) : nullptr;
    b.dub[h] = cv.take<R>(F); b.dvb[h] = cv.take<R>(F);
    b.chib[h] = d.ntr ? cv.take<R>(F * d.ntr) : nullptr;
    b.xpsb[h] = cv.take<double>(P2);
  }
  if (p.mo_spectral_nudge) {
    int km2, lm2;
    spectral_modes(d, p, km2, lm2);
    s.bvx = cv.take<R>((size_t)km2 * d.jx);
    s.bvy = cv.take<R>((size_t)lm2 * d.iy);
    s.cnudge = cv.take<R>(d.kz);
    D.spec = cv.take<R>((size_t)3 * d.kz * d.iy * km2);
  } else {
    s.bvx = s.bvy = s.cnudge = nullptr;
    D.spec = nullptr;
  }
  D.red_blocks = reduce_blocks(g);
  D.partials = cv.take<double>((size_t)D.red_blocks * 8);
  D.tmap = cv.take<char>((size_t)kTileShapes * kTmapSlots * kTmapBytes);
}

template <class R>
size_t arena_bytes(const mlc_dims &d, const mlc_params &p) {
  Dom<R> D{};
  Carver cv;
  carve_dom<R>(cv, D, make_geom(d, (int)sizeof(R)), d, p);
  return cv.off;
}

int validate_params(const mlc_params *p) {
  if (!p) return MLC_ERR_INVALID;
  if (!(p->dtsec > 0) || !(p->dx > 0) || !(p->mo_ztop > 0) || p->mo_nadv < 1 || p->mo_nsound < 1)
    return MLC_ERR_INVALID;
  if (!(p->dtbdys > 0) || p->nspgx < 3 || p->nspgd < 3) return MLC_ERR_INVALID;
  if (p->ipptls < 0 || p->ipptls > 5) return MLC_ERR_UNSUPPORTED;
  if (p->mo_spectral_nudge && !(p->dtrad > 0)) return MLC_ERR_INVALID;
  if (p->precision != MLC_PREC_FP64 && p->precision != MLC_PREC_MIXED) return MLC_ERR_INVALID;
  return MLC_OK;
}

int validate_dims(const mlc_dims *d, const mlc_params *p) {
  if (!d) return MLC_ERR_INVALID;
  if (d->jx < 10 || d->iy < 10 || d->kz < 4 || d->kz > kMaxLevels) return MLC_ERR_INVALID;
  // With these bounds (and at most kMaxSlots members) every grid dimension of
  // every launch stays within CUDA's limits (y and z below 65536).
  if (d->jx > kMaxExtent || d->iy > kMaxExtent) return MLC_ERR_TOO_LARGE;
  // kernels index within one 3-D field with 32-bit offsets
  if ((size_t)(d->jx + 32) * (size_t)d->iy * (size_t)(d->kz + 1) >= ((size_t)1 << 31))
    return MLC_ERR_TOO_LARGE;
  if (d->nqx < 2 || d->nqx > 10 || d->ntr < 0 || d->ntr > 8) return MLC_ERR_INVALID;
  // species per microphysics class (Main/mod_params.F90:1724-1736)
  if (p->ipptls >= 2 && d->nqx != (p->ipptls <= 3 ? 5 : p->ipptls == 4 ? 7 : 10))
    return MLC_ERR_INVALID;
  if (n_table_r(*d, *p, true) > kMaxFields) return MLC_ERR_UNSUPPORTED;
  // the tracer relaxation assumes disjoint south/north and west/east bands
  if (d->ntr > 0 && (d->jx - 1 < 2 * p->nspgx || d->iy - 1 < 2 * p->nspgx)) return MLC_ERR_UNSUPPORTED;
  if (p->mo_spectral_nudge) {
    int km2, lm2;
    spectral_modes(*d, *p, km2, lm2);
    if (km2 > kMaxModes || lm2 > kMaxModes) return MLC_ERR_UNSUPPORTED;
  }
  return MLC_OK;
}

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return MLC_OK;
  g_last_error = cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return MLC_ERR_NOMEM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return MLC_ERR_NODEVICE;
  return MLC_ERR_CUDA;
}

#define MLC_TRY(x)                                 \
  do {                                             \
    cudaError_t e_ = (x);                          \
    if (e_ != cudaSuccess) return cuda_status(e_); \
  } while (0)

#define MLC_CHK(x)               \
  do {                           \
    int s_ = (x);                \
    if (s_ != MLC_OK) return s_; \
  } while (0)

struct Member {
  bool used = false;
  mlc_dims dims{};
  Geom g{};
  Scal c{};
  void *raw = nullptr;   // the allocation (returned to the pool on removal)
  char *base = nullptr;  // 256-byte aligned start of the arena
  size_t bytes = 0;      // arena bytes
  Dom<double> dd{};      // descriptor of an FP64 member
  Dom<float> df{};       // descriptor of a mixed member
  bool have_static = false, have_state = false, have_bdy = false;
  // physics tendencies (allocated at the first mlc_member_set_tendencies;
  // live only between that call and the end of the open step)
  void *tend_raw = nullptr;
  size_t tend_bytes = 0;
  bool tend_live = false;
  int stall_polls = 0;   // test hook of the bounded waits (mlc_member_test_stall)
};

template <class R> Dom<R> &dom_of(Member &m);
template <> Dom<double> &dom_of<double>(Member &m) { return m.dd; }
template <> Dom<float> &dom_of<float>(Member &m) { return m.df; }

// What a recorded step graph depends on besides the device table contents.
struct GraphKey {
  LaunchGeom L;
  int any_copy;   // some member keeps non-advected species (ipptls = 0)
  int any_curv;   // some member has non-zero curvature terms
  int any_tke;    // the members carry TKE (ibltyp = 2)
};

}  // namespace

struct mlc_ctx {
  mlc_params prm{};
  bool mixed = false;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaMemPool_t pool = nullptr;
  std::vector<Member> mem;     // slots
  Clock *clks = nullptr;       // device, one per slot
  DiagDev *diags = nullptr;    // device, one per slot
  void *table = nullptr;       // device descriptor table (active members in slot order)
  double *staging = nullptr;   // layout conversion buffer shared by all members
  size_t staging_elems = 0;
  size_t budget = 0;           // bound on the bytes of all member arenas (0: none)
  size_t in_use = 0;           // bytes of all member arenas
  GraphKey key{};              // launch geometry and shapes of the next step
  bool table_dirty = true;
  cudaGraphExec_t graph = nullptr;
  GraphKey graph_key{};        // what the recorded graph was recorded with
  bool graph_valid = false;
  bool use_graphs = true;
  int launches_per_step = 0;
  bool step_open = false;      // between mlc_step_dynamics and mlc_step_finish
  // work lists of an uneven batch (one device buffer for all tilings) and the
  // launch shapes they were built for
  WorkItem *wl_buf = nullptr;
  size_t wl_cap = 0;           // entries
  bool wl_dirty = true;        // members changed since the lists were built
  int wl_key[6] = {-1, -1, -1, -1, -1, -1};
  const WorkItem *wl_ptr[7] = {};  // the lists in wl_buf (null: none) ...
  int wl_n[7] = {};                // ... and their lengths
};

namespace {

bool member_ok(const mlc_ctx *x, int m) {
  return x && m >= 0 && m < (int)x->mem.size() && x->mem[m].used;
}

// Grow the shared staging buffer to hold the packed state of extents d.
int ensure_staging(mlc_ctx *x, const mlc_dims &d) {
  const size_t need = state_elems(d);
  if (need <= x->staging_elems) return MLC_OK;
  if (x->staging) MLC_TRY(cudaFreeAsync(x->staging, x->stream));
  x->staging = nullptr;
  x->staging_elems = 0;
  void *p = nullptr;
  cudaError_t e = cudaMallocFromPoolAsync(&p, need * sizeof(double), x->pool, x->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return MLC_ERR_NOMEM;
  }
  x->staging = static_cast<double *>(p);
  x->staging_elems = need;
  return MLC_OK;
}

// ---- TMA tensor maps ---------------------------------------------------------
// The horizontal WAF loads each field's halo tile (rows I0-2 .. I0+nw+1, the
// warp range's 32*v columns at one level; hshape) with one tiled TMA copy,
// and the increment form the planes of theta_v, Exner and their vertical
// increments the same way.  The map's extents are the cross points (jx-1,
// iy-1, kz), so everything outside them reads as zero, as the kernels need.
// A copy must start on a 16-byte boundary: tile offsets step by 32*v - 4
// columns, a multiple of 16 bytes, and the first tile starts hshape_off
// columns left of its range so that its x times the element size is a
// multiple of 16; every box row is a multiple of 16 bytes.

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  }
  return fn;
}

template <class R>
int encode_tmaps(mlc_ctx *x, const Member &m, const Dom<R> &D) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return MLC_ERR_CUDA;
  const Geom &g = m.g;
  const int nf = n_table_r(m.dims, x->prm, sizeof(R) == sizeof(double));
  std::vector<CUtensorMap> maps((size_t)kTileShapes * kTmapSlots);
  std::memset(maps.data(), 0, maps.size() * sizeof(CUtensorMap));
  const size_t es = sizeof(R);
  const cuuint64_t dims[3] = {(cuuint64_t)(g.jx - 1), (cuuint64_t)(g.iy - 1), (cuuint64_t)g.kz};
  const cuuint32_t estr[3] = {1, 1, 1};
  auto encode = [&](CUtensorMap *mp, const void *base, size_t ebytes, HShape h) {
    const cuuint64_t strides[2] = {(cuuint64_t)g.P * ebytes, (cuuint64_t)g.PS * ebytes};
    const cuuint32_t box[3] = {(cuuint32_t)(32 * h.v + 2 * hshape_off((int)ebytes, h.v)),
                               (cuuint32_t)(h.nw + 4), 1};
    return enc(mp, ebytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3,
               const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  };
  const size_t F = g.field3();
  for (int t = 0; t < kTileShapes; ++t) {
    CUtensorMap *row = &maps[(size_t)t * kTmapSlots];
    for (int f = 0; f < nf; ++f)
      if (!encode(&row[f], D.wz[f], es, hshape((int)es, t))) return MLC_ERR_CUDA;
    if (x->mixed) {
      // double-float planes: hi at the allocation's start, lo F floats on
      const HShape hi = hshape_inc(t);
      const double *src[6] = {D.tetav[0], D.tetav[1], D.pai[0], D.pai[1], D.wz_d[0], D.wz_d[1]};
      for (int q = 0; q < 6; ++q) {
        const float *h = reinterpret_cast<const float *>(src[q]);
        if (!encode(&row[kMaxFields + 2 * q], h, 4, hi) ||
            !encode(&row[kMaxFields + 2 * q + 1], h + F, 4, hi))
          return MLC_ERR_CUDA;
      }
    }
  }
  MLC_TRY(cudaMemcpyAsync(const_cast<void *>(D.tmap), maps.data(), maps.size() * sizeof(CUtensorMap),
                          cudaMemcpyHostToDevice, x->stream));
  return cuda_status(cudaStreamSynchronize(x->stream));
}

// Give slot `slot` a member of extents d: allocate and zero its arena, reset
// its clock and diagnostics.  Every array starts at zero: s and w at the ring
// stay zero, as the reference's reset_tendencies and init_moloch leave them.
int add_member(mlc_ctx *x, int slot, const mlc_dims &d) {
  MLC_CHK(validate_dims(&d, &x->prm));
  Member m{};
  m.dims = d;
  m.g = make_geom(d, x->mixed ? 4 : 8);
  m.c = make_scal(x->prm);
  if (x->prm.mo_spectral_nudge) spectral_modes(d, x->prm, m.c.km2, m.c.lm2);
  m.bytes = x->mixed ? arena_bytes<float>(d, x->prm) : arena_bytes<double>(d, x->prm);
  if (x->budget && x->in_use + m.bytes > x->budget) return MLC_ERR_BUDGET;
  MLC_CHK(ensure_staging(x, d));
  cudaError_t e = cudaMallocFromPoolAsync(&m.raw, m.bytes + kAlign, x->pool, x->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return MLC_ERR_NOMEM;
  }
  m.base = reinterpret_cast<char *>(align_up(reinterpret_cast<uintptr_t>(m.raw)));
  Carver cv{m.base, 0};
  if (x->mixed) carve_dom<float>(cv, m.df, m.g, d, x->prm);
  else carve_dom<double>(cv, m.dd, m.g, d, x->prm);
  MLC_TRY(cudaMemsetAsync(m.base, 0, m.bytes, x->stream));
  MLC_TRY(cudaMemsetAsync(x->clks + slot, 0, sizeof(Clock), x->stream));
  MLC_TRY(cudaMemsetAsync(x->diags + slot, 0, sizeof(DiagDev), x->stream));
  MLC_TRY(cudaStreamSynchronize(x->stream));
  {
    const int st = x->mixed ? encode_tmaps<float>(x, m, m.df) : encode_tmaps<double>(x, m, m.dd);
    if (st != MLC_OK) {
      cudaFreeAsync(m.raw, x->stream);
      return st;
    }
  }
  m.used = true;
  x->mem[slot] = m;
  x->in_use += m.bytes;
  x->table_dirty = true;
  return MLC_OK;
}

int remove_member(mlc_ctx *x, int slot) {
  Member &m = x->mem[slot];
  // stream order puts the release after every step already enqueued
  MLC_TRY(cudaFreeAsync(m.raw, x->stream));
  if (m.tend_raw) MLC_TRY(cudaFreeAsync(m.tend_raw, x->stream));
  x->in_use -= m.bytes + m.tend_bytes;
  m = Member{};
  x->table_dirty = true;
  return MLC_OK;
}

// Upload the descriptor table of the active members and derive the launch
// geometry (maxima over the members; the launch shapes are kept).
template <class R>
int refresh(mlc_ctx *x) {
  if (!x->table_dirty) return MLC_OK;
  std::vector<Dom<R>> t;
  t.reserve(x->mem.size());
  GraphKey k = x->key;
  LaunchGeom &L = k.L;
  L.jx = L.iy = L.kz = 0;
  L.nadv_r = 0;
  L.nadv_d = x->mixed ? 2 : 0;
  L.red_blocks = 0;
  k.any_copy = 0;
  k.any_curv = 0;
  k.any_tke = 0;
  for (size_t slot = 0; slot < x->mem.size(); ++slot) {
    Member &m = x->mem[slot];
    if (!m.used) continue;
    Dom<R> D = dom_of<R>(m);
    D.g = m.g;
    D.c = m.c;
    D.clk = x->clks + slot;
    D.diag = x->diags + slot;
    D.active = 1;
    D.stall_polls = m.stall_polls;
    D.tend = m.tend_live ? static_cast<const R *>(m.tend_raw) : nullptr;
    t.push_back(D);
    L.jx = std::max(L.jx, m.g.jx);
    L.iy = std::max(L.iy, m.g.iy);
    L.kz = std::max(L.kz, m.g.kz);
    L.nadv_r = std::max(L.nadv_r, n_table_r(m.dims, x->prm, !x->mixed));
    L.red_blocks = std::max(L.red_blocks, D.red_blocks);
    if (x->prm.ipptls == 0 && m.dims.nqx > 1) k.any_copy = 1;
    if (m.c.curvature) k.any_curv = 1;
    if (m.c.tke) k.any_tke = 1;
  }
  L.nmem = (int)t.size();
  if (!t.empty()) {
    MLC_TRY(cudaMemcpyAsync(x->table, t.data(), t.size() * sizeof(Dom<R>), cudaMemcpyHostToDevice,
                            x->stream));
    MLC_TRY(cudaStreamSynchronize(x->stream));
  }
  x->key = k;
  x->table_dirty = false;
  x->wl_dirty = true;
  return MLC_OK;
}

// Work lists of an uneven batch (kernels read them through WorkItem; see
// mlc_device.cuh): one entry per block that has work, for each tiling the
// step launches, in the order of the grids they replace (tiles along j
// fastest).  A batch whose members all have the same extents keeps the plain
// grids.  Called before every launch sequence (never inside a capture); the
// lists follow the members and the launch shapes of x->key.L.
template <class R>
int ensure_lists(mlc_ctx *x) {
  LaunchGeom &L = x->key.L;
  std::vector<const Member *> act;
  for (const Member &m : x->mem)
    if (m.used) act.push_back(&m);
  bool uneven = false;
  for (const Member *m : act)
    uneven = uneven || m->g.jx != L.jx || m->g.iy != L.iy || m->g.kz != L.kz;
  const int key[6] = {uneven ? 1 : 0, L.col_x, L.col_y, L.vert_x, L.vert_y, L.htile};
  // the launch geometry always takes the lists from the context (a copy of
  // an older geometry may carry stale ones)
  auto apply = [&]() {
    L.wl_pt = x->wl_ptr[0]; L.wl_v4 = x->wl_ptr[1]; L.wl_solve = x->wl_ptr[2];
    L.wl_vert = x->wl_ptr[3]; L.wl_vinc = x->wl_ptr[4]; L.wl_h = x->wl_ptr[5];
    L.wl_hinc = x->wl_ptr[6];
    L.n_pt = x->wl_n[0]; L.n_v4 = x->wl_n[1]; L.n_solve = x->wl_n[2]; L.n_vert = x->wl_n[3];
    L.n_vinc = x->wl_n[4]; L.n_h = x->wl_n[5]; L.n_hinc = x->wl_n[6];
    return MLC_OK;
  };
  if (!x->wl_dirty && std::memcmp(key, x->wl_key, sizeof(key)) == 0) return apply();
  for (int q = 0; q < 7; ++q) {
    x->wl_ptr[q] = nullptr;
    x->wl_n[q] = 0;
  }
  std::memcpy(x->wl_key, key, sizeof(key));
  x->wl_key[0] = -1;  // valid only once the lists are built
  if (!uneven) {
    std::memcpy(x->wl_key, key, sizeof(key));
    x->wl_dirty = false;
    return apply();
  }
  const bool f64 = sizeof(R) == sizeof(double);
  std::vector<WorkItem> all;
  auto cdiv = [](int a, int b) { return (a + b - 1) / b; };
  auto push = [&](int m, int a, int b, int c) {
    all.push_back(WorkItem{(int16_t)m, (int16_t)a, (int16_t)b, (int16_t)c});
  };
  size_t off[7];
  // point kernels: col_x x col_y tiles over jx x iy, level chunks
  off[0] = all.size();
  for (int m = 0; m < (int)act.size(); ++m) {
    const Geom &g = act[m]->g;
    for (int kc = 0; kc < cdiv(g.kz, kPtLevels); ++kc)
      for (int bi = 0; bi < cdiv(g.iy, L.col_y); ++bi)
        for (int bj = 0; bj < cdiv(g.jx, L.col_x); ++bj) push(m, bj, bi, kc);
  }
  // four-column lanes: 128 x 4 tiles (mixed members)
  off[1] = all.size();
  if (!f64)
    for (int m = 0; m < (int)act.size(); ++m) {
      const Geom &g = act[m]->g;
      for (int kc = 0; kc < cdiv(g.kz, kPtLevels); ++kc)
        for (int bi = 0; bi < cdiv(g.iy, 4); ++bi)
          for (int bj = 0; bj < cdiv(g.jx, 128); ++bj) push(m, bj, bi, kc);
    }
  // column solves: 128-column segments of the rows i = 2 .. iy-2
  off[2] = all.size();
  for (int m = 0; m < (int)act.size(); ++m) {
    const Geom &g = act[m]->g;
    for (int r = 0; r < g.iy - 3; ++r)
      for (int bj = 0; bj < cdiv(g.jx - 1, f64 ? kSolveColsD : kSolveColsF); ++bj) push(m, bj, r, 0);
  }
  // vertical WAF: column tiles, the member's own fields of the R table
  off[3] = all.size();
  for (int m = 0; m < (int)act.size(); ++m) {
    const Geom &g = act[m]->g;
    const int nf = n_table_r(act[m]->dims, x->prm, f64);
    for (int bi = 0; bi < cdiv(g.iy - 1, L.vert_y); ++bi)
      for (int bj = 0; bj < cdiv(g.jx - 1, L.vert_x); ++bj)
        for (int f = 0; f < nf; ++f) push(m, bj, bi, f);
  }
  // the same for theta_v and Exner of mixed members
  off[4] = all.size();
  if (!f64)
    for (int m = 0; m < (int)act.size(); ++m) {
      const Geom &g = act[m]->g;
      for (int bi = 0; bi < cdiv(g.iy - 1, L.vert_y); ++bi)
        for (int bj = 0; bj < cdiv(g.jx - 1, L.vert_x); ++bj)
          for (int f = 0; f < 2; ++f) push(m, bj, bi, f);
    }
  // horizontal WAF tiles of the shape in use, every level
  auto htiles = [&](HShape h) {
    const int S = 32 * h.v - 4;
    for (int m = 0; m < (int)act.size(); ++m) {
      const Geom &g = act[m]->g;
      const int tj = cdiv(g.jx - 3 - hshape_ob0(h.v), S), ti = cdiv(g.iy - 1, h.nw);
      for (int k = 0; k < g.kz; ++k)
        for (int bi = 0; bi < ti; ++bi)
          for (int bj = 0; bj < tj; ++bj) push(m, bj, bi, k);
    }
  };
  off[5] = all.size();
  htiles(hshape((int)sizeof(R), L.htile));
  off[6] = all.size();
  if (!f64) htiles(hshape_inc(L.htile));
  const size_t total = all.size();
  if (total > x->wl_cap) {
    if (x->wl_buf) MLC_TRY(cudaFree(x->wl_buf));
    x->wl_buf = nullptr;
    x->wl_cap = 0;
    cudaError_t e = cudaMalloc(&x->wl_buf, total * sizeof(WorkItem));
    if (e != cudaSuccess) {
      cudaGetLastError();
      x->wl_buf = nullptr;
      return MLC_ERR_NOMEM;
    }
    x->wl_cap = total;
  }
  MLC_TRY(cudaMemcpyAsync(x->wl_buf, all.data(), total * sizeof(WorkItem), cudaMemcpyHostToDevice,
                          x->stream));
  MLC_TRY(cudaStreamSynchronize(x->stream));
  for (int q = 0; q < 7; ++q) {
    const size_t end = q == 6 ? total : off[q + 1];
    x->wl_n[q] = (int)(end - off[q]);
    x->wl_ptr[q] = x->wl_n[q] ? x->wl_buf + off[q] : nullptr;
  }
  std::memcpy(x->wl_key, key, sizeof(key));
  x->wl_dirty = false;
  return apply();
}

template <class R>
int refresh_all(mlc_ctx *x) {
  MLC_CHK(refresh<R>(x));
  return ensure_lists<R>(x);
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

#define REC(name, call)        \
  do {                         \
    if (rec) rec->begin(name); \
    call;                      \
    if (rec) rec->end();       \
  } while (0)

// Enqueue one model step (Main/mod_moloch.F90:312-446) of every active
// member on the context stream; returns the number of kernels launched.
// The offsets count the acoustic substeps (uvoff) and advection rounds
// (advoff) since the step began; with the roles in each member's clock they
// name the buffers every launch works on.  phase: kStepAll the whole step;
// kStepDynamics up to mkslice (:312-357), kStepFinish from status_update
// (:376-446) to the end, the two halves around the physics.
constexpr int kStepAll = 0, kStepDynamics = 1, kStepFinish = 2;
template <class R>
int enqueue_step(mlc_ctx *x, Recorder *rec = nullptr, int phase = kStepAll) {
  using K = Launch<R>;
  const LaunchGeom &L = x->key.L;
  const Dom<R> *d = static_cast<const Dom<R> *>(x->table);
  cudaStream_t s = x->stream;
  const int nadv = x->prm.mo_nadv, nsound = x->prm.mo_nsound;
  int nl = 0;
  for (int r = 0; r < nadv && phase != kStepFinish; ++r) {
    // ---- sound (Main/mod_moloch.F90:531-765) ----
    REC("sound_prep", K::sound_prep(L, d, r, s)); ++nl;
    for (int n = 0; n < nsound; ++n) {
      const int uvoff = r * nsound + n;
      REC("sound_div", K::sound_div(L, d, uvoff, s)); ++nl;
      REC("sound_solve", K::sound_solve(L, d, uvoff, r, n == nsound - 1, s)); ++nl;
      REC("sound_momentum", K::sound_momentum(L, d, uvoff, r, s)); ++nl;
    }
    // ---- advection (Main/mod_moloch.F90:767-1042) ----
    const int uvo = (r + 1) * nsound;
    REC("adv_prep", K::adv_prep(L, d, uvo, r, s)); ++nl;
    REC("adv_vertical", K::adv_vertical(L, d, r, s)); ++nl;
    if (L.nadv_d) { REC("adv_vertical_inc", K::adv_vertical_inc(L, d, r, s)); ++nl; }
    REC("adv_horizontal", K::adv_horizontal(L, d, uvo, r, s)); ++nl;
    if (L.nadv_d) { REC("adv_horizontal_inc", K::adv_horizontal_inc(L, d, uvo, r, s)); ++nl; }
    if (x->key.any_copy) { REC("adv_species_copy", K::adv_species_copy(L, d, r, s)); ++nl; }
    if (x->key.any_curv) { REC("adv_curvature", K::adv_curvature(L, d, r + 1, s)); ++nl; }
    REC("adv_back", K::adv_back(L, d, uvo, r + 1, s)); ++nl;
  }
  // ---- step end (Main/mod_moloch.F90:340-446) ----
  const int uvo = nadv * nsound, ao = nadv;
  if (phase != kStepFinish) {
    // the ring first: the point pass after it does tvirt, t and the relaxation
    if (x->prm.do_apply_bdy) { REC("bdy_ring", K::bdy_ring(L, d, uvo, ao, s)); ++nl; }
    REC("end_relax", K::end_relax(L, d, uvo, ao, s)); ++nl;
    if (x->prm.do_apply_bdy && x->prm.mo_spectral_nudge) {
      REC("bdy_spectral", K::bdy_spectral(L, d, uvo, ao, s));
      nl += 3;
    }
  }
  if (phase == kStepAll) {
    REC("end_cross", K::end_cross(L, d, uvo, ao, s)); ++nl;
  } else if (phase == kStepDynamics) {
    REC("end_mkslice", K::end_cross_split(L, d, uvo, ao, false, s)); nl += 2;
    return nl;
  } else {
    REC("end_status", K::end_cross_split(L, d, uvo, ao, true, s)); ++nl;
  }
  if (x->key.any_tke) { REC("end_tke", K::end_tke(L, d, phase == kStepAll, s)); ++nl; }
  REC("end_uvstag", K::end_uvstag(L, d, uvo, ao, s)); ++nl;
  REC("end_reduce", K::end_reduce(L, d, uvo, ao, s)); ++nl;
  return nl;
}

// Record the step into the context's graph: update the executable graph in
// place when the topology allows, instantiate a new one otherwise.
template <class R>
int record(mlc_ctx *x) {
  cudaGraph_t gr = nullptr;
  MLC_TRY(cudaStreamBeginCapture(x->stream, cudaStreamCaptureModeThreadLocal));
  const int nl = enqueue_step<R>(x);
  cudaError_t e = cudaStreamEndCapture(x->stream, &gr);
  if (e != cudaSuccess) return cuda_status(e);
  bool updated = false;
  if (x->graph) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(x->graph, gr, &info) == cudaSuccess) {
      updated = true;
    } else {
      cudaGetLastError();
      cudaGraphExecDestroy(x->graph);
      x->graph = nullptr;
    }
  }
  if (!updated) {
    e = cudaGraphInstantiate(&x->graph, gr, 0);
    if (e != cudaSuccess) {
      x->graph = nullptr;
      cudaGraphDestroy(gr);
      return cuda_status(e);
    }
  }
  cudaGraphDestroy(gr);
  x->graph_key = x->key;
  x->graph_valid = true;
  x->launches_per_step = nl;
  return MLC_OK;
}

bool ready(const mlc_ctx *x) {
  for (const Member &m : x->mem)
    if (m.used && (!m.have_static || !m.have_state || (x->prm.do_apply_bdy && !m.have_bdy)))
      return false;
  return true;
}

template <class R>
int step_impl(mlc_ctx *x, int nsteps) {
  MLC_CHK(refresh_all<R>(x));
  if (x->key.L.nmem == 0 || nsteps == 0) return MLC_OK;
  if (x->use_graphs) {
    if (!x->graph_valid || std::memcmp(&x->graph_key, &x->key, sizeof(GraphKey)) != 0)
      MLC_CHK(record<R>(x));
    for (int n = 0; n < nsteps; ++n) MLC_TRY(cudaGraphLaunch(x->graph, x->stream));
  } else {
    for (int n = 0; n < nsteps; ++n) x->launches_per_step = enqueue_step<R>(x);
  }
  return cuda_status(cudaGetLastError());
}

int step_any(mlc_ctx *x, int nsteps) {
  return x->mixed ? step_impl<float>(x, nsteps) : step_impl<double>(x, nsteps);
}

// ---- host <-> device transfers -------------------------------------------

Clock get_clock(mlc_ctx *x, int slot, int *st) {
  Clock c{};
  cudaError_t e = cudaMemcpyAsync(&c, x->clks + slot, sizeof(Clock), cudaMemcpyDeviceToHost, x->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(x->stream);
  *st = cuda_status(e);
  return c;
}

// Copy a packed (Fortran extents nj x ni x nk) host array into the padded
// device layout through the staging buffer at element offset `soff`.  One
// stream orders every copy and (un)pack, so consecutive fields may reuse the
// same staging slice.
// An FP64 array goes straight between the packed host array and the padded
// device layout in one pitched copy (rows of nj, ni rows of a plane on the
// host, iy on the device); a conversion to FP32 goes through the staging buffer.
cudaMemcpy3DParms pitched(const Geom &g, const double *host, double *dev, int nj, int ni, int nk,
                          bool to_device) {
  cudaMemcpy3DParms c{};
  cudaPitchedPtr hp = make_cudaPitchedPtr(const_cast<double *>(host), (size_t)nj * sizeof(double),
                                          (size_t)nj, (size_t)ni);
  cudaPitchedPtr dp = make_cudaPitchedPtr(dev, (size_t)g.P * sizeof(double), (size_t)g.P, (size_t)g.iy);
  c.srcPtr = to_device ? hp : dp;
  c.dstPtr = to_device ? dp : hp;
  c.extent = make_cudaExtent((size_t)nj * sizeof(double), (size_t)ni, (size_t)nk);
  c.kind = to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
  return c;
}

template <class R>
int put3(mlc_ctx *x, const Geom &g, const double *h, R *dst, int nj, int ni, int nk, size_t soff) {
  if (!h) return MLC_OK;
  if constexpr (sizeof(R) == sizeof(double)) {
    const cudaMemcpy3DParms c = pitched(g, h, reinterpret_cast<double *>(dst), nj, ni, nk, true);
    MLC_TRY(cudaMemcpy3DAsync(&c, x->stream));
    return MLC_OK;
  }
  const size_t n = (size_t)nj * ni * nk;
  if (soff + n > x->staging_elems) return MLC_ERR_INVALID;
  MLC_TRY(cudaMemcpyAsync(x->staging + soff, h, n * sizeof(double), cudaMemcpyHostToDevice, x->stream));
  Launch<R>::unpack3(x->staging + soff, dst, g, nj, ni, nk, x->stream);
  return MLC_OK;
}

// The same for a double-float field of a mixed member (planes of nplane
// elements: hi, then lo); an FP64 member takes the plain copy.
template <class R>
int put3x(mlc_ctx *x, const Geom &g, const double *h, double *dst, int nj, int ni, int nk,
          size_t soff, size_t nplane) {
  if (sizeof(R) == sizeof(double)) return put3<double>(x, g, h, dst, nj, ni, nk, soff);
  if (!h) return MLC_OK;
  const size_t n = (size_t)nj * ni * nk;
  if (soff + n > x->staging_elems) return MLC_ERR_INVALID;
  MLC_TRY(cudaMemcpyAsync(x->staging + soff, h, n * sizeof(double), cudaMemcpyHostToDevice, x->stream));
  Launch<R>::unpack3_df(x->staging + soff, dst, g, nj, ni, nk, nplane, x->stream);
  return MLC_OK;
}

template <class R>
int get3x(mlc_ctx *x, const Geom &g, const double *src, double *h, int nj, int ni, int nk,
          size_t soff, size_t nplane);

template <class R>
int get3(mlc_ctx *x, const Geom &g, const R *src, double *h, int nj, int ni, int nk, size_t soff) {
  if (!h) return MLC_OK;
  if constexpr (sizeof(R) == sizeof(double)) {
    const cudaMemcpy3DParms c =
        pitched(g, h, reinterpret_cast<double *>(const_cast<R *>(src)), nj, ni, nk, false);
    MLC_TRY(cudaMemcpy3DAsync(&c, x->stream));
    return MLC_OK;
  }
  const size_t n = (size_t)nj * ni * nk;
  if (soff + n > x->staging_elems) return MLC_ERR_INVALID;
  Launch<R>::pack3(src, x->staging + soff, g, nj, ni, nk, x->stream);
  MLC_TRY(cudaMemcpyAsync(h, x->staging + soff, n * sizeof(double), cudaMemcpyDeviceToHost, x->stream));
  return MLC_OK;
}

template <class R>
int get3x(mlc_ctx *x, const Geom &g, const double *src, double *h, int nj, int ni, int nk,
          size_t soff, size_t nplane) {
  if (sizeof(R) == sizeof(double)) return get3<double>(x, g, src, h, nj, ni, nk, soff);
  if (!h) return MLC_OK;
  const size_t n = (size_t)nj * ni * nk;
  if (soff + n > x->staging_elems) return MLC_ERR_INVALID;
  Launch<R>::pack3_df(src, x->staging + soff, g, nj, ni, nk, nplane, x->stream);
  MLC_TRY(cudaMemcpyAsync(h, x->staging + soff, n * sizeof(double), cudaMemcpyDeviceToHost, x->stream));
  return MLC_OK;
}

// A 1-D array of the field type that has no FP64 twin (written in both
// precisions).
template <class R>
int put1_as(mlc_ctx *x, const double *h, const R *dst, size_t n) {
  std::vector<R> tmp(n);
  for (size_t e = 0; e < n; ++e) tmp[e] = (R)h[e];
  MLC_TRY(cudaMemcpyAsync(W(dst), tmp.data(), n * sizeof(R), cudaMemcpyHostToDevice, x->stream));
  return cuda_status(cudaStreamSynchronize(x->stream));
}

// A 1-D array in the field type (mixed members keep FP32 copies).
template <class R>
int put1r(mlc_ctx *x, const double *h, const R *dst, size_t n) {
  if (sizeof(R) == sizeof(double)) return MLC_OK;  // aliases the FP64 array
  std::vector<R> tmp(n);
  for (size_t e = 0; e < n; ++e) tmp[e] = (R)h[e];
  MLC_TRY(cudaMemcpyAsync(W(dst), tmp.data(), n * sizeof(R), cudaMemcpyHostToDevice, x->stream));
  return cuda_status(cudaStreamSynchronize(x->stream));
}

// 2-D padded copy of a small host array (built on the host, then one copy).
template <class T>
int put2_host(mlc_ctx *x, const Geom &g, const T *h, T *dst, int nj, int ni) {
  std::vector<T> tmp((size_t)g.PS, T(0));
  for (int i = 0; i < ni; ++i)
    for (int j = 0; j < nj; ++j) tmp[(size_t)j + (size_t)i * g.P] = h[(size_t)j + (size_t)i * nj];
  MLC_TRY(cudaMemcpyAsync(dst, tmp.data(), tmp.size() * sizeof(T), cudaMemcpyHostToDevice, x->stream));
  return cuda_status(cudaStreamSynchronize(x->stream));
}

template <class R>
int put2r(mlc_ctx *x, const Geom &g, const std::vector<double> &h, const R *dst, int nj, int ni) {
  std::vector<R> tmp((size_t)nj * ni);
  for (size_t e = 0; e < tmp.size(); ++e) tmp[e] = (R)h[e];
  return put2_host<R>(x, g, tmp.data(), W(dst), nj, ni);
}

int put1(mlc_ctx *x, const double *h, const double *dst, size_t n) {
  MLC_TRY(cudaMemcpyAsync(W(dst), h, n * sizeof(double), cudaMemcpyHostToDevice, x->stream));
  return cuda_status(cudaStreamSynchronize(x->stream));
}

template <class R>
int bind_static_impl(mlc_ctx *x, Member &mb, const mlc_static_ptrs *s) {
  const Dom<R> &D = dom_of<R>(mb);
  const Stat<R> &a = D.sa;
  const Geom &g = mb.g;
  const mlc_dims &d = mb.dims;
  const mlc_params &p = x->prm;
  Scal &c = mb.c;
  const int jx = d.jx, iy = d.iy, kz = d.kz;
  if (!s->msfu || !s->msfv || !s->msfx || !s->ulat || !s->vlat || !s->hx || !s->hy || !s->fmz ||
      !s->fmzf || !s->rfmzu || !s->rfmzv || !s->zeta || !s->dz || !s->zita || !s->zitah ||
      !s->ffilt || !s->hefc || !s->ibnd_cr || !s->ibnd_ud || !s->ibnd_vd)
    return MLC_ERR_INVALID;
  if (d.ntr > 0 && !s->fcx) return MLC_ERR_INVALID;
  if (p.lrotllr && !s->rlat) return MLC_ERR_INVALID;
  // zone indices address rows 1..nspgx of hefc/fcx: reject anything else
  const size_t nd = (size_t)jx * iy;
  for (const int32_t *b : {s->ibnd_cr, s->ibnd_ud, s->ibnd_vd})
    for (size_t e = 0; e < nd; ++e)
      if (b[e] > p.nspgx || b[e] == 0 || b[e] < -1) return MLC_ERR_INVALID;
  c.rdzita = 1.0 / s->zita[kz - 1];
  c.rdzitaf = float(c.rdzita);
  // 3-D metric: one field at a time through the staging buffer
  MLC_CHK(put3<R>(x, g, s->fmz, W(a.fmz), jx - 1, iy - 1, kz, 0));
  MLC_CHK(put3<R>(x, g, s->fmzf, W(a.fmzf), jx - 1, iy - 1, kz + 1, 0));
  if (sizeof(R) != sizeof(double)) {
    // the hydrostatic factor of the mixed solve, cp*fmzf*dtrdz, in FP64
    const double dtrdz = c.dtsound * (1.0 / s->zita[kz - 1]);
    const size_t n = (size_t)(jx - 1) * (iy - 1) * (kz + 1);
    std::vector<double> cf(n);
    for (size_t e = 0; e < n; ++e) cf[e] = kCpd * s->fmzf[e] * dtrdz;
    MLC_CHK(put3x<R>(x, g, cf.data(), W(a.cfz), jx - 1, iy - 1, kz + 1, 0, g.PS * (size_t)(kz + 1)));
    MLC_TRY(cudaStreamSynchronize(x->stream));
  }
  MLC_CHK(put3<R>(x, g, s->rfmzu, W(a.rfmzu), jx, iy - 1, kz, 0));
  MLC_CHK(put3<R>(x, g, s->rfmzv, W(a.rfmzv), jx - 1, iy, kz, 0));
  MLC_CHK(put3<double>(x, g, s->zeta, W(a.zeta), jx - 1, iy - 1, kz, 0));
  MLC_CHK(put3<double>(x, g, s->dz, W(a.dz), jx - 1, iy - 1, kz, 0));
  if (sizeof(R) != sizeof(double)) {
    MLC_CHK(put3<R>(x, g, s->dz, W(a.dz_r), jx - 1, iy - 1, kz, 0));
    // the remainder dz - (float)dz, so that {dz_r, dz_lo} carries dz to FP64 accuracy
    const size_t n = (size_t)(jx - 1) * (iy - 1) * kz;
    std::vector<double> lo(n);
    for (size_t e = 0; e < n; ++e) lo[e] = s->dz[e] - (double)(float)s->dz[e];
    MLC_CHK(put3<R>(x, g, lo.data(), W(a.dz_lo), jx - 1, iy - 1, kz, 0));
    MLC_TRY(cudaStreamSynchronize(x->stream));
  }
  // vertical WAF ratios (dtrdz*fmz)/fmzf, Main/mod_moloch.F90:888-889
  {
    const double mo_dzita = s->zita[kz - 1];
    const double dtrdz = 0.5 * (c.dtstepa * (1.0 / mo_dzita));
    const size_t c2 = (size_t)(jx - 1) * (iy - 1);
    std::vector<double> zu(c2 * kz), zd(c2 * kz);
    for (int k = 0; k < kz; ++k)
      for (size_t e = 0; e < c2; ++e) {
        const double fz = s->fmz[e + c2 * k];
        zu[e + c2 * k] = dtrdz * fz / s->fmzf[e + c2 * k];
        zd[e + c2 * k] = dtrdz * fz / s->fmzf[e + c2 * (k + 1)];
      }
    MLC_CHK(put3<R>(x, g, zu.data(), W(a.zrfmu), jx - 1, iy - 1, kz, 0));
    MLC_CHK(put3<R>(x, g, zd.data(), W(a.zrfmd), jx - 1, iy - 1, kz, 0));
    MLC_TRY(cudaStreamSynchronize(x->stream));
  }
  // 2-D fields and init_moloch derivations (Main/mod_moloch.F90:258-271)
  std::vector<double> t2(nd);
  auto copy2 = [&](const double *h, size_t n) { t2.assign(h, h + n); };
  copy2(s->msfu, nd); MLC_CHK(put2r<R>(x, g, t2, a.msfu, jx, iy));
  copy2(s->msfv, nd); MLC_CHK(put2r<R>(x, g, t2, a.msfv, jx, iy));
  copy2(s->msfx, nd); MLC_CHK(put2r<R>(x, g, t2, a.msfx, jx, iy));
  for (size_t e = 0; e < nd; ++e) t2[e] = s->msfx[e] * s->msfx[e];
  MLC_CHK(put2r<R>(x, g, t2, a.mx2, jx, iy));
  for (size_t e = 0; e < nd; ++e) t2[e] = 1.0 / s->msfu[e];
  MLC_CHK(put2r<R>(x, g, t2, a.rmu, jx, iy));
  for (size_t e = 0; e < nd; ++e) t2[e] = 1.0 / s->msfv[e];
  MLC_CHK(put2r<R>(x, g, t2, a.rmv, jx, iy));
  copy2(s->hx, (size_t)jx * (iy - 1)); MLC_CHK(put2r<R>(x, g, t2, a.hx, jx, iy - 1));
  copy2(s->hy, (size_t)(jx - 1) * iy); MLC_CHK(put2r<R>(x, g, t2, a.hy, jx - 1, iy));
  t2.resize((size_t)jx * (iy - 1));
  for (size_t e = 0; e < t2.size(); ++e) t2[e] = kOmega2 * std::sin(s->ulat[e] * kDegrad);
  MLC_CHK(put2r<R>(x, g, t2, a.coru, jx, iy - 1));
  t2.resize((size_t)(jx - 1) * iy);
  for (size_t e = 0; e < t2.size(); ++e) t2[e] = kOmega2 * std::sin(s->vlat[e] * kDegrad);
  MLC_CHK(put2r<R>(x, g, t2, a.corv, jx - 1, iy));
  MLC_CHK(put2_host<int32_t>(x, g, s->ibnd_cr, W(a.ibnd_cr), jx, iy));
  MLC_CHK(put2_host<int32_t>(x, g, s->ibnd_ud, W(a.ibnd_ud), jx, iy));
  MLC_CHK(put2_host<int32_t>(x, g, s->ibnd_vd, W(a.ibnd_vd), jx, iy));
  // the relaxation zones are non-empty (ba%havebound)
  auto any_pos = [&](const int32_t *b) {
    for (size_t e = 0; e < nd; ++e) if (b[e] > 0) return 1;
    return 0;
  };
  c.hb_cr = any_pos(s->ibnd_cr); c.hb_ud = any_pos(s->ibnd_ud); c.hb_vd = any_pos(s->ibnd_vd);
  // the curvature terms vanish identically with uniform map factors
  {
    bool curv = p.lrotllr != 0;
    for (int i = 2; i <= iy - 2 && !curv; ++i)
      for (int j = 2; j <= jx - 2 && !curv; ++j) {
        const size_t e = (size_t)(j - 1) + (size_t)(i - 1) * jx;
        if ((s->msfu[e - 1] - s->msfu[e]) != 0.0 || (s->msfv[e - jx] - s->msfv[e]) != 0.0) curv = true;
      }
    c.curvature = curv ? 1 : 0;
  }
  // 1-D vertical arrays, Main/mod_moloch.F90:262-300
  std::vector<double> v1(kz + 1);
  for (int k = 1; k <= kz + 1; ++k) v1[k - 1] = gzita(s->zita[k - 1], p.mo_ztop, p.mo_a0);
  MLC_CHK(put1(x, v1.data(), a.gzitak, kz + 1));
  MLC_CHK(put1r<R>(x, v1.data(), a.gzitak_r, kz + 1));
  for (int k = 1; k <= kz; ++k) v1[k - 1] = gzita(s->zitah[k - 1], p.mo_ztop, p.mo_a0);
  MLC_CHK(put1(x, v1.data(), a.gzitakh, kz));
  MLC_CHK(put1r<R>(x, v1.data(), a.gzitakh_r, kz));
  for (int k = 1; k <= kz; ++k)
    v1[k - 1] = kNuMax * kDdamp * (1.0 / (k + 1.0) - 1.0 / (kz + 2.0));
  MLC_CHK(put1(x, v1.data(), a.xkdamp, kz));
  MLC_CHK(put1r<R>(x, v1.data(), a.xkdamp_r, kz));
  for (int k = 1; k <= kz; ++k)
    v1[k - 1] = kNuMax * (0.55 + 0.45 * ((double)(kz - k + 1) - 1.0) / ((double)kz - 1.0));
  MLC_CHK(put1(x, v1.data(), a.xknu, kz));
  MLC_CHK(put1r<R>(x, v1.data(), a.xknu_r, kz));
  MLC_CHK(put1(x, s->ffilt, a.ffilt, kz));
  MLC_CHK(put1r<R>(x, s->ffilt, a.ffilt_r, kz));
  {
    std::vector<double> tn(kz, 0.0);
    if (s->tnudge) tn.assign(s->tnudge, s->tnudge + kz);
    MLC_CHK(put1(x, tn.data(), a.tnudge, kz));
    MLC_CHK(put1r<R>(x, tn.data(), a.tnudge_r, kz));
  }
  // Levels nudged at the top: the member's own nztop, the last level with a
  // non-zero tnudge (bdyin sets tnudge > 0 exactly on levels 1..nztop,
  // Main/mod_bdycod.F90:507-537).  A level with tnudge = 0 would be left
  // unchanged by the nudging anyway, so members of one context may differ
  // in levels and terrain without sharing one nztop.
  c.nztop = 0;
  if (p.mo_top_nudge && s->tnudge)
    for (int k = 1; k <= kz; ++k)
      if (s->tnudge[k - 1] != 0.0) c.nztop = k;
  MLC_CHK(put1(x, s->hefc, a.hefc, (size_t)p.nspgx * kz));
  MLC_CHK(put1r<R>(x, s->hefc, a.hefc_r, (size_t)p.nspgx * kz));
  if (s->fcx) {
    MLC_CHK(put1(x, s->fcx, a.fcx, p.nspgx));
    MLC_CHK(put1r<R>(x, s->fcx, a.fcx_r, p.nspgx));
  }
  if (s->rlat) MLC_CHK(put1(x, s->rlat, a.rlat, iy));
  if (sizeof(R) == sizeof(double)) {
    // the acoustic substep's constant factors, in the kernels' operand order
    // (the same products the kernels formed every substep)
    const bool rot = p.lrotllr != 0;
    const double dtrdx = c.dtrdxs, dtrdy = c.dtrdxs, dxrdt = c.dxrdt, dts = c.dtsound;
    const double zfz = kGrav * dts;
    std::vector<double> xkd(kz), gkh(kz);
    for (int k = 1; k <= kz; ++k) {
      xkd[k - 1] = kNuMax * kDdamp * (1.0 / (k + 1.0) - 1.0 / (kz + 2.0));
      gkh[k - 1] = gzita(s->zitah[k - 1], p.mo_ztop, p.mo_a0);
    }
    const size_t nu = (size_t)jx * (iy - 1), nv = (size_t)(jx - 1) * iy, nc = (size_t)(jx - 1) * (iy - 1);
    std::vector<double> fu(nu * kz), fv(nv * kz), fc(nc * kz), gu(nu * kz), gv(nv * kz);
    std::vector<double> cu(nu), cvv(nv);
    for (int k = 0; k < kz; ++k)
      for (int i = 0; i < iy - 1; ++i)
        for (int j = 0; j < jx; ++j) {
          const size_t e = (size_t)j + (size_t)i * jx, e3 = e + nu * k;
          const double rmu = 1.0 / s->msfu[e];
          fu[e3] = rot ? dtrdx * s->rfmzu[e3] : dtrdx * s->rfmzu[e3] * rmu;
          gu[e3] = zfz * s->hx[e] * gkh[k];
        }
    for (int k = 0; k < kz; ++k)
      for (int i = 0; i < iy; ++i)
        for (int j = 0; j < jx - 1; ++j) {
          const size_t e2 = (size_t)j + (size_t)i * jx;          // msfv (jx, iy)
          const size_t e = (size_t)j + (size_t)i * (jx - 1), e3 = e + nv * k;
          const double rmv = 1.0 / s->msfv[e2];
          fv[e3] = dtrdy * s->rfmzv[e3] * rmv;
          gv[e3] = zfz * s->hy[e] * gkh[k];
        }
    for (int k = 0; k < kz; ++k)
      for (int i = 0; i < iy - 1; ++i)
        for (int j = 0; j < jx - 1; ++j) {
          const size_t e2 = (size_t)j + (size_t)i * jx;
          const size_t e3 = (size_t)j + (size_t)i * (jx - 1) + nc * k;
          const double mfac = rot ? s->msfx[e2] : s->msfx[e2] * s->msfx[e2];
          fc[e3] = s->fmz[e3] * mfac;
        }
    MLC_CHK(put3<double>(x, g, fu.data(), W(a.dv_cu), jx, iy - 1, kz, 0));
    MLC_CHK(put3<double>(x, g, fv.data(), W(a.dv_cv), jx - 1, iy, kz, 0));
    MLC_CHK(put3<double>(x, g, fc.data(), W(a.dv_cf), jx - 1, iy - 1, kz, 0));
    MLC_CHK(put3<double>(x, g, gu.data(), W(a.mo_gu), jx, iy - 1, kz, 0));
    MLC_CHK(put3<double>(x, g, gv.data(), W(a.mo_gv), jx - 1, iy, kz, 0));
    MLC_TRY(cudaStreamSynchronize(x->stream));
    for (int k = 0; k < kz; ++k)
      for (int i = 0; i < iy - 1; ++i)
        for (int j = 0; j < jx; ++j) {
          const size_t e = (size_t)j + (size_t)i * jx;
          fu[e + nu * k] = dxrdt * xkd[k] * s->msfu[e];
        }
    for (int k = 0; k < kz; ++k)
      for (int i = 0; i < iy; ++i)
        for (int j = 0; j < jx - 1; ++j) {
          const size_t e2 = (size_t)j + (size_t)i * jx;
          const size_t e = (size_t)j + (size_t)i * (jx - 1);
          fv[e + nv * k] = rot ? dxrdt * xkd[k] : dxrdt * xkd[k] * s->msfv[e2];
        }
    for (size_t e = 0; e < nu; ++e) cu[e] = kOmega2 * std::sin(s->ulat[e] * kDegrad) * dts;
    for (size_t e = 0; e < nv; ++e) cvv[e] = kOmega2 * std::sin(s->vlat[e] * kDegrad) * dts;
    MLC_CHK(put3<double>(x, g, fu.data(), W(a.mo_du), jx, iy - 1, kz, 0));
    MLC_CHK(put3<double>(x, g, fv.data(), W(a.mo_dv), jx - 1, iy, kz, 0));
    MLC_CHK(put3<double>(x, g, cu.data(), W(a.mo_cu), jx, iy - 1, 1, 0));
    MLC_CHK(put3<double>(x, g, cvv.data(), W(a.mo_cv), jx - 1, iy, 1, 0));
    MLC_TRY(cudaStreamSynchronize(x->stream));
    // the solve's factors, in the kernel's operand order: (bw*dtrdz)*fmz,
    // zcs2*fmz and dtrdz*fmz (dtrdz = dtsound*rdzita, zcs2 = dtrdz^2*R/cv)
    const double sdtrdz = c.dtsound * c.rdzita;
    const double zcs2 = (sdtrdz * sdtrdz) * kRdrcv;
    const int nsp = p.nspgx;
    std::vector<double> fa(nc * kz), fb(nc * kz);
    for (int k = 0; k < kz; ++k)
      for (int i = 0; i < iy - 1; ++i)
        for (int j = 0; j < jx - 1; ++j) {
          const size_t e2 = (size_t)j + (size_t)i * jx;
          const size_t e3 = (size_t)j + (size_t)i * (jx - 1) + nc * k;
          const int ib = s->ibnd_cr[e2];
          const double bw = ib > 0 ? 1.0 - s->hefc[(size_t)(ib - 1) + (size_t)k * nsp] : 1.0;
          fa[e3] = (bw * sdtrdz) * s->fmz[e3];
          fb[e3] = zcs2 * s->fmz[e3];
        }
    MLC_CHK(put3<double>(x, g, fa.data(), W(a.sv_a), jx - 1, iy - 1, kz, 0));
    MLC_CHK(put3<double>(x, g, fb.data(), W(a.sv_b), jx - 1, iy - 1, kz, 0));
    MLC_TRY(cudaStreamSynchronize(x->stream));
    for (size_t e = 0; e < nc * kz; ++e) fa[e] = sdtrdz * s->fmz[e];
    MLC_CHK(put3<double>(x, g, fa.data(), W(a.sv_c), jx - 1, iy - 1, kz, 0));
    MLC_TRY(cudaStreamSynchronize(x->stream));
  }
  if (p.mo_spectral_nudge) {
    // lowpass_init (Main/mod_bdycod.F90:3844-3896, one process: njcross =
    // jx-1, nicross = iy-1) in FP64, rows of the modes k = 1..2km over
    // j = 1..jx (jde) and l = 1..2lm over i = 1..iy (ide)
    if (!s->cnudge) return MLC_ERR_INVALID;
    const int km2 = c.km2, lm2 = c.lm2;
    const double dxa = kPi / (double)(jx - 2), dya = kPi / (double)(iy - 2);
    std::vector<double> bx((size_t)km2 * jx), by((size_t)lm2 * iy);
    for (int m = 1; m <= km2; ++m) {
      const double r = (double)m / (double)(km2 / 2);
      const double amp = std::sqrt(2.0 / (double)(jx - 1) * std::exp(-(r * r)));
      for (int j = 1; j <= jx; ++j) bx[(size_t)(m - 1) * jx + (j - 1)] = amp * std::sin(m * (j - 2) * dxa);
    }
    for (int l = 1; l <= lm2; ++l) {
      const double r = (double)l / (double)(lm2 / 2);
      const double amp = std::sqrt(2.0 / (double)(iy - 1) * std::exp(-(r * r)));
      for (int i = 1; i <= iy; ++i) by[(size_t)(l - 1) * iy + (i - 1)] = amp * std::sin(l * (i - 2) * dya);
    }
    MLC_CHK(put1_as<R>(x, bx.data(), a.bvx, bx.size()));
    MLC_CHK(put1_as<R>(x, by.data(), a.bvy, by.size()));
    MLC_CHK(put1_as<R>(x, s->cnudge, a.cnudge, kz));
  }
  MLC_TRY(cudaStreamSynchronize(x->stream));
  return MLC_OK;
}

template <class R>
int upload_state_impl(mlc_ctx *x, int slot, const mlc_state_ptrs *h) {
  Member &mb = x->mem[slot];
  int cst;
  const Clock ck = get_clock(x, slot, &cst);
  MLC_CHK(cst);
  const State<R> st = state_of(dom_of<R>(mb), ck.uv_role, ck.adv_role);
  const Geom &g = mb.g;
  const int jx = mb.dims.jx, iy = mb.dims.iy, kz = mb.dims.kz;
  size_t off = 0;
  const size_t c3 = (size_t)(jx - 1) * (iy - 1) * kz;
  auto adv = [&](size_t n) { size_t o = off; off += n; return o; };
  MLC_CHK(put3<R>(x, g, h->u, st.u, jx, iy - 1, kz, adv((size_t)jx * (iy - 1) * kz)));
  MLC_CHK(put3<R>(x, g, h->v, st.v, jx - 1, iy, kz, adv((size_t)(jx - 1) * iy * kz)));
  MLC_CHK(put3<R>(x, g, h->w, st.w, jx - 1, iy - 1, kz + 1, adv((size_t)(jx - 1) * (iy - 1) * (kz + 1))));
  MLC_CHK(put3x<R>(x, g, h->pai, st.pai, jx - 1, iy - 1, kz, adv(c3), g.field3()));
  MLC_CHK(put3x<R>(x, g, h->tetav, st.tetav, jx - 1, iy - 1, kz, adv(c3), g.field3()));
  R *f3[] = {st.t, st.tvirt, st.ux, st.vx, st.p, st.rho, st.qsat};
  const double *h3[] = {h->t, h->tvirt, h->ux, h->vx, h->p, h->rho, h->qsat};
  for (int q = 0; q < 7; ++q) MLC_CHK(put3<R>(x, g, h3[q], f3[q], jx - 1, iy - 1, kz, adv(c3)));
  const size_t F = g.field3();
  for (int n = 0; n < mb.dims.nqx && h->qx; ++n)
    MLC_CHK(put3<R>(x, g, h->qx + n * c3, st.qx + n * F, jx - 1, iy - 1, kz, adv(c3)));
  for (int n = 0; n < mb.dims.ntr && h->trac; ++n)
    MLC_CHK(put3<R>(x, g, h->trac + n * c3, st.trac + n * F, jx - 1, iy - 1, kz, adv(c3)));
  if (h->ps) {
    const size_t c2 = (size_t)(jx - 1) * (iy - 1);
    MLC_CHK(put3<double>(x, g, h->ps, st.ps, jx - 1, iy - 1, 1, adv(c2)));
  }
  if (h->tke && st.tke)
    MLC_CHK(put3<R>(x, g, h->tke, st.tke, jx - 1, iy - 1, kz + 1,
                    adv((size_t)(jx - 1) * (iy - 1) * (kz + 1))));
  // init_moloch: w(:,:,1) = 0 (Main/mod_moloch.F90:264-266)
  if (h->w) MLC_TRY(cudaMemsetAsync(st.w, 0, g.PS * sizeof(R), x->stream));
  return cuda_status(cudaStreamSynchronize(x->stream));
}

template <class R>
int download_state_impl(mlc_ctx *x, int slot, const mlc_state_ptrs *h) {
  Member &mb = x->mem[slot];
  int cst;
  const Clock ck = get_clock(x, slot, &cst);
  MLC_CHK(cst);
  // inside an open step the roles advance only at its end: the current
  // halves are those the step's last kernels work on
  const int uvo = x->step_open ? x->prm.mo_nadv * x->prm.mo_nsound : 0;
  const int ao = x->step_open ? x->prm.mo_nadv : 0;
  const State<R> st = state_of(dom_of<R>(mb), (ck.uv_role + uvo) & 1, (ck.adv_role + ao) & 1);
  const Geom &g = mb.g;
  const int jx = mb.dims.jx, iy = mb.dims.iy, kz = mb.dims.kz;
  size_t off = 0;
  const size_t c3 = (size_t)(jx - 1) * (iy - 1) * kz;
  auto adv = [&](size_t n) { size_t o = off; off += n; return o; };
  MLC_CHK(get3<R>(x, g, st.u, h->u, jx, iy - 1, kz, adv((size_t)jx * (iy - 1) * kz)));
  MLC_CHK(get3<R>(x, g, st.v, h->v, jx - 1, iy, kz, adv((size_t)(jx - 1) * iy * kz)));
  MLC_CHK(get3<R>(x, g, st.w, h->w, jx - 1, iy - 1, kz + 1, adv((size_t)(jx - 1) * (iy - 1) * (kz + 1))));
  MLC_CHK(get3x<R>(x, g, st.pai, h->pai, jx - 1, iy - 1, kz, adv(c3), g.field3()));
  MLC_CHK(get3x<R>(x, g, st.tetav, h->tetav, jx - 1, iy - 1, kz, adv(c3), g.field3()));
  const R *f3[] = {st.t, st.tvirt, st.ux, st.vx, st.p, st.rho, st.qsat};
  double *h3[] = {h->t, h->tvirt, h->ux, h->vx, h->p, h->rho, h->qsat};
  for (int q = 0; q < 7; ++q) MLC_CHK(get3<R>(x, g, f3[q], h3[q], jx - 1, iy - 1, kz, adv(c3)));
  const size_t F = g.field3();
  for (int n = 0; n < mb.dims.nqx && h->qx; ++n)
    MLC_CHK(get3<R>(x, g, st.qx + n * F, h->qx + n * c3, jx - 1, iy - 1, kz, adv(c3)));
  for (int n = 0; n < mb.dims.ntr && h->trac; ++n)
    MLC_CHK(get3<R>(x, g, st.trac + n * F, h->trac + n * c3, jx - 1, iy - 1, kz, adv(c3)));
  if (h->ps) {
    const size_t c2 = (size_t)(jx - 1) * (iy - 1);
    MLC_CHK(get3<double>(x, g, st.ps, h->ps, jx - 1, iy - 1, 1, adv(c2)));
  }
  if (h->tke && st.tke)
    MLC_CHK(get3<R>(x, g, st.tke, h->tke, jx - 1, iy - 1, kz + 1,
                    adv((size_t)(jx - 1) * (iy - 1) * (kz + 1))));
  return cuda_status(cudaStreamSynchronize(x->stream));
}

template <class R>
int set_boundary_impl(mlc_ctx *x, Member &mb, const mlc_bdy_ptrs *b) {
  const Bdy<R> &a = dom_of<R>(mb).bd;
  const Geom &g = mb.g;
  const mlc_dims &d = mb.dims;
  const mlc_params &p = x->prm;
  const int jx = d.jx, iy = d.iy, kz = d.kz;
  const size_t c3 = (size_t)(jx - 1) * (iy - 1) * kz;
  const size_t F = g.field3();
  for (int s = 0; s < 2; ++s) {
    if (!b->xtb[s] || !b->xqb[s] || !b->xpaib[s] || !b->dub[s] || !b->dvb[s] || !b->xpsb[s])
      return MLC_ERR_INVALID;
    if (p.present_qc && !b->xlb[s]) return MLC_ERR_INVALID;
    if (p.present_qi && !b->xib[s]) return MLC_ERR_INVALID;
    if (d.ntr > 0 && !b->chib[s]) return MLC_ERR_INVALID;
  }
  for (int s = 0; s < 2; ++s) {
    MLC_CHK(put3x<R>(x, g, b->xtb[s], W(a.xtb[s]), jx - 1, iy - 1, kz, 0, F));
    MLC_CHK(put3<R>(x, g, b->xqb[s], W(a.xqb[s]), jx - 1, iy - 1, kz, 0));
    MLC_CHK(put3x<R>(x, g, b->xpaib[s], W(a.xpaib[s]), jx - 1, iy - 1, kz, 0, F));
    if (p.present_qc) MLC_CHK(put3<R>(x, g, b->xlb[s], W(a.xlb[s]), jx - 1, iy - 1, kz, 0));
    if (p.present_qi) MLC_CHK(put3<R>(x, g, b->xib[s], W(a.xib[s]), jx - 1, iy - 1, kz, 0));
    MLC_CHK(put3<R>(x, g, b->dub[s], W(a.dub[s]), jx, iy - 1, kz, 0));
    MLC_CHK(put3<R>(x, g, b->dvb[s], W(a.dvb[s]), jx - 1, iy, kz, 0));
    for (int n = 0; n < d.ntr; ++n)
      MLC_CHK(put3<R>(x, g, b->chib[s] + n * c3, W(a.chib[s]) + n * F, jx - 1, iy - 1, kz, 0));
    MLC_CHK(put3<double>(x, g, b->xpsb[s], W(a.xpsb[s]), jx - 1, iy - 1, 1, 0));
    MLC_TRY(cudaStreamSynchronize(x->stream));
  }
  return MLC_OK;
}

void release(mlc_ctx *x) {
  if (!x) return;
  if (x->stream) cudaStreamSynchronize(x->stream);
  if (x->graph) cudaGraphExecDestroy(x->graph);
  for (Member &m : x->mem) {
    if (m.raw) cudaFreeAsync(m.raw, x->stream);
    if (m.tend_raw) cudaFreeAsync(m.tend_raw, x->stream);
  }
  if (x->staging) cudaFreeAsync(x->staging, x->stream);
  if (x->stream) cudaStreamSynchronize(x->stream);
  if (x->clks) cudaFree(x->clks);
  if (x->diags) cudaFree(x->diags);
  if (x->table) cudaFree(x->table);
  if (x->wl_buf) cudaFree(x->wl_buf);
  if (x->pool) cudaMemPoolDestroy(x->pool);
  if (x->stream) cudaStreamDestroy(x->stream);
  delete x;
}

// A context with `capacity` empty slots.
int create_common(const mlc_params *params, int capacity, size_t budget, mlc_ctx **out) {
  if (!out) return MLC_ERR_INVALID;
  *out = nullptr;
  MLC_CHK(validate_params(params));
  if (capacity < 1 || capacity > kMaxSlots) return MLC_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return MLC_ERR_NODEVICE;
  }
  mlc_ctx *x = new (std::nothrow) mlc_ctx();
  if (!x) return MLC_ERR_NOMEM;
  x->prm = *params;
  x->mixed = params->precision == MLC_PREC_MIXED;
  x->budget = budget;
  x->mem.assign(capacity, Member{});
  LaunchGeom &L = x->key.L;
  L.col_x = 32; L.col_y = 4;
  L.solve_x = 32; L.solve_y = 2;
  L.vert_x = 32; L.vert_y = 4;
  L.htile = 1;  // 64x8 tiles; the autotuner's fixed configuration is 32x8
  L.solve_df = 1;  // the mixed solve's recurrence to FP64 accuracy
  cudaError_t e = cudaGetDevice(&x->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&x->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = x->device;
    e = cudaMemPoolCreate(&x->pool, &props);
  }
  if (e == cudaSuccess) {
    // keep freed member arenas in the pool for the next join
    uint64_t keep = UINT64_MAX;
    e = cudaMemPoolSetAttribute(x->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  if (e == cudaSuccess) e = cudaMalloc(&x->clks, capacity * sizeof(Clock));
  if (e == cudaSuccess) e = cudaMalloc(&x->diags, capacity * sizeof(DiagDev));
  if (e == cudaSuccess)
    e = cudaMalloc(&x->table, capacity * std::max(sizeof(Dom<double>), sizeof(Dom<float>)));
  if (e == cudaSuccess) e = cudaMemsetAsync(x->clks, 0, capacity * sizeof(Clock), x->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(x->diags, 0, capacity * sizeof(DiagDev), x->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(x->stream);
  if (e == cudaSuccess) e = x->mixed ? Launch<float>::configure_sound() : Launch<double>::configure_sound();
  if (e == cudaSuccess) e = x->mixed ? Launch<float>::configure_advect() : Launch<double>::configure_advect();
  if (e != cudaSuccess) {
    cudaGetLastError();
    release(x);
    return cuda_status(e);
  }
  *out = x;
  return MLC_OK;
}

int create_members(const mlc_dims *dims, int stride, const mlc_params *params, int nmem, mlc_ctx **out) {
  if (!out) return MLC_ERR_INVALID;
  *out = nullptr;
  if (!dims || nmem < 1 || nmem > kMaxSlots) return MLC_ERR_INVALID;
  MLC_CHK(validate_params(params));
  for (int m = 0; m < nmem; ++m) MLC_CHK(validate_dims(dims + (size_t)m * stride, params));
  mlc_ctx *x = nullptr;
  MLC_CHK(create_common(params, nmem, 0, &x));
  for (int m = 0; m < nmem; ++m) {
    const int st = add_member(x, m, dims[(size_t)m * stride]);
    if (st != MLC_OK) {
      release(x);
      return st;
    }
  }
  *out = x;
  return MLC_OK;
}

// Diagnostics of every slot after the last step (out has one entry per slot).
int fetch_diags(mlc_ctx *x, int nsteps, mlc_diag *out) {
  const size_t n = x->mem.size();
  std::vector<DiagDev> dd(n);
  std::vector<Clock> ck(n);
  MLC_TRY(cudaMemcpyAsync(dd.data(), x->diags, n * sizeof(DiagDev), cudaMemcpyDeviceToHost, x->stream));
  MLC_TRY(cudaMemcpyAsync(ck.data(), x->clks, n * sizeof(Clock), cudaMemcpyDeviceToHost, x->stream));
  MLC_TRY(cudaStreamSynchronize(x->stream));
  bool bad = false, fault = false;
  for (size_t m = 0; m < n; ++m) {
    const bool used = x->mem[m].used;
    if (used && ck[m].nonfinite) bad = true;
    if (used && ck[m].fault) fault = true;
    if (!out) continue;
    std::memset(&out[m], 0, sizeof(out[m]));
    if (!used) continue;
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
  if (fault) {
    g_last_error = "a bounded device wait gave up (TMA tile load)";
    return MLC_ERR_CUDA;
  }
  return bad ? MLC_ERR_NONFINITE : MLC_OK;
}

}  // namespace

namespace {

template <class R>
int set_tendencies_impl(mlc_ctx *x, Member &mb, const mlc_tend_ptrs *t) {
  const Geom &g = mb.g;
  const int nf = 3 + mb.dims.nqx + mb.dims.ntr;
  const size_t F = g.field3();
  // tketen (kz+1 planes) follows the kz-plane fields when ibltyp = 2
  const size_t elems = (size_t)nf * F + (mb.c.tke ? F + g.PS : 0);
  if (!mb.tend_raw) {
    const size_t bytes = elems * sizeof(R);
    if (x->budget && x->in_use + bytes > x->budget) return MLC_ERR_BUDGET;
    cudaError_t e = cudaMallocFromPoolAsync(&mb.tend_raw, bytes, x->pool, x->stream);
    if (e != cudaSuccess) {
      cudaGetLastError();
      mb.tend_raw = nullptr;
      return MLC_ERR_NOMEM;
    }
    mb.tend_bytes = bytes;
    x->in_use += bytes;
  }
  R *base = static_cast<R *>(mb.tend_raw);
  // NULL arrays leave zero, as reset_tendencies does at every step's start
  MLC_TRY(cudaMemsetAsync(base, 0, elems * sizeof(R), x->stream));
  const int nj = mb.dims.jx - 3, ni = mb.dims.iy - 3, kz = mb.dims.kz;
  const size_t n3 = (size_t)nj * ni * kz;
  const size_t at22 = g.at2(2, 2);
  const double *h[3] = {t->tten, t->uten, t->vten};
  for (int f = 0; f < 3; ++f) MLC_CHK(put3<R>(x, g, h[f], base + (size_t)f * F + at22, nj, ni, kz, 0));
  for (int n = 0; n < mb.dims.nqx && t->qxten; ++n)
    MLC_CHK(put3<R>(x, g, t->qxten + n * n3, base + (size_t)(3 + n) * F + at22, nj, ni, kz, 0));
  for (int n = 0; n < mb.dims.ntr && t->chiten; ++n)
    MLC_CHK(put3<R>(x, g, t->chiten + n * n3, base + (size_t)(3 + mb.dims.nqx + n) * F + at22, nj, ni,
                    kz, 0));
  if (mb.c.tke && t->tketen)
    MLC_CHK(put3<R>(x, g, t->tketen, base + (size_t)nf * F + at22, nj, ni, kz + 1, 0));
  return cuda_status(cudaStreamSynchronize(x->stream));
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
  p->mo_spectral_nudge = 0;
  p->dtrad = 1800.0;  // Main/mod_params.F90:1229-1230
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
  // Share/mod_dynparam.F90:141,150-152 and Main/mod_params.F90 (ibltyp)
  p->bdy_use_lehmann = 0;
  p->ibltyp = 1;
  p->high_nudge = 3.0;
  p->medium_nudge = 2.0;
  p->low_nudge = 1.0;
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
    case MLC_ERR_BUDGET: return "request exceeds the device memory budget or the free slots";
    case MLC_ERR_TOO_LARGE: return "size beyond the fixed maximum";
    default: return "unknown status";
  }
}

size_t mlc_footprint_bytes(const mlc_dims *d, int precision) {
  if (!d) return 0;
  mlc_params p;
  mlc_default_params(&p);
  p.ipptls = d->nqx >= 5 ? 2 : 1;
  p.present_qc = p.present_qi = 1;
  p.nspgx = 34;
  const size_t arena = precision == MLC_PREC_MIXED ? arena_bytes<float>(*d, p) : arena_bytes<double>(*d, p);
  return arena + kAlign + state_elems(*d) * sizeof(double);
}

size_t mlc_member_footprint(const mlc_dims *d, const mlc_params *p) {
  if (!d || !p) return 0;
  const size_t arena = p->precision == MLC_PREC_MIXED ? arena_bytes<float>(*d, *p) : arena_bytes<double>(*d, *p);
  return arena;
}

int mlc_create_batch(const mlc_dims *dims, const mlc_params *params, int nmem, mlc_ctx **out) {
  return create_members(dims, 0, params, nmem, out);
}

int mlc_create_multi(const mlc_dims *dims, const mlc_params *params, int nmem, mlc_ctx **out) {
  return create_members(dims, 1, params, nmem, out);
}

int mlc_create(const mlc_dims *dims, const mlc_params *params, mlc_ctx **out) {
  return create_members(dims, 0, params, 1, out);
}

int mlc_create_pool(const mlc_params *params, int capacity, size_t budget_bytes, mlc_ctx **out) {
  return create_common(params, capacity, budget_bytes, out);
}

int mlc_pool_add(mlc_ctx *x, const mlc_dims *dims, int *slot) {
  if (!x || !dims || !slot) return MLC_ERR_INVALID;
  if (x->step_open) return MLC_ERR_STATE;
  *slot = -1;
  for (size_t m = 0; m < x->mem.size(); ++m)
    if (!x->mem[m].used) {
      MLC_CHK(add_member(x, (int)m, *dims));
      *slot = (int)m;
      return MLC_OK;
    }
  return MLC_ERR_BUDGET;
}

int mlc_pool_remove(mlc_ctx *x, int slot) {
  if (!member_ok(x, slot)) return MLC_ERR_INVALID;
  if (x->step_open) return MLC_ERR_STATE;
  return remove_member(x, slot);
}

size_t mlc_pool_bytes(const mlc_ctx *x) { return x ? x->in_use : 0; }

int mlc_member_bind_static(mlc_ctx *x, int m, const mlc_static_ptrs *s) {
  if (!member_ok(x, m) || !s) return MLC_ERR_INVALID;
  if (x->step_open) return MLC_ERR_STATE;
  if (!s->zita) return MLC_ERR_INVALID;
  Member &mb = x->mem[m];
  const int st = x->mixed ? bind_static_impl<float>(x, mb, s) : bind_static_impl<double>(x, mb, s);
  x->table_dirty = true;
  if (st == MLC_OK) mb.have_static = true;
  return st;
}

int mlc_bind_static(mlc_ctx *x, const mlc_static_ptrs *s) { return mlc_member_bind_static(x, 0, s); }

int mlc_member_upload_state(mlc_ctx *x, int m, const mlc_state_ptrs *h) {
  if (!member_ok(x, m) || !h) return MLC_ERR_INVALID;
  if (x->step_open) return MLC_ERR_STATE;
  const int st = x->mixed ? upload_state_impl<float>(x, m, h) : upload_state_impl<double>(x, m, h);
  if (st == MLC_OK) x->mem[m].have_state = true;
  return st;
}

int mlc_upload_state(mlc_ctx *x, const mlc_state_ptrs *h) { return mlc_member_upload_state(x, 0, h); }

int mlc_member_download_state(mlc_ctx *x, int m, const mlc_state_ptrs *h) {
  if (!member_ok(x, m) || !h) return MLC_ERR_INVALID;
  return x->mixed ? download_state_impl<float>(x, m, h) : download_state_impl<double>(x, m, h);
}

int mlc_download_state(mlc_ctx *x, const mlc_state_ptrs *h) {
  return mlc_member_download_state(x, 0, h);
}

// bdyin: new b0/b1 and the boundary clock.  The member's step counter, buffer
// roles and non-finite flag are kept.
int mlc_member_set_boundary(mlc_ctx *x, int m, const mlc_bdy_ptrs *b, double xbctime,
                            double dtbdys) {
  if (!member_ok(x, m) || !b || !(dtbdys > 0)) return MLC_ERR_INVALID;
  if (x->step_open) return MLC_ERR_STATE;
  Member &mb = x->mem[m];
  MLC_CHK(x->mixed ? set_boundary_impl<float>(x, mb, b) : set_boundary_impl<double>(x, mb, b));
  int cst;
  Clock ck = get_clock(x, m, &cst);
  MLC_CHK(cst);
  ck.xbctime = xbctime;
  MLC_TRY(cudaMemcpyAsync(x->clks + m, &ck, sizeof(Clock), cudaMemcpyHostToDevice, x->stream));
  MLC_TRY(cudaStreamSynchronize(x->stream));
  mb.c.dtbdys = dtbdys;
  mb.c.rtb = 1.0 / dtbdys;
  mb.have_bdy = true;
  x->table_dirty = true;
  return MLC_OK;
}

int mlc_set_boundary(mlc_ctx *x, const mlc_bdy_ptrs *b, double xbctime, double dtbdys) {
  return mlc_member_set_boundary(x, 0, b, xbctime, dtbdys);
}

int mlc_step_batch(mlc_ctx *x, int nsteps, mlc_diag *out) {
  if (!x || nsteps < 0) return MLC_ERR_INVALID;
  if (x->step_open) return MLC_ERR_STATE;
  if (!ready(x)) return MLC_ERR_STATE;
  MLC_CHK(step_any(x, nsteps));
  return fetch_diags(x, nsteps, out);
}

int mlc_step(mlc_ctx *x, int nsteps, mlc_diag *out) {
  if (!x) return MLC_ERR_INVALID;
  std::vector<mlc_diag> all(x->mem.size());
  const int st = mlc_step_batch(x, nsteps, all.data());
  if (out && st != MLC_ERR_INVALID && st != MLC_ERR_STATE) *out = all[0];
  return st;
}

// ---- the step split at the physics (Main/mod_moloch.F90:354-376) ----------

int mlc_step_dynamics(mlc_ctx *x) {
  if (!x) return MLC_ERR_INVALID;
  if (x->step_open || !ready(x)) return MLC_ERR_STATE;
  MLC_CHK(x->mixed ? refresh_all<float>(x) : refresh_all<double>(x));
  if (x->key.L.nmem == 0) return MLC_OK;
  if (x->mixed) enqueue_step<float>(x, nullptr, kStepDynamics);
  else enqueue_step<double>(x, nullptr, kStepDynamics);
  MLC_TRY(cudaGetLastError());
  x->step_open = true;
  return MLC_OK;
}

int mlc_member_set_tendencies(mlc_ctx *x, int m, const mlc_tend_ptrs *t) {
  if (!member_ok(x, m) || !t) return MLC_ERR_INVALID;
  if (!x->step_open) return MLC_ERR_STATE;
  Member &mb = x->mem[m];
  const int st = x->mixed ? set_tendencies_impl<float>(x, mb, t) : set_tendencies_impl<double>(x, mb, t);
  if (st != MLC_OK) return st;
  mb.tend_live = true;
  x->table_dirty = true;
  return MLC_OK;
}

int mlc_step_finish(mlc_ctx *x, mlc_diag *out) {
  if (!x) return MLC_ERR_INVALID;
  if (!x->step_open) return MLC_ERR_STATE;
  MLC_CHK(x->mixed ? refresh_all<float>(x) : refresh_all<double>(x));
  if (x->key.L.nmem > 0) {
    if (x->mixed) enqueue_step<float>(x, nullptr, kStepFinish);
    else enqueue_step<double>(x, nullptr, kStepFinish);
    MLC_TRY(cudaGetLastError());
  }
  x->step_open = false;
  // reset_tendencies: the next step starts from zero tendencies
  bool any = false;
  for (Member &m : x->mem) {
    any = any || m.tend_live;
    m.tend_live = false;
  }
  if (any) x->table_dirty = true;
  return fetch_diags(x, 1, out);
}

// ---- SAV restart files (Main/mod_savefile.F90, Main/mod_init.F90:421-450,941-966)

int mlc_member_write_sav(mlc_ctx *x, int m, const char *path, const char *idatex,
                         const char *calendar) {
  if (!member_ok(x, m) || !path) return MLC_ERR_INVALID;
  if (x->step_open) return MLC_ERR_STATE;  // a restart holds a whole step's state
  const mlc_dims d = x->mem[m].dims;
  const size_t jx = d.jx, iy = d.iy, kz = d.kz, c3 = (jx - 1) * (iy - 1) * kz;
  std::vector<double> u(jx * (iy - 1) * kz), v((jx - 1) * iy * kz), w((jx - 1) * (iy - 1) * (kz + 1));
  std::vector<double> t(c3), pai(c3), qx(c3 * d.nqx), ps((jx - 1) * (iy - 1)), trac(c3 * d.ntr);
  const bool tke = x->mem[m].c.tke != 0;
  std::vector<double> tk(tke ? (jx - 1) * (iy - 1) * (kz + 1) : 0);
  mlc_state_ptrs sp{};
  sp.u = u.data(); sp.v = v.data(); sp.w = w.data(); sp.t = t.data(); sp.pai = pai.data();
  sp.qx = qx.data(); sp.ps = ps.data(); sp.trac = d.ntr ? trac.data() : nullptr;
  sp.tke = tke ? tk.data() : nullptr;
  MLC_CHK(mlc_member_download_state(x, m, &sp));
  mlc_sav_fields f{u.data(), v.data(), w.data(), t.data(), pai.data(), qx.data(), ps.data(),
                   d.ntr ? trac.data() : nullptr, tke ? tk.data() : nullptr};
  return mlc_sav_write(path, &d, &f, idatex, calendar);
}

int mlc_member_read_sav(mlc_ctx *x, int m, const char *path) {
  if (!member_ok(x, m) || !path) return MLC_ERR_INVALID;
  if (x->step_open) return MLC_ERR_STATE;
  const mlc_dims d = x->mem[m].dims;
  const size_t jx = d.jx, iy = d.iy, kz = d.kz, c3 = (jx - 1) * (iy - 1) * kz;
  std::vector<double> u(jx * (iy - 1) * kz), v((jx - 1) * iy * kz), w((jx - 1) * (iy - 1) * (kz + 1));
  std::vector<double> t(c3), pai(c3), qx(c3 * d.nqx), ps((jx - 1) * (iy - 1)), trac(c3 * d.ntr);
  const bool tke = x->mem[m].c.tke != 0;
  std::vector<double> tk(tke ? (jx - 1) * (iy - 1) * (kz + 1) : 0);
  mlc_sav_fields f{u.data(), v.data(), w.data(), t.data(), pai.data(), qx.data(), ps.data(),
                   d.ntr ? trac.data() : nullptr, tke ? tk.data() : nullptr};
  MLC_CHK(mlc_sav_read(path, &d, &f, nullptr, 0));
  std::vector<double> su(u.size()), sv(v.size()), sw(w.size()), s3[9];
  for (auto &a : s3) a.resize(c3);
  std::vector<double> sq(qx.size()), sps(ps.size()), str(trac.size());
  mlc_state_ptrs sp{};
  sp.u = su.data(); sp.v = sv.data(); sp.w = sw.data(); sp.pai = s3[0].data(); sp.tetav = s3[1].data();
  sp.t = s3[2].data(); sp.tvirt = s3[3].data(); sp.ux = s3[4].data(); sp.vx = s3[5].data();
  sp.p = s3[6].data(); sp.rho = s3[7].data(); sp.qsat = s3[8].data(); sp.qx = sq.data();
  sp.ps = sps.data(); sp.trac = d.ntr ? str.data() : nullptr;
  sp.tke = tke ? tk.data() : nullptr;  // copied as read
  MLC_CHK(mlc_sav_restart_state(&d, &f, &sp));
  return mlc_member_upload_state(x, m, &sp);
}

int mlc_members(const mlc_ctx *x) { return x ? (int)x->mem.size() : 0; }

void mlc_destroy(mlc_ctx *x) { release(x); }

// mlc_step with the device time of the steps measured by CUDA events on the
// context stream (bracketing exactly the step launches).
int mlc_step_timed(mlc_ctx *x, int nsteps, mlc_diag *out, float *ms) {
  if (!x || !ms || nsteps < 0) return MLC_ERR_INVALID;
  if (x->step_open) return MLC_ERR_STATE;
  if (!ready(x)) return MLC_ERR_STATE;
  // descriptor upload and graph recording happen before the timed region
  MLC_CHK(step_any(x, 0));
  if (x->use_graphs && x->key.L.nmem > 0 &&
      (!x->graph_valid || std::memcmp(&x->graph_key, &x->key, sizeof(GraphKey)) != 0))
    MLC_CHK(x->mixed ? record<float>(x) : record<double>(x));
  cudaEvent_t e0, e1;
  MLC_TRY(cudaEventCreate(&e0));
  MLC_TRY(cudaEventCreate(&e1));
  MLC_TRY(cudaEventRecord(e0, x->stream));
  int st = step_any(x, nsteps);
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
  if (x->step_open) return MLC_ERR_STATE;
  if (!ready(x)) return MLC_ERR_STATE;
  MLC_CHK(step_any(x, 0));
  Recorder rec;
  rec.s = x->stream;
  if (x->key.L.nmem > 0)
    for (int n = 0; n < nsteps; ++n) {
      if (x->mixed) enqueue_step<float>(x, &rec);
      else enqueue_step<double>(x, &rec);
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
const int kVertCand[][2] = {{32, 4}, {32, 8}, {64, 2}, {32, 2}, {128, 1}};
constexpr int kNCol = 6, kNSolve = 5, kNVert = 5, kNTile = 4;

int group_of(const char *name) {
  if (!std::strcmp(name, "sound_solve")) return 1;
  if (!std::strcmp(name, "adv_vertical") || !std::strcmp(name, "adv_vertical_inc")) return 2;
  if (!std::strcmp(name, "adv_horizontal") || !std::strcmp(name, "adv_horizontal_inc")) return 3;
  if (!std::strcmp(name, "bdy_ring") || !std::strcmp(name, "end_reduce")) return -1;
  return 0;  // column kernels
}

bool shapes_fit(const LaunchGeom &L) {
  return L.col_x * L.col_y <= 1024 && L.vert_x * L.vert_y <= 1024;
}

// Per-group device time (ms) of `steps` eager steps with the shapes in x->key.L.
template <class R>
int time_groups(mlc_ctx *x, int steps, double ms[4]) {
  MLC_CHK(ensure_lists<R>(x));  // the trial's launch shapes
  Recorder rec;
  rec.s = x->stream;
  for (int n = 0; n < steps; ++n) enqueue_step<R>(x, &rec);
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

void set_shapes(LaunchGeom &L, int col, int solve, int vert, int tile) {
  L.col_x = kColCand[col][0]; L.col_y = kColCand[col][1];
  L.solve_x = kSolveCand[solve][0]; L.solve_y = kSolveCand[solve][1];
  L.vert_x = kVertCand[vert][0]; L.vert_y = kVertCand[vert][1];
  L.htile = tile;
}

template <class R>
int autotune_impl(mlc_ctx *x, int steps, mlc_tune_report *rep) {
  MLC_CHK(refresh_all<R>(x));
  if (x->key.L.nmem == 0) return MLC_ERR_STATE;
  // snapshot every member's arena and the clocks; each trial starts from it
  size_t total = x->mem.size() * sizeof(Clock);
  for (const Member &m : x->mem)
    if (m.used) total += m.bytes;
  char *snap = nullptr;
  if (cudaMallocFromPoolAsync(reinterpret_cast<void **>(&snap), total, x->pool, x->stream) != cudaSuccess) {
    cudaGetLastError();
    return MLC_ERR_NOMEM;
  }
  auto copy_all = [&](bool save) {
    size_t off = 0;
    for (const Member &m : x->mem) {
      if (!m.used) continue;
      if (save) cudaMemcpyAsync(snap + off, m.base, m.bytes, cudaMemcpyDeviceToDevice, x->stream);
      else cudaMemcpyAsync(m.base, snap + off, m.bytes, cudaMemcpyDeviceToDevice, x->stream);
      off += m.bytes;
    }
    const size_t nc = x->mem.size() * sizeof(Clock);
    if (save) cudaMemcpyAsync(snap + off, x->clks, nc, cudaMemcpyDeviceToDevice, x->stream);
    else cudaMemcpyAsync(x->clks, snap + off, nc, cudaMemcpyDeviceToDevice, x->stream);
  };
  copy_all(true);
  const LaunchGeom base = x->key.L;
  double best[4] = {1e30, 1e30, 1e30, 1e30};
  int pick[4] = {0, 0, 0, 0};
  int st = MLC_OK;
  const int ntrial = 6;
  for (int tr = 0; tr < ntrial && st == MLC_OK; ++tr) {
    LaunchGeom L = base;
    int idx[4] = {tr % kNCol, tr % kNSolve, tr % kNVert, tr % kNTile};
    set_shapes(L, idx[0], idx[1], idx[2], idx[3]);
    if (!shapes_fit(L)) {  // keep the base solve/vertical shapes for this trial
      L.solve_x = base.solve_x; L.solve_y = base.solve_y;
      L.vert_x = base.vert_x; L.vert_y = base.vert_y;
      idx[1] = idx[2] = 0;
    }
    x->key.L = L;
    double ms[4];
    copy_all(false);
    st = time_groups<R>(x, 1, ms);  // first use of the shapes
    if (st != MLC_OK) break;
    copy_all(false);
    st = time_groups<R>(x, steps, ms);
    if (st != MLC_OK) break;
    for (int q = 0; q < 4; ++q)
      if (ms[q] < best[q]) { best[q] = ms[q]; pick[q] = idx[q]; }
  }
  // the fixed configuration: 32 x 8 columns, tiles and vertical blocks, 32 x 2 solve
  LaunchGeom fixed = base;
  set_shapes(fixed, 1, 0, 1, 0);
  double msf[4] = {0, 0, 0, 0}, mst[4] = {0, 0, 0, 0};
  if (st == MLC_OK) {
    x->key.L = fixed;
    copy_all(false);
    st = time_groups<R>(x, steps, msf);
  }
  LaunchGeom tuned = base;
  set_shapes(tuned, pick[0], pick[1], pick[2], pick[3]);
  if (!shapes_fit(tuned)) tuned = base;
  if (st == MLC_OK) {
    x->key.L = tuned;
    copy_all(false);
    st = time_groups<R>(x, steps, mst);
  }
  copy_all(false);
  cudaFreeAsync(snap, x->stream);
  cudaStreamSynchronize(x->stream);
  if (st != MLC_OK) {
    x->key.L = base;
    return st;
  }
  x->key.L = tuned;  // the graph is recorded again at the next step
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
  if (x->step_open) return MLC_ERR_STATE;
  if (!ready(x)) return MLC_ERR_STATE;
  return x->mixed ? autotune_impl<float>(x, steps, rep) : autotune_impl<double>(x, steps, rep);
}

int mlc_set_launch_shapes(mlc_ctx *x, const mlc_tune_report *r) {
  if (!x || !r) return MLC_ERR_INVALID;
  if (x->step_open) return MLC_ERR_STATE;
  auto find = [](const int (*cand)[2], int n, int a, int b) {
    for (int q = 0; q < n; ++q)
      if (cand[q][0] == a && cand[q][1] == b) return q;
    return -1;
  };
  const int col = find(kColCand, kNCol, r->col_x, r->col_y);
  const int solve = find(kSolveCand, kNSolve, r->solve_x, r->solve_y);
  const int vert = find(kVertCand, kNVert, r->vert_x, r->vert_y);
  if (col < 0 || solve < 0 || vert < 0 || r->htile < 0 || r->htile >= kNTile) return MLC_ERR_INVALID;
  LaunchGeom L = x->key.L;
  set_shapes(L, col, solve, vert, r->htile);
  if (!shapes_fit(L)) return MLC_ERR_INVALID;
  x->key.L = L;  // the graph is recorded again at the next step
  return MLC_OK;
}

const char *mlc_last_error(void) { return g_last_error; }

// Kernels one mlc_step(ctx, 1) launches (for launch accounting).
int mlc_launches_per_step(const mlc_ctx *x) { return x ? x->launches_per_step : 0; }

// Run steps without graph capture (for tests of the capture path).
int mlc_set_graphs(mlc_ctx *x, int on) {
  if (!x) return MLC_ERR_INVALID;
  x->use_graphs = on != 0;
  return MLC_OK;
}

int mlc_member_test_stall(mlc_ctx *x, int m, int polls) {
  if (!member_ok(x, m) || polls < 0) return MLC_ERR_INVALID;
  if (x->step_open) return MLC_ERR_STATE;
  x->mem[m].stall_polls = polls;
  x->table_dirty = true;
  return MLC_OK;
}

int mlc_set_solve_precision(mlc_ctx *x, int df_recurrence) {
  if (!x) return MLC_ERR_INVALID;
  if (x->step_open) return MLC_ERR_STATE;
  x->key.L.solve_df = df_recurrence ? 1 : 0;
  return MLC_OK;
}

}  // extern "C"
