// mlc_restart.cpp -- SAV restart files of a MOLOCH domain (host code).
//
// The MOLOCH variables of RegCM's SAV file (Main/mod_savefile.F90:867-883,
// 1042-1046 definitions, :1128-1139, 1258-1260 data; read back :618-630)
// in the netCDF classic format, written and parsed here without the netCDF
// library: a header of dimensions, global attributes and variables, then
// each variable's values big-endian at its offset.  Fortran arrays
// (j fastest) are netCDF variables whose dimensions are listed slowest
// first, so the values go out in the Fortran array's own order.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/moloch_gb300_restart.h"
#include "mlc_constants.h"

namespace {

using namespace mlc;

constexpr uint32_t kNcDimension = 10, kNcVariable = 11, kNcAttribute = 12;
constexpr uint32_t kNcChar = 2, kNcFloat = 5, kNcDouble = 6;

struct NcDim {
  std::string name;
  uint64_t len;
};
struct NcVar {
  std::string name;
  std::vector<int> dims;  // slowest first
  const double *data = nullptr;
  uint32_t type = kNcDouble;
  uint64_t begin = 0, bytes = 0;
};

// ---- writer ----------------------------------------------------------------
struct Header {
  std::vector<uint8_t> b;
  bool w64;  // CDF-5: 64-bit counts and lengths
  void u32(uint32_t v) {
    for (int s = 24; s >= 0; s -= 8) b.push_back((uint8_t)(v >> s));
  }
  void u64(uint64_t v) {
    for (int s = 56; s >= 0; s -= 8) b.push_back((uint8_t)(v >> s));
  }
  void count(uint64_t v) { w64 ? u64(v) : u32((uint32_t)v); }
  void pad() {
    while (b.size() % 4) b.push_back(0);
  }
  void name(const std::string &s) {
    count(s.size());
    b.insert(b.end(), s.begin(), s.end());
    pad();
  }
};

std::vector<uint8_t> header(int version, const std::vector<NcDim> &dims,
                            const std::vector<std::pair<std::string, std::string>> &atts,
                            const std::vector<NcVar> &vars) {
  Header h{{}, version == 5};
  h.b = {'C', 'D', 'F', (uint8_t)version};
  h.count(0);  // numrecs: no record dimension
  h.u32(kNcDimension);
  h.count(dims.size());
  for (const NcDim &d : dims) {
    h.name(d.name);
    h.count(d.len);
  }
  if (atts.empty()) {
    h.u32(0);
    h.count(0);
  } else {
    h.u32(kNcAttribute);
    h.count(atts.size());
    for (const auto &a : atts) {
      h.name(a.first);
      h.u32(kNcChar);
      h.count(a.second.size());
      h.b.insert(h.b.end(), a.second.begin(), a.second.end());
      h.pad();
    }
  }
  h.u32(kNcVariable);
  h.count(vars.size());
  for (const NcVar &v : vars) {
    h.name(v.name);
    h.count(v.dims.size());
    for (int id : v.dims) h.count((uint64_t)id);
    h.u32(0);  // no variable attributes
    h.count(0);
    h.u32(v.type);
    // vsize: 32 bits in CDF-1/2 (the writer picks CDF-5 beyond them)
    h.count(v.bytes);
    if (version == 1) h.u32((uint32_t)v.begin);
    else h.u64(v.begin);
  }
  return h.b;
}

int write_file(const char *path, const std::vector<NcDim> &dims,
               const std::vector<std::pair<std::string, std::string>> &atts, std::vector<NcVar> &vars) {
  bool big = false;
  for (NcVar &v : vars) {
    uint64_t n = 1;
    for (int id : v.dims) n *= dims[(size_t)id].len;
    v.bytes = n * sizeof(double);
    if (v.bytes >= 0xFFFFFFFCull) big = true;
  }
  const int version = big ? 5 : 2;
  // offsets depend on the header's size, which does not depend on them
  uint64_t off = header(version, dims, atts, vars).size();
  for (NcVar &v : vars) {
    v.begin = off;
    off += v.bytes;
  }
  const std::vector<uint8_t> hd = header(version, dims, atts, vars);
  FILE *fp = std::fopen(path, "wb");
  if (!fp) return MLC_ERR_INVALID;
  bool ok = std::fwrite(hd.data(), 1, hd.size(), fp) == hd.size();
  std::vector<uint64_t> buf;
  for (const NcVar &v : vars) {
    const uint64_t n = v.bytes / sizeof(double);
    for (uint64_t e0 = 0; e0 < n && ok; e0 += (1u << 20)) {
      const uint64_t m = std::min<uint64_t>(n - e0, 1u << 20);
      buf.resize(m);
      for (uint64_t e = 0; e < m; ++e) {
        uint64_t x;
        std::memcpy(&x, v.data + e0 + e, 8);
        buf[e] = __builtin_bswap64(x);
      }
      ok = std::fwrite(buf.data(), 8, m, fp) == m;
    }
  }
  ok = (std::fclose(fp) == 0) && ok;
  return ok ? MLC_OK : MLC_ERR_INVALID;
}

// ---- reader ----------------------------------------------------------------
struct Reader {
  std::vector<uint8_t> b;
  size_t p = 0;
  bool w64 = false, bad = false;
  uint32_t u32() {
    if (p + 4 > b.size()) { bad = true; return 0; }
    uint32_t v = 0;
    for (int q = 0; q < 4; ++q) v = (v << 8) | b[p++];
    return v;
  }
  uint64_t u64() {
    if (p + 8 > b.size()) { bad = true; return 0; }
    uint64_t v = 0;
    for (int q = 0; q < 8; ++q) v = (v << 8) | b[p++];
    return v;
  }
  uint64_t count() { return w64 ? u64() : u32(); }
  std::string name() {
    const uint64_t n = count();
    if (bad || p + n > b.size()) { bad = true; return {}; }
    std::string s(reinterpret_cast<const char *>(b.data() + p), (size_t)n);
    p += (size_t)((n + 3) / 4 * 4);
    return s;
  }
};

size_t type_size(uint32_t t) {
  switch (t) {
    case 1: case 2: case 7: return 1;  // byte, char, ubyte
    case 3: case 8: return 2;          // short, ushort
    case 4: case 5: case 9: return 4;  // int, float, uint
    case 6: case 10: case 11: return 8;  // double, int64, uint64
    default: return 0;
  }
}

struct NcFile {
  std::vector<NcDim> dims;
  std::vector<NcVar> vars;
  std::string idatex;
};

// Parse the header of a classic-format file (CDF-1, CDF-2 or CDF-5).
int parse(FILE *fp, NcFile &f) {
  Reader r;
  // headers of these files are small; read a generous prefix
  r.b.resize(1 << 20);
  const size_t got = std::fread(r.b.data(), 1, r.b.size(), fp);
  r.b.resize(got);
  if (got < 8) return MLC_ERR_INVALID;
  if (r.b[0] == 0x89 && r.b[1] == 'H' && r.b[2] == 'D' && r.b[3] == 'F') return MLC_ERR_UNSUPPORTED;
  if (r.b[0] != 'C' || r.b[1] != 'D' || r.b[2] != 'F') return MLC_ERR_INVALID;
  const int version = r.b[3];
  if (version != 1 && version != 2 && version != 5) return MLC_ERR_UNSUPPORTED;
  r.p = 4;
  r.w64 = version == 5;
  r.count();  // numrecs
  uint32_t tag = r.u32();
  uint64_t n = r.count();
  if (tag == kNcDimension) {
    for (uint64_t q = 0; q < n && !r.bad; ++q) {
      NcDim d;
      d.name = r.name();
      d.len = r.count();
      f.dims.push_back(d);
    }
  }
  tag = r.u32();
  n = r.count();
  if (tag == kNcAttribute) {
    for (uint64_t q = 0; q < n && !r.bad; ++q) {
      const std::string nm = r.name();
      const uint32_t t = r.u32();
      const uint64_t ne = r.count();
      const size_t sz = type_size(t) * (size_t)ne;
      if (r.bad || type_size(t) == 0 || r.p + sz > r.b.size()) return MLC_ERR_INVALID;
      if (nm == "idatex" && t == kNcChar)
        f.idatex.assign(reinterpret_cast<const char *>(r.b.data() + r.p), sz);
      r.p += (sz + 3) / 4 * 4;
    }
  }
  tag = r.u32();
  n = r.count();
  if (tag != kNcVariable) return MLC_ERR_INVALID;
  for (uint64_t q = 0; q < n && !r.bad; ++q) {
    NcVar v;
    v.name = r.name();
    const uint64_t nd = r.count();
    if (nd > 64) return MLC_ERR_INVALID;
    for (uint64_t e = 0; e < nd && !r.bad; ++e) v.dims.push_back((int)r.count());
    const uint32_t at = r.u32();
    const uint64_t na = r.count();
    if (at == kNcAttribute) {
      for (uint64_t e = 0; e < na && !r.bad; ++e) {
        r.name();
        const uint32_t t = r.u32();
        const uint64_t ne = r.count();
        const size_t sz = type_size(t) * (size_t)ne;
        if (r.bad || type_size(t) == 0 || r.p + sz > r.b.size()) return MLC_ERR_INVALID;
        r.p += (sz + 3) / 4 * 4;
      }
    }
    v.type = r.u32();
    v.bytes = r.count();
    v.begin = version == 1 ? r.u32() : r.u64();
    for (int id : v.dims)
      if (id < 0 || (size_t)id >= f.dims.size()) return MLC_ERR_INVALID;
    f.vars.push_back(v);
  }
  return r.bad ? MLC_ERR_INVALID : MLC_OK;
}

// Read variable `name` with dimensions (slowest first) of lengths `shape`
// into dst (FP64; FP32 variables are widened).
int read_var(FILE *fp, const NcFile &f, const char *name, const std::vector<uint64_t> &shape, double *dst) {
  const NcVar *v = nullptr;
  for (const NcVar &c : f.vars)
    if (c.name == name) v = &c;
  if (!v || v->dims.size() != shape.size()) return MLC_ERR_INVALID;
  uint64_t n = 1;
  for (size_t q = 0; q < shape.size(); ++q) {
    const NcDim &d = f.dims[(size_t)v->dims[q]];
    if (d.len == 0 || d.len != shape[q]) return MLC_ERR_INVALID;  // record or wrong extent
    n *= shape[q];
  }
  if (v->type != kNcDouble && v->type != kNcFloat) return MLC_ERR_UNSUPPORTED;
  if (std::fseek(fp, (long)v->begin, SEEK_SET) != 0) return MLC_ERR_INVALID;
  const size_t es = v->type == kNcDouble ? 8 : 4;
  std::vector<uint8_t> buf;
  for (uint64_t e0 = 0; e0 < n; e0 += (1u << 20)) {
    const uint64_t m = std::min<uint64_t>(n - e0, 1u << 20);
    buf.resize((size_t)m * es);
    if (std::fread(buf.data(), es, (size_t)m, fp) != m) return MLC_ERR_INVALID;
    for (uint64_t e = 0; e < m; ++e) {
      if (es == 8) {
        uint64_t x;
        std::memcpy(&x, buf.data() + e * 8, 8);
        x = __builtin_bswap64(x);
        std::memcpy(dst + e0 + e, &x, 8);
      } else {
        uint32_t x;
        std::memcpy(&x, buf.data() + e * 4, 4);
        x = __builtin_bswap32(x);
        float y;
        std::memcpy(&y, &x, 4);
        dst[e0 + e] = (double)y;
      }
    }
  }
  return MLC_OK;
}

bool dims_ok(const mlc_dims *d) {
  return d && d->jx >= 4 && d->iy >= 4 && d->kz >= 1 && d->nqx >= 1 && d->ntr >= 0;
}

}  // namespace

extern "C" {

// write_savefile's MOLOCH part (Main/mod_savefile.F90:833-838 dimensions,
// :867-883 and :1042-1046 definitions, :1128-1139 and :1258-1260 values).
int mlc_sav_write(const char *path, const mlc_dims *d, const mlc_sav_fields *f, const char *idatex,
                  const char *calendar) {
  if (!path || !dims_ok(d) || !f || !f->u || !f->v || !f->w || !f->t || !f->pai || !f->qx || !f->ps)
    return MLC_ERR_INVALID;
  if (d->ntr > 0 && !f->trac) return MLC_ERR_INVALID;
  const uint64_t jx = (uint64_t)d->jx, iy = (uint64_t)d->iy, kz = (uint64_t)d->kz;
  enum { JC, IC, JD, ID, KH, KF, NQ, NT };
  std::vector<NcDim> dims = {{"jcross", jx - 1}, {"icross", iy - 1}, {"jdot", jx},
                             {"idot", iy},       {"khalf", kz},      {"kfull", kz + 1},
                             {"nqx", (uint64_t)d->nqx}};
  if (d->ntr > 0) dims.push_back({"ntr", (uint64_t)d->ntr});
  std::vector<NcVar> vars;
  auto add = [&](const char *nm, std::vector<int> ds, const double *p) {
    NcVar v;
    v.name = nm;
    v.dims = std::move(ds);
    v.data = p;
    vars.push_back(v);
  };
  add("atm_u", {KH, IC, JD}, f->u);
  add("atm_v", {KH, ID, JC}, f->v);
  add("atm_w", {KF, IC, JC}, f->w);
  add("atm_t", {KH, IC, JC}, f->t);
  add("atm_pai", {KH, IC, JC}, f->pai);
  add("atm_qx", {NQ, KH, IC, JC}, f->qx);
  if (f->tke) add("atm_tke", {KF, IC, JC}, f->tke);  // ibltyp = 2 (:884-887)
  add("ps", {IC, JC}, f->ps);
  if (d->ntr > 0) add("trac", {NT, KH, IC, JC}, f->trac);
  std::vector<std::pair<std::string, std::string>> atts;
  if (idatex) atts.push_back({"idatex", idatex});
  if (calendar) atts.push_back({"calendar", calendar});
  return write_file(path, dims, atts, vars);
}

int mlc_sav_read(const char *path, const mlc_dims *d, const mlc_sav_fields *f, char *idatex,
                 size_t idatex_len) {
  if (!path || !dims_ok(d) || !f || !f->u || !f->v || !f->w || !f->t || !f->pai || !f->qx || !f->ps)
    return MLC_ERR_INVALID;
  if (d->ntr > 0 && !f->trac) return MLC_ERR_INVALID;
  FILE *fp = std::fopen(path, "rb");
  if (!fp) return MLC_ERR_INVALID;
  NcFile nf;
  int st = parse(fp, nf);
  const uint64_t jx = (uint64_t)d->jx, iy = (uint64_t)d->iy, kz = (uint64_t)d->kz;
  const uint64_t nq = (uint64_t)d->nqx, nt = (uint64_t)d->ntr;
  if (st == MLC_OK) st = read_var(fp, nf, "atm_u", {kz, iy - 1, jx}, f->u);
  if (st == MLC_OK) st = read_var(fp, nf, "atm_v", {kz, iy, jx - 1}, f->v);
  if (st == MLC_OK) st = read_var(fp, nf, "atm_w", {kz + 1, iy - 1, jx - 1}, f->w);
  if (st == MLC_OK) st = read_var(fp, nf, "atm_t", {kz, iy - 1, jx - 1}, f->t);
  if (st == MLC_OK) st = read_var(fp, nf, "atm_pai", {kz, iy - 1, jx - 1}, f->pai);
  if (st == MLC_OK) st = read_var(fp, nf, "atm_qx", {nq, kz, iy - 1, jx - 1}, f->qx);
  if (st == MLC_OK && f->tke) st = read_var(fp, nf, "atm_tke", {kz + 1, iy - 1, jx - 1}, f->tke);
  if (st == MLC_OK) st = read_var(fp, nf, "ps", {iy - 1, jx - 1}, f->ps);
  if (st == MLC_OK && nt > 0) st = read_var(fp, nf, "trac", {nt, kz, iy - 1, jx - 1}, f->trac);
  std::fclose(fp);
  if (st == MLC_OK && idatex && idatex_len > 0) {
    const size_t n = std::min(idatex_len - 1, nf.idatex.size());
    std::memcpy(idatex, nf.idatex.data(), n);
    idatex[n] = '\0';
  }
  return st;
}

// Main/mod_init.F90:421-450 (copies) and :941-960 (diagnostics) in FP64.
int mlc_sav_restart_state(const mlc_dims *d, const mlc_sav_fields *f, const mlc_state_ptrs *st) {
  if (!dims_ok(d) || !f || !st || !f->u || !f->v || !f->w || !f->t || !f->pai || !f->qx || !f->ps)
    return MLC_ERR_INVALID;
  if (!st->u || !st->v || !st->w || !st->t || !st->pai || !st->qx || !st->ps || !st->p ||
      !st->qsat || !st->rho || !st->tvirt || !st->tetav)
    return MLC_ERR_INVALID;
  if (d->ntr > 0 && (!f->trac || !st->trac)) return MLC_ERR_INVALID;
  const size_t jx = (size_t)d->jx, iy = (size_t)d->iy, kz = (size_t)d->kz;
  const size_t c3 = (jx - 1) * (iy - 1) * kz;
  std::memcpy(st->u, f->u, jx * (iy - 1) * kz * sizeof(double));
  std::memcpy(st->v, f->v, (jx - 1) * iy * kz * sizeof(double));
  std::memcpy(st->w, f->w, (jx - 1) * (iy - 1) * (kz + 1) * sizeof(double));
  std::memcpy(st->t, f->t, c3 * sizeof(double));
  std::memcpy(st->pai, f->pai, c3 * sizeof(double));
  std::memcpy(st->qx, f->qx, c3 * (size_t)d->nqx * sizeof(double));
  std::memcpy(st->ps, f->ps, (jx - 1) * (iy - 1) * sizeof(double));
  if (d->ntr > 0) std::memcpy(st->trac, f->trac, c3 * (size_t)d->ntr * sizeof(double));
  if (f->tke && st->tke && st->tke != f->tke)
    std::memcpy(st->tke, f->tke, (jx - 1) * (iy - 1) * (kz + 1) * sizeof(double));
  for (size_t e = 0; e < c3; ++e) {
    const double t = f->t[e], pai = f->pai[e];
    const double p = std::pow(pai, kCpovr) * kP00;
    st->p[e] = p;
    st->qsat[e] = pfwsat(t, p);
    st->rho[e] = p / (kRgas * t);
    st->tvirt[e] = t * (1.0 + kEp1 * f->qx[e]);
    st->tetav[e] = st->tvirt[e] / pai;
  }
  if (st->ux) std::memset(st->ux, 0, c3 * sizeof(double));
  if (st->vx) std::memset(st->vx, 0, c3 * sizeof(double));
  return MLC_OK;
}

}  // extern "C"
