// mlc_noalloc.cu -- the mass budget of one domain without any allocation.
//
// Who needs this: a host model that keeps its fields in device memory it
// manages itself (a Fortran/OpenACC model whose memory manager owns the
// device heap, a pool that must not fragment, code that runs where
// cudaMalloc is not allowed, such as inside a callback or a region being
// captured into a graph) can hand the library pointers to its own arrays
// but cannot let the library call cudaMalloc for scratch.  This entry point
// computes the same sums as the budget of mlc_step (Main/mod_massck.F90:
// 77-170) from caller-owned device arrays, keeping its per-block partial
// sums in the file-scope device array below instead of allocating them.
//
// Limits and sharing rules:
// * the scratch holds kBudgetBlocks partial records; one block reduces up to
//   kBudgetRowsPerBlock rows (i, k), so a domain may have at most
//   kBudgetBlocks * kBudgetRowsPerBlock = 32768 rows ((iy-1) * kz); larger
//   domains are rejected with MLC_ERR_TOO_LARGE;
// * every GPU that loads the library holds the 256 KiB array until exit;
// * all calls share the one array: calls whose kernels overlap on the GPU
//   (different streams, or different host threads) race on it; serialise
//   them (one stream, or events);
// * every partial record the final pass reads is written by the same call
//   before it is read, so no part of the array has to start at zero.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "../../include/moloch_gb300.h"

namespace {

constexpr int kBudgetBlocks = 4096;
constexpr int kBudgetRowsPerBlock = 8;
constexpr int kBudgetRecord = 8;  // dry, dryadv, qmass, qadv, ps max, ps min, bad, pad
constexpr int kBudgetThreads = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_budget_scratch[kBudgetBlocks * kBudgetRecord];

// Host-side copy of the array's device address, per device, with the id of
// the CUDA context it was taken in.  In host code the name g_budget_scratch
// is only a stand-in: its device address comes from cudaGetSymbolAddress
// with the device current.  A cudaDeviceReset (or any new primary context)
// reloads the module at another address, so the cached address is used only
// while the current context's id is the one it was taken in; otherwise it is
// looked up again.
std::mutex g_mu;
double *g_scratch_ptr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};

// The unique id of the current CUDA context (0 if it cannot be read), from
// driver entry points fetched through the runtime (no link against libcuda).
unsigned long long current_context_id() {
  static PFN_cuCtxGetCurrent_v4000 get_ctx = nullptr;
  static PFN_cuCtxGetId_v12000 get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_ctx = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(p);
    cudaGetLastError();
  });
  if (!get_ctx || !get_id) return 0;
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (get_ctx(&c) != CUDA_SUCCESS || !c) return 0;
  if (get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

int scratch_for_current_device(double **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return MLC_ERR_NODEVICE;
  if (dev < 0 || dev >= kMaxDevices) return MLC_ERR_INVALID;
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev] || ctx == 0 || g_scratch_ctx[dev] != ctx) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_budget_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return MLC_ERR_CUDA;
    }
    g_scratch_ptr[dev] = static_cast<double *>(p);
    // the lookup makes the device's primary context current if none was
    g_scratch_ctx[dev] = ctx ? ctx : current_context_id();
  }
  *out = g_scratch_ptr[dev];
  return MLC_OK;
}

__device__ double tree_sum(double x, double *sh) {
  const int t = threadIdx.x;
  sh[t] = x;
  __syncthreads();
  for (int s = kBudgetThreads / 2; s > 0; s >>= 1) {
    if (t < s) sh[t] = sh[t] + sh[t + s];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

__device__ double tree_ext(double x, double *sh, bool take_max) {
  const int t = threadIdx.x;
  sh[t] = x;
  __syncthreads();
  for (int s = kBudgetThreads / 2; s > 0; s >>= 1) {
    if (t < s) sh[t] = take_max ? fmax(sh[t], sh[t + s]) : fmin(sh[t], sh[t + s]);
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

// Arrays are in the packed reference layout: cross (jx-1, iy-1, kz),
// u (jx, iy-1, kz), v (jx-1, iy, kz), qx (jx-1, iy-1, kz, nqx), ps (jx-1, iy-1).
__global__ void __launch_bounds__(kBudgetThreads) k_budget_partial(
    int jx, int iy, int kz, int nqx, double dx, double dt, const double *__restrict__ rho,
    const double *__restrict__ dz, const double *__restrict__ qx, const double *__restrict__ u,
    const double *__restrict__ v, const double *__restrict__ ps, double *scratch) {
  __shared__ double sh[kBudgetThreads];
  const int nc = jx - 1;
  const size_t c2 = (size_t)nc * (iy - 1);
  const size_t c3 = c2 * kz;
  auto cx = [&](int j, int i, int k) { return (size_t)(j - 1) + (size_t)nc * (i - 1) + c2 * (k - 1); };
  auto ux = [&](int j, int i, int k) {
    return (size_t)(j - 1) + (size_t)jx * (i - 1) + (size_t)jx * (iy - 1) * (k - 1);
  };
  auto vx = [&](int j, int i, int k) {
    return (size_t)(j - 1) + (size_t)nc * (i - 1) + (size_t)nc * iy * (k - 1);
  };
  const double dxsq = dx * dx;
  double dry = 0, dadv = 0, qm = 0, qadv = 0, pmax = -INFINITY, pmin = INFINITY, bad = 0;
  const int nrows = (iy - 1) * kz;
  const int r0 = blockIdx.x * kBudgetRowsPerBlock;
  for (int r = r0; r < min(r0 + kBudgetRowsPerBlock, nrows); ++r) {
    const int i = r % (iy - 1) + 1, k = r / (iy - 1) + 1;
    if (i >= 2 && i <= iy - 2) {
      for (int j = 2 + threadIdx.x; j <= jx - 2; j += kBudgetThreads) {
        const size_t o = cx(j, i, k);
        const double dzr = dz[o], rh = rho[o];
        dry += dxsq * dzr * rh;
        for (int n = 0; n < nqx; ++n) qm += qx[o + n * c3] * dxsq * dzr * rh;
      }
    }
    if (threadIdx.x == 0) {
      const size_t ow = cx(1, i, k), oe = cx(jx - 1, i, k);
      const double uw = u[ux(1, i, k)], ue = u[ux(jx, i, k)];
      dadv += uw * dt * dx * dz[ow] * rho[ow];
      dadv -= ue * dt * dx * dz[oe] * rho[oe];
      for (int n = 0; n < nqx; ++n) {
        qadv += qx[ow + n * c3] * uw * dt * dx * dz[ow] * rho[ow];
        qadv -= qx[oe + n * c3] * ue * dt * dx * dz[oe] * rho[oe];
      }
    }
    if (i == 1 || i == iy - 1) {
      const int iv = (i == 1) ? 1 : iy;
      const bool south = (i == 1);
      for (int j = 2 + threadIdx.x; j <= jx - 2; j += kBudgetThreads) {
        const size_t o = cx(j, i, k);
        const double vv = v[vx(j, iv, k)];
        const double fl = vv * dt * dx * dz[o] * rho[o];
        dadv = south ? dadv + fl : dadv - fl;
        for (int n = 0; n < nqx; ++n) {
          const double q = qx[o + n * c3] * vv * dt * dx * dz[o] * rho[o];
          qadv = south ? qadv + q : qadv - q;
        }
      }
    }
    if (k == 1 && i >= 2 && i <= iy - 2) {
      for (int j = 2 + threadIdx.x; j <= jx - 2; j += kBudgetThreads) {
        const double x = ps[(size_t)(j - 1) + (size_t)nc * (i - 1)];
        if (!isfinite(x)) bad = 1;
        else { pmax = fmax(pmax, x); pmin = fmin(pmin, x); }
      }
    }
  }
  dry = tree_sum(dry, sh);
  dadv = tree_sum(dadv, sh);
  qm = tree_sum(qm, sh);
  qadv = tree_sum(qadv, sh);
  bad = tree_sum(bad, sh);
  pmax = tree_ext(pmax, sh, true);
  pmin = tree_ext(pmin, sh, false);
  if (threadIdx.x == 0) {
    double *rec = scratch + (size_t)blockIdx.x * kBudgetRecord;
    rec[0] = dry; rec[1] = dadv; rec[2] = qm; rec[3] = qadv;
    rec[4] = pmax; rec[5] = pmin; rec[6] = bad; rec[7] = 0.0;
  }
}

__global__ void k_budget_final(const double *scratch, int nblocks, double *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double a[4] = {0, 0, 0, 0}, pmax = -INFINITY, pmin = INFINITY;
  bool bad = false;
  for (int b = 0; b < nblocks; ++b) {
    const double *rec = scratch + (size_t)b * kBudgetRecord;
    for (int q = 0; q < 4; ++q) a[q] += rec[q];
    pmax = fmax(pmax, rec[4]);
    pmin = fmin(pmin, rec[5]);
    if (rec[6] != 0.0) bad = true;
  }
  out[0] = a[0]; out[1] = a[1]; out[2] = a[2]; out[3] = a[3];
  out[4] = bad ? NAN : pmax;
  out[5] = bad ? NAN : pmin;
  out[6] = bad ? 1.0 : 0.0;
}

}  // namespace

extern "C" int mlc_mass_budget_noalloc(const mlc_dims *d, double dx, double dt,
                                       const double *rho, const double *dz, const double *qx,
                                       const double *u, const double *v, const double *ps,
                                       double *out, void *stream) {
  if (!d || !rho || !dz || !qx || !u || !v || !ps || !out) return MLC_ERR_INVALID;
  if (d->jx < 5 || d->iy < 5 || d->kz < 1 || d->nqx < 1) return MLC_ERR_INVALID;
  const long long nrows = (long long)(d->iy - 1) * d->kz;
  if (nrows > (long long)kBudgetBlocks * kBudgetRowsPerBlock) return MLC_ERR_TOO_LARGE;
  double *scratch = nullptr;
  const int st = scratch_for_current_device(&scratch);
  if (st != MLC_OK) return st;
  const int nblocks = (int)((nrows + kBudgetRowsPerBlock - 1) / kBudgetRowsPerBlock);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_budget_partial<<<nblocks, kBudgetThreads, 0, s>>>(d->jx, d->iy, d->kz, d->nqx, dx, dt, rho,
                                                      dz, qx, u, v, ps, scratch);
  k_budget_final<<<1, 32, 0, s>>>(scratch, nblocks, out);
  return cudaGetLastError() == cudaSuccess ? MLC_OK : MLC_ERR_CUDA;
}
