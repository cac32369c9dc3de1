// gsks_noalloc.cu -- FP64 kernel summation that allocates no memory.
//
// gsks_dgsks_device() obtains the scratch of its deterministic two-pass
// reduction (one partial sum per target row and source chunk) from the
// stream-ordered allocator on every call.  Some callers cannot let a library
// allocate device memory at all: a process whose device memory is handed out
// up front by a pool allocator (the pool already reserved the memory, so a
// cudaMalloc either fails or fragments the pool), or a latency-critical loop
// whose rules forbid any allocation after start-up.  For them,
// gsks_dgsks_device_noalloc() runs the same FP64 kernels with that scratch in
// a fixed array compiled into the library.
//
// The array holds GSKS_NOALLOC_MAX_PARTIAL doubles (8 MiB).  Every GPU that
// loads the library keeps it, and a 256-byte error word, until the process
// exits.  All calls on a device share the array and it keeps the contents of
// the last call; each call overwrites every entry it later reads, so nothing
// needs clearing.  Calls whose work overlaps on the GPU (two streams, or two
// host threads) race on the array: serialise them.
#include "gsks.h"
#include "gsks_internal.cuh"
#include "gsks_host.h"
#include "gsks_fp64_item.cuh"

#include <algorithm>
#include <mutex>

namespace gsks {
namespace {

constexpr size_t NOALLOC_MAX_PARTIAL = (size_t)1 << 20;   // doubles (8 MiB)
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) double g_noalloc_partial[NOALLOC_MAX_PARTIAL];
static __device__ __align__(256) int g_noalloc_err[64];

struct NoallocDevice {
  bool ready = false;
  double *partial = nullptr;  // device address of g_noalloc_partial
  int *err = nullptr;         // device address of g_noalloc_err
  int num_sms = 0;
};
NoallocDevice g_dev[NOALLOC_MAX_DEVICES];
std::mutex g_mu;

// Once per device, with that device current: the device addresses of the two
// arrays.  In host code the array names are host-side stand-ins, not device
// addresses, so they are never passed to a kernel directly.
int noalloc_setup(NoallocDevice *&out)
{
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "gsks_dgsks_device_noalloc");
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return set_status(GSKS_ERR_ARG, "gsks_dgsks_device_noalloc");
  std::lock_guard<std::mutex> lock(g_mu);
  NoallocDevice &d = g_dev[dev];
  if (!d.ready) {
    void *p = nullptr, *q = nullptr;
    if ((e = cudaGetSymbolAddress(&p, g_noalloc_partial)) != cudaSuccess)
      return cuda_status(e, "cudaGetSymbolAddress(partial)");
    if ((e = cudaGetSymbolAddress(&q, g_noalloc_err)) != cudaSuccess)
      return cuda_status(e, "cudaGetSymbolAddress(err)");
    if ((e = cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
      return cuda_status(e, "cudaDeviceGetAttribute");
    d.partial = (double *)p;
    d.err = (int *)q;
    d.ready = true;
  }
  out = &d;
  return GSKS_OK;
}

}  // namespace
}  // namespace gsks

using namespace gsks;

extern "C" int gsks_dgsks_device_noalloc(ks_t *kernel, int m, int n, int k,
                                         double *u, const int *umap,
                                         const double *XA, const double *XA2, const int *amap,
                                         const double *XB, const double *XB2, const int *bmap,
                                         const double *w, const int *wmap, void *stream)
{
  note_launches(0);
  if (m < 0 || n < 0 || k < 0) return set_status(GSKS_ERR_ARG, "gsks_dgsks_device_noalloc");
  if (m == 0 || n == 0 || k == 0) return set_status(GSKS_OK, nullptr);
  int st = check_kernel(kernel, k);
  if (st) return set_status(st, "gsks_dgsks_device_noalloc");
  if (!u || !XA || !XB || !w) return set_status(GSKS_ERR_ARG, "gsks_dgsks_device_noalloc");
  if (kt_uses_norms(kernel->type) && (!XA2 || !XB2))
    return set_status(GSKS_ERR_ARG, "gsks_dgsks_device_noalloc");

  // The partial sums of one call need at least one slot per target row
  // (rounded up to the 64-row tile): m above 2^20 cannot fit the array.
  const size_t ldp_need = ((size_t)m + fp64cfg::BM - 1) / fp64cfg::BM * fp64cfg::BM;
  if (ldp_need > NOALLOC_MAX_PARTIAL) return set_status(GSKS_ERR_TOO_LARGE, "gsks_dgsks_device_noalloc");

  NoallocDevice *d = nullptr;
  if ((st = noalloc_setup(d)) != GSKS_OK) return st;

  // Same decomposition as gsks_dgsks_device, with the number of source chunks
  // capped so that chunks x rows fits the array.  fp64_plan keeps nsc * ntm
  // below 32 * SMs + ntm (or nsc = 1), i.e. under 2^20 partials for up to 256
  // SMs (GB300 has 152): the cap is a guard for larger devices.
  Fp64Plan p = fp64_plan(m, n, k, d->num_sms);
  if (p.partial_elems > NOALLOC_MAX_PARTIAL) {
    const long long nsc_max = std::max<long long>(1, (long long)(NOALLOC_MAX_PARTIAL / (size_t)p.ldp));
    int chunk = (int)((n + nsc_max - 1) / nsc_max);
    chunk = (chunk + fp64cfg::BN - 1) / fp64cfg::BN * fp64cfg::BN;
    p.chunk = chunk;
    p.nsc = (n + chunk - 1) / chunk;
    p.grid = (int)std::min<long long>((long long)p.ntm * p.nsc, (long long)std::max(1, d->num_sms) * 2);
    p.partial_elems = (size_t)p.nsc * p.ldp;
  }

  FusedArgs a{};
  a.m = m; a.n = n; a.k = k;
  a.XA = XA; a.XA2 = XA2; a.amap = amap;
  a.XB = XB; a.XB2 = XB2; a.bmap = bmap;
  a.w = w; a.wmap = wmap;
  a.kp = make_kparams(kernel, kernel->hi, kernel->hj);
  a.kp.coinc = coincidence_eps(k);
  a.nxa = -1; a.nxb = -1;   // maps are not range-checked on this path
  a.partial = d->partial;
  a.err = d->err;
  const int launches = fp64_launch(a, p, u, umap, (cudaStream_t)stream);
  if (launches < 0) return set_status(GSKS_ERR_KERNEL_TYPE, "gsks_dgsks_device_noalloc");
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e, "gsks_dgsks_device_noalloc");
  note_launches(launches);
  return set_status(GSKS_OK, nullptr);
}
