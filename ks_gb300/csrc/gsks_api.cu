// gsks_api.cu -- the C ABI of libgsks.so (ks.h + gsks.h).
//
// Host-side layer between C callers and the sm_103a kernels:
//   * argument and kernel-descriptor checks with status codes in place of
//     the reference's printf + exit (frame/dgsks.c:393-468);
//   * per-thread contexts (CUDA stream, pinned staging, device buffers), so
//     that dgsks() may be called concurrently from many host threads as the
//     reference's batched driver does (frame/omp_dgsks_list.cpp:366-396);
//   * host-pointer calls: the rows named by the maps are gathered into pinned
//     buffers, copied once, evaluated with identity maps, and u is scattered
//     back in target order (u[umap[i]] = result[i], i ascending,
//     frame/dgsks_ref.c:454-459).  umap is meant to be injective within one
//     call; for repeated entries this path keeps the last writer, whereas the
//     reference's result then depends on its OpenMP schedule and blocking;
//   * device-pointer calls run in place on the caller's stream.
#include "gsks.h"
#include "gsks_internal.cuh"
#include "gsks_host.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace gsks {

thread_local int tl_status = GSKS_OK;
thread_local int tl_precision = -1;
thread_local int tl_launches = 0;

static bool verbose()
{
  static int v = -1;
  if (v < 0) { const char *e = getenv("GSKS_VERBOSE"); v = (e && *e && *e != '0') ? 1 : 0; }
  return v == 1;
}

int set_status(int s, const char *where)
{
  tl_status = s;
  if (s != GSKS_OK && verbose())
    fprintf(stderr, "gsks: %s: %s\n", where ? where : "", gsks_error_string(s));
  return s;
}

int cuda_status(cudaError_t e, const char *where)
{
  if (e == cudaSuccess) return GSKS_OK;
  if (verbose()) fprintf(stderr, "gsks: %s: %s\n", where, cudaGetErrorString(e));
  if (e == cudaErrorMemoryAllocation) return set_status(GSKS_ERR_ALLOC, where);
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
    return set_status(GSKS_ERR_NO_DEVICE, where);
  return set_status(GSKS_ERR_CUDA, where);
}

void note_launches(int n) { tl_launches = n; }

// ---------------------------------------------------------------------------
bool DevBuf::ensure(size_t bytes)
{
  if (bytes <= cap) return true;
  if (p) { cudaFree(p); p = nullptr; cap = 0; }
  size_t want = std::max<size_t>(bytes + bytes / 4, 256);
  if (cudaMalloc(&p, want) != cudaSuccess) { p = nullptr; return false; }
  cap = want;
  return true;
}
void DevBuf::release() { if (p) cudaFree(p); p = nullptr; cap = 0; }

bool PinBuf::ensure(size_t bytes)
{
  if (bytes <= cap) return true;
  if (p) { cudaFreeHost(p); p = nullptr; cap = 0; }
  size_t want = std::max<size_t>(bytes + bytes / 4, 256);
  if (cudaMallocHost(&p, want) != cudaSuccess) { p = nullptr; return false; }
  cap = want;
  return true;
}
void PinBuf::release() { if (p) cudaFreeHost(p); p = nullptr; cap = 0; }

Ctx::~Ctx()
{
  // Runs at host-thread exit; the CUDA runtime may already be gone at
  // process teardown, in which case the frees fail harmlessly.
  for (DevBuf *b : {&partial, &err, &dA, &dA2, &dB, &dB2, &dw, &du, &dhi, &dhj, &dwork, &rmaps, &serr, &stats})
    b->release();
  for (PinBuf *b : {&hA, &hA2, &hB, &hB2, &hw, &hu, &hhi, &hhj}) b->release();
  if (stream) cudaStreamDestroy(stream);
}

static thread_local std::unique_ptr<Ctx> tl_ctx;

Ctx *get_ctx()
{
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) { cuda_status(e, "cudaGetDevice"); return nullptr; }
  if (tl_ctx && tl_ctx->device == dev) return tl_ctx.get();
  std::unique_ptr<Ctx> c(new Ctx);
  c->device = dev;
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) {
    cuda_status(e, "cudaStreamCreate");
    return nullptr;
  }
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev);
  if (!c->err.ensure(sizeof(int))) { set_status(GSKS_ERR_ALLOC, "context"); return nullptr; }
  cudaMemset(c->err.p, 0, sizeof(int));
  tl_ctx = std::move(c);
  return tl_ctx.get();
}

int effective_precision()
{
  if (tl_precision < 0) {
    const char *e = getenv("GSKS_PRECISION");
    tl_precision = GSKS_FP64;
    if (e && (!strncmp(e, "split", 5) || !strcmp(e, "bf16x3"))) tl_precision = GSKS_SPLIT_BF16X3;
  }
  return tl_precision;
}

// Kernel-descriptor checks and the Laplace parameter overwrite
// (frame/dgsks.c:420-468; the reference prints and carries on for a missing
// bandwidth vector or k < 3, and exits for an illegal type).
int check_kernel(ks_t *ker, int k)
{
  if (!ker) return GSKS_ERR_ARG;
  switch (ker->type) {
    case KS_GAUSSIAN: case KS_POLYNOMIAL: case KS_TANH: case KS_QUARTIC:
    case KS_MULTIQUADRATIC: case KS_EPANECHNIKOV:
      return GSKS_OK;
    case KS_GAUSSIAN_VAR_BANDWIDTH:
      return (ker->hi && ker->hj) ? GSKS_OK : GSKS_ERR_BANDWIDTH;
    case KS_LAPLACE:
      if (k < 3) return GSKS_ERR_LAPLACE_K;
      ker->powe = 0.5 * (2.0 - (double)k);
      ker->scal = tgamma(0.5 * k + 1.0) / ((double)k * (double)(k - 2) * pow(M_PI, 0.5 * k));
      return GSKS_OK;
    default:
      return GSKS_ERR_KERNEL_TYPE;
  }
}

bool is_device_pointer(const void *p)
{
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) { cudaGetLastError(); return false; }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

static int host_threads_for(size_t work)
{
#ifdef _OPENMP
  if (work < (1u << 16)) return 1;
  return std::max(1, std::min(omp_get_max_threads(), 16));
#else
  (void)work;
  return 1;
#endif
}

// One side of a host-pointer call gathered by the GPU straight from the
// caller's (pageable) host arrays: row i of dX is X[map[i]], and the row's
// norm, bandwidth and R values (u or w, nrhs interleaved columns) come along.
// One warp per row, lanes over the coordinates.  The maps were checked on the
// host first (no negative entry).
__global__ void __launch_bounds__(256) gather_rows(int cnt, int k, int R, const int *__restrict__ map,
                                                   const int *__restrict__ vmap, const double *__restrict__ X,
                                                   const double *__restrict__ X2, const double *__restrict__ hv,
                                                   const double *__restrict__ val, double *__restrict__ dX,
                                                   double *__restrict__ dX2, double *__restrict__ dh,
                                                   double *__restrict__ dval)
{
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < cnt; i += nw) {
    const int p = map[i], q = vmap[i];
    const double *src = X + (size_t)p * k;
    double *dst = dX + (size_t)i * k;
    for (int e = lane; e < k; e += 32) dst[e] = src[e];
    if (lane == 0) {
      if (X2) dX2[i] = X2[p];
      if (hv) dh[i] = hv[p];
    }
    for (int r = lane; r < R; r += 32) dval[(size_t)i * R + r] = val[(size_t)q * R + r];
  }
}

// Whether this device's kernels may read pageable host memory (coherent
// access through the host page tables, as on Grace-Blackwell): then the host
// calls gather on the GPU.  GSKS_HOST_GATHER=cpu keeps the gather on the host.
static bool host_direct(Ctx *c)
{
  const char *e = getenv("GSKS_HOST_GATHER");
  if (e && !strcmp(e, "cpu")) return false;
  if (c->host_direct < 0) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, c->device) != cudaSuccess) {
      cudaGetLastError();
      v = 0;
    }
    c->host_direct = v ? 1 : 0;
  }
  return c->host_direct == 1;
}

extern "C" int gsks_host_gather_on_device(void)
{
  Ctx *c = get_ctx();
  if (!c) return -1;
  return host_direct(c) ? 1 : 0;
}

// Gather the rows a host-pointer call names into pinned buffers and copy
// them to the device (or, where the GPU reads host memory, gather them on the
// GPU).  On return `v` describes packed, identity-mapped data.
int stage_host(Ctx *c, const ks_t *ker, int m, int n, int k,
               const double *u, const int *umap,
               const double *XA, const double *XA2, const int *amap,
               const double *XB, const double *XB2, const int *bmap,
               const double *w, const int *wmap, Staged &v, int nrhs)
{
  const bool norms = kt_uses_norms(ker->type);
  const bool varbw = ker->type == KS_GAUSSIAN_VAR_BANDWIDTH;
  if (norms && (!XA2 || !XB2)) return GSKS_ERR_ARG;

  const size_t mk = (size_t)m * k, nk = (size_t)n * k;
  // u and w keep their nrhs interleaved columns (u[umap[i] * nrhs + r])
  const size_t R = (size_t)std::max(nrhs, 1);
  bool ok = c->hA.ensure(mk * 8) && c->hB.ensure(nk * 8) && c->hu.ensure((size_t)m * R * 8) &&
            c->hw.ensure((size_t)n * R * 8) && c->dA.ensure(mk * 8) && c->dB.ensure(nk * 8) &&
            c->du.ensure((size_t)m * R * 8) && c->dw.ensure((size_t)n * R * 8);
  if (ok && norms)
    ok = c->hA2.ensure((size_t)m * 8) && c->hB2.ensure((size_t)n * 8) &&
         c->dA2.ensure((size_t)m * 8) && c->dB2.ensure((size_t)n * 8);
  if (ok && varbw)
    ok = c->hhi.ensure((size_t)m * 8) && c->hhj.ensure((size_t)n * 8) &&
         c->dhi.ensure((size_t)m * 8) && c->dhj.ensure((size_t)n * 8);
  if (!ok) return GSKS_ERR_ALLOC;

  if (host_direct(c)) {
    // the maps are checked on the host (negative entries), then one gather
    // kernel per side reads the caller's arrays
    const int nt = host_threads_for((size_t)std::max(m, n) * 16);
    int bad = 0;
#pragma omp parallel for num_threads(nt) reduction(| : bad) schedule(static)
    for (int i = 0; i < std::max(m, n); i++) {
      if (i < m && (amap[i] < 0 || umap[i] < 0)) bad = 1;
      if (i < n && (bmap[i] < 0 || wmap[i] < 0)) bad = 1;
    }
    if (bad) return GSKS_ERR_MAP_RANGE;
    const int R_ = (int)R;
    const int grid = std::max(1, c->num_sms * 8);
    gather_rows<<<grid, 256, 0, c->stream>>>(m, k, R_, amap, umap, XA, norms ? XA2 : nullptr, varbw ? ker->hi : nullptr,
                                               u, (double *)c->dA.p, (double *)c->dA2.p, (double *)c->dhi.p,
                                               (double *)c->du.p);
    gather_rows<<<grid, 256, 0, c->stream>>>(n, k, R_, bmap, wmap, XB, norms ? XB2 : nullptr, varbw ? ker->hj : nullptr,
                                               w, (double *)c->dB.p, (double *)c->dB2.p, (double *)c->dhj.p,
                                               (double *)c->dw.p);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e, "gather_rows");
    note_launches(2);
    v.A = (const double *)c->dA.p; v.B = (const double *)c->dB.p;
    v.A2 = norms ? (const double *)c->dA2.p : nullptr;
    v.B2 = norms ? (const double *)c->dB2.p : nullptr;
    v.hi = varbw ? (const double *)c->dhi.p : nullptr;
    v.hj = varbw ? (const double *)c->dhj.p : nullptr;
    v.u = (double *)c->du.p; v.w = (const double *)c->dw.p;
    return GSKS_OK;
  }

  double *hA = (double *)c->hA.p, *hB = (double *)c->hB.p;
  double *hA2 = (double *)c->hA2.p, *hB2 = (double *)c->hB2.p;
  double *hhi = (double *)c->hhi.p, *hhj = (double *)c->hhj.p;
  double *hu = (double *)c->hu.p, *hw = (double *)c->hw.p;
  const size_t rowb = (size_t)k * sizeof(double);
  cudaStream_t s = c->stream;

  // Gather the rows the maps name into the pinned buffers and copy them, in
  // chunks: the calling thread issues a chunk's copy while the team gathers
  // the next one.  Maps are checked as they are read.
  const int nt = host_threads_for(std::max(mk, nk));
  const int ch = std::max(1024, (int)((4u << 20) / std::max(rowb, (size_t)8)));   // rows per chunk (~4 MiB)
  int bad = 0;
  cudaError_t e = cudaSuccess;
#pragma omp parallel num_threads(nt)
  {
    for (int side = 0; side < 2; side++) {
      const int cnt = side ? n : m;
      const int *map = side ? bmap : amap, *vmap = side ? wmap : umap;
      const double *X = side ? XB : XA, *X2 = side ? XB2 : XA2, *hv = side ? ker->hj : ker->hi;
      const double *val = side ? w : u;
      double *hX = side ? hB : hA, *hX2 = side ? hB2 : hA2, *hh = side ? hhj : hhi, *hval = side ? hw : hu;
      for (int r0 = 0; r0 < cnt; r0 += ch) {
        const int r1 = std::min(cnt, r0 + ch);
#pragma omp for schedule(static)
        for (int i = r0; i < r1; i++) {
          const int p = map[i], q = vmap[i];
          if (p < 0 || q < 0) {
#pragma omp atomic write
            bad = 1;
            continue;
          }
          memcpy(hX + (size_t)i * k, X + (size_t)p * k, rowb);
          if (norms) hX2[i] = X2[p];
          if (varbw) hh[i] = hv[p];
          for (size_t r = 0; r < R; r++) hval[(size_t)i * R + r] = val[(size_t)q * R + r];
        }
        // (the loop's barrier: the chunk is complete)
#pragma omp master
        {
          double *dX = (double *)(side ? c->dB.p : c->dA.p);
          if (e == cudaSuccess)
            e = cudaMemcpyAsync(dX + (size_t)r0 * k, hX + (size_t)r0 * k, (size_t)(r1 - r0) * rowb,
                                cudaMemcpyHostToDevice, s);
        }
      }
    }
  }
  if (bad) return GSKS_ERR_MAP_RANGE;
#define GSKS_CP(dst, src, bytes) \
  if (e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s)
  GSKS_CP(c->du.p, hu, (size_t)m * R * 8);
  GSKS_CP(c->dw.p, hw, (size_t)n * R * 8);
  if (norms) { GSKS_CP(c->dA2.p, hA2, (size_t)m * 8); GSKS_CP(c->dB2.p, hB2, (size_t)n * 8); }
  if (varbw) { GSKS_CP(c->dhi.p, hhi, (size_t)m * 8); GSKS_CP(c->dhj.p, hhj, (size_t)n * 8); }
#undef GSKS_CP
  if (e != cudaSuccess) return cuda_status(e, "stage_host copy");

  v.A = (const double *)c->dA.p; v.B = (const double *)c->dB.p;
  v.A2 = norms ? (const double *)c->dA2.p : nullptr;
  v.B2 = norms ? (const double *)c->dB2.p : nullptr;
  v.hi = varbw ? (const double *)c->dhi.p : nullptr;
  v.hj = varbw ? (const double *)c->dhj.p : nullptr;
  v.u = (double *)c->du.p; v.w = (const double *)c->dw.p;
  return GSKS_OK;
}

// Copy the evaluated u back and scatter it in target order.
int unstage_host(Ctx *c, int m, double *u, const int *umap, int nrhs)
{
  const size_t R = (size_t)std::max(nrhs, 1);
  cudaError_t e = cudaMemcpyAsync(c->hu.p, c->du.p, (size_t)m * R * 8, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_status(e, "unstage_host");
  const double *hu = (const double *)c->hu.p;
  for (int i = 0; i < m; i++)
    for (size_t r = 0; r < R; r++) u[(size_t)umap[i] * R + r] = hu[(size_t)i * R + r];
  return GSKS_OK;
}

SyncErrScope::SyncErrScope(Ctx *ctx) : c(ctx)
{
  ok = c->serr.ensure(2 * sizeof(int)) &&
       cudaMemsetAsync(c->serr.p, 0, 2 * sizeof(int), c->stream) == cudaSuccess;
  if (ok) c->cur_err = (int *)c->serr.p;
}

int SyncErrScope::finish()
{
  if (!ok) return GSKS_ERR_ALLOC;
  int flags = 0;
  cudaError_t e = cudaMemcpyAsync(&flags, c->serr.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_status(e, "device error flags");
  if (flags & DEVERR_TIMEOUT) return GSKS_ERR_TIMEOUT;
  if (flags & DEVERR_MAP_RANGE) return GSKS_ERR_MAP_RANGE;
  return GSKS_OK;
}

int read_device_errors(Ctx *c)
{
  int flags = 0;
  if (cudaMemcpyAsync(&flags, c->err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess)
    return -1;
  cudaStreamSynchronize(c->stream);
  if (flags) cudaMemsetAsync(c->err.p, 0, sizeof(int), c->stream);
  return flags;
}

KParams make_kparams(const ks_t *ker, const double *hi, const double *hj)
{
  KParams kp;
  kp.type = ker->type; kp.scal = ker->scal; kp.cons = ker->cons; kp.powe = ker->powe;
  kp.hi = hi; kp.hj = hj;
  kp.coinc = 0.0;
  kp.pmode = POW_GENERAL; kp.pint = 0;
  const double p = ker->powe;
  if (fabs(p) <= 511.0 && p == rint(p)) { kp.pmode = POW_INT; kp.pint = (int)p; }
  else if (fabs(p) <= 511.0 && 2.0 * p == rint(2.0 * p)) { kp.pmode = POW_HALF; kp.pint = (int)floor(p); }
  kp.fscal = (float)kp.scal; kp.fcons = (float)kp.cons; kp.fpowe = (float)kp.powe; kp.fpad = 0.0f;
  return kp;
}

// Relative size of the rounding noise of the assembled squared distance:
// |fl(aa - 2 x.y + bb) - d2| <= ~2k u (aa + bb) with u = 2^-53.
double coincidence_eps(int k) { return 4.0 * (double)std::max(k, 1) * 0x1p-53; }

// Enqueue one fused evaluation on stream s.  Maps may be nullptr (identity).
int enqueue_fused(Ctx *c, const ks_t *ker, int m, int n, int k,
                  double *u, const int *umap,
                  const double *XA, const double *XA2, const int *amap, int nxa,
                  const double *XB, const double *XB2, const int *bmap, int nxb,
                  const double *w, const int *wmap, const double *hi, const double *hj,
                  int precision, cudaStream_t s, bool stream_ordered_alloc, int nrhs)
{
  // nrhs > 1: interleaved u and w, each K formed once (up to 4)
  if (precision == GSKS_SPLIT_BF16X3)
    return enqueue_split(c, ker, m, n, k, u, umap, XA, XA2, amap, nxa, XB, XB2, bmap, nxb,
                         w, wmap, hi, hj, s, stream_ordered_alloc, std::max(nrhs, 1));
  if (precision != GSKS_FP64) return GSKS_ERR_PRECISION;

  Fp64Plan p = fp64_plan(m, n, k, c->num_sms);
  const size_t pbytes = p.partial_elems * sizeof(double) * (size_t)std::max(nrhs, 1);
  double *partial = nullptr;
  if (stream_ordered_alloc) {
    cudaError_t e = cudaMallocAsync((void **)&partial, pbytes, s);
    if (e != cudaSuccess) return cuda_status(e, "cudaMallocAsync");
  } else {
    if (!c->partial.ensure(pbytes)) return GSKS_ERR_ALLOC;
    partial = (double *)c->partial.p;
  }
  FusedArgs a{};
  a.m = m; a.n = n; a.k = k;
  a.XA = XA; a.XA2 = XA2; a.amap = amap;
  a.XB = XB; a.XB2 = XB2; a.bmap = bmap;
  a.w = w; a.wmap = wmap;
  a.kp = make_kparams(ker, hi, hj);
  a.kp.coinc = coincidence_eps(k);
  a.nxa = nxa; a.nxb = nxb;
  a.partial = partial;
  a.err = err_word(c);
  a.nrhs = std::max(nrhs, 1);
  int launches = fp64_launch(a, p, u, umap, s);
  if (launches < 0) return GSKS_ERR_KERNEL_TYPE;
  cudaError_t e = cudaGetLastError();
  if (stream_ordered_alloc) cudaFreeAsync(partial, s);
  if (e != cudaSuccess) return cuda_status(e, "fp64 launch");
  note_launches(launches);
  return GSKS_OK;
}

// ---- several right-hand sides -------------------------------------------
// u and w hold nrhs interleaved columns, as the reference lays them out for
// KS_RHS > 1 (u[umap[i] * KS_RHS + r], w[wmap[j] * KS_RHS + r]).  Both forms
// take up to four in one pass, each kernel value multiplied by every weight
// column.  Otherwise (more than four, or a split layout without room for the
// extra weights) right-hand side r is one evaluation with the maps
// umap[i] * nrhs + r and wmap[j] * nrhs + r, built on the device, and the
// kernel values are evaluated again for every r.
__global__ void rhs_map_kernel(int cnt, const int *__restrict__ map, int nrhs, int r, int *__restrict__ out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cnt) out[i] = (map ? map[i] : i) * nrhs + r;
}

int enqueue_rhs(Ctx *c, const ks_t *ker, int m, int n, int k, int nrhs, double *u, const int *umap,
                const double *XA, const double *XA2, const int *amap, int nxa,
                const double *XB, const double *XB2, const int *bmap, int nxb,
                const double *w, const int *wmap, const double *hi, const double *hj,
                int precision, cudaStream_t s, bool stream_ordered_alloc)
{
  if (nrhs <= 4) {   // one pass, each K formed once
    const int st = enqueue_fused(c, ker, m, n, k, u, umap, XA, XA2, amap, nxa, XB, XB2, bmap, nxb, w, wmap, hi, hj,
                                 precision, s, stream_ordered_alloc, nrhs);
    // the split form's sweep of several columns needs more shared memory than
    // some layouts leave (the Laplace table beyond k = 64): one sweep per column
    if (!(st == GSKS_ERR_TOO_LARGE && precision == GSKS_SPLIT_BF16X3 && nrhs > 1 && k <= 1024)) return st;
  }
  const size_t bytes = ((size_t)m + n) * sizeof(int);
  int *maps = nullptr;
  if (stream_ordered_alloc) {
    const cudaError_t e = cudaMallocAsync((void **)&maps, bytes, s);
    if (e != cudaSuccess) return cuda_status(e, "rhs maps");
  } else {
    if (!c->rmaps.ensure(bytes)) return GSKS_ERR_ALLOC;
    maps = (int *)c->rmaps.p;
  }
  int st = GSKS_OK, launches = 0;
  for (int r = 0; r < nrhs && st == GSKS_OK; r++) {
    rhs_map_kernel<<<(m + 255) / 256, 256, 0, s>>>(m, umap, nrhs, r, maps);
    rhs_map_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, wmap, nrhs, r, maps + m);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { st = cuda_status(e, "rhs maps"); break; }
    st = enqueue_fused(c, ker, m, n, k, u, maps, XA, XA2, amap, nxa, XB, XB2, bmap, nxb, w, maps + m, hi, hj,
                       precision, s, stream_ordered_alloc);
    launches += 2 + tl_launches;
  }
  if (stream_ordered_alloc) cudaFreeAsync(maps, s);
  tl_launches = launches;
  return st;
}

}  // namespace gsks

using namespace gsks;

// ===========================================================================
extern "C" {

int gsks_last_error(void) { return tl_status; }

const char *gsks_error_string(int code)
{
  switch (code) {
    case GSKS_OK: return "success";
    case GSKS_ERR_ARG: return "invalid argument";
    case GSKS_ERR_KERNEL_TYPE: return "illegal kernel type";
    case GSKS_ERR_BANDWIDTH: return "bandwidth vector has not been initialized";
    case GSKS_ERR_LAPLACE_K: return "laplace kernel only supports k > 2";
    case GSKS_ERR_MAP_RANGE: return "map index out of range";
    case GSKS_ERR_CUDA: return "CUDA runtime error";
    case GSKS_ERR_ALLOC: return "allocation failed";
    case GSKS_ERR_LIST: return "alist, blist and wlist must have the same sizes";
    case GSKS_ERR_PRECISION: return "unsupported precision";
    case GSKS_ERR_NO_DEVICE: return "no CUDA device";
    case GSKS_ERR_TOO_LARGE: return "size exceeds the supported maximum";
    case GSKS_ERR_TIMEOUT: return "a bounded wait in a kernel gave up; the result is incomplete";
    default: return "unknown status";
  }
}

int gsks_set_precision(int precision)
{
  if (precision != GSKS_FP64 && precision != GSKS_SPLIT_BF16X3)
    return set_status(GSKS_ERR_PRECISION, "gsks_set_precision");
  tl_precision = precision;
  return set_status(GSKS_OK, nullptr);
}

int gsks_get_precision(void) { return effective_precision(); }

int gsks_last_launch_count(void) { return tl_launches; }

int gsks_device_errors(void)
{
  Ctx *c = get_ctx();
  if (!c) return -1;
  if (cudaDeviceSynchronize() != cudaSuccess) return -1;
  return read_device_errors(c);
}

int dgsks_status(ks_t *kernel, int m, int n, int k,
                 double *u, int *umap,
                 double *XA, double *XA2, int *amap,
                 double *XB, double *XB2, int *bmap,
                 double *w, int *wmap)
{
  NvtxRange nvtx_("dgsks");
  tl_launches = 0;
  if (m < 0 || n < 0 || k < 0) return set_status(GSKS_ERR_ARG, "dgsks");
  // early return before the kernel-type switch, as frame/dgsks.c:394-397
  if (m == 0 || n == 0 || k == 0) return set_status(GSKS_OK, nullptr);
  int st = check_kernel(kernel, k);
  if (st) return set_status(st, "dgsks");
  if (!u || !umap || !XA || !amap || !XB || !bmap || !w || !wmap)
    return set_status(GSKS_ERR_ARG, "dgsks");
  Ctx *c = get_ctx();
  if (!c) return tl_status;
  const int prec = effective_precision();
  SyncErrScope se(c);

  if (is_device_pointer(XA)) {
    st = enqueue_fused(c, kernel, m, n, k, u, umap, XA, XA2, amap, -1, XB, XB2, bmap, -1,
                       w, wmap, kernel->hi, kernel->hj, prec, c->stream, false);
    if (st) return set_status(st, "dgsks");
    return set_status(se.finish(), "dgsks");
  }

  Staged v;
  st = stage_host(c, kernel, m, n, k, u, umap, XA, XA2, amap, XB, XB2, bmap, w, wmap, v);
  if (st) return set_status(st, "dgsks");
  st = enqueue_fused(c, kernel, m, n, k, v.u, nullptr, v.A, v.A2, nullptr, m, v.B, v.B2,
                     nullptr, n, v.w, nullptr, v.hi, v.hj, prec, c->stream, false);
  if (st) return set_status(st, "dgsks");
  // the flags first: a timed-out evaluation leaves u untouched
  if ((st = se.finish()) != GSKS_OK) return set_status(st, "dgsks");
  st = unstage_host(c, m, u, umap);
  return set_status(st, "dgsks");
}

void dgsks(ks_t *kernel, int m, int n, int k,
           double *u, int *umap,
           double *XA, double *XA2, int *amap,
           double *XB, double *XB2, int *bmap,
           double *w, int *wmap)
{
  (void)dgsks_status(kernel, m, n, k, u, umap, XA, XA2, amap, XB, XB2, bmap, w, wmap);
}

int gsks_dgsks_device(ks_t *kernel, int m, int n, int k,
                      double *u, const int *umap,
                      const double *XA, const double *XA2, const int *amap, int nxa,
                      const double *XB, const double *XB2, const int *bmap, int nxb,
                      const double *w, const int *wmap,
                      int precision, void *stream)
{
  NvtxRange nvtx_("gsks_dgsks_device");
  tl_launches = 0;
  if (m < 0 || n < 0 || k < 0) return set_status(GSKS_ERR_ARG, "gsks_dgsks_device");
  if (m == 0 || n == 0 || k == 0) return set_status(GSKS_OK, nullptr);
  int st = check_kernel(kernel, k);
  if (st) return set_status(st, "gsks_dgsks_device");
  if (!u || !XA || !XB || !w) return set_status(GSKS_ERR_ARG, "gsks_dgsks_device");
  if (kt_uses_norms(kernel->type) && (!XA2 || !XB2))
    return set_status(GSKS_ERR_ARG, "gsks_dgsks_device");
  Ctx *c = get_ctx();
  if (!c) return tl_status;
  st = enqueue_fused(c, kernel, m, n, k, u, umap, XA, XA2, amap, nxa, XB, XB2, bmap, nxb,
                     w, wmap, kernel->hi, kernel->hj, precision, (cudaStream_t)stream, true);
  return set_status(st, "gsks_dgsks_device");
}

int gsks_dgsks_device_rhs(ks_t *kernel, int m, int n, int k, int nrhs,
                          double *u, const int *umap,
                          const double *XA, const double *XA2, const int *amap, int nxa,
                          const double *XB, const double *XB2, const int *bmap, int nxb,
                          const double *w, const int *wmap,
                          int precision, void *stream)
{
  NvtxRange nvtx_("gsks_dgsks_device_rhs");
  tl_launches = 0;
  if (m < 0 || n < 0 || k < 0 || nrhs < 1) return set_status(GSKS_ERR_ARG, "gsks_dgsks_device_rhs");
  if (m == 0 || n == 0 || k == 0) return set_status(GSKS_OK, nullptr);
  int st = check_kernel(kernel, k);
  if (st) return set_status(st, "gsks_dgsks_device_rhs");
  if (!u || !XA || !XB || !w) return set_status(GSKS_ERR_ARG, "gsks_dgsks_device_rhs");
  if (kt_uses_norms(kernel->type) && (!XA2 || !XB2))
    return set_status(GSKS_ERR_ARG, "gsks_dgsks_device_rhs");
  Ctx *c = get_ctx();
  if (!c) return tl_status;
  st = enqueue_rhs(c, kernel, m, n, k, nrhs, u, umap, XA, XA2, amap, nxa, XB, XB2, bmap, nxb,
                   w, wmap, kernel->hi, kernel->hj, precision, (cudaStream_t)stream, true);
  return set_status(st, "gsks_dgsks_device_rhs");
}

int dgsks_rhs(ks_t *kernel, int m, int n, int k, int nrhs,
              double *u, int *umap,
              double *XA, double *XA2, int *amap,
              double *XB, double *XB2, int *bmap,
              double *w, int *wmap)
{
  NvtxRange nvtx_("dgsks_rhs");
  tl_launches = 0;
  if (m < 0 || n < 0 || k < 0 || nrhs < 1) return set_status(GSKS_ERR_ARG, "dgsks_rhs");
  if (m == 0 || n == 0 || k == 0) return set_status(GSKS_OK, nullptr);
  int st = check_kernel(kernel, k);
  if (st) return set_status(st, "dgsks_rhs");
  if (!u || !umap || !XA || !amap || !XB || !bmap || !w || !wmap) return set_status(GSKS_ERR_ARG, "dgsks_rhs");
  Ctx *c = get_ctx();
  if (!c) return tl_status;
  const int prec = effective_precision();
  SyncErrScope se(c);
  if (is_device_pointer(XA)) {
    st = enqueue_rhs(c, kernel, m, n, k, nrhs, u, umap, XA, XA2, amap, -1, XB, XB2, bmap, -1, w, wmap,
                     kernel->hi, kernel->hj, prec, c->stream, false);
    if (st) return set_status(st, "dgsks_rhs");
    return set_status(se.finish(), "dgsks_rhs");
  }
  Staged v;
  st = stage_host(c, kernel, m, n, k, u, umap, XA, XA2, amap, XB, XB2, bmap, w, wmap, v, nrhs);
  if (st) return set_status(st, "dgsks_rhs");
  st = enqueue_rhs(c, kernel, m, n, k, nrhs, v.u, nullptr, v.A, v.A2, nullptr, m, v.B, v.B2, nullptr, n, v.w,
                   nullptr, v.hi, v.hj, prec, c->stream, false);
  if (st) return set_status(st, "dgsks_rhs");
  if ((st = se.finish()) != GSKS_OK) return set_status(st, "dgsks_rhs");
  st = unstage_host(c, m, u, umap, nrhs);
  return set_status(st, "dgsks_rhs");
}

int gsks_norms_device(int N, int k, const double *X, double *X2, void *stream)
{
  if (N < 0 || k < 0 || (N > 0 && (!X || !X2))) return set_status(GSKS_ERR_ARG, "gsks_norms_device");
  cudaError_t e = norms_launch(N, k, X, X2, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_status(e, "gsks_norms_device");
  tl_launches = N > 0 ? 1 : 0;
  return set_status(GSKS_OK, nullptr);
}

double *ks_malloc_aligned(int m, int n, int size)
{
  void *ptr = nullptr;
  size_t bytes = (size_t)(m > 0 ? m : 0) * (size_t)(n > 0 ? n : 0) * (size_t)(size > 0 ? size : 0);
  if (bytes == 0) bytes = 64;
  if (posix_memalign(&ptr, 64, bytes) != 0) {
    set_status(GSKS_ERR_ALLOC, "ks_malloc_aligned");
    return nullptr;
  }
  set_status(GSKS_OK, nullptr);
  return (double *)ptr;
}

static ks_t wrapper_kernel(int type, double scal, double cons, double powe, double *h)
{
  ks_t ker;
  memset(&ker, 0, sizeof(ker));
  ker.type = (ks_type)type;
  ker.scal = scal; ker.cons = cons; ker.powe = powe;
  ker.hi = h; ker.hj = h; ker.h = h;
  return ker;
}

void dgsks_wrapper(int m, int n, int k, double *u, int *umap,
                   double *XA, double *XA2, int *amap,
                   double *XB, double *XB2, int *bmap,
                   double *w, int *wmap,
                   int type, double scal, double cons, double powe, double *h)
{
  ks_t ker = wrapper_kernel(type, scal, cons, powe, h);
  dgsks(&ker, m, n, k, u, umap, XA, XA2, amap, XB, XB2, bmap, w, wmap);
}

void dgsks_ref_wrapper(int m, int n, int k, double *u, int *umap,
                       double *XA, double *XA2, int *amap,
                       double *XB, double *XB2, int *bmap,
                       double *w, int *wmap,
                       int type, double scal, double cons, double powe, double *h)
{
  ks_t ker = wrapper_kernel(type, scal, cons, powe, h);
  dgsks_ref(&ker, m, n, k, u, umap, XA, XA2, amap, XB, XB2, bmap, w, wmap);
}

}  // extern "C"
