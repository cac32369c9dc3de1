// gsks_single.cu -- sgsks: the kernel summation on FP32 arrays.
//
// The reference declares no single-precision entry (its single-precision
// micro-kernels are stubs).  Here sgsks gathers the rows the maps name into
// FP64 staging, converting as it goes: host arrays into the pinned buffers,
// device arrays with a gather kernel.  The squared norms are recomputed in
// FP64 from the converted coordinates, so they match them exactly.  The
// evaluation is then dgsks's, in the precision the switch selects, and
// u[umap[i]] is written back rounded to FP32.
#include "gsks.h"
#include "gsks_internal.cuh"
#include "gsks_host.h"

#include <algorithm>
#include <cstring>
#include <omp.h>

namespace gsks {
namespace {

// rows i < cnt: out[i k + p] = X[map[i] k + p], out2[i] = |out_i|^2 (FP64),
// outh[i] = h[map[i]] (when h), outv[i] = val[vmap[i]]; a negative index sets *bad.
__global__ void gather_rows_f32(int cnt, int k, const float *__restrict__ X, const int *__restrict__ map,
                                const double *__restrict__ h, const float *__restrict__ val,
                                const int *__restrict__ vmap, double *__restrict__ out, double *__restrict__ out2,
                                double *__restrict__ outh, double *__restrict__ outv, int *bad)
{
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < cnt; i += warps) {
    const int p = map[i], q = vmap[i];
    if (p < 0 || q < 0) {
      if (lane == 0) atomicOr(bad, 1);
      continue;
    }
    double s = 0.0;
    for (int c = lane; c < k; c += 32) {
      const double x = (double)X[(size_t)p * k + c];
      out[(size_t)i * k + c] = x;
      s = fma(x, x, s);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
      out2[i] = s;
      if (h) outh[i] = h[p];
      outv[i] = (double)val[q];
    }
  }
}

__global__ void scatter_u_f32(int m, const double *__restrict__ ud, const int *__restrict__ umap,
                              float *__restrict__ u)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) u[umap[i]] = (float)ud[i];
}

}  // namespace
}  // namespace gsks

using namespace gsks;

int sgsks_status(ks_t *kernel, int m, int n, int k,
                 float *u, int *umap,
                 float *XA, float *XA2, int *amap,
                 float *XB, float *XB2, int *bmap,
                 float *w, int *wmap)
{
  NvtxRange nvtx_("sgsks");
  (void)XA2; (void)XB2;   // recomputed in FP64 from the converted coordinates
  if (m < 0 || n < 0 || k < 0) return set_status(GSKS_ERR_ARG, "sgsks");
  if (m == 0 || n == 0 || k == 0) return set_status(GSKS_OK, nullptr);
  int st = check_kernel(kernel, k);
  if (st) return set_status(st, "sgsks");
  if (!u || !umap || !XA || !amap || !XB || !bmap || !w || !wmap) return set_status(GSKS_ERR_ARG, "sgsks");
  Ctx *c = get_ctx();
  if (!c) return gsks_last_error();
  const bool varbw = kernel->type == KS_GAUSSIAN_VAR_BANDWIDTH;
  const size_t mk = (size_t)m * k, nk = (size_t)n * k;
  bool ok = c->dA.ensure(mk * 8) && c->dB.ensure(nk * 8) && c->dA2.ensure((size_t)m * 8) &&
            c->dB2.ensure((size_t)n * 8) && c->du.ensure((size_t)m * 8) && c->dw.ensure((size_t)n * 8);
  if (ok && varbw) ok = c->dhi.ensure((size_t)m * 8) && c->dhj.ensure((size_t)n * 8);
  if (!ok) return set_status(GSKS_ERR_ALLOC, "sgsks");
  double *dA = (double *)c->dA.p, *dB = (double *)c->dB.p, *dA2 = (double *)c->dA2.p, *dB2 = (double *)c->dB2.p;
  double *du = (double *)c->du.p, *dw = (double *)c->dw.p;
  double *dhi = varbw ? (double *)c->dhi.p : nullptr, *dhj = varbw ? (double *)c->dhj.p : nullptr;
  cudaStream_t s = c->stream;
  const int prec = effective_precision();
  SyncErrScope se(c);   // clears both words of the synchronous calls' flags
  if (!se.ok) return set_status(GSKS_ERR_ALLOC, "sgsks");

  if (is_device_pointer(XA)) {
    int *bad = (int *)c->serr.p + 1;   // the gather's map-check flag
    cudaError_t e = cudaSuccess;
    const int blocks = std::max(1, std::min(1024, (std::max(m, n) + 7) / 8));
    gather_rows_f32<<<blocks, 256, 0, s>>>(m, k, XA, amap, varbw ? kernel->hi : nullptr, u, umap, dA, dA2, dhi, du,
                                           bad);
    gather_rows_f32<<<blocks, 256, 0, s>>>(n, k, XB, bmap, varbw ? kernel->hj : nullptr, w, wmap, dB, dB2, dhj, dw,
                                           bad);
    int hbad = 0;
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e, "sgsks gather");
    if (hbad) return set_status(GSKS_ERR_MAP_RANGE, "sgsks");
    st = enqueue_fused(c, kernel, m, n, k, du, nullptr, dA, dA2, nullptr, m, dB, dB2, nullptr, n, dw, nullptr, dhi,
                       dhj, prec, s, false);
    if (st) return set_status(st, "sgsks");
    if ((st = se.finish()) != GSKS_OK) return set_status(st, "sgsks");   // a timed-out evaluation leaves u as it was
    scatter_u_f32<<<(m + 255) / 256, 256, 0, s>>>(m, du, umap, u);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e, "sgsks");
    return set_status(GSKS_OK, nullptr);
  }

  // host arrays: convert while gathering into the pinned buffers
  ok = c->hA.ensure(mk * 8) && c->hB.ensure(nk * 8) && c->hA2.ensure((size_t)m * 8) &&
       c->hB2.ensure((size_t)n * 8) && c->hu.ensure((size_t)m * 8) && c->hw.ensure((size_t)n * 8);
  if (ok && varbw) ok = c->hhi.ensure((size_t)m * 8) && c->hhj.ensure((size_t)n * 8);
  if (!ok) return set_status(GSKS_ERR_ALLOC, "sgsks");
  int bad = 0;
  for (int side = 0; side < 2; side++) {
    const int cnt = side ? n : m;
    const int *map = side ? bmap : amap, *vmap = side ? wmap : umap;
    const float *X = side ? XB : XA, *val = side ? w : u;
    const double *hv = varbw ? (side ? kernel->hj : kernel->hi) : nullptr;
    double *hX = (double *)(side ? c->hB.p : c->hA.p), *hX2 = (double *)(side ? c->hB2.p : c->hA2.p);
    double *hh = (double *)(side ? c->hhj.p : c->hhi.p), *hval = (double *)(side ? c->hw.p : c->hu.p);
#pragma omp parallel for schedule(static) if (cnt * (size_t)k > 65536)
    for (int i = 0; i < cnt; i++) {
      const int p = map[i], q = vmap[i];
      if (p < 0 || q < 0) {
#pragma omp atomic write
        bad = 1;
        continue;
      }
      double sq = 0.0;
      for (int c2 = 0; c2 < k; c2++) {
        const double x = (double)X[(size_t)p * k + c2];
        hX[(size_t)i * k + c2] = x;
        sq += x * x;
      }
      hX2[i] = sq;
      if (hv) hh[i] = hv[p];
      hval[i] = (double)val[q];
    }
  }
  if (bad) return set_status(GSKS_ERR_MAP_RANGE, "sgsks");
  cudaError_t e = cudaSuccess;
#define GSKS_CP(dst, src, bytes) \
  if (e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s)
  GSKS_CP(dA, c->hA.p, mk * 8);
  GSKS_CP(dB, c->hB.p, nk * 8);
  GSKS_CP(dA2, c->hA2.p, (size_t)m * 8);
  GSKS_CP(dB2, c->hB2.p, (size_t)n * 8);
  GSKS_CP(du, c->hu.p, (size_t)m * 8);
  GSKS_CP(dw, c->hw.p, (size_t)n * 8);
  if (varbw) { GSKS_CP(dhi, c->hhi.p, (size_t)m * 8); GSKS_CP(dhj, c->hhj.p, (size_t)n * 8); }
#undef GSKS_CP
  if (e != cudaSuccess) return cuda_status(e, "sgsks copy");
  st = enqueue_fused(c, kernel, m, n, k, du, nullptr, dA, dA2, nullptr, m, dB, dB2, nullptr, n, dw, nullptr, dhi,
                     dhj, prec, s, false);
  if (st) return set_status(st, "sgsks");
  if ((st = se.finish()) != GSKS_OK) return set_status(st, "sgsks");
  e = cudaMemcpyAsync(c->hu.p, du, (size_t)m * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e, "sgsks");
  const double *hu = (const double *)c->hu.p;
  for (int i = 0; i < m; i++) u[umap[i]] = (float)hu[i];
  return set_status(GSKS_OK, nullptr);
}

void sgsks(ks_t *kernel, int m, int n, int k,
           float *u, int *umap,
           float *XA, float *XA2, int *amap,
           float *XB, float *XB2, int *bmap,
           float *w, int *wmap)
{
  (void)sgsks_status(kernel, m, n, k, u, umap, XA, XA2, amap, XB, XB2, bmap, w, wmap);
}
