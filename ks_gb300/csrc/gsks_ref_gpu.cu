// gsks_ref_gpu.cu -- dgsks_ref(): the unfused GEMM + kernel + GEMV evaluation.
//
// The reference's dgsks_ref (frame/dgsks_ref.c:94-535) collects the points,
// forms C = rank_k_scale * A^T B, applies the kernel function element-wise,
// and computes u += C w.  This file does the same on the GPU in three
// separate FP64 passes over a materialised block of C (row blocks sized to a
// bounded buffer), independently of the fused kernel in gsks_fp64.cu, so the
// two can cross-check each other.  The per-element operation order is the
// reference's; unlike the fused kernel, no clamp of the squared distance.
#include "gsks.h"
#include "gsks_internal.cuh"
#include "gsks_host.h"
#include <algorithm>

namespace gsks {
namespace {

__device__ __forceinline__ double ref_kvalue(int type, double c, double aa, double bb,
                                             double hi, double hj, const KParams &kp)
{
  switch (type) {
    case KS_GAUSSIAN: c += aa; c += bb; c *= kp.scal; return exp(c);
    case KS_GAUSSIAN_VAR_BANDWIDTH: c += aa; c += bb; c *= -0.5; c *= hi; c *= hj; return exp(c);
    case KS_POLYNOMIAL:
      c *= kp.scal; c += kp.cons;
      if (kp.powe == 2.0) return c * c;
      if (kp.powe == 4.0) { c = c * c; return c * c; }
      return pow(c, kp.powe);
    case KS_LAPLACE:
      c += aa; c += bb;
      if (c < fmax(1e-15, kp.coinc * (aa + bb))) c = 1.79e308;
      return pow(c, kp.powe) * kp.scal;
    case KS_TANH: c *= kp.scal; c += kp.cons; return tanh(c);
    case KS_QUARTIC:
      c += aa; c += bb;
      if (c < 1.0) { c = 1.0 - c; return (15.0 / 16.0) * c * c; }
      return 0.0;
    case KS_MULTIQUADRATIC: c += aa; c += bb; c += kp.cons; return c;
    default:  // KS_EPANECHNIKOV
      c += aa; c += bb;
      if (c < 1.0) { c = 1.0 - c; return 0.75 * c; }
      return 0.0;
  }
}

// C[j*mb + r] = rks * <A[row(i0+r)], B[row(j)]>, summed in coordinate order.
__global__ void ref_gemm(int mb, int i0, int n, int k, double rks,
                         const double *__restrict__ XA, const int *__restrict__ amap,
                         const double *__restrict__ XB, const int *__restrict__ bmap,
                         double *__restrict__ C)
{
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (r >= mb || j >= n) return;
  const int pa = amap ? amap[i0 + r] : i0 + r;
  const int pb = bmap ? bmap[j] : j;
  const double *a = XA + (size_t)pa * k, *b = XB + (size_t)pb * k;
  double s = 0.0;
  for (int p = 0; p < k; p++) s += a[p] * b[p];
  C[(size_t)j * mb + r] = s * rks;
}

__global__ void ref_apply(int mb, int i0, int n, KParams kp,
                          const double *__restrict__ XA2, const int *__restrict__ amap,
                          const double *__restrict__ XB2, const int *__restrict__ bmap,
                          double *__restrict__ C)
{
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)mb * n) return;
  const int r = (int)(e % mb), j = (int)(e / mb);
  const int pa = amap ? amap[i0 + r] : i0 + r;
  const int pb = bmap ? bmap[j] : j;
  const bool norms = kt_uses_norms(kp.type);
  const double aa = norms ? XA2[pa] : 0.0, bb = norms ? XB2[pb] : 0.0;
  const bool vb = kp.type == KS_GAUSSIAN_VAR_BANDWIDTH;
  C[e] = ref_kvalue(kp.type, C[e], aa, bb, vb ? kp.hi[pa] : 0.0, vb ? kp.hj[pb] : 0.0, kp);
}

// us = u[umap[i]] + sum_j C[i,j] w[wmap[j]] in source order; then scatter.
__global__ void ref_gemv(int mb, int i0, int n, const double *__restrict__ C,
                         const double *__restrict__ w, const int *__restrict__ wmap,
                         double *__restrict__ u, const int *__restrict__ umap)
{
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= mb) return;
  const int pu = umap ? umap[i0 + r] : i0 + r;
  double s = u[pu];
  for (int j = 0; j < n; j++) s += C[(size_t)j * mb + r] * w[wmap ? wmap[j] : j];
  u[pu] = s;
}

int enqueue_ref(Ctx *c, const ks_t *ker, int m, int n, int k, double *u, const int *umap,
                const double *XA, const double *XA2, const int *amap,
                const double *XB, const double *XB2, const int *bmap,
                const double *w, const int *wmap, const double *hi, const double *hj,
                cudaStream_t s)
{
  const double rks = (ker->type == KS_POLYNOMIAL || ker->type == KS_TANH) ? 1.0 : -2.0;
  const size_t cap_elems = (size_t)32 << 20;  // 256 MiB block of C
  const int mb_max = (int)std::max<size_t>(1, std::min<size_t>((size_t)m, cap_elems / (size_t)n));
  if (!c->dwork.ensure((size_t)mb_max * n * sizeof(double))) return GSKS_ERR_ALLOC;
  double *C = (double *)c->dwork.p;
  KParams kp = make_kparams(ker, hi, hj);
  kp.coinc = coincidence_eps(k);
  int launches = 0;
  for (int i0 = 0; i0 < m; i0 += mb_max) {
    const int mb = std::min(mb_max, m - i0);
    dim3 blk(32, 8), grd((mb + 31) / 32, (n + 7) / 8);
    ref_gemm<<<grd, blk, 0, s>>>(mb, i0, n, k, rks, XA, amap, XB, bmap, C);
    const size_t tot = (size_t)mb * n;
    ref_apply<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(mb, i0, n, kp, XA2, amap, XB2, bmap, C);
    ref_gemv<<<(mb + 127) / 128, 128, 0, s>>>(mb, i0, n, C, w, wmap, u, umap);
    launches += 3;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e, "dgsks_ref launch");
  note_launches(launches);
  return GSKS_OK;
}

}  // namespace
}  // namespace gsks

using namespace gsks;

extern "C" void dgsks_ref(ks_t *kernel, int m, int n, int k,
                          double *u, int *umap,
                          double *XA, double *XA2, int *amap,
                          double *XB, double *XB2, int *bmap,
                          double *w, int *wmap)
{
  NvtxRange nvtx_("dgsks_ref");
  note_launches(0);
  if (m < 0 || n < 0 || k < 0) { set_status(GSKS_ERR_ARG, "dgsks_ref"); return; }
  if (m == 0 || n == 0 || k == 0) { set_status(GSKS_OK, nullptr); return; }
  int st = check_kernel(kernel, k);
  if (st) { set_status(st, "dgsks_ref"); return; }
  if (!u || !umap || !XA || !amap || !XB || !bmap || !w || !wmap) {
    set_status(GSKS_ERR_ARG, "dgsks_ref");
    return;
  }
  Ctx *c = get_ctx();
  if (!c) return;
  if (is_device_pointer(XA)) {
    st = enqueue_ref(c, kernel, m, n, k, u, umap, XA, XA2, amap, XB, XB2, bmap, w, wmap,
                     kernel->hi, kernel->hj, c->stream);
    if (!st) {
      cudaError_t e = cudaStreamSynchronize(c->stream);
      if (e != cudaSuccess) st = cuda_status(e, "dgsks_ref");
    }
    set_status(st, "dgsks_ref");
    return;
  }
  Staged v;
  st = stage_host(c, kernel, m, n, k, u, umap, XA, XA2, amap, XB, XB2, bmap, w, wmap, v);
  if (!st)
    st = enqueue_ref(c, kernel, m, n, k, v.u, nullptr, v.A, v.A2, nullptr, v.B, v.B2, nullptr,
                     v.w, nullptr, v.hi, v.hj, c->stream);
  if (!st) st = unstage_host(c, m, u, umap);
  set_status(st, "dgsks_ref");
}
