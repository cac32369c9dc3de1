// gsks_fp64.cu -- plain FP64 form of the fused kernel summation (sm_103a).
//
// A work item is (a tile of up to BM targets gathered through amap) x (a
// chunk of sources gathered through bmap).  It forms the rank-k inner
// products with DFMA in 4x4 register tiles, assembles the kernel value in
// registers and folds K * w into per-row sums, so the kernel matrix never
// leaves registers.  Each item writes one partial sum per row; a second pass
// adds the partials of a row in a fixed order into u (deterministic, no
// floating-point atomics).
//
// Replaces the reference's BLIS loop nest and x86 micro-kernels:
//   frame/dgsks.c:367-776 (jc/pc/ic loops, gather-packing :70-213),
//   micro_kernel/x86_64/sandybridge/ks_*_int_d8x4.c (rank-k + kernel + sum).
// The batched form (gsks_list.cu) runs the same item over a size-sorted queue
// of (task, target tile, source chunk) items in one persistent launch.
//
// GB300 note: FP64 issues at a small fraction of the FP32 rate on this part,
// so the design keeps the FP64 instruction count per pair at k + O(1) and
// leaves every other pipe (loads, shared memory, integer) lightly used.
#include "gsks_internal.cuh"
#include "gsks_fp64_item.cuh"
#include <algorithm>

namespace gsks {

namespace {

template <int KT, int R>
__global__ void __launch_bounds__(fp64cfg::NT, 2) fp64_tiles(FusedArgs a)
{
  __shared__ Fp64Smem sm;
  const int items = a.ntm * a.nsc;
  for (int item = blockIdx.x; item < items; item += gridDim.x) {
    const int ti = item % a.ntm;
    const int sc = item / a.ntm;
    const int i0 = ti * fp64cfg::BM;
    const int j0 = sc * a.chunk;
    fp64_item<KT, R>(a, a.kp, sm, i0, min(fp64cfg::BM, a.m - i0), j0, min(a.chunk, a.n - j0),
                     a.partial + (size_t)sc * a.ldp + i0);
  }
}

// u[umap[i] R + q] += sum over chunks of the chunk partials of right-hand
// side q, in chunk order.
__global__ void fp64_reduce(int m, int nsc, int ldp, int R, long long rstride, const double *__restrict__ partial,
                            double *__restrict__ u, const int *__restrict__ umap)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const size_t p = (size_t)(umap ? umap[i] : i) * R;
  for (int q = 0; q < R; q++) {
    double s = 0.0;
    for (int c = 0; c < nsc; c++) s += partial[(size_t)q * rstride + (size_t)c * ldp + i];
    u[p + q] += s;
  }
}

// One warp per point: X2[p] = sum_q X[p*k+q]^2.
__global__ void norms_kernel(int N, int k, const double *__restrict__ X, double *__restrict__ X2)
{
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= N) return;
  const double *x = X + (size_t)warp * k;
  double s = 0.0;
  for (int q = lane; q < k; q += 32) s = fma(x[q], x[q], s);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (lane == 0) X2[warp] = s;
}

template <int KT>
void launch_tiles(const FusedArgs &a, int grid, cudaStream_t s)
{
  switch (a.nrhs) {
    case 2: fp64_tiles<KT, 2><<<grid, fp64cfg::NT, 0, s>>>(a); break;
    case 3: fp64_tiles<KT, 3><<<grid, fp64cfg::NT, 0, s>>>(a); break;
    case 4: fp64_tiles<KT, 4><<<grid, fp64cfg::NT, 0, s>>>(a); break;
    default: fp64_tiles<KT, 1><<<grid, fp64cfg::NT, 0, s>>>(a); break;
  }
}
}  // namespace

Fp64Plan fp64_plan(int m, int n, int k, int num_sms)
{
  (void)k;
  using namespace fp64cfg;
  Fp64Plan p{};
  p.ntm = (m + BM - 1) / BM;
  const int slots = std::max(1, num_sms) * 2;
  const long long want = (long long)slots * 16;
  const int max_nsc = (n + BN - 1) / BN;
  long long nsc = (want + p.ntm - 1) / p.ntm;
  nsc = std::max<long long>(1, std::min<long long>(nsc, max_nsc));
  int chunk = (int)((n + nsc - 1) / nsc);
  chunk = ((chunk + BN - 1) / BN) * BN;
  p.chunk = chunk;
  p.nsc = (n + chunk - 1) / chunk;
  const long long items = (long long)p.ntm * p.nsc;
  p.grid = (int)std::min<long long>(items, slots);
  p.ldp = p.ntm * BM;
  p.partial_elems = (size_t)p.nsc * p.ldp;
  return p;
}

int fp64_launch(const FusedArgs &a0, const Fp64Plan &p, double *u, const int *umap,
                cudaStream_t s)
{
  FusedArgs a = a0;
  a.ntm = p.ntm; a.nsc = p.nsc; a.chunk = p.chunk; a.ldp = p.ldp;
  if (a.nrhs < 1 || a.nrhs > fp64cfg::RMAX) a.nrhs = 1;
  a.rstride = (long long)p.nsc * p.ldp;
  switch (a.kp.type) {
    case KS_GAUSSIAN: launch_tiles<KS_GAUSSIAN>(a, p.grid, s); break;
    case KS_POLYNOMIAL: launch_tiles<KS_POLYNOMIAL>(a, p.grid, s); break;
    case KS_LAPLACE: launch_tiles<KS_LAPLACE>(a, p.grid, s); break;
    case KS_GAUSSIAN_VAR_BANDWIDTH: launch_tiles<KS_GAUSSIAN_VAR_BANDWIDTH>(a, p.grid, s); break;
    case KS_TANH: launch_tiles<KS_TANH>(a, p.grid, s); break;
    case KS_QUARTIC: launch_tiles<KS_QUARTIC>(a, p.grid, s); break;
    case KS_MULTIQUADRATIC: launch_tiles<KS_MULTIQUADRATIC>(a, p.grid, s); break;
    case KS_EPANECHNIKOV: launch_tiles<KS_EPANECHNIKOV>(a, p.grid, s); break;
    default: return -1;
  }
  fp64_reduce<<<(a.m + 255) / 256, 256, 0, s>>>(a.m, p.nsc, p.ldp, a.nrhs, a.rstride, a.partial, u, umap);
  return 2;
}

cudaError_t norms_launch(int N, int k, const double *X, double *X2, cudaStream_t s)
{
  if (N <= 0) return cudaSuccess;
  const int threads = 256;
  const long long blocks = ((long long)N * 32 + threads - 1) / threads;
  norms_kernel<<<(unsigned)blocks, threads, 0, s>>>(N, k, X, X2);
  return cudaGetLastError();
}

}  // namespace gsks
