// gsks_fp64_item.cuh -- one FP64 work item: a target tile x a source chunk.
//
// Shared by the single-call kernel (gsks_fp64.cu) and the batched persistent
// kernel (gsks_list.cu).  256 threads as 16 x 16; thread (tx, ty) owns rows
// ty + 16 r and columns tx + 16 c (r, c < 4) of each 64 x 64 pair tile, so the
// A reads of a warp are two broadcast addresses and the B reads one 128-byte
// line.  Points are gathered through the maps into k-chunks of shared memory
// (coordinates beyond k are zero and add nothing to the inner product).
#pragma once
#include "gsks_internal.cuh"

namespace gsks {

namespace fp64cfg {
constexpr int BM = 64;    // targets per tile
constexpr int BN = 64;    // sources per tile
constexpr int KC = 16;    // k chunk staged in shared memory
constexpr int NT = 256;   // threads per CTA
constexpr int TM = 4, TN = 4;
constexpr int RMAX = 4;   // right-hand sides evaluated together
}  // namespace fp64cfg

struct Fp64Smem {
  double As[fp64cfg::KC][fp64cfg::BM + 1];
  double Bs[fp64cfg::KC][fp64cfg::BN + 1];
  double aa[fp64cfg::BM], hi[fp64cfg::BM];
  double bb[fp64cfg::BN], hj[fp64cfg::BN], w[fp64cfg::RMAX][fp64cfg::BN];
  long long arow[fp64cfg::BM], brow[fp64cfg::BN];
};

// Rows a0 .. a0+rows-1 of the call (positions in amap), sources b0 ..
// b0+cols-1 (positions in bmap / wmap).  out[r] = sum_j K(r, j) w(j) for
// r < rows.  With R right-hand sides (w[wmap[j] R + q]) each K(r, j) is
// formed once and out[q rstride + r] receives right-hand side q.  Must be
// called by all NT threads of the block.
template <int KT, int R = 1>
__device__ __forceinline__ void fp64_item(const FusedArgs &a, const KParams &kp, Fp64Smem &sm,
                                          int a0, int rows, int b0, int cols, double *out)
{
  using namespace fp64cfg;
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int k = a.k;

  __syncthreads();  // the previous item is done with shared memory
  if (tid < BM) {
    long long off = 0;
    double aav = 0.0, hiv = 0.0;
    if (tid < rows) {
      int p = a.amap ? __ldg(a.amap + a0 + tid) : a0 + tid;
      if (a.nxa >= 0 && (p < 0 || p >= a.nxa)) { atomicOr(a.err, DEVERR_MAP_RANGE); p = 0; }
      off = (long long)p * k;
      if (kt_uses_norms(KT)) aav = __ldg(a.XA2 + p);
      if (KT == KS_GAUSSIAN_VAR_BANDWIDTH) hiv = __ldg(kp.hi + p);
    }
    sm.arow[tid] = off; sm.aa[tid] = aav; sm.hi[tid] = hiv;
  }

  double racc[TM][R];
#pragma unroll
  for (int r = 0; r < TM; r++)
#pragma unroll
    for (int q = 0; q < R; q++) racc[r][q] = 0.0;

  for (int j0 = 0; j0 < cols; j0 += BN) {
    const int ncols = min(BN, cols - j0);
    __syncthreads();  // the previous source tile's metadata is consumed
    if (tid < BN) {
      long long off = 0;
      double bbv = 0.0, hjv = 0.0, wv[R];
#pragma unroll
      for (int q = 0; q < R; q++) wv[q] = 0.0;
      if (tid < ncols) {
        const int j = b0 + j0 + tid;
        int p = a.bmap ? __ldg(a.bmap + j) : j;
        if (a.nxb >= 0 && (p < 0 || p >= a.nxb)) { atomicOr(a.err, DEVERR_MAP_RANGE); p = 0; }
        off = (long long)p * k;
        if (kt_uses_norms(KT)) bbv = __ldg(a.XB2 + p);
        if (KT == KS_GAUSSIAN_VAR_BANDWIDTH) hjv = __ldg(kp.hj + p);
        const size_t wj = (size_t)(a.wmap ? __ldg(a.wmap + j) : j) * R;
#pragma unroll
        for (int q = 0; q < R; q++) wv[q] = __ldg(a.w + wj + q);
      }
      sm.brow[tid] = off; sm.bb[tid] = bbv; sm.hj[tid] = hjv;
#pragma unroll
      for (int q = 0; q < R; q++) sm.w[q][tid] = wv[q];
    }

    double acc[TM][TN];
#pragma unroll
    for (int r = 0; r < TM; r++)
#pragma unroll
      for (int c = 0; c < TN; c++) acc[r][c] = 0.0;

    for (int k0 = 0; k0 < k; k0 += KC) {
      const int kc = min(KC, k - k0);
      __syncthreads();  // metadata visible; previous chunk consumed
      for (int e = tid; e < BM * KC; e += NT) {
        const int r = e / KC, kk = e - r * KC;
        double v = 0.0;
        if (r < rows && kk < kc) v = __ldg(a.XA + sm.arow[r] + k0 + kk);
        sm.As[kk][r] = v;
      }
      for (int e = tid; e < BN * KC; e += NT) {
        const int c = e / KC, kk = e - c * KC;
        double v = 0.0;
        if (c < ncols && kk < kc) v = __ldg(a.XB + sm.brow[c] + k0 + kk);
        sm.Bs[kk][c] = v;
      }
      __syncthreads();
      if (kc == KC) {
#pragma unroll
        for (int kk = 0; kk < KC; kk++) {
          double av[TM], bv[TN];
#pragma unroll
          for (int r = 0; r < TM; r++) av[r] = sm.As[kk][ty + 16 * r];
#pragma unroll
          for (int c = 0; c < TN; c++) bv[c] = sm.Bs[kk][tx + 16 * c];
#pragma unroll
          for (int r = 0; r < TM; r++)
#pragma unroll
            for (int c = 0; c < TN; c++) acc[r][c] = fma(av[r], bv[c], acc[r][c]);
        }
      } else {
        for (int kk = 0; kk < kc; kk++) {
          double av[TM], bv[TN];
#pragma unroll
          for (int r = 0; r < TM; r++) av[r] = sm.As[kk][ty + 16 * r];
#pragma unroll
          for (int c = 0; c < TN; c++) bv[c] = sm.Bs[kk][tx + 16 * c];
#pragma unroll
          for (int r = 0; r < TM; r++)
#pragma unroll
            for (int c = 0; c < TN; c++) acc[r][c] = fma(av[r], bv[c], acc[r][c]);
        }
      }
    }

    // Epilogue: kernel function and weighted sum, in registers.
#pragma unroll
    for (int r = 0; r < TM; r++) {
      const int rr = ty + 16 * r;
      const double aav = sm.aa[rr], hiv = sm.hi[rr];
      double s[R];
#pragma unroll
      for (int q = 0; q < R; q++) s[q] = 0.0;
#pragma unroll
      for (int c = 0; c < TN; c++) {
        const int cc = tx + 16 * c;
        if (cc < ncols) {
          const double kv = kfun64<KT>(acc[r][c], aav, sm.bb[cc], hiv, sm.hj[cc], kp);
#pragma unroll
          for (int q = 0; q < R; q++) s[q] = fma(kv, sm.w[q][cc], s[q]);
        }
      }
#pragma unroll
      for (int q = 0; q < R; q++) racc[r][q] += s[q];
    }
  }

  // Row sums: the 16 threads of a half-warp share the same rows.
#pragma unroll
  for (int r = 0; r < TM; r++) {
#pragma unroll
    for (int q = 0; q < R; q++)
#pragma unroll
      for (int off = 8; off > 0; off >>= 1)
        racc[r][q] += __shfl_xor_sync(0xffffffffu, racc[r][q], off);
  }
  if (tx == 0) {
#pragma unroll
    for (int r = 0; r < TM; r++) {
      const int rr = ty + 16 * r;
      if (rr < rows) {
#pragma unroll
        for (int q = 0; q < R; q++) out[(size_t)q * a.rstride + rr] = racc[r][q];
      }
    }
  }
}

}  // namespace gsks
