// gsks_split.cu -- split-precision tensor-core form of the kernel summation.
//
// The rank-k inner products run on the 5th-generation tensor cores
// (tcgen05.mma, accumulators in TMEM); the kernel function runs in FP32; FP64
// is kept for the squared norms, for the distance of pairs flagged by an
// error bound, and for the per-target accumulation of u.
//
// Operand split (per call, in FP64, in split_pack):
//   x'' = alpha (x - c)            c: centre of the call's bounding box (distance
//                                  kernels; 0 for polynomial / tanh); alpha folds
//                                  the Gaussian scale: alpha^2 = -scal log2(e)
//   x'' / sigma * 2^7 = a1 + a2 + a3 with a1 = rint(.) an integer |a1| <= 128
//                                  and a2, a3 the two FP16 roundings of the rest
//                                  (sigma: a power of two >= max |x''|)
// so each coordinate carries ~30 significant bits.  Products a1*b1 are exact
// 14-bit integers; their k-sum stays below 2^24 for k <= 1024, so the "H"
// accumulator is exact in FP32 whatever the tensor core's accumulation order.
// The next terms (a1 b2 + a2 b1 + a2 b2 + a1 b3 + a3 b1, 2^-8 and below
// relative) go to a second accumulator "L".  x''.y'' = sigma^2 2^-14 (H + L).
//
// Epilogue (one thread per target row, 128 rows = the 128 TMEM lanes):
//   d2 = |x''|^2 + |y''|^2 - 2 x''.y'' assembled as an unevaluated FP32 sum
//   t + lo: the norms are split on a common grid so that their high parts add
//   exactly, -2 sigma^2 2^-14 H is exact, and Fast2Sum captures the last
//   rounding (|x''|^2 + |y''|^2 >= |2 x''.y''|).  The Gaussian value is
//   2^-t (1 - ln2 lo) with the SFU's ex2.  Pairs whose distance the bound says
//   is not resolved (Laplace near coincidence; cancellation when the points sit
//   far from the centre) are recomputed in FP64 from the pool coordinates.
// Row sums: FP32 within a 128-source tile (4 interleaved partial sums), FP64
// across tiles; one partial per (row, source chunk); a fixed-order reduction
// adds the partials into u (deterministic).
//
// Pipeline (one CTA per SM, persistent over (target tile, source chunk) items):
//   warp 0      producer: bulk copies (TMA engine) of the target tile image
//               (resident for the item) and of the source tile images (2 stages)
//   warp 1      MMA issuer: 6 x k/16 tcgen05.mma per source tile into one of
//               two TMEM accumulator pairs (double buffered)
//   warps 2..5  epilogue: tcgen05.ld of the accumulators, kernel function,
//               weighted row sums
// Every wait is bounded; on a timeout the CTA records an error, drains and
// frees its tensor memory.
#include "gsks.h"
#include "gsks_internal.cuh"
#include "gsks_host.h"
#include "gsks_sm100.cuh"

#include <cuda_fp16.h>
#include <algorithm>
#include <cmath>

namespace gsks {
namespace split {

using namespace sm100;

constexpr int BM = 128;             // targets per tile (TMEM lanes)
constexpr int BN = 128;             // sources per tile
constexpr int KPAD_MAX = 64;        // padded k of the target-resident kernel
constexpr int NSTAGE = 3;           // source-tile operand stages
constexpr int NMETA = 4;            // source-tile metadata ring
constexpr int NBLK = 3;             // slices per operand
constexpr int EPI_GROUPS = 4;          // column groups of the epilogue
constexpr int EPI_WARPS = 4 * EPI_GROUPS;
constexpr int NTHREADS = 32 * (2 + EPI_WARPS);
constexpr long long WAIT_LIMIT = 1LL << 32;   // clock cycles (~2 s) per wait
constexpr uint32_t TMEM_COLS = 512;           // 2 buffers x (H, L) x 128 columns

struct PtMeta {          // 32 bytes per point, appended to each tile image
  float n_hi, n_lo;      // |x''|^2 = n_hi + n_lo, n_hi on the call's grid q
  float w;               // sources: w[wmap[j]]; targets: unused
  float h;               // var-bandwidth factor (targets: -0.5 log2e hi; sources: hj)
  int pos;               // position in amap / bmap, -1 for padding
  int pad[3];
};

struct Params {          // per call, computed on the device
  double alpha, sigma, inv_sigma, q;
  double g;              // 2 sigma^2 2^-14: d2 = g (nu_i + nu_j - H - L)
  float rc;              // -g as a float
  float t_flag;          // flag pairs with t < t_flag ...
  float rho;             // ... or t < rho * (n_i + n_j)
  int centred;
  int any_flag;          // some pair may be flagged
  int exact_t1;          // nu_i + nu_j - H is exact in FP32
  int gfast;             // Gaussian without flags: low norm parts folded into w / row factors
  float c0h, c0l;        // Laplace: scal^(1/m), m = -powe, as a double-float
};

__host__ __device__ inline size_t blk_bytes(int rows, int kpad) { return (size_t)rows * kpad * 2; }
__host__ __device__ inline size_t tile_bytes(int rows, int kpad)
{
  return NBLK * blk_bytes(rows, kpad) + (size_t)rows * sizeof(PtMeta);
}

// k is processed in chunks of KCH (the whole padded k when it is smaller);
// beyond KPAD_MAX the target tile no longer stays resident and both operands
// stream through the stages chunk by chunk.
constexpr int KCH = 64;
__host__ __device__ inline int kchunk(int kpad) { return kpad < KCH ? kpad : KCH; }

// Byte offset, inside a 128-row tile image, of the 16-byte row segment
// (slice b, k-group kg, row r): chunk-major, then slice, then the no-swizzle
// K-major core-matrix layout of the chunk (k-group, row, 8 elements).
__host__ __device__ inline size_t img_off(int b, int kg, int r, int kpad)
{
  const int kc = kchunk(kpad), gpc = kc / 8;
  const int c = kg / gpc, kgc = kg - c * gpc;
  return (size_t)c * NBLK * BM * kc * 2 + (size_t)b * BM * kc * 2 + (size_t)kgc * BM * 16 + (size_t)r * 16;
}

// Shared-memory plan of split_tiles for a padded k.
struct SmemLayout {
  bool resident;       // the target tile stays in shared memory for the item
  int kc, nch;         // k-chunk and number of chunks
  int nstage;          // operand stages
  size_t chunk_op;     // bytes of one operand's chunk (3 slices x 128 rows x kc)
  size_t chunk_al;     // chunk_op rounded up to 1 KiB
  size_t stage_bytes;  // one stage: the source chunk, or both operands' chunks
  size_t a_region;     // target image (resident) or target metadata
};
__host__ __device__ inline SmemLayout smem_layout(int kpad)
{
  SmemLayout L;
  L.kc = kchunk(kpad);
  L.nch = kpad / L.kc;
  L.resident = (L.nch == 1);
  L.chunk_op = (size_t)NBLK * BM * L.kc * 2;
  L.chunk_al = (L.chunk_op + 1023) & ~(size_t)1023;
  L.nstage = L.resident ? NSTAGE : 2;
  L.stage_bytes = L.resident ? L.chunk_al : 2 * L.chunk_al;
  L.a_region = L.resident ? ((tile_bytes(BM, kpad) + 1023) & ~(size_t)1023)
                          : (((size_t)BM * sizeof(PtMeta) + 1023) & ~(size_t)1023);
  return L;
}

// ---------------------------------------------------------------------------
// Ordered 64-bit keys of doubles, so that integer min/max is the double's.
__device__ __forceinline__ long long dkey(double v)
{
  long long b = __double_as_longlong(v);
  return b >= 0 ? b : b ^ 0x7FFFFFFFFFFFFFFFLL;
}
__device__ __forceinline__ double dval(long long k)
{
  return __longlong_as_double(k >= 0 ? k : k ^ 0x7FFFFFFFFFFFFFFFLL);
}

__global__ void bbox_init(int k, long long *bbox)
{
  for (int p = threadIdx.x + blockIdx.x * blockDim.x; p < k; p += blockDim.x * gridDim.x) {
    bbox[p] = 0x7FFFFFFFFFFFFFFFLL;
    bbox[k + p] = (long long)0x8000000000000000ULL;
  }
}

// Per-dimension min / max over the gathered targets and sources.
__global__ void bbox_kernel(int m, int n, int k, const double *__restrict__ XA, const int *__restrict__ amap,
                            const double *__restrict__ XB, const int *__restrict__ bmap, long long *bbox)
{
  extern __shared__ long long sb[];
  for (int p = threadIdx.x; p < k; p += blockDim.x) {
    sb[p] = 0x7FFFFFFFFFFFFFFFLL;
    sb[k + p] = (long long)0x8000000000000000ULL;
  }
  __syncthreads();
  const long long total = (long long)(m + n) * k;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)blockDim.x * gridDim.x) {
    const int pt = (int)(e / k), p = (int)(e - (long long)pt * k);
    double v;
    if (pt < m) v = XA[(size_t)(amap ? amap[pt] : pt) * k + p];
    else v = XB[(size_t)(bmap ? bmap[pt - m] : pt - m) * k + p];
    const long long key = dkey(v);
    atomicMin(&sb[p], key);
    atomicMax(&sb[k + p], key);
  }
  __syncthreads();
  for (int p = threadIdx.x; p < k; p += blockDim.x) {
    atomicMin(&bbox[p], sb[p]);
    atomicMax(&bbox[k + p], sb[k + p]);
  }
}

// Centre, scales and the flag thresholds from the bounding box (one block).
__global__ void params_kernel(int k, int kt, double scal, double powe, float tau, const long long *bbox,
                              double *centre, Params *P)
{
  __shared__ double s_sq[1024], s_mx[1024];
  const bool dist = kt_uses_norms(kt);
  double sq = 0.0, mx = 0.0;
  for (int p = threadIdx.x; p < k; p += blockDim.x) {
    const double lo = dval(bbox[p]), hi = dval(bbox[k + p]);
    double c = 0.0, half;
    if (dist) { c = 0.5 * (lo + hi); half = 0.5 * (hi - lo); }
    else half = fmax(fabs(lo), fabs(hi));
    centre[p] = c;
    sq += half * half;
    mx = fmax(mx, half);
  }
  s_sq[threadIdx.x] = sq; s_mx[threadIdx.x] = mx;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {   // fixed-order tree: deterministic
    if ((int)threadIdx.x < s) {
      s_sq[threadIdx.x] += s_sq[threadIdx.x + s];
      s_mx[threadIdx.x] = fmax(s_mx[threadIdx.x], s_mx[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double log2e = 1.4426950408889634;
    const double alpha = (kt == KS_GAUSSIAN) ? sqrt(-scal * log2e) : 1.0;
    const double maxabs = alpha * s_mx[0];
    double sigma = maxabs > 0.0 ? exp2(ceil(log2(maxabs))) : 1.0;
    if (sigma < maxabs) sigma *= 2.0;
    const double nbound = alpha * alpha * s_sq[0];        // >= any |x''|^2
    const double q = exp2(ceil(log2(2.0 * nbound + 1e-300)) - 23.0);
    P->alpha = alpha; P->sigma = sigma; P->inv_sigma = 1.0 / sigma; P->q = q;
    P->g = 2.0 * sigma * sigma * 0x1p-14;
    P->rc = (float)(-P->g);
    P->centred = dist ? 1 : 0;
    // Absolute error bound of the assembled d2 (in the scaled units): rounding
    // of the L accumulator and of the split norms, plus the slicing remainder.
    // (Calibrated: over a 16384-pair tile at k = 64, sigma = 1, the largest
    // |t + lo - d2| was 1.4e-7, and this expression gives 1.6e-7 there.)
    const double delta = 2.0 * (sigma * sigma * (double)k * 0x1p-31) +
                         2.0 * sigma * sqrt((double)k) * sqrt(nbound) * 0x1p-30 + 2.0 * q * 0x1p-23;
    float t_flag = -1.0f, rho = 0.0f;
    if (kt == KS_GAUSSIAN) {
      // relative error of 2^-d2 is ln2 * delta; pairs with t >= 126 underflow anyway
      if (delta * 0.6931471805599453 > tau) t_flag = 126.0f;
    } else if (kt == KS_GAUSSIAN_VAR_BANDWIDTH) {
      if (delta > tau) t_flag = 3.0e38f;      // bound not usable per pair: recheck all near pairs
    } else if (kt == KS_LAPLACE) {
      rho = 0x1p-10f;                         // coincident points and near-cancellation
      t_flag = (float)(fabs(powe) * delta / tau);
      // (c0 / d2)^m stays below 2^120 for d2 above c0 2^(-120/m)
      const double mm = -powe, c0 = pow(scal, 1.0 / mm);
      P->c0h = (float)c0;
      P->c0l = (float)(c0 - (double)P->c0h);
      t_flag = fmaxf(t_flag, (float)(c0 * exp2(-120.0 / mm) * 1.001));
    } else if (dist) {
      rho = 0.0f;                             // compact / polynomial in d2: absolute error only
    }
    P->t_flag = t_flag; P->rho = rho;
    P->any_flag = (t_flag > 0.0f || rho > 0.0f) ? 1 : 0;
    // |x''|^2 + |y''|^2 lies on the grid q and -2 sigma^2 2^-14 H on the grid
    // 2 sigma^2 2^-14; when the latter is a multiple of q their sum is exact
    // (it stays below 2^24 q), and only the small L term needs Fast2Sum.
    P->exact_t1 = (q <= 2.0 * sigma * sigma * 0x1p-14) ? 1 : 0;
    P->gfast = (kt == KS_GAUSSIAN && P->exact_t1 && !P->any_flag) ? 1 : 0;
  }
}

// Tile images: per tile, NBLK slice blocks in the no-swizzle K-major core-matrix
// layout (element (r, p) at (p/8)*rows*16 + r*16 + (p%8)*2 bytes), then the
// point metadata.  One thread per point.
__global__ void pack_kernel(int side, int npts, int k, int kpad, const double *__restrict__ X,
                            const int *__restrict__ map, const double *__restrict__ w,
                            const int *__restrict__ wmap, const double *__restrict__ hvec, int kt,
                            const double *__restrict__ centre, const Params *__restrict__ P,
                            uint8_t *__restrict__ img)
{
  const int tile = blockIdx.x, r = threadIdx.x;
  const int pt = tile * BM + r;
  const bool valid = pt < npts;
  const int pidx = valid ? (map ? map[pt] : pt) : 0;
  const double *x = X + (size_t)pidx * k;
  const double alpha = P->alpha, inv_sigma = P->inv_sigma;
  const bool centred = P->centred != 0;
  uint8_t *base = img + (size_t)tile * tile_bytes(BM, kpad);
  const size_t bb = blk_bytes(BM, kpad);
  double nrm = 0.0;
  for (int kg = 0; kg < kpad / 8; kg++) {
    __align__(16) __half s1[8], s2[8], s3[8];
#pragma unroll
    for (int e = 0; e < 8; e++) {
      const int p = kg * 8 + e;
      double a1 = 0.0, r1 = 0.0;
      __half h2 = __float2half_rn(0.0f), h3 = __float2half_rn(0.0f);
      if (valid && p < k) {
        const double xv = alpha * (x[p] - (centred ? centre[p] : 0.0));
        const double t = xv * inv_sigma * 128.0;
        a1 = rint(t);
        r1 = t - a1;                                   // |r1| <= 0.5, exact
        h2 = __float2half_rn((float)r1);
        const double r2 = r1 - (double)__half2float(h2);
        h3 = __float2half_rn((float)r2);
        // The norm of the represented point restricted to the products the
        // tensor cores form (a1a1 + 2a1a2 + a2a2 + 2a1a3), so that the
        // assembled d2 of identical points is 0 up to the FP32 accumulations.
        const double f2 = (double)__half2float(h2), f3 = (double)__half2float(h3);
        nrm += (a1 * a1 + 2.0 * a1 * f2 + f2 * f2 + 2.0 * a1 * f3) * (1.0 / 16384.0);
      }
      s1[e] = __float2half_rn((float)a1);              // exact: |a1| <= 128
      s2[e] = h2;
      s3[e] = h3;
    }
    *(uint4 *)(base + img_off(0, kg, r, kpad)) = *(const uint4 *)s1;
    *(uint4 *)(base + img_off(1, kg, r, kpad)) = *(const uint4 *)s2;
    *(uint4 *)(base + img_off(2, kg, r, kpad)) = *(const uint4 *)s3;
  }
  (void)bb;
  // The norm in units of the accumulators: nu = |x''|^2 / g with
  // g = 2 sigma^2 2^-14, so that d2 = g (nu_i + nu_j - H - L).  nu is split on
  // the grid q / g (a power of two): its high parts and H add exactly.
  const double g = P->g;
  const double nu = nrm * (P->sigma * P->sigma) / g;
  const double qg = P->q / g;
  const double nh = rint(nu / qg) * qg;
  const double nl = nu - nh;
  PtMeta mt;
  mt.n_hi = (float)nh;
  mt.n_lo = (float)nl;
  mt.w = 0.0f;
  mt.h = 0.0f;
  if (side == 1 && valid) mt.w = (float)w[wmap ? wmap[pt] : pt];
  if (P->gfast) {
    // Gaussian: 2^-(g nl) is a per-point factor; fold it into w for sources
    // and into a row factor for targets (applied to the row sum)
    const double f = exp2(-g * nl);
    mt.n_lo = 0.0f;
    if (side == 1) mt.w = valid ? (float)(w[wmap ? wmap[pt] : pt] * f) : 0.0f;
    else mt.h = (float)f;
  }
  if (kt == KS_GAUSSIAN_VAR_BANDWIDTH && valid) {
    const double hv = hvec[pidx];
    mt.h = side == 0 ? (float)(-0.5 * 1.4426950408889634 * hv) : (float)hv;
  }
  mt.pos = valid ? pt : -1;
  mt.pad[0] = mt.pad[1] = mt.pad[2] = 0;
  ((PtMeta *)(base + NBLK * bb))[r] = mt;
}

// ---------------------------------------------------------------------------
struct TileArgs {
  int m, n, k, kpad, kt;
  int ntm, ntn, nsc, chunk_tiles;   // items = ntm * nsc; chunk = source tiles per item
  const uint8_t *imgA, *imgB;
  const double *XA, *XB;            // pool coordinates (FP64) for the rechecks
  const int *amap, *bmap, *wmap;
  const double *w;
  const double *hi, *hj;
  KParams kp;                       // FP64 descriptor for the rechecks
  const Params *P;
  double *partial;                  // [nsc][ldp]
  int ldp;
  int *err;
  float *dump;                      // test hook: H, L, t, lo, K of CTA 0's first tile
};

struct SplitSmem {
  uint64_t a_full, a_empty;
  uint64_t b_full[NSTAGE], b_empty[NSTAGE];
  uint64_t m_full[NMETA], m_empty[NMETA];
  uint64_t t_full[2], t_empty[2];
  uint64_t drain;
  uint32_t tmem_base;
  int abort;
  int never;             // stays 0: an abort flag for the drain waits
  double rsum[2][EPI_GROUPS - 1][BM];   // row sums of epilogue groups 1.., by item parity
};

// Double-float (unevaluated FP32 pair) product, a *= b: Dekker's product with
// the FMA giving the exact error of the high product.
__device__ __forceinline__ void df_mul(float &ah, float &al, float bh, float bl)
{
  const float p = ah * bh;
  float e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, e);
  e = fmaf(al, bh, e);
  const float s = p + e;
  al = e - (s - p);
  ah = s;
}

// Double-float reciprocal, a = 1 / a, one Newton step on the FP32 quotient.
__device__ __forceinline__ void df_rcp(float &ah, float &al)
{
  float q = rcp_approx(ah);
  q = fmaf(q, fmaf(-ah, q, 1.0f), q);        // Newton step: q to ~1 ulp of 1/ah
  float r = fmaf(-ah, q, 1.0f);
  r = fmaf(-al, q, r);
  const float ql = q * r;
  const float s = q + ql;
  al = ql - (s - q);
  ah = s;
}

// FP32 kernel value from the double-float squared distance t + lo (scaled
// units) or, for inner-product kernels, from c = x.y.
template <int KT>
__device__ __forceinline__ float kval32(float t, float lo, float c, float hrow, float hcol, const KParams &kp)
{
  if constexpr (KT == KS_GAUSSIAN) {
    const float e = ex2_approx(-t);
    return fmaf(e, -0.69314718f * lo, e);
  } else if constexpr (KT == KS_GAUSSIAN_VAR_BANDWIDTH) {
    // arg2 = (t + lo) * hrow * hcol, hrow = -0.5 log2e hi
    const float f = hrow * hcol;
    const float a = t * f;
    const float ae = fmaf(t, f, -a) + lo * f;
    const float e = ex2_approx(a);
    return fmaf(e, 0.69314718f * ae, e);
  } else if constexpr (KT == KS_POLYNOMIAL) {
    const float v = fmaf((float)kp.scal, c, (float)kp.cons);
    if (kp.pmode == POW_INT) {
      int e = kp.pint < 0 ? -kp.pint : kp.pint;
      float r = 1.0f, b = v;
      for (;;) { if (e & 1) r *= b; e >>= 1; if (!e) break; b *= b; }
      return kp.pint < 0 ? 1.0f / r : r;
    }
    return ex2_approx((float)kp.powe * __log2f(v));
  } else if constexpr (KT == KS_LAPLACE) {
    // scal * d2^powe with powe = -m < 0 (k >= 3), evaluated as (c0 / d2)^m with
    // c0 = scal^(1/m): the intermediates stay in the FP32 range for every d2
    // whose kernel value does (smaller d2 are flagged and done in FP64).  The
    // base is a double-float through binary powering: m up to 32 would
    // amplify a single FP32 rounding of d2 m-fold.  hrow / hcol carry c0.
    float bh = t, bl = lo;
    df_rcp(bh, bl);
    df_mul(bh, bl, hrow, hcol);
    const int m = -kp.pint - (kp.pmode == POW_HALF ? 1 : 0);   // integer part of -powe
    float rh = 1.0f, rl = 0.0f, ph = bh, pl = bl;
#pragma unroll
    for (int bit = 0; bit < 9; bit++) {      // fixed trip count (m < 512), uniform branches
      if (m & (1 << bit)) df_mul(rh, rl, ph, pl);
      if (m >> (bit + 1)) df_mul(ph, pl, ph, pl);
    }
    if (kp.pmode == POW_HALF) {
      const float sh = sqrtf(bh);
      const float sl = (fmaf(-sh, sh, bh) + bl) / (2.0f * sh);   // sqrt(bh + bl) = sh + sl
      df_mul(rh, rl, sh, sl);
    }
    return rh + rl;
  } else if constexpr (KT == KS_TANH) {
    const float v = fmaf((float)kp.scal, c, (float)kp.cons);
    const float av = fabsf(v);
    float r;
    if (av < 0.125f) {
      const float v2 = v * v;  // tanh series v - v^3/3 + 2v^5/15 - 17v^7/315
      r = v * fmaf(v2, fmaf(v2, fmaf(v2, -17.0f / 315.0f, 2.0f / 15.0f), -1.0f / 3.0f), 1.0f);
    } else {
      const float e = ex2_approx(2.0f * 1.44269504f * av);
      r = 1.0f - 2.0f / (e + 1.0f);
      r = copysignf(r, v);
    }
    return r;
  } else if constexpr (KT == KS_QUARTIC) {
    const float d = t + lo;
    if (d < 1.0f) { const float u = 1.0f - d; return 0.9375f * u * u; }
    return 0.0f;
  } else if constexpr (KT == KS_MULTIQUADRATIC) {
    return (t + (float)kp.cons) + lo;
  } else {  // Epanechnikov
    const float d = t + lo;
    return d < 1.0f ? 0.75f * (1.0f - d) : 0.0f;
  }
}

// FP64 recheck of one flagged pair from the pool coordinates (the distance
// assembly of near-coincident pairs is kept in FP64).
template <int KT>
__device__ double recheck64(const TileArgs &a, int ipos, int jpos)
{
  const int pa = a.amap ? a.amap[ipos] : ipos;
  const int pb = a.bmap ? a.bmap[jpos] : jpos;
  const double *x = a.XA + (size_t)pa * a.k, *y = a.XB + (size_t)pb * a.k;
  double d2 = 0.0;
  for (int p = 0; p < a.k; p++) { const double d = x[p] - y[p]; d2 = fma(d, d, d2); }
  const double wv = a.w[a.wmap ? a.wmap[jpos] : jpos];
  double kv;
  if constexpr (KT == KS_GAUSSIAN) kv = exp(d2 * a.kp.scal);
  else if constexpr (KT == KS_GAUSSIAN_VAR_BANDWIDTH) kv = exp(((d2 * -0.5) * a.hi[pa]) * a.hj[pb]);
  else if constexpr (KT == KS_LAPLACE) {
    if (d2 < 1e-15) d2 = 1.79e308;
    kv = pow_class(d2, a.kp) * a.kp.scal;
  } else if constexpr (KT == KS_QUARTIC) {
    kv = d2 < 1.0 ? (15.0 / 16.0) * (1.0 - d2) * (1.0 - d2) : 0.0;
  } else if constexpr (KT == KS_MULTIQUADRATIC) kv = d2 + a.kp.cons;
  else if constexpr (KT == KS_EPANECHNIKOV) kv = d2 < 1.0 ? 0.75 * (1.0 - d2) : 0.0;
  else kv = 0.0;
  return kv * wv;
}

// Squared distance t + lo (double-float, scaled units) of one pair from its
// accumulators and split norms.
// In units of the accumulators the distance is nu_i + nu_j - H - L; rc = -g
// scales it back (exactly: g is a power of two).
template <bool EXACT>
__device__ __forceinline__ void assemble(float H, float L, float an_hi, float an_lo, float bn_hi, float bn_lo,
                                         float rc, float &t, float &lo, float &s)
{
  s = an_hi + bn_hi;                          // exact on the grid q / g
  float tt, ee;
  if constexpr (EXACT) {
    const float t1 = s - H;                   // exact: H is an integer and q / g divides 1
    tt = t1 - L;
    ee = (t1 - tt) - L;                       // Fast2Sum
  } else {
    const float u1 = s - L;
    const float e1 = (s - u1) - L;            // Fast2Sum: |s| >= |L|
    tt = u1 - H;
    const float e2 = (u1 - tt) - H;           // Fast2Sum: |u1| >= |H|
    ee = e1 + e2;
  }
  t = tt * -rc;
  lo = ((an_lo + bn_lo) + ee) * -rc;
  s *= -rc;
}

// NC columns of one row, Gaussian with the low norm parts folded into the
// source weights and the row factor: kv = 2^-(g tt) (1 - ln2 g ee).
template <int NC>
__device__ __forceinline__ void epi_chunk_gfast(const uint32_t (&h)[NC], const uint32_t (&l)[NC],
                                                const PtMeta *__restrict__ bm, float an_hi, float rc,
                                                float (&acc)[4])
{
  const float cg = 0.69314718f * rc;          // -ln2 g
#pragma unroll
  for (int j = 0; j < NC; j++) {
    const float4 m0 = *(const float4 *)&bm[j];   // nu_hi, 0, w', h
    const float w = m0.z;
    const float H = __uint_as_float(h[j]), L = __uint_as_float(l[j]);
    const float t1 = (an_hi + m0.x) - H;      // exact
    const float tt = t1 - L;
    const float ee = (t1 - tt) - L;
    const float e = ex2_approx(tt * rc);      // 2^-(g tt)
    const float kv = fmaf(e, cg * ee, e);
    acc[j & 3] = fmaf(kv, w, acc[j & 3]);
  }
}

// NC columns of one row, distance kernels.  Returns the flagged columns.
template <int KT, bool EXACT, bool FLAGS, int NC>
__device__ __forceinline__ uint32_t epi_chunk(const uint32_t (&h)[NC], const uint32_t (&l)[NC],
                                              const PtMeta *__restrict__ bm, const PtMeta &am, float rc,
                                              const Params *P, const KParams &kp, float (&acc)[4])
{
  uint32_t flags = 0;
  float t_flag = 0.f, rho = 0.f;
  if constexpr (FLAGS) { t_flag = P->t_flag; rho = P->rho; }
#pragma unroll
  for (int j = 0; j < NC; j++) {
    const float4 m0 = *(const float4 *)&bm[j];   // n_hi, n_lo, w, h
    float t, lo, s;
    assemble<EXACT>(__uint_as_float(h[j]), __uint_as_float(l[j]), am.n_hi, am.n_lo, m0.x, m0.y, rc, t, lo, s);
    float kv;
    if constexpr (KT == KS_LAPLACE) kv = kval32<KT>(t, lo, 0.f, P->c0h, P->c0l, kp);
    else kv = kval32<KT>(t, lo, 0.f, am.h, m0.w, kp);
    if constexpr (FLAGS) {
      if (t < t_flag || t < rho * s) { flags |= 1u << j; kv = 0.f; }
    }
    // padding columns carry w = 0 and finite distances
    acc[j & 3] = fmaf(kv, m0.z, acc[j & 3]);
  }
  return flags;
}

// NC columns of one row, inner-product kernels (polynomial, tanh).
template <int KT, int NC>
__device__ __forceinline__ void epi_chunk_ip(const uint32_t (&h)[NC], const uint32_t (&l)[NC],
                                             const PtMeta *__restrict__ bm, int valid, float rc,
                                             const KParams &kp, float (&acc)[4])
{
#pragma unroll
  for (int j = 0; j < NC; j++) {
    const float w = bm[j].w;
    const float cc = fmaf(__uint_as_float(l[j]), rc, __uint_as_float(h[j]) * rc) * -0.5f;  // x.y
    const float kv = kval32<KT>(0.f, 0.f, cc, 0.f, 0.f, kp);
    acc[j & 3] += (j < valid) ? kv * w : 0.f;      // the kernel of a padding column may be NaN
  }
}

// Test hook: raw accumulators and epilogue values of NC columns from c0.
template <int KT, int NC>
__device__ void dump_chunk(float *dump, int row, int c0, const uint32_t (&h)[NC], const uint32_t (&l)[NC],
                           const PtMeta *bm, const PtMeta &am, float rc, const KParams &kp)
{
  for (int j = 0; j < NC; j++) {
    const int c = c0 + j;
    float *dp = dump + ((size_t)row * BN + c) * 5;
    const float H = __uint_as_float(h[j]), L = __uint_as_float(l[j]);
    dp[0] = H; dp[1] = L;
    if constexpr (kt_uses_norms(KT)) {
      float t, lo, s;
      assemble<false>(H, L, am.n_hi, am.n_lo, bm[j].n_hi, bm[j].n_lo, rc, t, lo, s);
      dp[2] = 0.f;
      if constexpr (KT != KS_LAPLACE) dp[2] = kval32<KT>(t, lo, 0.f, am.h, bm[j].h, kp);
      dp[3] = t; dp[4] = lo;
    } else {
      dp[2] = kval32<KT>(0.f, 0.f, fmaf(L, rc, H * rc) * -0.5f, 0.f, 0.f, kp);
      dp[3] = dp[4] = 0.f;
    }
  }
}

template <int KT>
__global__ void __launch_bounds__(NTHREADS, 1) split_tiles(TileArgs a)
{
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *sm = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int kpad = a.kpad;
  const SmemLayout L = smem_layout(kpad);
  const bool resident = L.resident;
  const size_t a_bytes = tile_bytes(BM, kpad), b_bytes = tile_bytes(BN, kpad);
  const size_t a_op = NBLK * blk_bytes(BM, kpad);     // operand part of a tile image
  const size_t meta_bytes = (size_t)BM * sizeof(PtMeta);
  uint8_t *sA = sm;                                   // target image (resident) or target meta
  uint8_t *sAmeta = resident ? sA + a_op : sA;
  uint8_t *sStage = sm + L.a_region;
  uint8_t *sBm = sStage + L.nstage * L.stage_bytes;   // NMETA source metadata slots
  SplitSmem *S = (SplitSmem *)(sBm + NMETA * meta_bytes);
  volatile int *abort = &S->abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int items = a.ntm * a.nsc;

  if (threadIdx.x == 0) {
    mbar_init(&S->a_full, 1);
    mbar_init(&S->a_empty, 1 + EPI_WARPS);
    for (int s = 0; s < NSTAGE; s++) { mbar_init(&S->b_full[s], 1); mbar_init(&S->b_empty[s], 1); }
    for (int s = 0; s < NMETA; s++) { mbar_init(&S->m_full[s], 1); mbar_init(&S->m_empty[s], EPI_WARPS); }
    for (int b = 0; b < 2; b++) { mbar_init(&S->t_full[b], 1); mbar_init(&S->t_empty[b], EPI_WARPS); }
    mbar_init(&S->drain, 1);
    S->abort = 0;
    S->never = 0;
    fence_mbar_init();
  }
  if (warp == 0) { tmem_alloc(&S->tmem_base, TMEM_COLS); tmem_relinquish(); }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S->tmem_base;

  if (warp == 0) {
    // ---------------- producer ----------------
    // Resident (k <= KPAD_MAX): the target tile image once per item, the source
    // operands once per tile.  Streaming: the target metadata once per item,
    // then per tile and k-chunk one stage holding both operands' chunk.
    if (lane == 0) {
      int g = 0, tt = 0;
      int a_issued = -1;                  // item index of the last target copy
      int b_last[NSTAGE], m_last[NMETA];  // use count of the last copy per stage / meta slot
      for (int s = 0; s < NSTAGE; s++) b_last[s] = -1;
      for (int s = 0; s < NMETA; s++) m_last[s] = -1;
      bool stop = false;
      for (int it = 0, item = blockIdx.x; item < items && !*abort && !stop; it++, item += gridDim.x) {
        const int ti = item % a.ntm, sc = item / a.ntm;
        if (it > 0 && !mbar_wait(&S->a_empty, (it - 1) & 1, abort, WAIT_LIMIT)) break;
        const uint8_t *imgA = a.imgA + (size_t)ti * a_bytes;
        if (resident) {
          mbar_arrive_expect_tx(&S->a_full, (uint32_t)a_bytes);
          bulk_g2s(sA, imgA, (uint32_t)a_bytes, &S->a_full);
        } else {
          mbar_arrive_expect_tx(&S->a_full, (uint32_t)meta_bytes);
          bulk_g2s(sAmeta, imgA + a_op, (uint32_t)meta_bytes, &S->a_full);
        }
        a_issued = it;
        const int t0 = sc * a.chunk_tiles, t1 = min(a.ntn, t0 + a.chunk_tiles);
        for (int tj = t0; tj < t1 && !stop; tj++, tt++) {
          const uint8_t *imgB = a.imgB + (size_t)tj * b_bytes;
          for (int c = 0; c < L.nch; c++, g++) {
            const int st = g % L.nstage, u = g / L.nstage;
            if (u > 0 && !mbar_wait(&S->b_empty[st], (u - 1) & 1, abort, WAIT_LIMIT)) { stop = true; break; }
            uint8_t *dst = sStage + st * L.stage_bytes;
            if (resident) {
              mbar_arrive_expect_tx(&S->b_full[st], (uint32_t)L.chunk_op);
              bulk_g2s(dst, imgB, (uint32_t)L.chunk_op, &S->b_full[st]);
            } else {
              mbar_arrive_expect_tx(&S->b_full[st], (uint32_t)(2 * L.chunk_op));
              bulk_g2s(dst, imgA + (size_t)c * L.chunk_op, (uint32_t)L.chunk_op, &S->b_full[st]);
              bulk_g2s(dst + L.chunk_al, imgB + (size_t)c * L.chunk_op, (uint32_t)L.chunk_op, &S->b_full[st]);
            }
            b_last[st] = u;
          }
          if (stop) break;
          const int ms = tt % NMETA, mu = tt / NMETA;
          if (mu > 0 && !mbar_wait(&S->m_empty[ms], (mu - 1) & 1, abort, WAIT_LIMIT)) break;
          mbar_arrive_expect_tx(&S->m_full[ms], (uint32_t)meta_bytes);
          bulk_g2s(sBm + ms * meta_bytes, imgB + a_op, (uint32_t)meta_bytes, &S->m_full[ms]);
          m_last[ms] = mu;
        }
      }
      // On an abort, let the copies already issued land before the CTA exits
      // (each wait bounded; a copy's phase may also have completed long ago).
      if (*abort) {
        volatile int *nev = &S->never;
        if (a_issued >= 0) mbar_wait(&S->a_full, a_issued & 1, nev, 1LL << 28);
        for (int s = 0; s < NSTAGE; s++)
          if (b_last[s] >= 0) mbar_wait(&S->b_full[s], b_last[s] & 1, nev, 1LL << 28);
        for (int s = 0; s < NMETA; s++)
          if (m_last[s] >= 0) mbar_wait(&S->m_full[s], m_last[s] & 1, nev, 1LL << 28);
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const uint32_t idesc = idesc_f16_f32(BM, BN);
      const uint32_t lbo = BM * 16, sbo = 128;        // BM == BN
      const uint32_t blk = (uint32_t)BM * L.kc * 2;   // one slice block of one chunk
      int g = 0, tc = 0;
      bool stop = false;
      for (int it = 0, item = blockIdx.x; item < items && !*abort && !stop; it++, item += gridDim.x) {
        const int sc = item / a.ntm;
        if (!mbar_wait(&S->a_full, it & 1, abort, WAIT_LIMIT)) break;
        const int t0 = sc * a.chunk_tiles, t1 = min(a.ntn, t0 + a.chunk_tiles);
        for (int tj = t0; tj < t1 && !stop; tj++, tc++) {
          const int buf = tc & 1;
          if (tc >= 2 && !mbar_wait(&S->t_empty[buf], ((tc >> 1) - 1) & 1, abort, WAIT_LIMIT)) { stop = true; break; }
          const uint32_t dH = tmem + buf * 256, dL = tmem + buf * 256 + 128;
          for (int c = 0; c < L.nch; c++, g++) {
            const int st = g % L.nstage;
            if (!mbar_wait(&S->b_full[st], (g / L.nstage) & 1, abort, WAIT_LIMIT)) { stop = true; break; }
            tc_fence_after();
            const uint32_t sbase = smem_addr(sStage + st * L.stage_bytes);
            const uint32_t a0 = resident ? smem_addr(sA) : sbase;
            const uint32_t b0 = resident ? sbase : sbase + (uint32_t)L.chunk_al;
            for (int s = 0; s < L.kc / 16; s++) {
              auto da = [&](int b) { return desc_noswizzle(a0 + b * blk + (uint32_t)s * 2 * lbo, lbo, sbo); };
              auto db = [&](int b) { return desc_noswizzle(b0 + b * blk + (uint32_t)s * 2 * lbo, lbo, sbo); };
              const uint32_t acc = (c > 0 || s > 0) ? 1u : 0u;
              umma_f16(dH, da(0), db(0), idesc, acc);
              umma_f16(dL, da(0), db(1), idesc, acc);
              umma_f16(dL, da(1), db(0), idesc, 1);
              umma_f16(dL, da(1), db(1), idesc, 1);
              umma_f16(dL, da(0), db(2), idesc, 1);
              umma_f16(dL, da(2), db(0), idesc, 1);
            }
            umma_commit(&S->b_empty[st]);
          }
          if (stop) break;
          umma_commit(&S->t_full[buf]);
        }
        umma_commit(&S->a_empty);
      }
      umma_commit(&S->drain);
      mbar_wait(&S->drain, 0, &S->never, 1LL << 30);
    }
  } else {
    // ---------------- epilogue (warps 2 .. 2+EPI_WARPS-1) ----------------
    // EPI_GROUPS groups of four warps; group g takes columns [32g, 32g+32) of
    // every tile, each warp the 32 TMEM lanes (= target rows) of its
    // sub-partition, in two 16-column TMEM loads.
    const int ew = warp - 2;
    const int grp = ew >> 2;
    const int qd = warp & 3;
    const int row = qd * 32 + lane;
    const Params *P = a.P;
    const float rc = P->rc;
    const bool flags_on = P->any_flag != 0, exact = P->exact_t1 != 0, gfast = P->gfast != 0;
    int g = 0, tc = 0;
    for (int it = 0, item = blockIdx.x; item < items && !*abort; it++, item += gridDim.x) {
      const int ti = item % a.ntm, sc = item / a.ntm;
      if (!mbar_wait(&S->a_full, it & 1, abort, WAIT_LIMIT)) break;
      const PtMeta am = ((const PtMeta *)sAmeta)[row];
      __syncwarp();
      if (lane == 0) mbar_arrive(&S->a_empty);
      double racc = 0.0;
      const int t0 = sc * a.chunk_tiles, t1 = min(a.ntn, t0 + a.chunk_tiles);
      bool ok = true;
      for (int tj = t0; tj < t1; tj++, g++, tc++) {
        const int ms = g % NMETA, buf = tc & 1;
        if (!mbar_wait(&S->t_full[buf], (tc >> 1) & 1, abort, WAIT_LIMIT)) { ok = false; break; }
        if (!mbar_wait(&S->m_full[ms], (g / NMETA) & 1, abort, WAIT_LIMIT)) { ok = false; break; }
        tc_fence_after();
        const PtMeta *bm = (const PtMeta *)(sBm + ms * meta_bytes);
        const int ncols = min(BN, a.n - tj * BN);
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        const uint32_t tH = tmem + ((uint32_t)(qd * 32) << 16) + buf * 256;
#pragma unroll 1
        for (int half = 0; half < 2; half++) {
          const int c0 = grp * 32 + half * 16;
          uint32_t h[16], l[16];
          tmem_ld16(tH + c0, h);
          tmem_ld16(tH + 128 + c0, l);
          tmem_ld_wait();
          if constexpr (KT == KS_GAUSSIAN) {
            if (gfast) {
              epi_chunk_gfast<16>(h, l, bm + c0, am.n_hi, rc, acc);
              if (a.dump && blockIdx.x == 0 && tc == 0) dump_chunk<KT, 16>(a.dump, row, c0, h, l, bm + c0, am, rc, a.kp);
              continue;
            }
          }
          if constexpr (kt_uses_norms(KT)) {
            uint32_t flags = 0;
            if (exact) {
              if (flags_on) flags = epi_chunk<KT, true, true, 16>(h, l, bm + c0, am, rc, P, a.kp, acc);
              else epi_chunk<KT, true, false, 16>(h, l, bm + c0, am, rc, P, a.kp, acc);
            } else {
              if (flags_on) flags = epi_chunk<KT, false, true, 16>(h, l, bm + c0, am, rc, P, a.kp, acc);
              else epi_chunk<KT, false, false, 16>(h, l, bm + c0, am, rc, P, a.kp, acc);
            }
            // FP64 rechecks of the flagged pairs of these 16 columns
            while (flags) {
              const int j = __ffs(flags) - 1;
              flags &= flags - 1;
              const int c = c0 + j;
              if (c < ncols && am.pos >= 0) racc += recheck64<KT>(a, am.pos, bm[c].pos);
            }
          } else {
            epi_chunk_ip<KT, 16>(h, l, bm + c0, ncols - c0, rc, a.kp, acc);
          }
          if (a.dump && blockIdx.x == 0 && tc == 0) dump_chunk<KT, 16>(a.dump, row, c0, h, l, bm + c0, am, rc, a.kp);
        }
        racc += ((double)acc[0] + (double)acc[1]) + ((double)acc[2] + (double)acc[3]);
        tc_fence_before();
        __syncwarp();
        if (lane == 0) { mbar_arrive(&S->t_empty[buf]); mbar_arrive(&S->m_empty[ms]); }
      }
      if (!ok) break;
      // combine the groups' row sums in group order (double-buffered by item parity)
      double (*xs)[BM] = S->rsum[it & 1];
      if (grp > 0) xs[grp - 1][row] = racc;
      asm volatile("bar.sync 1, %0;" ::"n"(32 * EPI_WARPS) : "memory");
      if (grp == 0) {
        for (int q = 0; q < EPI_GROUPS - 1; q++) racc += xs[q][row];
        const int grow = ti * BM + row;
        if (KT == KS_GAUSSIAN && gfast) racc *= (double)am.h;   // the row's low-norm factor
        if (grow < a.m) a.partial[(size_t)sc * a.ldp + grow] = racc;
      }
    }
  }

  __syncthreads();
  if (*abort && threadIdx.x == 0) atomicOr(a.err, DEVERR_TIMEOUT);
  if (warp == 0) { tc_fence_after(); tmem_dealloc(tmem, TMEM_COLS); }
}

// u[umap[i]] += sum over chunks of the chunk partials, in chunk order.
__global__ void split_reduce(int m, int nsc, int ldp, const double *__restrict__ partial, double *__restrict__ u,
                             const int *__restrict__ umap)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  double s = 0.0;
  for (int c = 0; c < nsc; c++) s += partial[(size_t)c * ldp + i];
  u[umap ? umap[i] : i] += s;
}

template <int KT>
cudaError_t launch_tiles_t(const TileArgs &a, int grid, size_t smem, cudaStream_t s)
{
  // The attribute is per function and device; raise it to what this launch needs.
  static int attr_bytes[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64 || attr_bytes[dev] < (int)smem) {
    cudaError_t e = cudaFuncSetAttribute(split_tiles<KT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64) attr_bytes[dev] = (int)smem;
  }
  split_tiles<KT><<<grid, NTHREADS, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_tiles(const TileArgs &a, int grid, size_t smem, cudaStream_t s)
{
  switch (a.kt) {
    case KS_GAUSSIAN: return launch_tiles_t<KS_GAUSSIAN>(a, grid, smem, s);
    case KS_GAUSSIAN_VAR_BANDWIDTH: return launch_tiles_t<KS_GAUSSIAN_VAR_BANDWIDTH>(a, grid, smem, s);
    case KS_POLYNOMIAL: return launch_tiles_t<KS_POLYNOMIAL>(a, grid, smem, s);
    case KS_LAPLACE: return launch_tiles_t<KS_LAPLACE>(a, grid, smem, s);
    case KS_TANH: return launch_tiles_t<KS_TANH>(a, grid, smem, s);
    case KS_QUARTIC: return launch_tiles_t<KS_QUARTIC>(a, grid, smem, s);
    case KS_MULTIQUADRATIC: return launch_tiles_t<KS_MULTIQUADRATIC>(a, grid, smem, s);
    default: return launch_tiles_t<KS_EPANECHNIKOV>(a, grid, smem, s);
  }
}

size_t smem_bytes(int kpad)
{
  const SmemLayout L = smem_layout(kpad);
  return 1024 /* alignment slack */ + L.a_region + L.nstage * L.stage_bytes + NMETA * (size_t)BN * sizeof(PtMeta) +
         sizeof(SplitSmem) + 64;
}

}  // namespace split

// Test hook state (gsks_split_debug_dump): per host thread.
thread_local float *tl_split_dump = nullptr;
thread_local void *tl_split_params = nullptr;

// ---------------------------------------------------------------------------
int enqueue_split(Ctx *c, const ks_t *ker, int m, int n, int k, double *u, const int *umap,
                  const double *XA, const double *XA2, const int *amap, int nxa,
                  const double *XB, const double *XB2, const int *bmap, int nxb,
                  const double *w, const int *wmap, const double *hi, const double *hj,
                  cudaStream_t s, bool stream_ordered_alloc)
{
  using namespace split;
  (void)XA2; (void)XB2; (void)nxa; (void)nxb;
  // padded k: a multiple of the MMA k-step (16) up to one chunk, of the chunk beyond
  const int kpad = k <= KCH ? (k + 15) / 16 * 16 : (k + KCH - 1) / KCH * KCH;
  if (kpad > 1024) return GSKS_ERR_TOO_LARGE;   // the exact head accumulation needs k <= 1024
  const int ntm = (m + BM - 1) / BM, ntn = (n + BN - 1) / BN;
  const int sms = std::max(1, c->num_sms);
  int nsc = (int)std::min<long long>(ntn, std::max<long long>(1, (8LL * sms + ntm - 1) / ntm));
  const int chunk_tiles = (ntn + nsc - 1) / nsc;
  nsc = (ntn + chunk_tiles - 1) / chunk_tiles;
  const int ldp = ntm * BM;

  // workspace: params | centre | bbox | A images | B images | partials
  auto al = [](size_t x) { return (x + 1023) & ~(size_t)1023; };
  const size_t o_params = 0;
  const size_t o_centre = al(sizeof(Params));
  const size_t o_bbox = o_centre + al((size_t)k * 8);
  const size_t o_a = o_bbox + al((size_t)2 * k * 8);
  const size_t o_b = o_a + al((size_t)ntm * tile_bytes(BM, kpad));
  const size_t o_p = o_b + al((size_t)ntn * tile_bytes(BN, kpad));
  const size_t total = o_p + al((size_t)nsc * ldp * 8);
  uint8_t *ws = nullptr;
  if (stream_ordered_alloc) {
    cudaError_t e = cudaMallocAsync((void **)&ws, total, s);
    if (e != cudaSuccess) return cuda_status(e, "split workspace");
  } else {
    if (!c->dwork.ensure(total)) return GSKS_ERR_ALLOC;
    ws = (uint8_t *)c->dwork.p;
  }
  Params *P = (Params *)(ws + o_params);
  double *centre = (double *)(ws + o_centre);
  long long *bbox = (long long *)(ws + o_bbox);

  // Per-pair relative error budget of a kernel value before its pair is
  // recomputed in FP64; random per-pair errors of this size keep the summed
  // result well inside 1e-6.
  const float tau = 5e-7f;
  bbox_init<<<1, 256, 0, s>>>(k, bbox);
  {
    const long long tot = (long long)(m + n) * k;
    const int blocks = (int)std::min<long long>(4LL * sms, std::max<long long>(1, (tot + 255) / 256));
    bbox_kernel<<<blocks, 256, 2 * k * sizeof(long long), s>>>(m, n, k, XA, amap, XB, bmap, bbox);
  }
  params_kernel<<<1, 1024, 0, s>>>(k, ker->type, ker->scal, ker->powe, tau, bbox, centre, P);
  pack_kernel<<<ntm, BM, 0, s>>>(0, m, k, kpad, XA, amap, nullptr, nullptr, hi, ker->type, centre, P, ws + o_a);
  pack_kernel<<<ntn, BN, 0, s>>>(1, n, k, kpad, XB, bmap, w, wmap, hj, ker->type, centre, P, ws + o_b);

  TileArgs a{};
  a.m = m; a.n = n; a.k = k; a.kpad = kpad; a.kt = ker->type;
  a.ntm = ntm; a.ntn = ntn; a.nsc = nsc; a.chunk_tiles = chunk_tiles;
  a.imgA = ws + o_a; a.imgB = ws + o_b;
  a.XA = XA; a.XB = XB; a.amap = amap; a.bmap = bmap; a.wmap = wmap; a.w = w;
  a.hi = hi; a.hj = hj;
  a.kp = make_kparams(ker, hi, hj);
  a.kp.coinc = coincidence_eps(k);
  a.P = P;
  a.partial = (double *)(ws + o_p);
  a.ldp = ldp;
  a.err = (int *)c->err.p;
  a.dump = tl_split_dump;
  if (tl_split_params) {
    cudaMemcpyAsync(tl_split_params, P, sizeof(Params), cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync((uint8_t *)tl_split_params + 64, centre, (size_t)k * 8, cudaMemcpyDeviceToDevice, s);
  }
  const int grid = std::min(ntm * nsc, sms);
  cudaError_t e = launch_tiles(a, grid, smem_bytes(kpad), s);
  if (e == cudaSuccess) {
    split_reduce<<<(m + 255) / 256, 256, 0, s>>>(m, nsc, ldp, a.partial, u, umap);
    e = cudaGetLastError();
  }
  if (stream_ordered_alloc) cudaFreeAsync(ws, s);
  if (e != cudaSuccess) return cuda_status(e, "split launch");
  note_launches(7);
  return GSKS_OK;
}

}  // namespace gsks

using namespace gsks;

// Test hook: one split-precision evaluation (device pointers, Gaussian-type
// inputs as gsks_dgsks_device) that also writes, for the first tile of CTA 0,
// the raw accumulators and epilogue values of every (row, column):
// dump[(row*128 + col)*5 + {0: H, 1: L, 2: K, 3: t, 4: lo}], and the call's
// scales to params_out (alpha, sigma, inv_sigma, q at byte 0; the centre, k
// doubles, at byte 64).
extern "C" int gsks_split_debug_dump(ks_t *kernel, int m, int n, int k, double *u, const int *umap,
                                     const double *XA, const int *amap, const double *XB, const int *bmap,
                                     const double *w, const int *wmap, float *dump, void *params_out,
                                     void *stream)
{
  Ctx *c = get_ctx();
  if (!c) return gsks_last_error();
  int st = check_kernel(kernel, k);
  if (st) return set_status(st, "gsks_split_debug_dump");
  tl_split_dump = dump;
  tl_split_params = params_out;
  st = enqueue_split(c, kernel, m, n, k, u, umap, XA, nullptr, amap, -1, XB, nullptr, bmap, -1, w, wmap,
                     kernel->hi, kernel->hj, (cudaStream_t)stream, true);
  tl_split_dump = nullptr;
  tl_split_params = nullptr;
  return set_status(st, "gsks_split_debug_dump");
}
