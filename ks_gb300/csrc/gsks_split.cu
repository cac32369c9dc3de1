// gsks_split.cu -- split-precision tensor-core form of the kernel summation.
//
// The rank-k inner products run on the 5th-generation tensor cores
// (tcgen05.mma, accumulators in TMEM); the kernel function runs in FP32; FP64
// is kept for the squared norms, for the distance of pairs flagged by an
// error bound, and for the per-target accumulation of u.
//
// Operand split (per call, pack_kernel):
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
// Epilogue (one thread per target row and 32-column group):
//   d2 = |x''|^2 + |y''|^2 - 2 x''.y'' assembled as an unevaluated FP32 sum
//   t + lo: the norms are split on a common grid so that their high parts add
//   exactly, -2 sigma^2 2^-14 H is exact, and Fast2Sum captures the last
//   rounding.  Gaussian-type values are 2^-t (1 - ln2 lo) with the SFU's ex2,
//   Laplace values come from a table-driven log2 with an exact integer
//   exponent.  Pairs whose distance an error bound says is not resolved
//   (Laplace near coincidence; narrow bandwidths relative to the data's extent)
//   are recomputed from the pool coordinates, and rows whose values over a
//   32-column group all fall below the FP32 range are redone in FP64.
// Row sums: FP32 within a 32-column group (4 interleaved partial sums), FP64
// across groups and tiles; one partial per (row, source chunk); a fixed-order
// reduction adds the partials into u (deterministic).
//
// Pipeline (one CTA per SM, persistent over work items = (target tile, run of
// source tiles)):
//   warp 0       producer: bulk copies (TMA engine) of the target tile image,
//                resident for the item when k <= 64 (3 source stages), else
//                both operands streamed in 64-wide k chunks (2 stages)
//   warp 1       MMA issuer: 6 tcgen05.mma per 16-wide k step into one of two
//                TMEM accumulator pairs (double buffered, 512 columns); the
//                whole warp runs the loop, one elected lane issues (the
//                epilogue warps of its SM sub-partition otherwise starve it
//                of issue slots and the tensor core idles)
//   warps 2..17  epilogue: 4 column groups x 4 TMEM sub-partitions, tcgen05.ld
//                of 16 columns at a time, kernel function, weighted row sums
// The batched form (KS_LIST) runs the same pipeline over a table of items
// from many tasks, each task with its own tiles, kernel and thresholds.
// Every wait is bounded; on a timeout the CTA records an error, drains and
// frees its tensor memory.
#include "gsks.h"
#include "gsks_internal.cuh"
#include "gsks_host.h"
#include "gsks_sm100.cuh"

#include <cuda_fp16.h>
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

namespace gsks {
namespace split {

using namespace sm100;

constexpr int BM = 128;             // targets per tile (TMEM lanes)
constexpr int BN = 128;             // sources per tile
constexpr int KPAD_MAX = 64;        // padded k of the target-resident kernel
constexpr int NSTAGE = 3;           // source-tile operand stages
constexpr int LTAB = 256;           // Laplace log2 table entries
constexpr size_t SMEM_MAX = 232448; // dynamic shared memory per block (227 KB)
constexpr int NMETA = 3;            // source-tile metadata ring
constexpr int NBLK = 3;             // slices per operand
constexpr int EPI_GROUPS = 4;          // column groups of the epilogue
constexpr int EPI_WARPS = 4 * EPI_GROUPS;
constexpr int NTHREADS = 32 * (2 + EPI_WARPS);
constexpr long long WAIT_LIMIT = 1LL << 32;   // clock cycles (~2 s) per wait
constexpr uint32_t TMEM_COLS = 512;           // 2 buffers x (H, L) x 128 columns

struct PtMeta {          // target tiles: 32 bytes per point, appended to the image
  float n_hi, n_lo;      // |x''|^2 = n_hi + n_lo, n_hi on the call's grid q
  float w;               // unused
  float h;               // var-bandwidth factor -0.5 log2e hi (gfast: the row factor)
  int pos;               // position in amap, -1 for padding
  int pad[3];            // [1] var-bandwidth: low part of h (float bits)
};

// Source tiles: the same 32 bytes per point as a structure of arrays, so that
// one 16-byte shared-memory load serves four columns of one field.
struct SrcMeta {
  float n_hi[BN], n_lo[BN];
  float w[BN];           // w[wmap[j]] (gfast: times the column's low-norm factor)
  float h[BN];           // var-bandwidth factor hj
  int pos[BN];           // position in bmap, -1 for padding
  float wsum[BN];        // column 32g: sum of |w| over columns 32g..32g+31
  float hlo[BN];         // var-bandwidth: low part of h
  int pad[BN];
};
static_assert(sizeof(SrcMeta) == BN * sizeof(PtMeta), "both metadata blocks take 32 bytes per point");

// Several right-hand sides in one sweep: up to RMAX weight columns per source,
// each kernel value multiplied by all of them.  Source tiles then carry 48
// bytes of metadata per point: the 32 of SrcMeta (w = column 0, wsum = the
// sum over columns of |w|), then the other columns' weights and a pad.
constexpr int RMAX = 4;
struct SrcMetaX {
  SrcMeta m;
  float wx[RMAX - 1][BN];
  float pad2[BN];
};
static_assert(sizeof(SrcMetaX) == BN * 48, "48 bytes per point with several right-hand sides");
__host__ __device__ constexpr size_t smeta_pt(int nr) { return nr > 1 ? 48 : 32; }
// Weights of column r of a source tile's metadata.
__device__ __forceinline__ const float *wrow(const SrcMeta *bm, int r)
{
  return r == 0 ? bm->w : reinterpret_cast<const SrcMetaX *>(bm)->wx[r - 1];
}

__device__ __forceinline__ float4 ld4(const float *p) { return *(const float4 *)p; }
__device__ __forceinline__ float f4(const float4 &v, int i) { return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w; }

// Laplace: K = scal d2^powe = 2^(log2 scal + powe log2 d2), powe = -P/2,
// log2 scal = ls13 2^-13 + lsf.
struct LapParam {
  int P, ls13;
  float lsf, mh;         // mh = -P/2
  float tover;           // d2 below tover: K may exceed the FP32 range
  int c0, p4096;         // ls13 + 127 P 4096 and P 4096: E = c0 - p4096 (bits >> 23) - P z
  int pad;
};

struct Params {          // per call, computed on the device
  double alpha, sigma, inv_sigma, q;
  double g;              // 2 sigma^2 2^-14: d2 = g (nu_i + nu_j - H - L)
  float rc;              // -g as a float
  float t_flag;          // flag pairs with t < t_flag ...
  float rho;             // ... or t < rho * (n_i + n_j)
  float nbmax;           // bound of every |x''|^2 (scaled units): n_j <= nbmax
  int centred;
  int any_flag;          // some pair may be flagged
  int exact_t1;          // nu_i + nu_j - H is exact in FP32
  int gfast;             // Gaussian without flags: low norm parts folded into w / row factors
  int ff_ok;             // coordinates within 2^50: float-pair rechecks stay in range
  LapParam lap;          // Laplace exponent constants
  double delta;          // absolute error bound of the assembled d2 (scaled units)
  // List form: the bounding box's largest half-extent and sum of squared
  // half-extents, centred (distance tasks) and uncentred (inner-product
  // tasks); each task's scale follows from them (task_params_kernel).
  double mx_c, sq_c, mx_u, sq_u;
  int k;
  // Polynomial kernels of integer power 1..4 (anch): each target row carries
  // an anchor v0 near its values v = cons + scal x.y; the epilogue sums
  // K - v0^p in FP32 and the reduction adds v0^p times the sum of the
  // weights in FP64.  sg = scal * g / 2 maps accumulator units to v.
  int anch;
  float sg;
  int pw;                // anch: the power
  double pscal, pcons;   // anch: the kernel's scal and cons
};

// Kernel selector of the batched (list) form: the epilogue dispatches on each
// task's type, with the task's own tile scale.
constexpr int KS_LIST = 99;

// Epilogue parameters of one task (a single call uses one, built from Params).
// The list form copies each item's entry into shared memory with the target
// tile (a bulk copy: 16-byte multiple).
struct __align__(16) TaskParam {
  KParams kp;
  float t_flag, rho;     // flag pairs with t < t_flag or t < rho * (n_i + n_j)
  float s2, s2l;         // Gaussian rechecks from pool coordinates: scal * log2(e) = s2 + s2l
  LapParam lap;          // Laplace
  int any_flag;
  int centred;           // distance kernels: coordinates taken relative to the centre
  float rc;              // -g of the task's scale (d2 = g (nu_i + nu_j - H - L))
  int exact;             // nu_i + nu_j - H is exact in FP32 at that scale
  // the task's tile images: coordinate -> slice units, sigma^2, g and the norm
  // grid q (list form; Gaussian tasks are scaled by their bandwidth)
  double sc, sig2, g, q;
  int gfast;             // Gaussian without flags: low norm parts folded (as Params::gfast)
  int anch;              // polynomial of power 1..4 summed around row anchors (as Params::anch)
  float sg;              // scal * g / 2 (anch)
  float nbmax;           // bound of every point's |x''|^2 at the task's scale (the flag test)
  double kcoin;          // Laplace: the value at coincident points (the reference's clamp), else 0
  double pad2;
};
static_assert(sizeof(TaskParam) % 16 == 0, "TaskParam is copied by the bulk-copy engine");

// Laplace: the value of a pair whose points coincide (d2 below 1e-15 in FP64
// takes the reference's clamp, d2 = 1.79e308, as recheck64 does).
__device__ __forceinline__ double lap_coincident(const KParams &kp)
{
  return pow_class(1.79e308, kp) * kp.scal;
}

// One work item of the list form: a target tile and a range of source tiles of
// one task; the rows' partial sums go to partial[out + row].
struct SplitItem {
  int a_tile, b0, b1, task;
  long long out;
  int rows, pad;
};

// One task of the list form as the row rescue sees it: its targets are list
// positions a0 .. a0 + m - 1, its sources b0 .. b0 + n - 1, and target row r's
// chunk sums sit at partial[pbase + c * m + r], c < nsc.
struct SplitTaskGeo {
  long long pbase;
  int a0, m, b0, n, nsc, pad;
};

__host__ __device__ inline size_t blk_bytes(int rows, int kpad) { return (size_t)rows * kpad * 2; }
// mpt: metadata bytes per point (32; 48 for source tiles of several right-hand sides)
__host__ __device__ inline size_t tile_bytes(int rows, int kpad, size_t mpt = sizeof(PtMeta))
{
  return NBLK * blk_bytes(rows, kpad) + (size_t)rows * mpt;
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
  size_t smeta;        // one source-metadata slot (BN points)
  int tab_sh;          // Laplace table: log2 of its copies (0 or 3), -1 without table
};
__host__ __device__ inline size_t smem_fixed(const SmemLayout &L);

// kt: the kernel selector (the Laplace table is sized for KS_LAPLACE and KS_LIST).
// The table is replicated eight times when it fits, one copy per bank group of
// a quarter warp, so that table lookups never conflict; the resident Laplace
// form then keeps two source stages instead of three (its epilogue, not the
// copies, sets the pace).
// nr: right-hand sides of the sweep (1, or RMAX: larger source metadata).
__host__ __device__ inline SmemLayout smem_layout(int kpad, int kt, int nr = 1)
{
  SmemLayout L;
  L.smeta = (size_t)BN * smeta_pt(nr);
  L.kc = kchunk(kpad);
  L.nch = kpad / L.kc;
  L.resident = (L.nch == 1);
  L.chunk_op = (size_t)NBLK * BM * L.kc * 2;
  L.chunk_al = (L.chunk_op + 1023) & ~(size_t)1023;
  const bool tab = kt == KS_LAPLACE || kt == KS_LIST;
  L.nstage = L.resident ? (tab ? 2 : NSTAGE) : 2;
  L.stage_bytes = L.resident ? L.chunk_al : 2 * L.chunk_al;
  L.a_region = L.resident ? ((tile_bytes(BM, kpad) + 1023) & ~(size_t)1023)
                          : (((size_t)BM * sizeof(PtMeta) + 1023) & ~(size_t)1023);
  L.tab_sh = -1;
  if (tab) {
    L.tab_sh = 3;
    if (smem_fixed(L) + ((size_t)LTAB << 3) * 16 > SMEM_MAX) L.tab_sh = 0;
  }
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

// Map entry -> pool index; an entry outside [0, npool) (npool >= 0) raises
// DEVERR_MAP_RANGE and reads point 0 instead.
__device__ __forceinline__ int pool_index(const int *map, int pos, int npool, int *err)
{
  int p = map ? map[pos] : pos;
  if (npool >= 0 && (p < 0 || p >= npool)) { atomicOr(err, DEVERR_MAP_RANGE); p = 0; }
  return p;
}

// Per-dimension min / max over the gathered targets and sources.  Every thread
// keeps one dimension (the grid-wide thread count is rounded down to a
// multiple of k; at least k threads are launched) and folds its points in
// registers; one shared and one global atomic per thread and bound.
__global__ void bbox_kernel(int m, int n, int k, const double *__restrict__ XA, const int *__restrict__ amap,
                            int nxa, const double *__restrict__ XB, const int *__restrict__ bmap, int nxb,
                            int *err, long long *bbox)
{
  extern __shared__ long long sb[];
  for (int p = threadIdx.x; p < k; p += blockDim.x) {
    sb[p] = 0x7FFFFFFFFFFFFFFFLL;
    sb[k + p] = (long long)0x8000000000000000ULL;
  }
  __syncthreads();
  const long long nthr = (long long)blockDim.x * gridDim.x;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long per = nthr / k;                      // points advanced per step
  if (tid < per * k) {
    const int p = (int)(tid % k);
    long long lo = 0x7FFFFFFFFFFFFFFFLL, hi = (long long)0x8000000000000000ULL;
#pragma unroll 4
    for (long long pt = tid / k; pt < (long long)m + n; pt += per) {
      double v;
      if (pt < m) v = XA[(size_t)pool_index(amap, (int)pt, nxa, err) * k + p];
      else v = XB[(size_t)pool_index(bmap, (int)(pt - m), nxb, err) * k + p];
      const long long key = dkey(v);
      lo = min(lo, key);
      hi = max(hi, key);
    }
    atomicMin(&sb[p], lo);
    atomicMax(&sb[k + p], hi);
  }
  __syncthreads();
  for (int p = threadIdx.x; p < k; p += blockDim.x) {
    atomicMin(&bbox[p], sb[p]);
    atomicMax(&bbox[k + p], sb[k + p]);
  }
}

__device__ LapParam lap_param(double scal, double powe)
{
  LapParam L;
  L.P = (int)rint(-2.0 * powe);
  const double ls = log2(scal);
  const double l13 = fmin(fmax(floor(ls * 8192.0), -0x1p30), 0x1p30);   // scal beyond the FP64 range: clamped
  L.ls13 = (int)l13;
  L.lsf = (float)(ls - l13 / 8192.0);
  L.mh = -0.5f * (float)L.P;
  const double mm = -powe;
  L.tover = (float)(pow(scal, 1.0 / mm) * exp2(-120.0 / mm) * 1.001);   // K = 2^120 at d2 = c0 2^(-120/m)
  L.c0 = L.ls13 + 127 * 4096 * L.P;
  L.p4096 = 4096 * L.P;
  L.pad = 0;
  return L;
}

// Centre, scales and the flag thresholds from the bounding box (one block).
// kt = KS_LIST: the list form, whose tasks mix centred (distance) and
// uncentred (inner-product) kernels: the centre is the box's, the scale covers
// the uncentred coordinates too, and the thresholds are set per task later.
__global__ void params_kernel(int k, int kt, double scal, double cons, double powe, float tau, const long long *bbox,
                              double *centre, Params *P)
{
  __shared__ double s_sq[1024], s_mx[1024], s_sqc[1024], s_mxc[1024];
  const bool dist = kt_uses_norms(kt);
  double sq = 0.0, mx = 0.0, sqc = 0.0, mxc = 0.0;
  for (int p = threadIdx.x; p < k; p += blockDim.x) {
    const double lo = dval(bbox[p]), hi = dval(bbox[k + p]);
    double c = 0.0, half;
    const double halfc = 0.5 * (hi - lo);
    if (kt == KS_LIST) { c = 0.5 * (lo + hi); half = fmax(fabs(lo), fabs(hi)); }
    else if (dist) { c = 0.5 * (lo + hi); half = halfc; }
    else half = fmax(fabs(lo), fabs(hi));
    centre[p] = c;
    sq += half * half;
    mx = fmax(mx, half);
    sqc += halfc * halfc;
    mxc = fmax(mxc, halfc);
  }
  s_sq[threadIdx.x] = sq; s_mx[threadIdx.x] = mx;
  s_sqc[threadIdx.x] = sqc; s_mxc[threadIdx.x] = mxc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {   // fixed-order tree: deterministic
    if ((int)threadIdx.x < s) {
      s_sq[threadIdx.x] += s_sq[threadIdx.x + s];
      s_mx[threadIdx.x] = fmax(s_mx[threadIdx.x], s_mx[threadIdx.x + s]);
      s_sqc[threadIdx.x] += s_sqc[threadIdx.x + s];
      s_mxc[threadIdx.x] = fmax(s_mxc[threadIdx.x], s_mxc[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    P->k = k;
    P->mx_c = s_mxc[0]; P->sq_c = s_sqc[0];
    P->mx_u = s_mx[0]; P->sq_u = s_sq[0];
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
    P->delta = delta;
    float t_flag = -1.0f, rho = 0.0f;
    if (kt == KS_GAUSSIAN) {
      // relative error of 2^-d2 is ln2 * delta; pairs with t >= 126 underflow anyway
      if (delta * 0.6931471805599453 > tau) t_flag = 126.0f;
    } else if (kt == KS_GAUSSIAN_VAR_BANDWIDTH) {
      // relative error of 2^(f d2) is ln2 f delta: pairs with a bandwidth
      // product f above this cap (and no underflow) are rechecked
      t_flag = (float)(tau / (0.6931471805599453 * delta));
    } else if (kt == KS_LAPLACE) {
      rho = 0x1p-10f;                         // coincident points and near-cancellation
      t_flag = (float)(fabs(powe) * delta / tau);
      // K stays below 2^120 for d2 above c0 2^(-120/m), c0 = scal^(1/m)
      const double mm = -powe, c0 = pow(scal, 1.0 / mm);
      t_flag = fmaxf(t_flag, (float)(c0 * exp2(-120.0 / mm) * 1.001));
      P->lap = lap_param(scal, powe);
    } else if (dist) {
      rho = 0.0f;                             // compact / polynomial in d2: absolute error only
    }
    P->t_flag = t_flag; P->rho = rho;
    P->nbmax = (float)(nbound * (1.0 + 0x1p-20));
    P->any_flag = (t_flag > 0.0f || rho > 0.0f) ? 1 : 0;
    // |x''|^2 + |y''|^2 lies on the grid q and -2 sigma^2 2^-14 H on the grid
    // 2 sigma^2 2^-14; when the latter is a multiple of q their sum is exact
    // (it stays below 2^24 q), and only the small L term needs Fast2Sum.
    P->exact_t1 = (q <= 2.0 * sigma * sigma * 0x1p-14) ? 1 : 0;
    P->gfast = (kt == KS_GAUSSIAN && P->exact_t1 && !P->any_flag) ? 1 : 0;
    P->ff_ok = (s_mx[0] <= 0x1p50) ? 1 : 0;
    P->anch = ((kt == KS_POLYNOMIAL && powe == rint(powe) && powe >= 1.0 && powe <= 4.0) || kt == KS_TANH ||
               kt == KS_QUARTIC || kt == KS_MULTIQUADRATIC || kt == KS_EPANECHNIKOV) ? 1 : 0;
    P->sg = (float)(scal * 0.5 * P->g);
    P->pw = (int)powe;
    P->pscal = scal;
    P->pcons = cons;
  }

}

// Per task of the list form, the per-dimension min and max (ordered keys)
// over its targets (XA through a_idx) and sources (XB through b_idx):
// tbox[t][0][p], tbox[t][1][p]; each task's box is also folded into the
// global one (bbox, from bbox_init) with one atomic per dimension and bound.
// One block per task, the threads over (dimension, stride of points).
__global__ void __launch_bounds__(256) list_box_kernel(int ntask, int k, const SplitTaskGeo *__restrict__ tg,
                                                       const double *__restrict__ XA, const int *__restrict__ a_idx,
                                                       int nxa, const double *__restrict__ XB,
                                                       const int *__restrict__ b_idx, int nxb, int *err,
                                                       long long *__restrict__ tbox, long long *__restrict__ bbox)
{
  __shared__ long long slo[256], shi[256];
  const int t = blockIdx.x;
  if (t >= ntask) return;
  const SplitTaskGeo G = tg[t];
  const int npts = G.m + G.n, tid = threadIdx.x;
  for (int p0 = 0; p0 < k; p0 += blockDim.x) {
    const int cols = min((int)blockDim.x, k - p0);
    const int sub = blockDim.x / cols;
    const int c = tid % cols, grp = tid / cols;
    long long lo = 0x7FFFFFFFFFFFFFFFLL, hi = (long long)0x8000000000000000ULL;
    if (grp < sub) {
      const int p = p0 + c;
      for (int q = grp; q < npts; q += sub) {
        const double v = q < G.m ? XA[(size_t)pool_index(a_idx, G.a0 + q, nxa, err) * k + p]
                                 : XB[(size_t)pool_index(b_idx, G.b0 + q - G.m, nxb, err) * k + p];
        const long long key = dkey(v);
        lo = min(lo, key);
        hi = max(hi, key);
      }
    }
    slo[tid] = lo;
    shi[tid] = hi;
    __syncthreads();
    if (tid < cols) {
      for (int q = 1; q < sub; q++) { lo = min(lo, slo[q * cols + tid]); hi = max(hi, shi[q * cols + tid]); }
      tbox[(size_t)t * 2 * k + p0 + tid] = lo;
      tbox[(size_t)t * 2 * k + k + p0 + tid] = hi;
      if (npts > 0) {
        atomicMin(&bbox[p0 + tid], lo);
        atomicMax(&bbox[k + p0 + tid], hi);
      }
    }
    __syncthreads();
  }
}

// Per-task parameters of the list form: the scale of the task's tile images
// and the flag thresholds, by the rules of params_kernel with the task's own
// kernel.  Distance tasks take the centred box, inner-product tasks the
// uncentred one; Gaussian tasks fold their bandwidth into the coordinates
// (scaled units, as a single call), the others keep them unscaled.
//
// Every task takes its own box (tbox: ordered keys of the per-dimension min
// and max over the task's targets and sources, list_box_kernel): distance
// tasks are centred on the box's centre (tcen[t k + p], written here), and
// the scale follows the task's own extent, so that spatially local tasks (a
// tree code's near-field blocks) keep a small distance error bound however
// far they lie from the other tasks.
__global__ void task_params_kernel(int ntask, const KParams *__restrict__ kps, const Params *__restrict__ P,
                                   float tau, TaskParam *__restrict__ out, const long long *__restrict__ tbox,
                                   double *__restrict__ tcen)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntask) return;
  const KParams kp = kps[t];
  const bool centred = kt_uses_norms(kp.type);
  const double s2 = kp.scal * 1.4426950408889634;
  const double alpha = kp.type == KS_GAUSSIAN ? sqrt(fmax(-s2, 0.0)) : 1.0;
  double mx_c = 0.0, sq_c = 0.0, mx_u = 0.0, sq_u = 0.0;
  {
    const int k = P->k;
    const long long *lo = tbox + (size_t)t * 2 * k, *hi = lo + k;
    const bool empty = lo[0] > hi[0];   // a task without points (no items either)
    for (int p = 0; p < k; p++) {
      const double a = empty ? 0.0 : dval(lo[p]), b = empty ? 0.0 : dval(hi[p]);
      const double hc = 0.5 * (b - a), hu = fmax(fabs(a), fabs(b));
      tcen[(size_t)t * k + p] = 0.5 * (a + b);
      mx_c = fmax(mx_c, hc); sq_c += hc * hc;
      mx_u = fmax(mx_u, hu); sq_u += hu * hu;
    }
  }
  const double maxabs = alpha * (centred ? mx_c : mx_u);
  double sigma = maxabs > 0.0 ? exp2(ceil(log2(maxabs))) : 1.0;
  if (sigma < maxabs) sigma *= 2.0;
  const double nbound = alpha * alpha * (centred ? sq_c : sq_u);
  const double q = exp2(ceil(log2(2.0 * nbound + 1e-300)) - 23.0);
  const double g = 2.0 * sigma * sigma * 0x1p-14;
  const int k = P->k;
  const double delta = 2.0 * (sigma * sigma * (double)k * 0x1p-31) +
                       2.0 * sigma * sqrt((double)k) * sqrt(nbound) * 0x1p-30 + 2.0 * q * 0x1p-23;
  TaskParam T;
  T.kp = kp;
  T.t_flag = -1.0f; T.rho = 0.0f; T.s2 = T.s2l = 0.0f; T.lap = LapParam{0, 0, 0.f, 0.f, 0.f, 0, 0, 0};
  T.centred = centred ? 1 : 0;
  T.sc = alpha / sigma * 128.0;
  T.sig2 = sigma * sigma;
  T.g = g;
  T.q = q;
  T.rc = (float)(-g);
  T.exact = (q <= g) ? 1 : 0;
  T.gfast = 0;
  T.anch = ((kp.type == KS_POLYNOMIAL && kp.pmode == POW_INT && kp.pint >= 1 && kp.pint <= 4) ||
            kp.type == KS_TANH) ? 1 : 0;
  T.sg = (float)(kp.scal * 0.5 * g);
  T.nbmax = (float)(nbound * (1.0 + 0x1p-20));
  if (kp.type == KS_GAUSSIAN) {
    T.s2 = (float)s2;                      // the rechecks work from the pool coordinates
    T.s2l = (float)(s2 - (double)T.s2);
    // scaled units: the relative error of 2^-d2 is ln2 delta; pairs with
    // d2 >= 126 underflow anyway
    if (0.6931471805599453 * delta > tau) T.t_flag = 126.0f;
    T.gfast = (T.exact && T.t_flag < 0.0f) ? 1 : 0;
  } else if (kp.type == KS_GAUSSIAN_VAR_BANDWIDTH) {
    T.t_flag = (float)(tau / (0.6931471805599453 * delta));   // cap on f, as params_kernel
  } else if (kp.type == KS_LAPLACE) {
    T.rho = 0x1p-10f;
    T.t_flag = (float)(fabs(kp.powe) * delta / tau);
    const double mm = -kp.powe, c0 = pow(kp.scal, 1.0 / mm);
    T.t_flag = fmaxf(T.t_flag, (float)(c0 * exp2(-120.0 / mm) * 1.001));
    T.lap = lap_param(kp.scal, kp.powe);
  }
  T.kcoin = kp.type == KS_LAPLACE ? lap_coincident(kp) : 0.0;
  T.pad2 = 0.0;
  T.any_flag = (T.t_flag > 0.0f || T.rho > 0.0f) ? 1 : 0;
  out[t] = T;
}

// Float-pair copy of n / k points: Xf[i] = (hi, lo), hi + lo = the
// coordinate to 2^-48.  Without a map, of the pool's first points; with one
// (a single call's gathered rows), row r of the copy is pool point map[r]
// (entries outside [0, npool), npool >= 0, read point 0).  With P != nullptr
// (a single call) only when the call may flag pairs.
__global__ void pool_split(long long n, int k, const double *__restrict__ X, const int *__restrict__ map, int npool,
                           float2 *__restrict__ Xf, const Params *P)
{
  if (P && !P->any_flag) return;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)blockDim.x * gridDim.x) {
    size_t src = (size_t)i;
    if (map) {
      const long long r = i / k;
      int p = map[r];
      if (npool >= 0 && (p < 0 || p >= npool)) p = 0;
      src = (size_t)p * k + (size_t)(i - r * k);
    }
    const double v = X[src];
    const float h = (float)v;
    Xf[i] = make_float2(h, (float)(v - (double)h));
  }
}

// Sums over the sources j0 .. j1-1 of every coordinate (ysum[p] = inv_n times
// the sum, p < k) and of the weights (*wsum), in FP64 and in a fixed order:
// the block's threads take the k + 1 columns in passes, each column split
// over equal strided groups of sources, the groups then added in order.
// sh: blockDim.x doubles of shared memory.
__device__ void block_source_sums(int j0, int j1, int k, const double *__restrict__ X,
                                  const int *__restrict__ map, int npool, int *err,
                                  const double *__restrict__ w, const int *__restrict__ wmap, double inv_n,
                                  double *ysum, double *wsum, double *sh)
{
  const int kk = k + 1, t = threadIdx.x;
  for (int p0 = 0; p0 < kk; p0 += blockDim.x) {
    const int cols = min((int)blockDim.x, kk - p0);
    const int sub = blockDim.x / cols;           // threads per column
    const int c = t % cols, grp = t / cols;
    double s = 0.0;
    if (grp < sub) {
      const int p = p0 + c;
      for (int j = j0 + grp; j < j1; j += sub)
        s += p < k ? X[(size_t)pool_index(map, j, npool, err) * k + p] : w[wmap ? wmap[j] : j];
    }
    sh[t] = s;
    __syncthreads();
    if (t < cols) {
      double r = 0.0;
      for (int q = 0; q < sub; q++) r += sh[q * cols + t];
      if (p0 + t < k) ysum[p0 + t] = r * inv_n;
      else *wsum = r;
    }
    __syncthreads();
  }
}

// Anchor point of a single call's polynomial, tanh and compact / multiquadratic
// kernels (the sources' mean and mean squares per coordinate) and the sum of
// all weights.  Any point inside the sources' hull keeps each row's anchor
// value within the range of that row's values, so the mean of a strided
// sample of at most ANCHOR_SAMPLE sources serves: anchor_coords blocks (cb,
// sb) take 32 coordinates of ANCHOR_SB-th of the sample each.  The weight sum
// covers every source (anchor_weights: contiguous ranges, fixed-order tree).
// anchor_final adds the partials in order.  All of it deterministic.
constexpr int ANCHOR_SAMPLE = 2048;
constexpr int ANCHOR_SB = 16;       // sample blocks of anchor_coords
constexpr int ANCHOR_WPER = 4096;   // weights per block of the weight sum

// cpart[(sb * 2 + 0) * k + p]: sum of coordinate p over sample block sb;
// cpart[(sb * 2 + 1) * k + p]: the sum of its squares.
__global__ void __launch_bounds__(256) anchor_coords(int n, int k, const double *__restrict__ XB,
                                                     const int *__restrict__ bmap, int nxb, int *err,
                                                     double *__restrict__ cpart)
{
  __shared__ double sh[2][256];
  const int t = threadIdx.x, lane = t & 31, wp = t >> 5;
  const int S = min(n, ANCHOR_SAMPLE), stride = n / S;
  const int per = (S + ANCHOR_SB - 1) / ANCHOR_SB;
  const int q0 = blockIdx.y * per, q1 = min(S, q0 + per);
  const int p = blockIdx.x * 32 + lane;
  double s = 0.0, s2 = 0.0;
  if (p < k) {
#pragma unroll 8
    for (int q = q0 + wp; q < q1; q += 8) {
      const double y = XB[(size_t)pool_index(bmap, q * stride, nxb, err) * k + p];
      s += y;
      s2 = fma(y, y, s2);
    }
  }
  sh[0][t] = s;
  sh[1][t] = s2;
  __syncthreads();
  if (wp == 0 && p < k) {
    double r = 0.0, r2 = 0.0;
    for (int q = 0; q < 8; q++) { r += sh[0][q * 32 + lane]; r2 += sh[1][q * 32 + lane]; }
    cpart[((size_t)blockIdx.y * 2 + 0) * k + p] = r;
    cpart[((size_t)blockIdx.y * 2 + 1) * k + p] = r2;
  }
}

// wpart[b * nrhs + r]: the sum of weight column r over sources b ANCHOR_WPER ..
__global__ void __launch_bounds__(256) anchor_weights(int n, const double *__restrict__ w,
                                                      const int *__restrict__ wmap, int nrhs,
                                                      double *__restrict__ wpart)
{
  __shared__ double sh[256];
  const int t = threadIdx.x, b = blockIdx.x;
  const int j0 = b * ANCHOR_WPER, j1 = min(n, j0 + ANCHOR_WPER);
  for (int r = 0; r < nrhs; r++) {
    double s = 0.0;
    for (int j = j0 + t; j < j1; j += 256) s += w[(size_t)(wmap ? wmap[j] : j) * nrhs + r];
    sh[t] = s;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
      if (t < h) sh[t] += sh[t + h];
      __syncthreads();
    }
    if (t == 0) wpart[(size_t)b * nrhs + r] = sh[0];
    __syncthreads();
  }
}

// ybar[p], ybsq[p]: the sample's mean and mean square of coordinate p;
// wsum[r]: the sum of weight column r.
__global__ void anchor_final(int n, int k, int nwb, int nrhs, const double *__restrict__ cpart,
                             const double *__restrict__ wpart, double *__restrict__ ybar,
                             double *__restrict__ ybsq, double *__restrict__ wsum)
{
  const double inv = 1.0 / (double)min(n, ANCHOR_SAMPLE);
  for (int p = threadIdx.x; p < k; p += blockDim.x) {
    double a = 0.0, b = 0.0;
    for (int sb = 0; sb < ANCHOR_SB; sb++) {
      a += cpart[((size_t)sb * 2 + 0) * k + p];
      b += cpart[((size_t)sb * 2 + 1) * k + p];
    }
    ybar[p] = a * inv;
    ybsq[p] = b * inv;
  }
  for (int r = threadIdx.x; r < nrhs; r += blockDim.x) {
    double a = 0.0;
    for (int b = 0; b < nwb; b++) a += wpart[(size_t)b * nrhs + r];
    wsum[r] = a;
  }
}

// The same per task of the list form (one block per task; tasks that are not
// anchored, or empty, are skipped): ybar[t * k ..] and wsum[t].
__global__ void list_anchor(int ntask, int k, const TaskParam *__restrict__ tp, const SplitTaskGeo *__restrict__ tg,
                            const double *__restrict__ XB, const int *__restrict__ b_idx, int nxb,
                            const double *__restrict__ w, const int *__restrict__ w_idx, int *err,
                            double *__restrict__ ybar, double *__restrict__ wsum)
{
  extern __shared__ double sh_sum[];
  const int t = blockIdx.x;
  if (t >= ntask || !tp[t].anch || tg[t].n <= 0 || tg[t].m <= 0) return;
  const SplitTaskGeo G = tg[t];
  block_source_sums(G.b0, G.b0 + G.n, k, XB, b_idx, nxb, err, w, w_idx, 1.0 / (double)G.n,
                    ybar + (size_t)t * k, wsum + t, sh_sum);
}

// Tile images: per tile, NBLK slice blocks in the no-swizzle K-major core-matrix
// layout (element (r, p) at (p/8)*rows*16 + r*16 + (p%8)*2 bytes), then the
// point metadata.  One thread per point.
// List form (tiles != nullptr): tile t packs positions tiles[t].x ..
// tiles[t].x + tiles[t].y - 1 of the CSR list `map`, for task tile_task[t].
__global__ void pack_kernel(int side, int npts, int k, int kpad, const double *__restrict__ X,
                            const int *__restrict__ map, int npool, int *err, const double *__restrict__ w,
                            const int *__restrict__ wmap, const double *__restrict__ hvec, int kt,
                            const double *__restrict__ centre, const Params *__restrict__ P,
                            uint8_t *__restrict__ img, const int2 *__restrict__ tiles,
                            const int *__restrict__ tile_task, const TaskParam *__restrict__ tp,
                            const double *__restrict__ ybar, double *__restrict__ rowc, int nrhs = 1,
                            const double *__restrict__ ybsq = nullptr)
{
  // nrhs > 1 (sources of several right-hand sides): w holds nrhs interleaved
  // columns and the tiles carry RMAX weights per point (SrcMetaX)
  const int tile = blockIdx.x, r = threadIdx.x;
  int pt = tile * BM + r;
  bool valid = pt < npts;
  bool centred = P->centred != 0;
  if (tiles) {
    const int2 tl = tiles[tile];
    const TaskParam &T = tp[tile_task[tile]];
    pt = tl.x + r;
    valid = r < tl.y;
    centred = T.centred != 0;
    kt = T.kp.type;
    hvec = side == 0 ? T.kp.hi : T.kp.hj;
  }
  const int pidx = valid ? pool_index(map, pt, npool, err) : 0;
  const double *x = X + (size_t)pidx * k;
  // the centre: the call's, or (list form) the task's own (centre + task k)
  const double *cen = tiles ? centre + (size_t)tile_task[tile] * k : centre;
  // coordinate -> slice units: the call's scale, or the list task's
  const TaskParam *TT = tiles ? &tp[tile_task[tile]] : nullptr;
  const double sc = TT ? TT->sc : P->alpha * P->inv_sigma * 128.0;
  const double sig2 = TT ? TT->sig2 : P->sigma * P->sigma;
  const bool gfast = TT ? TT->gfast != 0 : P->gfast != 0;
  uint8_t *base = img + (size_t)tile * tile_bytes(BM, kpad, side == 1 ? smeta_pt(nrhs > 1 ? RMAX : 1) : sizeof(PtMeta));
  const size_t bb = blk_bytes(BM, kpad);
  // The norm of the represented point restricted to the products the tensor
  // cores form (a1a1 + 2a1a2 + a2a2 + 2a1a3), so that the assembled d2 of
  // identical points is 0 up to the FP32 accumulations.  Every term is an
  // integer multiple of 2^-48 (halves are multiples of 2^-24): summed exactly
  // in integers, a1a1 at scale 1, 2a1(a2 + a3) at 2^24, a2a2 at 2^48.  FP64
  // instructions issue slowly here; the slicing uses six per coordinate.
  int n_i = 0;
  long long n_a = 0, n_b = 0;
  for (int kg = 0; kg < kpad / 8; kg++) {
    __align__(16) __half s1[8], s2[8], s3[8];
#pragma unroll
    for (int e = 0; e < 8; e++) {
      const int p = kg * 8 + e;
      float a1 = 0.0f;
      __half h2 = __float2half_rn(0.0f), h3 = __float2half_rn(0.0f);
      if (valid && p < k) {
        const double t = (centred ? x[p] - cen[p] : x[p]) * sc;   // the difference is exact near the centre
        a1 = rintf((float)t);                          // |a1| <= 128
        const float r1 = (float)(t - (double)a1);      // |r1| <= 1/2 (+ a rounding at ties)
        h2 = __float2half_rn(r1);
        h3 = __float2half_rn(r1 - __half2float(h2));   // the difference is exact in FP32
        const int ia = (int)a1;
        const int F2 = (int)(__half2float(h2) * 16777216.0f), F3 = (int)(__half2float(h3) * 16777216.0f);
        n_i += ia * ia;
        n_a += (long long)(2 * ia) * (F2 + F3);
        n_b += (long long)F2 * F2;
      }
      s1[e] = __float2half_rn(a1);                     // exact
      s2[e] = h2;
      s3[e] = h3;
    }
    *(uint4 *)(base + img_off(0, kg, r, kpad)) = *(const uint4 *)s1;
    *(uint4 *)(base + img_off(1, kg, r, kpad)) = *(const uint4 *)s2;
    *(uint4 *)(base + img_off(2, kg, r, kpad)) = *(const uint4 *)s3;
  }
  const double nrm = ((double)n_i + (double)n_a * 0x1p-24 + (double)n_b * 0x1p-48) * (1.0 / 16384.0);
  (void)bb;
  // The norm in units of the accumulators: nu = |x''|^2 / g with
  // g = 2 sigma^2 2^-14, so that d2 = g (nu_i + nu_j - H - L).  nu is split on
  // the grid q / g (a power of two): its high parts and H add exactly.
  const double g = TT ? TT->g : P->g;
  const double nu = nrm * sig2 / g;
  const double qg = (TT ? TT->q : P->q) / g;
  const double nh = rint(nu / qg) * qg;
  const double nl = nu - nh;
  PtMeta mt;
  mt.n_hi = (float)nh;
  mt.n_lo = (float)nl;
  mt.w = 0.0f;
  mt.h = 0.0f;
  const size_t wi = valid ? (size_t)(wmap ? wmap[pt] : pt) * (nrhs > 1 ? nrhs : 1) : 0;   // weight column 0
  double wf = 1.0;                 // the Gaussian fast path's source factor
  if (side == 1 && valid) mt.w = (float)w[wi];
  if (gfast) {
    // Gaussian: 2^-(g nl) is a per-point factor; fold it into w for sources
    // and into a row factor for targets (applied to the row sum)
    const double f = exp2(-g * nl);
    mt.n_lo = 0.0f;
    if (side == 1) { mt.w = valid ? (float)(w[wi] * f) : 0.0f; wf = f; }
    else mt.h = (float)f;
  }
  mt.pos = valid ? pt : -1;
  mt.pad[0] = mt.pad[1] = mt.pad[2] = 0;
  if (kt == KS_GAUSSIAN_VAR_BANDWIDTH && valid) {
    // the factor as a float pair h + pad[1]: an FP32 factor alone would put a
    // relative error of 2^-24 on exponents of up to 126
    const double hv = side == 0 ? -0.5 * 1.4426950408889634 * hvec[pidx] : hvec[pidx];
    mt.h = (float)hv;
    mt.pad[1] = __float_as_int((float)(hv - (double)mt.h));
  }
  const bool anch = side == 0 && (TT ? TT->anch != 0 : P->anch != 0);
  if (anch) {
    // Polynomial and tanh rows summed around an anchor: H0 = x.ybar in
    // accumulator units (x.y = (g/2)(H + L)), rounded to an integer so that
    // H - H0 is exact, and v0 = cons + scal (g/2) H0; the row keeps H0 (n_hi)
    // and, for the polynomial, the binomial coefficients c_i = C(p, i)
    // v0^(p-i), i = 1..p-1 (n_lo, w, h), rowc v0^p in FP64; for tanh, t0 =
    // tanh(v0) and 1 - t0^2 (n_lo, w), rowc t0 in FP64.  Padding rows: zero.
    if (kt_uses_norms(kt)) {
      // Compact and multiquadratic kernels (functions of d2): the anchor is
      // d0^2 = |x - ybar|^2 + mean |y - ybar|^2, the rows' mean squared
      // distance to the sources; the row keeps d0^2 (w), K(d0^2) in FP32 (h)
      // and 1 - d0^2 (pad[0]); rowc gets K(d0^2) in FP64.  The norms stay.
      mt.w = mt.h = 0.0f;
      mt.pad[0] = 0;
      if (valid) {
        double d0 = 0.0;
        for (int p = 0; p < k; p++) {
          const double dx = x[p] - ybar[p];
          d0 = fma(dx, dx, d0) + (ybsq[p] - ybar[p] * ybar[p]);
        }
        const double c = 1.0 - d0;
        double K0;
        if (kt == KS_QUARTIC) K0 = d0 < 1.0 ? (15.0 / 16.0) * c * c : 0.0;
        else if (kt == KS_EPANECHNIKOV) K0 = d0 < 1.0 ? 0.75 * c : 0.0;
        else K0 = d0 + (TT ? TT->kp.cons : P->pcons);
        mt.w = (float)d0;
        mt.h = (float)K0;
        mt.pad[0] = __float_as_int((float)c);
        rowc[pt] = K0;
      }
    } else {
    mt.n_hi = mt.n_lo = mt.w = mt.h = 0.0f;
    if (valid) {
      const double *yb = ybar + (TT ? (size_t)tile_task[tile] * k : 0);
      double A = 0.0;
      for (int p = 0; p < k; p++) A = fma(x[p], yb[p], A);
      const double G = 0.5 * g;
      const double H0 = fmin(fmax(rint(A / G), -0x1p24), 0x1p24);
      const double scal = TT ? TT->kp.scal : P->pscal, cons = TT ? TT->kp.cons : P->pcons;
      const int pw = TT ? TT->kp.pint : P->pw;
      const double v0 = fma(scal * G, H0, cons);
      const double v2 = v0 * v0;
      double c1 = 1.0, c2 = 0.0, c3 = 0.0, vp = v0;
      if (kt == KS_TANH) { vp = tanh(v0); c1 = vp; c2 = 1.0 - vp * vp; c3 = v0; }
      else if (pw == 2) { c1 = 2.0 * v0; vp = v2; }
      else if (pw == 3) { c1 = 3.0 * v2; c2 = 3.0 * v0; vp = v2 * v0; }
      else if (pw == 4) { c1 = 4.0 * v2 * v0; c2 = 6.0 * v2; c3 = 4.0 * v0; vp = v2 * v2; }
      mt.n_hi = (float)H0;
      mt.n_lo = (float)c1;
      mt.w = (float)c2;
      mt.h = (float)c3;
      rowc[pt] = vp;
    }
    }
  }
  if (side == 0) {
    ((PtMeta *)(base + NBLK * bb))[r] = mt;
    return;
  }
  // sources: sum of |w| (over the weight columns) over each group of 32
  // columns, kept with the group's first column (the underflow test of the
  // exponential kernels)
  float wa = fabsf(mt.w);
  SrcMeta *sm = (SrcMeta *)(base + NBLK * bb);
  if (nrhs > 1) {
    SrcMetaX *sx = (SrcMetaX *)sm;
    for (int c = 1; c < RMAX; c++) {
      const float wc = (valid && c < nrhs) ? (float)(w[wi + c] * wf) : 0.0f;
      sx->wx[c - 1][r] = wc;
      wa += fabsf(wc);
    }
    sx->pad2[r] = 0.0f;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) wa += __shfl_xor_sync(0xffffffffu, wa, o);
  sm->n_hi[r] = mt.n_hi; sm->n_lo[r] = mt.n_lo; sm->w[r] = mt.w; sm->h[r] = mt.h;
  sm->pos[r] = mt.pos;
  sm->wsum[r] = (r & 31) == 0 ? wa : 0.0f;
  sm->hlo[r] = __int_as_float(mt.pad[1]);
  sm->pad[r] = 0;
}

// ---------------------------------------------------------------------------
struct TileArgs {
  int m, n, k, kpad, kt;
  int ntm, ntn, nsc, chunk_tiles;   // items = ntm * nsc; chunk = source tiles per item
  const uint8_t *imgA, *imgB;
  const double *XA, *XB;            // pool coordinates (FP64) for the rechecks
  const float2 *XAf, *XBf;          // float-pair copies for the rechecks (or nullptr)
  int ffpos;                        // the copies are indexed by position (else by pool point)
  unsigned long long *nrecheck;     // count of rechecked pairs (or nullptr)
  int nrhs;                         // interleaved columns of u and w (the FP64 weights of the rechecks)
  const int *amap, *bmap, *wmap;
  int nxa, nxb;                     // pool sizes for the map range checks (-1: unchecked)
  const double *w;
  const double *hi, *hj;
  KParams kp;                       // FP64 descriptor for the rechecks
  const Params *P;
  double *partial;                  // [nsc][ldp]
  float *pskip;                     // W sums of the groups left to the row rescue (the partial layout)
  int ldp;
  int *err;
  long long wait_limit;             // clock cycles before a wait gives up
  int stall;                        // test hook: the producer issues nothing (the waits run out)
  // list form: explicit work items and per-task parameters (nullptr otherwise)
  const SplitItem *tab;
  int ntab;
  const TaskParam *tp;
  const int *btile_cols;            // valid columns of each source tile
  int *next_item;                   // work counter (zero at launch): items after the first gridDim.x
};

// Geometry of work item `item`: target tile, source-tile range, task, the
// partial offset of row 0 and the number of valid rows.
struct ItemGeo {
  int ti, t0, t1, task, rows;
  long long out;
};
__device__ __forceinline__ ItemGeo item_geo(const TileArgs &a, int item)
{
  ItemGeo g;
  if (a.tab) {
    const SplitItem it = a.tab[item];
    g.ti = it.a_tile; g.t0 = it.b0; g.t1 = it.b1; g.task = it.task; g.out = it.out; g.rows = it.rows;
  } else {
    g.ti = item % a.ntm;
    const int sc = item / a.ntm;
    g.t0 = sc * a.chunk_tiles;
    g.t1 = min(a.ntn, g.t0 + a.chunk_tiles);
    g.task = 0;
    g.out = (long long)sc * a.ldp + (long long)g.ti * BM;
    g.rows = min(BM, a.m - g.ti * BM);
  }
  return g;
}

struct SplitSmem {
  uint64_t a_full, a_empty;
  uint64_t b_full[NSTAGE], b_empty[NSTAGE];
  uint64_t m_full[NMETA], m_empty[NMETA];
  uint64_t t_full[2], t_empty[2];
  uint64_t r_full[2], r_empty[2];       // row-sum exchange of the epilogue groups, by item parity
  uint64_t drain;
  uint32_t tmem_base;
  int abort;
  int never;             // stays 0: an abort flag for the drain waits
  double rsum[2][EPI_GROUPS - 1][BM];   // row sums of epilogue groups 1.., by item parity
  float rskip[2][EPI_GROUPS - 1][BM];   // their skipped-group weights (pskip)
  float rq[EPI_WARPS][32];              // per epilogue warp: recheck values (recheck_warp)
  TaskParam tslot[2];    // list form: the current items' task parameters, by item parity
  int islot[2];          // the current items (-1: no work left), by item parity
};


// Shared memory without the Laplace table (which follows SplitSmem).
__host__ __device__ inline size_t smem_fixed(const SmemLayout &L)
{
  return 1024 /* alignment slack */ + L.a_region + L.nstage * L.stage_bytes + NMETA * L.smeta + sizeof(SplitSmem) +
         64;
}

// The largest non-table layout (resident k = KPAD_MAX, NSTAGE source stages)
// fits the shared memory of a block.
static_assert(1024 + ((NBLK * (size_t)BM * KPAD_MAX * 2 + (size_t)BM * sizeof(PtMeta) + 1023) & ~(size_t)1023) +
                      NSTAGE * ((NBLK * (size_t)BM * KPAD_MAX * 2 + 1023) & ~(size_t)1023) +
                      NMETA * (size_t)BN * sizeof(PtMeta) + sizeof(SplitSmem) + 64 <= SMEM_MAX,
              "split_tiles shared memory");
// The streaming layout (k beyond KPAD_MAX: two stages of both operands' 64-wide
// chunks) with one copy of the Laplace table (the list form) fits too.
static_assert(1024 + (((size_t)BM * sizeof(PtMeta) + 1023) & ~(size_t)1023) +
                      2 * 2 * ((NBLK * (size_t)BM * KCH * 2 + 1023) & ~(size_t)1023) +
                      NMETA * (size_t)BN * sizeof(PtMeta) + sizeof(SplitSmem) + 64 + ((sizeof(SplitSmem) + 15) & 15) +
                      (size_t)LTAB * 16 <= SMEM_MAX,
              "split_tiles shared memory (streaming, table)");

template <int KT>
__device__ __forceinline__ const TaskParam &pick_task(const TaskParam &slot, const TaskParam &single)
{
  if constexpr (KT == KS_LIST) return slot;
  else return single;
}


// Laplace table: for i in [0, 256), c_i ~ 1 / (1 + (i + 1/2) / 256) with 12
// significant bits (so that r = f c_i - 1 is exact up to one rounding of a
// value below 2^-8.8), and -log2(c_i) as an integer on the 2^-12 grid (bits in
// .z) plus an FP32 remainder (.y).  Filled once per CTA in FP64.
// Entry i sits at tab[(i << sh) + g] for each of the 2^sh copies g.
// With L (a single call's Laplace parameters), .w holds c0 - P z (int bits):
// the entry's part of the exponent, folded (laplace_val2<true>).
__device__ void laplace_table(float4 *tab, int sh, const LapParam *L = nullptr)
{
  for (int i = threadIdx.x; i < LTAB; i += blockDim.x) {
    const double fm = 1.0 + (i + 0.5) / LTAB;
    const double c = rint(4096.0 / fm) / 4096.0;
    const double T = -log2(c);
    const double th = rint(T * 4096.0);
    const float4 v = make_float4((float)c, (float)(T - th / 4096.0), __int_as_float((int)th),
                                 L ? __int_as_float(L->c0 - L->P * (int)th) : 0.f);
    for (int g = 0; g < (1 << sh); g++) tab[(i << sh) + g] = v;
  }
}

// A thread's view of the table: its copy and the copies' stride.  An entry is
// read with one 16-byte shared load (an ordinary float4 read whose last field
// goes unused is split by the compiler into an 8- and a 4-byte load, which
// conflict across the copies' banks: twice the shared-memory wavefronts, taken
// from the tensor core's operand reads).  The entry of an FP32 value with bits
// u is number (u >> 15) & 255 (its top 8 mantissa bits); its byte offset, that
// number << (sh + 4), is formed as (u >> (11 - sh)) & (255 << (sh + 4)).
struct LTab {
  uint32_t base;        // shared address of this lane's copy
  int shr;              // 11 - sh
  uint32_t mask;        // 255 << (sh + 4)
  __device__ __forceinline__ LTab(const float4 *p, int sh)
      : base(smem_addr(p)), shr(11 - sh), mask(255u << (sh + 4)) {}
  // the entry for the FP32 bits u
  __device__ __forceinline__ float4 at_bits(uint32_t u) const
  {
    float4 v;
    asm("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "r"(base + ((u >> shr) & mask)));
    return v;
  }
};

// scal * d2^powe for the double-float d2 = t + lo, powe = -P/2, as
// 2^(log2 scal + powe log2 d2).  log2 d2 = e + (-log2 c_i) + log2(1 + r) +
// lo / (t ln2) with t = 2^e f, i the top 8 bits of f and r = f c_i - 1; the
// series of log2(1 + r) to r^4 (|r| < 2^-8.8).  The exponent's integer and
// 2^-13-grid parts are formed exactly in int32, the rest in FP32, so that the
// result carries a relative error of a few 1e-7 for every P up to 1022.
// Values below 2^-126 flush to zero (rows of such values are redone in FP64).
__device__ __forceinline__ float laplace_core(float t, float lo, const LTab &tab, const LapParam &L,
                                              int &n)
{
  const uint32_t u = __float_as_uint(t);
  const int e = (int)(u >> 23) - 127;
  const float4 tb = tab.at_bits(u);
  const float f = __uint_as_float((u & 0x007fffffu) | 0x3f800000u);
  const float r = fmaf(f, tb.x, -1.0f);
  const float p = r * fmaf(r, fmaf(r, fmaf(r, -0.36067376f, 0.48089835f), -0.72134752f), 1.44269504f);
  const float llo = (tb.y + p) + lo * rcp_approx(t) * 1.44269504f;
  const int lhi = e * 4096 + __float_as_int(tb.z);          // log2 d2 on the 2^-12 grid
  const int E = L.ls13 - L.P * lhi;                          // 2^-13 units
  const float arg = fmaf((float)(E & 8191), 0x1p-13f, fmaf(L.mh, llo, L.lsf));
  n = E >> 13;
  return ex2_approx(arg);
}
__device__ __forceinline__ float laplace_val(float t, float lo, const LTab &tab, const LapParam &L)
{
  int n;
  const float y = laplace_core(t, lo, tab, L, n);
  return n >= -126 ? y * __int_as_float((n + 127) << 23) : 0.0f;
}

// laplace_val of two columns, the floating-point part in packed FP32 pairs (the
// series one term shorter: its error stays far below the per-pair budget).
// FOLD: the table was built with this call's parameters (.w = c0 - P z).
template <bool FOLD = false>
__device__ __forceinline__ uint64_t laplace_val2(uint64_t T, uint64_t LO, const LTab &tab, const LapParam &L)
{
  const float t0 = lo2(T), t1 = hi2(T);
  const uint32_t u0 = __float_as_uint(t0), u1 = __float_as_uint(t1);
  const float4 b0 = tab.at_bits(u0), b1 = tab.at_bits(u1);
  const uint64_t F = pk2(__uint_as_float((u0 & 0x007fffffu) | 0x3f800000u),
                         __uint_as_float((u1 & 0x007fffffu) | 0x3f800000u));
  const uint64_t R = fma2(F, pk2(b0.x, b1.x), pk2(-1.0f, -1.0f));
  // log2(1 + r) to r^3: the omitted -log2(e) r^4 / 4 is below 2^-36.7 (|r| < 2^-8.8),
  // 2^-27.7 relative on K even at P = 1022
  uint64_t Q = fma2(R, pk2(0.48089835f, 0.48089835f), pk2(-0.72134752f, -0.72134752f));
  Q = mul2(R, fma2(R, Q, pk2(1.44269504f, 1.44269504f)));
  const uint64_t RT = pk2(rcp_approx(t0), rcp_approx(t1));
  const uint64_t LLO = fma2(mul2(LO, RT), pk2(1.44269504f, 1.44269504f), add2(pk2(b0.y, b1.y), Q));
  // the exponent in 2^-13 units, ls13 - P (4096 (e - 127) + z), with the
  // constant terms folded into c0 and p4096
  const int E0 = (FOLD ? __float_as_int(b0.w) : L.c0 - L.P * __float_as_int(b0.z)) - L.p4096 * (int)(u0 >> 23);
  const int E1 = (FOLD ? __float_as_int(b1.w) : L.c0 - L.P * __float_as_int(b1.z)) - L.p4096 * (int)(u1 >> 23);
  // its fraction (E mod 8192) 2^-13 exactly: the float 2^23 + (E & 8191) times
  // 2^-13 is 1024 + fraction, and the FMA with -1024 rounds nothing
  const uint64_t FR = fma2(pk2(__uint_as_float(0x4B000000u | (uint32_t)(E0 & 8191)),
                               __uint_as_float(0x4B000000u | (uint32_t)(E1 & 8191))),
                           pk2(0x1p-13f, 0x1p-13f), pk2(-1024.0f, -1024.0f));
  const uint64_t ARG = add2(FR, fma2(pk2(L.mh, L.mh), LLO, pk2(L.lsf, L.lsf)));
  // 2^n, zero below 2^-126
  const int n0 = E0 >> 13, n1 = E1 >> 13;
  const float s0 = __int_as_float(max(n0 + 127, 0) << 23), s1 = __int_as_float(max(n1 + 127, 0) << 23);
  return mul2(pk2(ex2_approx(lo2(ARG)), ex2_approx(hi2(ARG))), pk2(s0, s1));
}

// 2^n y in FP64, n in the normal FP64 exponent range (beyond it, 0 or inf;
// the rechecks send results below the normal range through FP64).
__device__ __forceinline__ double scale2(float y, int n)
{
  if (n < -1022) return 0.0;
  if (n > 1023) return (double)y * 0x1p1023 * 2.0;
  return (double)y * __longlong_as_double((long long)(n + 1023) << 52);
}

// 2^((t + lo)(ph + pl)) for a double-float distance and a double-float factor
// (ph + pl <= 0): the product's rounding and the low parts enter through the
// first-order term.
__device__ __forceinline__ float exp2_prod(float t, float lo, float ph, float pl)
{
  const float a = t * ph;
  const float ae = fmaf(t, ph, -a) + fmaf(lo, ph, t * pl);
  const float e = ex2_approx(a);
  return fmaf(e, 0.69314718f * ae, e);
}

// exp2_prod of two columns in packed FP32 pairs.
__device__ __forceinline__ uint64_t exp2_prod2(uint64_t T, uint64_t LO, uint64_t PH, uint64_t PL)
{
  const uint64_t A = mul2(T, PH);
  const uint64_t AE = add2(fma2(T, PH, sub2(0, A)), fma2(LO, PH, mul2(T, PL)));
  const uint64_t E = pk2(ex2_approx(lo2(A)), ex2_approx(hi2(A)));
  return fma2(E, mul2(pk2(0.69314718f, 0.69314718f), AE), E);
}

// 2^((t + lo)(ph + pl)) as exp2_prod, returned in FP64 so that values below
// the FP32 range keep their size (the integer part of the exponent is applied
// in FP64).
__device__ __forceinline__ double exp2_prod_wide(float t, float lo, float ph, float pl, bool &deep)
{
  const float a = t * ph;
  const float ae = fmaf(t, ph, -a) + fmaf(lo, ph, t * pl);
  const float n = floorf(a);
  // results in the FP64 subnormal band go through FP64; below it FP64 gives 0 too
  deep = n < -1020.0f && n > -1090.0f;
  if (n <= -1090.0f) return 0.0;
  const float f = (a - n) + ae;                  // a - n is exact
  const float e = ex2_approx(f);
  return scale2(e, (int)n);
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
    const float v = fmaf(kp.fscal, c, kp.fcons);
    if (kp.pmode == POW_INT) {
      int e = kp.pint < 0 ? -kp.pint : kp.pint;
      float r = 1.0f, b = v;
      for (;;) { if (e & 1) r *= b; e >>= 1; if (!e) break; b *= b; }
      return kp.pint < 0 ? 1.0f / r : r;
    }
    return ex2_approx(kp.fpowe * __log2f(v));
  } else if constexpr (KT == KS_TANH) {
    const float v = fmaf(kp.fscal, c, kp.fcons);
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
    return (t + kp.fcons) + lo;
  } else {  // Epanechnikov
    const float d = t + lo;
    return d < 1.0f ? 0.75f * (1.0f - d) : 0.0f;
  }
}

// FP64 recheck of one flagged pair from the pool coordinates (the distance
// assembly of near-coincident pairs is kept in FP64): the kernel value.
template <int KT>
__device__ double recheck64(const TileArgs &a, const KParams &kp, int pa, int pb)
{
  const double *x = a.XA + (size_t)pa * a.k, *y = a.XB + (size_t)pb * a.k;
  double d2 = 0.0;
  for (int p = 0; p < a.k; p++) { const double d = x[p] - y[p]; d2 = fma(d, d, d2); }
  double kv;
  if constexpr (KT == KS_GAUSSIAN) kv = exp(d2 * kp.scal);
  else if constexpr (KT == KS_GAUSSIAN_VAR_BANDWIDTH) kv = exp(((d2 * -0.5) * kp.hi[pa]) * kp.hj[pb]);
  else if constexpr (KT == KS_LAPLACE) {
    if (d2 < 1e-15) d2 = 1.79e308;
    kv = pow_class(d2, kp) * kp.scal;
  } else if constexpr (KT == KS_QUARTIC) {
    kv = d2 < 1.0 ? (15.0 / 16.0) * (1.0 - d2) * (1.0 - d2) : 0.0;
  } else if constexpr (KT == KS_MULTIQUADRATIC) kv = d2 + kp.cons;
  else if constexpr (KT == KS_EPANECHNIKOV) kv = d2 < 1.0 ? 0.75 * (1.0 - d2) : 0.0;
  else kv = 0.0;
  return kv;
}

// Weight r (of a.nrhs interleaved columns) of source position jpos, in FP64.
__device__ __forceinline__ double wcol64(const TileArgs &a, int jpos, int r)
{
  return a.w[(size_t)(a.wmap ? a.wmap[jpos] : jpos) * (a.nrhs > 1 ? a.nrhs : 1) + r];
}

// One coordinate of a float-pair squared distance: (u - v)^2 added to the
// double-float (sh, sl) by a TwoSum difference, an exact square by FMA and a
// TwoSum accumulation.
__device__ __forceinline__ void ff_acc(float2 u, float2 v, float &sh, float &sl)
{
  const float s = u.x - v.x;                       // TwoSum(u.x, -v.x)
  const float bv = s - u.x;
  float e = (u.x - (s - bv)) + (-v.x - bv);
  e += u.y - v.y;
  const float dh = s + e, dl = e - (dh - s);       // Fast2Sum
  const float q = dh * dh;
  const float qe = fmaf(dh, dh, -q) + 2.f * dh * dl;
  const float t = sh + q;                          // TwoSum(sh, q)
  const float z = t - sh;
  sl += ((sh - (t - z)) + (q - z)) + qe;
  sh = t;
}

// Squared distance of two points given as float pairs (about 2^-44
// relative), returned as the float pair th + tl.  Even and odd coordinates go
// to two accumulators, combined at the end in a fixed order, which halves the
// dependency chain; where both rows are 16-byte aligned, 16-byte loads of two
// coordinates, four in flight, so that the loads of a long row overlap
// instead of waiting one after another.
__device__ __forceinline__ void ff_dist2(const float2 *__restrict__ x, const float2 *__restrict__ y, int k,
                                         float &th, float &tl)
{
  float sh0 = 0.f, sl0 = 0.f, sh1 = 0.f, sl1 = 0.f;
  int p = 0;
  if (((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15) == 0) {
    const float4 *__restrict__ x4 = reinterpret_cast<const float4 *>(x);
    const float4 *__restrict__ y4 = reinterpret_cast<const float4 *>(y);
    const int k2 = k >> 1;
#pragma unroll 4
    for (int q = 0; q < k2; q++) {
      const float4 a = __ldg(x4 + q), b = __ldg(y4 + q);
      ff_acc(make_float2(a.x, a.y), make_float2(b.x, b.y), sh0, sl0);
      ff_acc(make_float2(a.z, a.w), make_float2(b.z, b.w), sh1, sl1);
    }
    p = k2 << 1;
  }
  for (; p < k; p++) ff_acc(x[p], y[p], sh0, sl0);
  // (sh0 + sl0) + (sh1 + sl1): TwoSum of the high parts, then the low parts
  const float t = sh0 + sh1;
  const float z = t - sh0;
  const float e = ((sh0 - (t - z)) + (sh1 - z)) + (sl0 + sl1);
  th = t + e;
  tl = e - (th - t);
}

// Recheck of one pair: its kernel value (the caller applies the weights).
// The list form keeps float-pair copies of the pools:
// there the squared distance is summed in float-pair arithmetic (TwoSum per
// coordinate difference, exact square by FMA; about 2^-44 relative) and the
// kernel value is formed in FP32 from it, as in the main epilogue; FP64
// instructions issue too slowly on this GPU to recheck many pairs.  Coincident
// and overflowing Laplace pairs, the other kernels and the single-call form go
// through FP64.
template <int KT, bool PRE = false>
__device__ double recheck(const TileArgs &a, const TaskParam &T, const LTab &ltab, int ipos, int jpos)
{
  int pa = a.amap ? a.amap[ipos] : ipos;
  int pb = a.bmap ? a.bmap[jpos] : jpos;
  if (a.nxa >= 0 && (pa < 0 || pa >= a.nxa)) pa = 0;   // flagged by pack_kernel
  if (a.nxb >= 0 && (pb < 0 || pb >= a.nxb)) pb = 0;
  if constexpr (KT == KS_LAPLACE) {
    if (pa == pb && a.XA == a.XB) return T.kcoin;   // the same pool point twice
  }
  if constexpr (KT == KS_GAUSSIAN || KT == KS_GAUSSIAN_VAR_BANDWIDTH ||
                KT == KS_LAPLACE) {
    if (a.XAf && a.P->ff_ok && (a.tab || a.P->any_flag)) {   // the copies exist
      // (a single call builds them only when it may flag pairs)
      const float2 *x = a.XAf + (size_t)(a.ffpos ? ipos : pa) * a.k;
      const float2 *y = a.XBf + (size_t)(a.ffpos ? jpos : pb) * a.k;
      double hf = 0.0;
      if constexpr (KT == KS_GAUSSIAN_VAR_BANDWIDTH) hf = T.kp.hi[pa] * T.kp.hj[pb];
      if constexpr (PRE && KT != KS_LAPLACE) {
        // an FP32 estimate first: exponents beyond -1100 are 0 in FP64 as well
        float e2 = 0.f;
        for (int p = 0; p < a.k; p++) { const float d = x[p].x - y[p].x; e2 = fmaf(d, d, e2); }
        const float fexp = KT == KS_GAUSSIAN_VAR_BANDWIDTH ? (float)(0.7213475204444817 * hf) : -T.s2;
        if (e2 * fexp > 1111.0f) return 0.0;
      }
      float th, tl;
      ff_dist2(x, y, a.k, th, tl);
      bool deep = false;
      if constexpr (KT == KS_GAUSSIAN) {
        const double v = exp2_prod_wide(th, tl, T.s2, T.s2l, deep);
        if (!deep) return v;
      } else if constexpr (KT == KS_GAUSSIAN_VAR_BANDWIDTH) {
        const double f = -0.5 * 1.4426950408889634 * hf;
        const float fh = (float)f, fl = (float)(f - (double)fh);
        const double v = exp2_prod_wide(th, tl, fh, fl, deep);
        if (!deep) return v;
      } else {
        if (th > T.lap.tover && th >= 1e-15f) {
          int n;
          const float y = laplace_core(th, tl, ltab, T.lap, n);
          if (n >= -1020) return scale2(y, n);
          if (n <= -1090) return 0.0;
        }
        // equal points: recheck64's clamp (see recheck_lap_warp)
        if (th == 0.0f && tl == 0.0f) return T.kcoin;
      }
    }
  }
  return recheck64<KT>(a, T.kp, pa, pb);
}

// ff_dist2 by a whole warp for one pair (every lane passes the same rows):
// lane l takes coordinates l, l + 32, ... (coalesced loads, two accumulators),
// then a butterfly of TwoSums adds the lanes' double-float partials.  TwoSum
// is exact whichever operand comes first, so every lane ends with the same
// float pair; the order is fixed (deterministic).
__device__ __forceinline__ void ff_dist2_warp(const float2 *__restrict__ x, const float2 *__restrict__ y, int k,
                                              float &th, float &tl)
{
  const int lane = threadIdx.x & 31;
  float sh0 = 0.f, sl0 = 0.f, sh1 = 0.f, sl1 = 0.f;
  int p = lane;
#pragma unroll 2
  for (; p + 32 < k; p += 64) {
    const float2 u0 = __ldg(x + p), v0 = __ldg(y + p), u1 = __ldg(x + p + 32), v1 = __ldg(y + p + 32);
    ff_acc(u0, v0, sh0, sl0);
    ff_acc(u1, v1, sh1, sl1);
  }
  if (p < k) ff_acc(__ldg(x + p), __ldg(y + p), sh0, sl0);
  float h, l;
  {
    const float t = sh0 + sh1, z = t - sh0;
    const float e = ((sh0 - (t - z)) + (sh1 - z)) + (sl0 + sl1);
    h = t + e;
    l = e - (h - t);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(0xffffffffu, h, o), l2 = __shfl_xor_sync(0xffffffffu, l, o);
    const float t = h + h2, z = t - h;
    const float e = ((h - (t - z)) + (h2 - z)) + (l + l2);
    h = t + e;
    l = e - (h - t);
  }
  th = h;
  tl = l;
}

// Rows of at least this many coordinates are rechecked by a whole warp per
// pair (ff_dist2_warp), shorter ones by one lane per pair (ff_dist2).
constexpr int WARP_RECHECK_K = 256;

// One flagged Laplace pair, rechecked by the whole warp: the float-pair
// distance with the lanes over the coordinates (ff_dist2_warp, whose butterfly
// leaves the same th + tl in every lane), then the table-driven value, in FP64
// in every lane.  Coincident and overflowing pairs, values beyond the FP64
// normal range and pools without the float-pair copies go through recheck64
// on lane 0.  (One lane per pair would chain a row's dependent loads while the
// other 31 lanes wait, and every warp of the block waits for that warp at the
// next accumulator buffer.)
__device__ double recheck_lap_warp(const TileArgs &a, const TaskParam &T, const LTab &ltab, int ipos, int jpos)
{
  int pa = a.amap ? a.amap[ipos] : ipos;
  int pb = a.bmap ? a.bmap[jpos] : jpos;
  if (a.nxa >= 0 && (pa < 0 || pa >= a.nxa)) pa = 0;   // flagged by pack_kernel
  if (a.nxb >= 0 && (pb < 0 || pb >= a.nxb)) pb = 0;
  if (pa == pb && a.XA == a.XB) return T.kcoin;   // the same pool point twice
  if (a.XAf && a.P->ff_ok && (a.tab || a.P->any_flag)) {   // the copies exist
    const float2 *x = a.XAf + (size_t)(a.ffpos ? ipos : pa) * a.k;
    const float2 *y = a.XBf + (size_t)(a.ffpos ? jpos : pb) * a.k;
    float th, tl;
    ff_dist2_warp(x, y, a.k, th, tl);
    if (th > T.lap.tover && th >= 1e-15f) {
      int n;
      const float v = laplace_core(th, tl, ltab, T.lap, n);
      if (n >= -1020) return scale2(v, n);
      if (n <= -1090) return 0.0;
    }
    // equal points: every coordinate difference lies below the float-pair
    // resolution, so the FP64 distance is below 1e-15 as well and takes
    // recheck64's clamp
    if (th == 0.0f && tl == 0.0f) return T.kcoin;
  }
  double r = 0.0;
  if ((threadIdx.x & 31) == 0) r = recheck64<KS_LAPLACE>(a, T.kp, pa, pb);
  return __shfl_sync(0xffffffffu, r, 0);
}

// A flagged pair of the Gaussian kinds, FP64-free: the flag rules select pairs
// whose value lies in the FP32 range, so the value (float-pair distance from
// the pools' float-pair copies, then exp2_prod) times the column's FP32 weight
// is formed in FP32 like the main path's.  Needs the copies (ffp).
// WARP: called by the whole warp for the same pair (ff_dist2_warp).
template <int KT, bool WARP = false>
__device__ __forceinline__ float recheck_f(const TileArgs &a, const TaskParam &T, int ipos, float ah, float ahl,
                                           const SrcMeta *__restrict__ bm, int c)
{
  const int jpos = bm->pos[c];
  int pa = a.amap ? a.amap[ipos] : ipos;
  int pb = a.bmap ? a.bmap[jpos] : jpos;
  if (a.nxa >= 0 && (pa < 0 || pa >= a.nxa)) pa = 0;   // flagged by pack_kernel
  if (a.nxb >= 0 && (pb < 0 || pb >= a.nxb)) pb = 0;
  float th, tl;
  const float2 *x = a.XAf + (size_t)(a.ffpos ? ipos : pa) * a.k, *y = a.XBf + (size_t)(a.ffpos ? jpos : pb) * a.k;
  if constexpr (WARP) ff_dist2_warp(x, y, a.k, th, tl);
  else ff_dist2(x, y, a.k, th, tl);
  float ph, pl;
  if constexpr (KT == KS_GAUSSIAN_VAR_BANDWIDTH) {
    // (-0.5 log2e hi) hj from the row's and the column's float pairs
    const float hc = bm->h[c], hl = bm->hlo[c];
    ph = ah * hc;
    pl = fmaf(ah, hc, -ph) + fmaf(ah, hl, ahl * hc);
  } else {
    ph = T.s2;
    pl = T.s2l;
  }
  return exp2_prod(th, tl, ph, pl);   // the caller applies the column's weights
}

// The flagged pairs of one warp's 32 rows (lanes) x 32 columns, all lanes
// working: the flags are numbered lane by lane (fl: this lane's columns, bit
// j = column 32 grp + j), 32 per round; each lane finds one, and either
// rechecks it (recheck_f, short rows) or the warp rechecks the round's pairs
// one after another with its lanes over the coordinates (long rows: coalesced
// loads instead of 32 rows read side by side).  Each row adds its own values
// in their order (through the warp's 32-float scratch wq) to add, their
// magnitudes to fchk.
template <int KT, int NR>
__device__ __forceinline__ void recheck_warp(const TileArgs &a, const TaskParam &T, const PtMeta &am,
                                             const SrcMeta *__restrict__ bm, int grp, uint32_t fl,
                                             float *wq, float (&add)[NR], float &fchk)
{
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int cnt = __popc(fl);
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(full, incl, o);
    if (lane >= o) incl += y;
  }
  const int excl = incl - cnt;
  const int tot = __shfl_sync(full, incl, 31);
  if (lane == 0 && a.nrecheck) atomicAdd(a.nrecheck, (unsigned long long)tot);
  for (int base = 0; base < tot; base += 32) {
    const int e = base + lane;
    int L = 0;                       // the owner: lanes before it have incl <= e
#pragma unroll
    for (int st = 16; st > 0; st >>= 1) {
      const int v = __shfl_sync(full, incl, L + st - 1);
      if (v <= e) L += st;
    }
    L = min(L, 31);                  // e >= tot: no entry
    const uint32_t flL = __shfl_sync(full, fl, L);
    const int exL = __shfl_sync(full, excl, L);
    const int posL = __shfl_sync(full, am.pos, L);
    const float hL = __shfl_sync(full, am.h, L);
    const float hlL = __shfl_sync(full, __int_as_float(am.pad[1]), L);
    float kv = 0.f;
    int col = -1;
    if (e < tot) {
      uint32_t mk = flL;             // its (e - exL)-th flagged column
      for (int i = e - exL; i > 0 && mk; i--) mk &= mk - 1;
      if (mk) col = grp * 32 + __ffs(mk) - 1;
    }
    if (a.k >= WARP_RECHECK_K) {
      const int ne = min(32, tot - base);
      for (int q = 0; q < ne; q++) {
        const int cq = __shfl_sync(full, col, q);
        const int pq = __shfl_sync(full, posL, q);
        const float hq = __shfl_sync(full, hL, q), hlq = __shfl_sync(full, hlL, q);
        if (cq >= 0) {
          const float r = recheck_f<KT, true>(a, T, pq, hq, hlq, bm, cq);
          if (lane == q) kv = r;
        }
      }
    } else if (col >= 0) {
      kv = recheck_f<KT>(a, T, posL, hL, hlL, bm, col);
    }
    const int q1 = min(incl, base + 32) - base;
#pragma unroll
    for (int r = 0; r < NR; r++) {   // each weight column: the values through wq, rows in order
      wq[lane] = col >= 0 ? kv * wrow(bm, r)[col] : 0.f;
      __syncwarp();
      for (int q = max(excl, base) - base; q < q1; q++) {
        const float x = wq[q];
        add[r] += x;
        fchk += fabsf(x);
      }
      __syncwarp();
    }
  }
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

// assemble for two columns at once (packed FP32 pairs; the same operations and
// roundings per column).  NRC = (-rc, -rc).
template <bool EXACT>
__device__ __forceinline__ void assemble2(uint64_t H, uint64_t L, uint64_t AN, uint64_t ANL, uint64_t BN,
                                          uint64_t BNL, uint64_t NRC, uint64_t &T, uint64_t &LO, uint64_t &S)
{
  const uint64_t s = add2(AN, BN);
  uint64_t tt, ee;
  if constexpr (EXACT) {
    const uint64_t t1 = sub2(s, H);
    tt = sub2(t1, L);
    ee = sub2(sub2(t1, tt), L);
  } else {
    const uint64_t u1 = sub2(s, L);
    const uint64_t e1 = sub2(sub2(s, u1), L);
    tt = sub2(u1, H);
    const uint64_t e2 = sub2(sub2(u1, tt), H);
    ee = add2(e1, e2);
  }
  T = mul2(tt, NRC);
  LO = mul2(add2(add2(ANL, BNL), ee), NRC);
  S = mul2(s, NRC);
}

// NC columns of one row, Gaussian with the low norm parts folded into the
// source weights and the row factor: kv = 2^-(g tt) (1 - ln2 g ee), times
// the NR weight columns (acc[r]).
template <int NC, int NR>
__device__ __forceinline__ void epi_chunk_gfast(const uint32_t (&h)[NC], const uint32_t (&l)[NC],
                                                const SrcMeta *__restrict__ bm, int c0, float an_hi, float rc,
                                                float (&acc)[NR][4])
{
  // two columns per instruction (packed FP32 pairs); column j feeds acc[.][j & 3]
  const float cg = 0.69314718f * rc;          // -ln2 g
  const uint64_t AN = pk2(an_hi, an_hi), RC = pk2(rc, rc), CG = pk2(cg, cg);
  uint64_t A01[NR], A23[NR];
#pragma unroll
  for (int r = 0; r < NR; r++) { A01[r] = pk2(acc[r][0], acc[r][1]); A23[r] = pk2(acc[r][2], acc[r][3]); }
#pragma unroll
  for (int j4 = 0; j4 < NC; j4 += 4) {
    const float4 nh = ld4(&bm->n_hi[c0 + j4]);                              // nu_hi
    float4 ww[NR];                                                          // w' of each column
#pragma unroll
    for (int r = 0; r < NR; r++) ww[r] = ld4(wrow(bm, r) + c0 + j4);
#pragma unroll
    for (int q = 0; q < 4; q += 2) {
      const int j = j4 + q;
      const uint64_t H = pk2(__uint_as_float(h[j]), __uint_as_float(h[j + 1]));
      const uint64_t L = pk2(__uint_as_float(l[j]), __uint_as_float(l[j + 1]));
      const uint64_t t1 = sub2(add2(AN, pk2(f4(nh, q), f4(nh, q + 1))), H);   // exact
      const uint64_t tt = sub2(t1, L);
      const uint64_t ee = sub2(sub2(t1, tt), L);
      const uint64_t ar = mul2(tt, RC);
      const uint64_t E = pk2(ex2_approx(lo2(ar)), ex2_approx(hi2(ar)));       // 2^-(g tt)
      const uint64_t kv = fma2(E, mul2(CG, ee), E);
#pragma unroll
      for (int r = 0; r < NR; r++) {
        const uint64_t W = pk2(f4(ww[r], q), f4(ww[r], q + 1));
        if (q == 0) A01[r] = fma2(kv, W, A01[r]);
        else A23[r] = fma2(kv, W, A23[r]);
      }
    }
  }
#pragma unroll
  for (int r = 0; r < NR; r++) {
    acc[r][0] = lo2(A01[r]); acc[r][1] = hi2(A01[r]); acc[r][2] = lo2(A23[r]); acc[r][3] = hi2(A23[r]);
  }
}

// NC columns of one row, distance kernels, NR weight columns.  Returns the
// flagged columns.
template <int KT, bool EXACT, bool FLAGS, int NC, int NR, bool FOLD = false>
__device__ __forceinline__ uint32_t epi_chunk(const uint32_t (&h)[NC], const uint32_t (&l)[NC],
                                              const SrcMeta *__restrict__ bm, int c0, const PtMeta &am, float rc,
                                              const TaskParam &T, const LTab &ltab,
                                              float (&acc)[NR][4], float &amin)
{
  const KParams &kp = T.kp;
  uint32_t flags = 0;
  // flag test: t < t_flag or t < rho (n_i + n_j), tested against the row's
  // bound max(t_flag, rho (n_i + nbmax)) (a superset: the extra pairs are
  // rechecked exactly), one comparison per column
  float t_flag = 0.f;
  if constexpr (FLAGS) t_flag = fmaxf(T.t_flag, T.rho * fmaf(am.n_hi, -rc, T.nbmax));
  const uint64_t AN = pk2(am.n_hi, am.n_hi), ANL = pk2(am.n_lo, am.n_lo), NRC = pk2(-rc, -rc);
#pragma unroll
  for (int j4 = 0; j4 < NC; j4 += 4) {
    const float4 nh = ld4(&bm->n_hi[c0 + j4]), nl = ld4(&bm->n_lo[c0 + j4]);
    float4 ww[NR];
#pragma unroll
    for (int r = 0; r < NR; r++) ww[r] = ld4(wrow(bm, r) + c0 + j4);
    float4 hh = make_float4(0.f, 0.f, 0.f, 0.f), hl = hh;
    if constexpr (KT == KS_GAUSSIAN_VAR_BANDWIDTH) { hh = ld4(&bm->h[c0 + j4]); hl = ld4(&bm->hlo[c0 + j4]); }
    uint64_t T2[2], LO2[2], S2[2];
#pragma unroll
    for (int p2 = 0; p2 < 2; p2++) {
      const int j = j4 + 2 * p2;
      assemble2<EXACT>(pk2(__uint_as_float(h[j]), __uint_as_float(h[j + 1])),
                       pk2(__uint_as_float(l[j]), __uint_as_float(l[j + 1])), AN, ANL,
                       pk2(f4(nh, 2 * p2), f4(nh, 2 * p2 + 1)), pk2(f4(nl, 2 * p2), f4(nl, 2 * p2 + 1)), NRC,
                       T2[p2], LO2[p2], S2[p2]);
    }
    uint64_t KV2[2] = {0, 0};
    if constexpr (KT == KS_LAPLACE) {
      KV2[0] = laplace_val2<FOLD>(T2[0], LO2[0], ltab, T.lap);
      KV2[1] = laplace_val2<FOLD>(T2[1], LO2[1], ltab, T.lap);
    } else if constexpr (KT == KS_GAUSSIAN_VAR_BANDWIDTH) {
      // factor h_i h_j (negative) as a float pair, two columns at a time
      const uint64_t AH = pk2(am.h, am.h), AHL = pk2(__int_as_float(am.pad[1]), __int_as_float(am.pad[1]));
#pragma unroll
      for (int p2 = 0; p2 < 2; p2++) {
        const uint64_t HC = pk2(f4(hh, 2 * p2), f4(hh, 2 * p2 + 1)), HL = pk2(f4(hl, 2 * p2), f4(hl, 2 * p2 + 1));
        const uint64_t PH = mul2(AH, HC);
        const uint64_t PL = add2(fma2(AH, HC, sub2(0, PH)), fma2(AH, HL, mul2(AHL, HC)));
        KV2[p2] = exp2_prod2(T2[p2], LO2[p2], PH, PL);
      }
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int j = j4 + q;
      const float t = (q & 1) ? hi2(T2[q >> 1]) : lo2(T2[q >> 1]);
      const float lo = (q & 1) ? hi2(LO2[q >> 1]) : lo2(LO2[q >> 1]);
      const float s = (q & 1) ? hi2(S2[q >> 1]) : lo2(S2[q >> 1]);
      float kv;
      if constexpr (KT == KS_LAPLACE || KT == KS_GAUSSIAN_VAR_BANDWIDTH)
        kv = (q & 1) ? hi2(KV2[q >> 1]) : lo2(KV2[q >> 1]);
      else if constexpr (KT == KS_QUARTIC || KT == KS_EPANECHNIKOV || KT == KS_MULTIQUADRATIC) {
        if (T.anch) {
          // K - K(d0^2) from e = d2 - d0^2 (t - d0^2 is exact near the anchor)
          const float e = (t - am.w) + lo;
          const float d = t + lo, c = __int_as_float(am.pad[0]);
          if constexpr (KT == KS_MULTIQUADRATIC) kv = e;
          else if (d >= 1.0f) kv = -am.h;                                       // K = 0
          else if (c <= 0.0f) kv = kval32<KT>(t, lo, 0.f, 0.f, 0.f, kp);        // K(d0^2) = 0
          else if constexpr (KT == KS_EPANECHNIKOV) kv = -0.75f * e;
          else kv = 0.9375f * e * (e - 2.0f * c);
        } else {
          kv = kval32<KT>(t, lo, 0.f, am.h, 0.f, kp);
        }
      }
      else kv = kval32<KT>(t, lo, 0.f, am.h, 0.f, kp);
      // smallest exponent (log2 units) of the exponential kernels' values: the
      // row rescue is needed only if some value is not 0 in FP64 either
      if constexpr (KT == KS_GAUSSIAN) amin = fminf(amin, t);
      else if constexpr (KT == KS_GAUSSIAN_VAR_BANDWIDTH) amin = fminf(amin, -am.h * f4(hh, q) * t);
      if constexpr (FLAGS) {
        if constexpr (KT == KS_GAUSSIAN_VAR_BANDWIDTH) {
          const float f = -am.h * f4(hh, q);      // 0.5 log2(e) h_i h_j
          if (f > t_flag && t * f < 126.f) { flags |= 1u << j; kv = 0.f; }
        } else {
          if (t < t_flag) { flags |= 1u << j; kv = 0.f; }
        }
      }
      // padding columns carry w = 0 and finite distances
#pragma unroll
      for (int r = 0; r < NR; r++) acc[r][q] = fmaf(kv, f4(ww[r], q), acc[r][q]);
    }
  }
  return flags;
}

// NC columns of one row, inner-product kernels (polynomial, tanh).  PW in
// 1..4: a polynomial of that integer power, multiplied out; its values are
// finite on padding columns (x.y = 0 there), whose weight 0 then needs no mask.
template <int KT, int NC, int NR, int PW = 0>
__device__ __forceinline__ void epi_chunk_ip(const uint32_t (&h)[NC], const uint32_t (&l)[NC],
                                             const SrcMeta *__restrict__ bm, int c0, int valid, float rc,
                                             const KParams &kp, float (&acc)[NR][4])
{
  // two columns per instruction where the kernel allows it (packed FP32 pairs)
  const uint64_t RC = pk2(rc, rc), MH = pk2(-0.5f, -0.5f);
  const float sc = kp.fscal, cn = kp.fcons;
  const uint64_t SC = pk2(sc, sc), CN = pk2(cn, cn);
  const bool ipow = KT == KS_POLYNOMIAL && kp.pmode == POW_INT;
  uint64_t A[NR][2];
#pragma unroll
  for (int r = 0; r < NR; r++) { A[r][0] = pk2(acc[r][0], acc[r][1]); A[r][1] = pk2(acc[r][2], acc[r][3]); }
#pragma unroll
  for (int j4 = 0; j4 < NC; j4 += 4) {
    float4 ww[NR];
#pragma unroll
    for (int r = 0; r < NR; r++) ww[r] = ld4(wrow(bm, r) + c0 + j4);
#pragma unroll
    for (int p2 = 0; p2 < 2; p2++) {
      const int j = j4 + 2 * p2;
      const uint64_t H = pk2(__uint_as_float(h[j]), __uint_as_float(h[j + 1]));
      const uint64_t L = pk2(__uint_as_float(l[j]), __uint_as_float(l[j + 1]));
      const uint64_t CC = mul2(fma2(L, RC, mul2(H, RC)), MH);          // x.y
      if constexpr (PW > 0) {
        const uint64_t V = fma2(SC, CC, CN);
        uint64_t R = V;
        if constexpr (PW == 2) R = mul2(V, V);
        if constexpr (PW == 3) R = mul2(mul2(V, V), V);
        if constexpr (PW == 4) { R = mul2(V, V); R = mul2(R, R); }
#pragma unroll
        for (int r = 0; r < NR; r++)
          A[r][p2] = fma2(R, pk2(f4(ww[r], 2 * p2), f4(ww[r], 2 * p2 + 1)), A[r][p2]);
        continue;
      }
      float k0, k1;
      if (ipow) {
        // (scal x.y + cons)^p by binary powering on both columns
        const uint64_t V = fma2(SC, CC, CN);
        int e = kp.pint < 0 ? -kp.pint : kp.pint;
        uint64_t R = pk2(1.0f, 1.0f), B = V;
        for (;;) {
          if (e & 1) R = mul2(R, B);
          e >>= 1;
          if (!e) break;
          B = mul2(B, B);
        }
        k0 = lo2(R); k1 = hi2(R);
        if (kp.pint < 0) { k0 = 1.0f / k0; k1 = 1.0f / k1; }
      } else {
        k0 = kval32<KT>(0.f, 0.f, lo2(CC), 0.f, 0.f, kp);
        k1 = kval32<KT>(0.f, 0.f, hi2(CC), 0.f, 0.f, kp);
      }
      // the kernel of a padding column may be NaN (its weight is 0)
      if (j >= valid) k0 = 0.f;
      if (j + 1 >= valid) k1 = 0.f;
#pragma unroll
      for (int r = 0; r < NR; r++)
        A[r][p2] = fma2(pk2(k0, k1), pk2(f4(ww[r], 2 * p2), f4(ww[r], 2 * p2 + 1)), A[r][p2]);
    }
  }
#pragma unroll
  for (int r = 0; r < NR; r++) {
    acc[r][0] = lo2(A[r][0]); acc[r][1] = hi2(A[r][0]); acc[r][2] = lo2(A[r][1]); acc[r][3] = hi2(A[r][1]);
  }
}

// NC columns of one row, polynomial of integer power PW in 1..4, summed
// around the row's anchor v0: v = v0 + d with d = sg ((H - H0) + L) (H - H0
// exact: both are integers below 2^24), and
//   K - v0^PW = d (c1 + d (c2 + d (c3 + d)))   (binomial expansion, Horner
// form, c_i = C(PW, i) v0^(PW-i) from the row's metadata).  The reduction adds
// v0^PW times the sum of all weights in FP64, so the FP32 sums carry only the
// variation of K around v0^PW: where K sits on a large constant (v near cons,
// the sum of K w cancelling), FP32 rounding of K itself would otherwise
// dominate the error.  Padding columns: finite values, weight 0.
template <int NC, int PW, int NR>
__device__ __forceinline__ void epi_chunk_anchor(const uint32_t (&h)[NC], const uint32_t (&l)[NC],
                                                 const SrcMeta *__restrict__ bm, int c0, const PtMeta &am, float sg,
                                                 float (&acc)[NR][4])
{
  const uint64_t H0 = pk2(am.n_hi, am.n_hi), SG = pk2(sg, sg);
  const uint64_t C1 = pk2(am.n_lo, am.n_lo), C2 = pk2(am.w, am.w), C3 = pk2(am.h, am.h);
  uint64_t A[NR][2];
#pragma unroll
  for (int r = 0; r < NR; r++) { A[r][0] = pk2(acc[r][0], acc[r][1]); A[r][1] = pk2(acc[r][2], acc[r][3]); }
#pragma unroll
  for (int j4 = 0; j4 < NC; j4 += 4) {
    float4 ww[NR];
#pragma unroll
    for (int r = 0; r < NR; r++) ww[r] = ld4(wrow(bm, r) + c0 + j4);
#pragma unroll
    for (int p2 = 0; p2 < 2; p2++) {
      const int j = j4 + 2 * p2;
      const uint64_t H = pk2(__uint_as_float(h[j]), __uint_as_float(h[j + 1]));
      const uint64_t L = pk2(__uint_as_float(l[j]), __uint_as_float(l[j + 1]));
      const uint64_t D = mul2(add2(sub2(H, H0), L), SG);
      uint64_t R;
      if constexpr (PW == 1) R = D;
      else if constexpr (PW == 2) R = mul2(D, add2(D, C1));
      else if constexpr (PW == 3) R = mul2(D, fma2(D, add2(D, C2), C1));
      else R = mul2(D, fma2(D, fma2(D, add2(D, C3), C2), C1));
#pragma unroll
      for (int r = 0; r < NR; r++)
        A[r][p2] = fma2(R, pk2(f4(ww[r], 2 * p2), f4(ww[r], 2 * p2 + 1)), A[r][p2]);
    }
  }
#pragma unroll
  for (int r = 0; r < NR; r++) {
    acc[r][0] = lo2(A[r][0]); acc[r][1] = hi2(A[r][0]); acc[r][2] = lo2(A[r][1]); acc[r][3] = hi2(A[r][1]);
  }
}

// tanh in FP32: its series for |v| < 1/8, else from 2^(2 log2(e) |v|).
__device__ __forceinline__ float tanh32(float v)
{
  const float av = fabsf(v);
  if (av < 0.125f) {
    const float v2 = v * v;   // v - v^3/3 + 2v^5/15 - 17v^7/315
    return v * fmaf(v2, fmaf(v2, fmaf(v2, -17.0f / 315.0f, 2.0f / 15.0f), -1.0f / 3.0f), 1.0f);
  }
  const float e = ex2_approx(2.0f * 1.44269504f * av);
  return copysignf(1.0f - 2.0f / (e + 1.0f), v);
}

// NC columns of one row, tanh summed around the row's anchor v0: with d =
// v - v0 = sg ((H - H0) + L) and, for |d| < 1/8, tau = tanh(d),
//   tanh(v) - t0 = tau (1 - t0^2) / (1 + t0 tau),   t0 = tanh(v0)
// (the addition theorem; the denominator stays above 7/8); farther from the
// anchor, tanh(v0 + d) - t0 directly.  t0, 1 - t0^2 and v0 come from the
// row's metadata; the reduction adds t0 times the sum of the weights in FP64.
template <int NC, int NR>
__device__ __forceinline__ void epi_chunk_tanh_anchor(const uint32_t (&h)[NC], const uint32_t (&l)[NC],
                                                      const SrcMeta *__restrict__ bm, int c0, const PtMeta &am,
                                                      float sg, float (&acc)[NR][4])
{
  const float t0 = am.n_lo, s0 = am.w;
#pragma unroll
  for (int j4 = 0; j4 < NC; j4 += 4) {
    float4 ww[NR];
#pragma unroll
    for (int r = 0; r < NR; r++) ww[r] = ld4(wrow(bm, r) + c0 + j4);
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int j = j4 + q;
      const float d = ((__uint_as_float(h[j]) - am.n_hi) + __uint_as_float(l[j])) * sg;
      float kv;
      if (fabsf(d) < 0.125f) {
        const float tau = tanh32(d);
        kv = tau * s0 / fmaf(t0, tau, 1.0f);
      } else {
        kv = tanh32(am.h + d) - t0;
      }
#pragma unroll
      for (int r = 0; r < NR; r++) acc[r][q] = fmaf(kv, f4(ww[r], q), acc[r][q]);
    }
  }
}

// Row sums of one work item.  The FP32 sums of the 32-column groups
// accumulate as an unevaluated FP32 pair hi + lo (TwoSum per tile, about
// 2^-48 relative per addition): FP32 instructions only, since FP64 ones issue
// at 1/64 of the FP32 rate here and every epilogue warp would queue on that
// pipe at the end of each tile.  Sums of values rechecked in FP64 enter as
// their FP32 pair when below 2^120 (values below the FP32 range vanish there:
// a row whose values all lie that low is redone in FP64, and elsewhere they
// are below 2^-126 against values of the row that are not); a larger one (a
// Laplace value of nearly coincident points) sends the row to the FP64 redo
// instead (tile_epilogue).
constexpr double ROW_PAIR_MAX = 0x1p120;
template <int NR>
struct RowAcc {
  float hi[NR], lo[NR];
  __device__ __forceinline__ void zero()
  {
#pragma unroll
    for (int r = 0; r < NR; r++) { hi[r] = 0.f; lo[r] = 0.f; }
  }
  __device__ __forceinline__ void add(int r, float v)
  {
    const float s = hi[r] + v;
    const float bv = s - hi[r];
    lo[r] += (hi[r] - (s - bv)) + (v - bv);
    hi[r] = s;
  }
  __device__ __forceinline__ void add64(int r, double v)
  {
    const float h = (float)v;
    add(r, h);
    lo[r] += (float)(v - (double)h);
  }
  // the item's row sum r in FP64 (an infinite hi passes through unchanged)
  __device__ __forceinline__ double total(int r) const
  {
    const double h = (double)hi[r];
    return isfinite(hi[r]) ? h + (double)lo[r] : h;
  }
};

// Kernels whose FP32 values may fall below the FP32 range while FP64 keeps
// them (the row rescue of tile_epilogue).
__host__ __device__ constexpr bool kt_rescue(int kt)
{
  return kt == KS_GAUSSIAN || kt == KS_GAUSSIAN_VAR_BANDWIDTH || kt == KS_LAPLACE;
}

// One warp's share of one tile (32 columns of its 32 rows): TMEM loads, kernel
// values, weighted sums (NR weight columns), rechecks of the flagged pairs.
// Adds the row sums of these columns to racc (column r), and to bsk the columns' sum
// of |w| (over the weight columns) where every value of the 32 columns lies
// below 2^-96.  The 32 columns are summed in FP32 (four interleaved partial
// sums) and enter the FP64 row sum with one conversion and one add: FP64
// instructions issue at a small fraction of the FP32 rate here.
template <int KT, bool LISTED, int NR>
__device__ __forceinline__ void tile_epilogue(const TileArgs &a, const TaskParam &T, uint32_t tH, int grp, int row,
                                              const SrcMeta *bm, int ncols, const PtMeta &am, float rc, bool exact,
                                              bool gfast, const LTab &ltab, RowAcc<NR> &racc,
                                              float &bsk, float *wq)
{
  // Gaussian kinds with the pools' float-pair copies: flagged pairs are
  // collected over the 32 columns (fl32) and rechecked by the whole warp
  constexpr bool GK = KT == KS_GAUSSIAN || KT == KS_GAUSSIAN_VAR_BANDWIDTH;
  uint32_t fl32 = 0;
  float acc[NR][4];
#pragma unroll
  for (int r = 0; r < NR; r++) acc[r][0] = acc[r][1] = acc[r][2] = acc[r][3] = 0.f;
  double rchk[NR];
#pragma unroll
  for (int r = 0; r < NR; r++) rchk[r] = 0.0;
  float fchk = 0.f;                 // |rechecked values|, for the underflow test
  bool nchk = false;
  float amin = gfast ? 0.f : 3.0e38f;   // see epi_chunk (not tracked by the Gaussian fast path)
  // float-pair copies of the pools exist (a single call builds them only when
  // it may flag pairs)
  const bool ffp = a.XAf && a.P->ff_ok && (a.tab || a.P->any_flag);
  // a single call's Laplace table carries the call's exponent constants
  constexpr bool FOLD = KT == KS_LAPLACE && !LISTED;
  // columns per TMEM load: 8 for the kernels with the most live state per column (the list
  // form's Laplace too: its kernel holds every epilogue variant; and several weight columns)
  constexpr int NCH = (KT == KS_GAUSSIAN_VAR_BANDWIDTH || (KT == KS_LAPLACE && LISTED) || NR > 1) ? 8 : 16;
#pragma unroll 1
  for (int part = 0; part < 32 / NCH; part++) {
    const int c0 = grp * 32 + part * NCH;
    uint32_t h[NCH], l[NCH];
    tmem_ld<NCH>(tH + c0, h);
    tmem_ld<NCH>(tH + 128 + c0, l);
    tmem_ld_wait();
    if constexpr (KT == KS_GAUSSIAN) {
      if (gfast) { epi_chunk_gfast<NCH, NR>(h, l, bm, c0, am.n_hi, rc, acc); continue; }
    }
    if constexpr (kt_uses_norms(KT)) {
      uint32_t flags = 0;
      const bool fl = T.any_flag != 0;
      if (exact) {
        if (fl) flags = epi_chunk<KT, true, true, NCH, NR, FOLD>(h, l, bm, c0, am, rc, T, ltab, acc, amin);
        else epi_chunk<KT, true, false, NCH, NR, FOLD>(h, l, bm, c0, am, rc, T, ltab, acc, amin);
      } else {
        if (fl) flags = epi_chunk<KT, false, true, NCH, NR, FOLD>(h, l, bm, c0, am, rc, T, ltab, acc, amin);
        else epi_chunk<KT, false, false, NCH, NR, FOLD>(h, l, bm, c0, am, rc, T, ltab, acc, amin);
      }
      if constexpr (GK) {
        if (ffp) {
          fl32 |= flags << (part * NCH);
          flags = 0;
        }
      }
      // Laplace rechecks of long rows with few flagged pairs in the warp: the
      // warp takes them one after another (each lane's own in column order,
      // as below), its lanes over the coordinates.  Short rows, or many
      // flagged pairs, one lane per pair (the lanes in parallel).
      constexpr unsigned full = 0xffffffffu;
      if (KT == KS_LAPLACE && a.k >= 32 && __any_sync(full, flags != 0) &&
          __reduce_add_sync(full, (unsigned)__popc(flags)) <= 8) {
        const int lane = threadIdx.x & 31;
        for (uint32_t pend = __ballot_sync(full, flags != 0); pend; pend = __ballot_sync(full, flags != 0)) {
          const int src = __ffs(pend) - 1;
          const int j = __ffs(__shfl_sync(full, flags, src)) - 1;
          if (lane == src) flags &= flags - 1;
          const int c = c0 + j;
          const int ipos = __shfl_sync(full, am.pos, src);
          if (c < ncols && ipos >= 0) {
            const int jpos = bm->pos[c];
            const double kv = recheck_lap_warp(a, T, ltab, ipos, jpos);
            if (lane == src && a.nrecheck) atomicAdd(a.nrecheck, 1ull);
            if (lane == src && kv != 0.0) {   // (coincident points: often exactly 0)
#pragma unroll
              for (int r = 0; r < NR; r++) {
                const double v = kv * wcol64(a, jpos, r);
                rchk[r] += v;
                fchk += fabsf((float)v);
              }
              nchk = true;
            }
          }
        }
      }
      // rechecks of the flagged pairs of these columns (one lane each)
      while (flags) {
        const int j = __ffs(flags) - 1;
        flags &= flags - 1;
        const int c = c0 + j;
        if (c < ncols && am.pos >= 0) {
          const int jpos = bm->pos[c];
          const double kv = recheck<KT>(a, T, ltab, am.pos, jpos);
          if (a.nrecheck) atomicAdd(a.nrecheck, 1ull);
#pragma unroll
          for (int r = 0; r < NR; r++) {
            const double v = kv * wcol64(a, jpos, r);
            rchk[r] += v;
            fchk += fabsf((float)v);
          }
          nchk = true;
        }
      }
    } else if constexpr (KT == KS_POLYNOMIAL) {
      const int pw = T.kp.pmode == POW_INT ? T.kp.pint : 0;
      if (T.anch) {
        if (pw == 3) epi_chunk_anchor<NCH, 3, NR>(h, l, bm, c0, am, T.sg, acc);
        else if (pw == 2) epi_chunk_anchor<NCH, 2, NR>(h, l, bm, c0, am, T.sg, acc);
        else if (pw == 4) epi_chunk_anchor<NCH, 4, NR>(h, l, bm, c0, am, T.sg, acc);
        else epi_chunk_anchor<NCH, 1, NR>(h, l, bm, c0, am, T.sg, acc);
      }
      else if (pw == 2) epi_chunk_ip<KT, NCH, NR, 2>(h, l, bm, c0, ncols - c0, rc, T.kp, acc);
      else if (pw == 3) epi_chunk_ip<KT, NCH, NR, 3>(h, l, bm, c0, ncols - c0, rc, T.kp, acc);
      else if (pw == 4) epi_chunk_ip<KT, NCH, NR, 4>(h, l, bm, c0, ncols - c0, rc, T.kp, acc);
      else if (pw == 1) epi_chunk_ip<KT, NCH, NR, 1>(h, l, bm, c0, ncols - c0, rc, T.kp, acc);
      else epi_chunk_ip<KT, NCH, NR>(h, l, bm, c0, ncols - c0, rc, T.kp, acc);
    } else if constexpr (KT == KS_TANH) {
      if (T.anch) epi_chunk_tanh_anchor<NCH, NR>(h, l, bm, c0, am, T.sg, acc);
      else epi_chunk_ip<KT, NCH, NR>(h, l, bm, c0, ncols - c0, rc, T.kp, acc);
    } else {
      epi_chunk_ip<KT, NCH, NR>(h, l, bm, c0, ncols - c0, rc, T.kp, acc);
    }
  }
  if constexpr (GK) {
    if (ffp) {
      const int nv = ncols - grp * 32;   // valid columns of the group
      if (am.pos < 0 || nv <= 0) fl32 = 0;
      else if (nv < 32) fl32 &= (1u << nv) - 1u;
      if (__any_sync(0xffffffffu, fl32 != 0)) {
        float add[NR];
#pragma unroll
        for (int r = 0; r < NR; r++) add[r] = 0.f;
        recheck_warp<KT, NR>(a, T, am, bm, grp, fl32, wq, add, fchk);
#pragma unroll
        for (int r = 0; r < NR; r++) acc[r][0] += add[r];
      }
    }
  }
  float fs[NR], fsa = 0.f;
#pragma unroll
  for (int r = 0; r < NR; r++) {
    fs[r] = (acc[r][0] + acc[r][1]) + (acc[r][2] + acc[r][3]);
    fsa += fabsf(fs[r]);
  }
  if constexpr (kt_rescue(KT)) {
    // Kernel values over these 32 columns all below 2^-96 (FP32 flushes values
    // below 2^-126 to zero, FP64 keeps them down to 2^-1074): the columns add
    // less than 2^-96 W to the row, and whether that matters depends on the
    // rest of the row, summed by other warps and work items.  W goes to bsk;
    // the reduction redoes the rows where it may matter (split_rescue,
    // list_rescue).
    const float W = bm->wsum[grp * 32];
    if (am.pos >= 0 && fsa + fchk < 0x1p-96f * W && (KT == KS_LAPLACE || amin < 1111.0f)) bsk += W;
  }
#pragma unroll
  for (int r = 0; r < NR; r++) {
    racc.add(r, fs[r]);
    if (nchk) {
      // an infinite skipped-group bound makes the reduction redo the row in
      // FP64 (split_rescue / list_rescue): the value stays out of the pair
      if (fabs(rchk[r]) < ROW_PAIR_MAX) racc.add64(r, rchk[r]);
      else if (am.pos >= 0) bsk = __int_as_float(0x7f800000);
    }
  }
}

// NR: weight columns of one sweep (1, or RMAX for several right-hand sides;
// the list form takes 1).
template <int KT, int NR>
__global__ void __launch_bounds__(NTHREADS, 1) split_tiles(TileArgs a)
{
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *sm = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int kpad = a.kpad;
  const SmemLayout L = smem_layout(kpad, KT, NR);
  const bool resident = L.resident;
  const size_t a_bytes = tile_bytes(BM, kpad), b_bytes = tile_bytes(BN, kpad, smeta_pt(NR));
  const size_t a_op = NBLK * blk_bytes(BM, kpad);     // operand part of a tile image
  const size_t meta_bytes = (size_t)BM * sizeof(PtMeta);
  uint8_t *sA = sm;                                   // target image (resident) or target meta
  uint8_t *sAmeta = resident ? sA + a_op : sA;
  uint8_t *sStage = sm + L.a_region;
  uint8_t *sBm = sStage + L.nstage * L.stage_bytes;   // NMETA source metadata slots
  SplitSmem *S = (SplitSmem *)(sBm + NMETA * L.smeta);
  volatile int *abort = &S->abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int items = a.tab ? a.ntab : a.ntm * a.nsc;

  if (threadIdx.x == 0) {
    mbar_init(&S->a_full, 1);
    mbar_init(&S->a_empty, 1 + EPI_WARPS);
    for (int s = 0; s < NSTAGE; s++) { mbar_init(&S->b_full[s], 1); mbar_init(&S->b_empty[s], 1); }
    for (int s = 0; s < NMETA; s++) { mbar_init(&S->m_full[s], 1); mbar_init(&S->m_empty[s], EPI_WARPS); }
    for (int b = 0; b < 2; b++) { mbar_init(&S->t_full[b], 1); mbar_init(&S->t_empty[b], EPI_WARPS); }
    for (int b = 0; b < 2; b++) {   // one arrive per thread: groups 1.. fill, group 0 empties
      mbar_init(&S->r_full[b], 32 * 4 * (EPI_GROUPS - 1));
      mbar_init(&S->r_empty[b], 32 * 4);
    }
    mbar_init(&S->drain, 1);
    S->abort = 0;
    S->never = 0;
    fence_mbar_init();
  }
  if (warp == 0) { tmem_alloc(&S->tmem_base, TMEM_COLS); tmem_relinquish(); }
  float4 *tab_base = (float4 *)((uint8_t *)S + ((sizeof(SplitSmem) + 15) & ~(size_t)15));
  if constexpr (KT == KS_LAPLACE || KT == KS_LIST) laplace_table(tab_base, L.tab_sh, KT == KS_LAPLACE ? &a.P->lap : nullptr);

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S->tmem_base;

  if (warp == 0) {
    // ---------------- producer ----------------
    // Resident (k <= KPAD_MAX): the target tile image once per item, the source
    // operands once per tile.  Streaming: the target metadata once per item,
    // then per tile and k-chunk one stage holding both operands' chunk.
    if (lane == 0 && !a.stall) {
      int g = 0, tt = 0;
      int a_issued = -1;                  // item index of the last target copy
      int b_last[NSTAGE], m_last[NMETA];  // use count of the last copy per stage / meta slot
      for (int s = 0; s < NSTAGE; s++) b_last[s] = -1;
      for (int s = 0; s < NMETA; s++) m_last[s] = -1;
      bool stop = false;
      // Items are taken from the work counter, so that CTAs with cheap items
      // take more of them; the item goes to the other roles through islot
      // (written before the arrive on a_full, which releases it).
      int item = blockIdx.x;
      for (int it = 0; !*abort && !stop; it++) {
        if (it > 0 && !mbar_wait(&S->a_empty, (it - 1) & 1, abort, a.wait_limit)) break;
        if (item >= items) {
          S->islot[it & 1] = -1;
          mbar_arrive(&S->a_full);
          break;
        }
        S->islot[it & 1] = item;
        const int next = atomicAdd(a.next_item, 1) + (int)gridDim.x;   // in flight while this item's copies issue
        const ItemGeo G = item_geo(a, item);
        const uint8_t *imgA = a.imgA + (size_t)G.ti * a_bytes;
        // slot it & 1 was last read for item it - 2, which every epilogue warp
        // has finished once it arrived on a_empty for item it - 1
        const uint32_t tp_bytes = a.tab ? (uint32_t)sizeof(TaskParam) : 0u;
        if (resident) {
          mbar_arrive_expect_tx(&S->a_full, (uint32_t)a_bytes + tp_bytes);
          bulk_g2s(sA, imgA, (uint32_t)a_bytes, &S->a_full);
        } else {
          mbar_arrive_expect_tx(&S->a_full, (uint32_t)meta_bytes + tp_bytes);
          bulk_g2s(sAmeta, imgA + a_op, (uint32_t)meta_bytes, &S->a_full);
        }
        if (tp_bytes) bulk_g2s(&S->tslot[it & 1], a.tp + G.task, tp_bytes, &S->a_full);
        a_issued = it;
        for (int tj = G.t0; tj < G.t1 && !stop; tj++, tt++) {
          const uint8_t *imgB = a.imgB + (size_t)tj * b_bytes;
          for (int c = 0; c < L.nch; c++, g++) {
            const int st = g % L.nstage, u = g / L.nstage;
            if (u > 0 && !mbar_wait(&S->b_empty[st], (u - 1) & 1, abort, a.wait_limit)) { stop = true; break; }
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
          if (mu > 0 && !mbar_wait(&S->m_empty[ms], (mu - 1) & 1, abort, a.wait_limit)) break;
          mbar_arrive_expect_tx(&S->m_full[ms], (uint32_t)L.smeta);
          bulk_g2s(sBm + ms * L.smeta, imgB + a_op, (uint32_t)L.smeta, &S->m_full[ms]);
          m_last[ms] = mu;
        }
        item = next;
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
    // The whole warp runs the loop (waits and descriptors stay warp-uniform;
    // a wait's outcome is made uniform with __all_sync), and the elected lane
    // (lane 0 of the converged warp) issues the MMAs and commits.  A start
    // address advances the descriptor's address field (address >> 4, 14 bits)
    // by offset >> 4, without carry for shared-memory addresses below 256 KB.
    {
      const unsigned full = 0xffffffffu;
      const uint32_t idesc = idesc_f16_f32(BM, BN);
      const uint32_t lbo = BM * 16, sbo = 128;        // BM == BN
      const uint32_t blk = (uint32_t)BM * L.kc * 2;   // one slice block of one chunk
      const uint64_t bstep = blk >> 4, sstep = (2 * lbo) >> 4;
      const int nks = L.kc / 16;
      int g = 0, tc = 0;
      bool stop = false;
      for (int it = 0; !stop; it++) {
        if (!__all_sync(full, *abort == 0 && mbar_wait(&S->a_full, it & 1, abort, a.wait_limit))) break;
        const int item = __shfl_sync(full, ((volatile int *)S->islot)[it & 1], 0);
        if (item < 0) break;
        const ItemGeo G = item_geo(a, item);
        for (int tj = G.t0; tj < G.t1 && !stop; tj++, tc++) {
          const int buf = tc & 1;
          if (tc >= 2 && !__all_sync(full, mbar_wait(&S->t_empty[buf], ((tc >> 1) - 1) & 1, abort, a.wait_limit))) {
            stop = true;
            break;
          }
          const uint32_t dH = tmem + buf * 256, dL = tmem + buf * 256 + 128;
          for (int c = 0; c < L.nch; c++, g++) {
            const int st = g % L.nstage;
            if (!__all_sync(full, mbar_wait(&S->b_full[st], (g / L.nstage) & 1, abort, a.wait_limit))) {
              stop = true;
              break;
            }
            tc_fence_after();
            const uint32_t sbase = smem_addr(sStage + st * L.stage_bytes);
            const uint32_t a0 = resident ? smem_addr(sA) : sbase;
            const uint32_t b0 = resident ? sbase : sbase + (uint32_t)L.chunk_al;
            // every descriptor of the chunk first, then all its MMAs back to
            // back from the elected lane (no dependent work between them)
            const uint64_t dA0 = desc_noswizzle(a0, lbo, sbo), dB0 = desc_noswizzle(b0, lbo, sbo);
            uint64_t As[4], Bs[4];
#pragma unroll
            for (int s = 0; s < 4; s++) { As[s] = dA0 + (uint64_t)s * sstep; Bs[s] = dB0 + (uint64_t)s * sstep; }
            const bool last = c == L.nch - 1;
            if (elect_one()) {
#pragma unroll
              for (int s = 0; s < 4; s++) {
                if (s < nks) {
                  const uint32_t acc = (c > 0 || s > 0) ? 1u : 0u;
                  umma_f16(dH, As[s], Bs[s], idesc, acc);                      // a1 b1
                  umma_f16(dL, As[s], Bs[s] + bstep, idesc, acc);              // a1 b2
                  umma_f16(dL, As[s] + bstep, Bs[s], idesc, 1);                // a2 b1
                  umma_f16(dL, As[s] + bstep, Bs[s] + bstep, idesc, 1);        // a2 b2
                  umma_f16(dL, As[s], Bs[s] + 2 * bstep, idesc, 1);            // a1 b3
                  umma_f16(dL, As[s] + 2 * bstep, Bs[s], idesc, 1);            // a3 b1
                }
              }
              umma_commit(&S->b_empty[st]);
              if (last) umma_commit(&S->t_full[buf]);
            }
            __syncwarp();
          }
          if (stop) break;
        }
        if (elect_one()) umma_commit(&S->a_empty);
        __syncwarp();
      }
      if (elect_one()) umma_commit(&S->drain);
      __syncwarp();
      mbar_wait(&S->drain, 0, &S->never, 1LL << 30);
    }
  } else {
    // ---------------- epilogue (warps 2 .. 2+EPI_WARPS-1) ----------------
    // EPI_GROUPS groups of four warps; group g takes columns [32g, 32g+32) of
    // every tile, each warp the 32 TMEM lanes (= target rows) of its
    // sub-partition, in two 16-column TMEM loads.
    const int ew = warp - 2;
    const int grp = ew >> 2;
    float *wq = S->rq[ew];
    const LTab ltab{tab_base + (L.tab_sh > 0 ? (lane & ((1 << L.tab_sh) - 1)) : 0), L.tab_sh > 0 ? L.tab_sh : 0};
    const int qd = warp & 3;
    const int row = qd * 32 + lane;
    const Params *P = a.P;
    const float rc = P->rc;
    const bool exact = P->exact_t1 != 0, gfast = P->gfast != 0;
    TaskParam T0;                                  // the single call's parameters
    if constexpr (KT != KS_LIST) {
      const double s2 = a.kp.scal * 1.4426950408889634;   // Gaussian rechecks from pool coordinates
      T0.kp = a.kp; T0.t_flag = P->t_flag; T0.rho = P->rho; T0.nbmax = P->nbmax;
      T0.s2 = (float)s2; T0.s2l = (float)(s2 - (double)T0.s2);
      T0.lap = P->lap; T0.any_flag = P->any_flag; T0.centred = P->centred;
      T0.anch = P->anch; T0.sg = P->sg;
      T0.kcoin = KT == KS_LAPLACE ? lap_coincident(a.kp) : 0.0;
    }
    int g = 0, tc = 0;
    for (int it = 0; !*abort; it++) {
      if (!mbar_wait(&S->a_full, it & 1, abort, a.wait_limit)) break;
      const int item = ((volatile int *)S->islot)[it & 1];
      if (item < 0) break;
      const ItemGeo G = item_geo(a, item);
      const TaskParam &T = pick_task<KT>(S->tslot[it & 1], T0);
      const PtMeta am = ((const PtMeta *)sAmeta)[row];
      __syncwarp();
      if (lane == 0) mbar_arrive(&S->a_empty);
      RowAcc<NR> ra;
      ra.zero();
      float bsk = 0.0f;
      bool ok = true;
      for (int tj = G.t0; tj < G.t1; tj++, g++, tc++) {
        const int ms = g % NMETA, buf = tc & 1;
        if (!mbar_wait(&S->t_full[buf], (tc >> 1) & 1, abort, a.wait_limit)) { ok = false; break; }
        if (!mbar_wait(&S->m_full[ms], (g / NMETA) & 1, abort, a.wait_limit)) { ok = false; break; }
        tc_fence_after();
        const SrcMeta *bm = (const SrcMeta *)(sBm + ms * L.smeta);
        const int ncols = a.tab ? a.btile_cols[tj] : min(BN, a.n - tj * BN);
        const uint32_t tH = tmem + ((uint32_t)(qd * 32) << 16) + buf * 256;
        if constexpr (KT == KS_LIST) {
          const float lrc = T.rc;              // the task's scale (centred or not)
          const bool lexact = T.exact != 0;
          switch (T.kp.type) {
            case KS_GAUSSIAN:   // scaled units, as a single call
              tile_epilogue<KS_GAUSSIAN, false, 1>(a, T, tH, grp, row, bm, ncols, am, lrc, lexact, T.gfast != 0, ltab, ra, bsk, wq); break;
            case KS_GAUSSIAN_VAR_BANDWIDTH:
              tile_epilogue<KS_GAUSSIAN_VAR_BANDWIDTH, false, 1>(a, T, tH, grp, row, bm, ncols, am, lrc, lexact, false, ltab, ra, bsk, wq); break;
            case KS_POLYNOMIAL:
              tile_epilogue<KS_POLYNOMIAL, false, 1>(a, T, tH, grp, row, bm, ncols, am, lrc, lexact, false, ltab, ra, bsk, wq); break;
            case KS_LAPLACE:
              tile_epilogue<KS_LAPLACE, true, 1>(a, T, tH, grp, row, bm, ncols, am, lrc, lexact, false, ltab, ra, bsk, wq); break;
            case KS_TANH:
              tile_epilogue<KS_TANH, false, 1>(a, T, tH, grp, row, bm, ncols, am, lrc, lexact, false, ltab, ra, bsk, wq); break;
            case KS_QUARTIC:
              tile_epilogue<KS_QUARTIC, false, 1>(a, T, tH, grp, row, bm, ncols, am, lrc, lexact, false, ltab, ra, bsk, wq); break;
            case KS_MULTIQUADRATIC:
              tile_epilogue<KS_MULTIQUADRATIC, false, 1>(a, T, tH, grp, row, bm, ncols, am, lrc, lexact, false, ltab, ra, bsk, wq); break;
            default:
              tile_epilogue<KS_EPANECHNIKOV, false, 1>(a, T, tH, grp, row, bm, ncols, am, lrc, lexact, false, ltab, ra, bsk, wq); break;
          }
        } else {
          tile_epilogue<KT, false, NR>(a, T, tH, grp, row, bm, ncols, am, rc, exact, gfast, ltab, ra, bsk, wq);
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) { mbar_arrive(&S->t_empty[buf]); mbar_arrive(&S->m_empty[ms]); }
      }
      if (!ok) break;
      double racc[NR];
#pragma unroll
      for (int r = 0; r < NR; r++) racc[r] = ra.total(r);
      if constexpr (NR > 1) {
        // several right-hand sides: every group writes its own partials (no
        // exchange): partial[((r nsc + sc) groups + grp) ldp + i], pskip
        // [(sc groups + grp) ldp + i]; the reduction adds them in that order
        const bool rowf = KT == KS_GAUSSIAN && gfast;   // the row's low-norm factor
        const long long sc = G.t0 / a.chunk_tiles, i = (long long)G.ti * BM + row;
        if (row < G.rows) {
#pragma unroll
          for (int r = 0; r < NR; r++)
            a.partial[((r * a.nsc + sc) * EPI_GROUPS + grp) * a.ldp + i] = rowf ? racc[r] * (double)am.h : racc[r];
          if (a.pskip) a.pskip[(sc * EPI_GROUPS + grp) * a.ldp + i] = rowf ? bsk * am.h : bsk;
        }
        continue;
      }
      // Combine the groups' row sums in group order, through a slot per item
      // parity: groups 1.. write theirs and arrive on r_full, group 0 waits,
      // reads and arrives on r_empty.  Every wait is bounded (a block-wide
      // barrier here could wait forever for a warp whose earlier wait gave up).
      const int rb = it & 1, ru = it >> 1;   // slot, and its earlier uses
      double (*xs)[BM] = S->rsum[rb];
      float (*xb)[BM] = S->rskip[rb];
      if (grp > 0) {
        if (ru > 0 && !mbar_wait(&S->r_empty[rb], (ru - 1) & 1, abort, a.wait_limit)) break;
        xs[grp - 1][row] = racc[0];
        xb[grp - 1][row] = bsk;
        mbar_arrive(&S->r_full[rb]);
      } else {
        if (!mbar_wait(&S->r_full[rb], ru & 1, abort, a.wait_limit)) break;
        for (int q = 0; q < EPI_GROUPS - 1; q++) { racc[0] += xs[q][row]; bsk += xb[q][row]; }
        mbar_arrive(&S->r_empty[rb]);
        const bool rowf = KT == KS_LIST ? (T.kp.type == KS_GAUSSIAN && T.gfast != 0) : (KT == KS_GAUSSIAN && gfast);
        if (rowf) {                               // the row's low-norm factor
          racc[0] *= (double)am.h;
          bsk *= am.h;
        }
        if (row < G.rows) {
          a.partial[G.out + row] = racc[0];
          if (a.pskip) a.pskip[G.out + row] = bsk;
        }
      }
    }
  }

  __syncthreads();
  if (*abort && threadIdx.x == 0) atomicOr(a.err, DEVERR_TIMEOUT);
  if (warp == 0) { tc_fence_after(); tmem_dealloc(tmem, TMEM_COLS); }
}

// u[umap[i]] += sum over chunks of the chunk partials, in chunk order.
// Groups of columns whose values all lay below 2^-96 were left out of the row
// sums (pskip holds their sums of |w|, b): their part of row i is below
// 2^-96 b.  Where that could reach 2^-27 of |s| (in practice: rows whose
// every value is that small) the row goes to the rescue list instead.
// Anchored polynomial rows (rowc != nullptr): the row's v0^p times the sum of
// all weights, wsum[r], is added in FP64.
// NR > 1 (several right-hand sides, nrhs <= NR interleaved in u): the
// partials of every (column r, chunk, epilogue group), in that order; a row is
// rescued when the skipped groups could matter for any of its columns.
template <int NR>
__global__ void split_reduce(int m, int nsc, int ldp, const double *__restrict__ partial,
                             const float *__restrict__ pskip, double *__restrict__ u, const int *__restrict__ umap,
                             int *__restrict__ rlist, int *__restrict__ rcount, const double *__restrict__ rowc,
                             const double *__restrict__ wsum, int nrhs)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  if constexpr (NR == 1) {
    double s = 0.0;
    float b = 0.0f;
    for (int c = 0; c < nsc; c++) s += partial[(size_t)c * ldp + i];
    if (rowc) s += rowc[i] * *wsum;
    if (pskip) {
      for (int c = 0; c < nsc; c++) b += pskip[(size_t)c * ldp + i];
      if (b > 0.0f && fabs(s) < 0x1p-69 * (double)b) {
        rlist[atomicAdd(rcount, 1)] = i;
        return;
      }
    }
    u[umap ? umap[i] : i] += s;
  } else {
    double s[NR];
    double smin = 1e300;
#pragma unroll
    for (int r = 0; r < NR; r++) {
      s[r] = 0.0;
      if (r >= nrhs) continue;
      for (int c = 0; c < nsc * EPI_GROUPS; c++) s[r] += partial[((size_t)r * nsc * EPI_GROUPS + c) * ldp + i];
      if (rowc) s[r] += rowc[i] * wsum[r];
      smin = fmin(smin, fabs(s[r]));
    }
    if (pskip) {
      float b = 0.0f;
      for (int c = 0; c < nsc * EPI_GROUPS; c++) b += pskip[(size_t)c * ldp + i];
      if (b > 0.0f && smin < 0x1p-69 * (double)b) {
        rlist[atomicAdd(rcount, 1)] = i;
        return;
      }
    }
    const size_t ui = (size_t)(umap ? umap[i] : i) * nrhs;
#pragma unroll
    for (int r = 0; r < NR; r++)
      if (r < nrhs) u[ui + r] += s[r];
  }
}

// The rows of the rescue list, one warp per row: every pair of the row from
// the pool coordinates (recheck: float-pair distances, values in the FP64
// range), summed in FP64 in a fixed order.
template <int KT, int NR>
__global__ void __launch_bounds__(256) split_rescue(TileArgs a, const int *__restrict__ rlist,
                                                    const int *__restrict__ rcount, double *__restrict__ u,
                                                    const int *__restrict__ umap)
{
  __shared__ float4 tab[LTAB];
  if constexpr (KT == KS_LAPLACE) laplace_table(tab, 0);
  __syncthreads();
  const LTab ltab{tab, 0};
  const Params *P = a.P;
  TaskParam T;
  {
    const double s2 = a.kp.scal * 1.4426950408889634;
    T.kp = a.kp; T.t_flag = P->t_flag; T.rho = P->rho;
    T.s2 = (float)s2; T.s2l = (float)(s2 - (double)T.s2);
    T.lap = P->lap; T.any_flag = P->any_flag; T.centred = P->centred;
    T.kcoin = KT == KS_LAPLACE ? lap_coincident(a.kp) : 0.0;
  }
  const int nr = *rcount, lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < nr; e += nw) {
    const int i = rlist[e];
    const int nr = a.nrhs > 1 ? a.nrhs : 1;
    double r[NR];
#pragma unroll
    for (int q = 0; q < NR; q++) r[q] = 0.0;
    for (int j = lane; j < a.n; j += 32) {
      const double kv = recheck<KT, true>(a, T, ltab, i, j);
#pragma unroll
      for (int q = 0; q < NR; q++)
        if (q < nr) r[q] += kv * wcol64(a, j, q);
    }
#pragma unroll
    for (int q = 0; q < NR; q++) {
#pragma unroll
      for (int o = 16; o; o >>= 1) r[q] += __shfl_xor_sync(0xffffffffu, r[q], o);
      if (lane == 0 && q < nr) u[(size_t)(umap ? umap[i] : i) * nr + q] += r[q];
    }
  }
}

template <int NR>
cudaError_t launch_rescue_t(const TileArgs &a, int grid, const int *rlist, const int *rcount, double *u,
                            const int *umap, cudaStream_t s)
{
  switch (a.kt) {
    case KS_GAUSSIAN: split_rescue<KS_GAUSSIAN, NR><<<grid, 256, 0, s>>>(a, rlist, rcount, u, umap); break;
    case KS_GAUSSIAN_VAR_BANDWIDTH:
      split_rescue<KS_GAUSSIAN_VAR_BANDWIDTH, NR><<<grid, 256, 0, s>>>(a, rlist, rcount, u, umap); break;
    case KS_LAPLACE: split_rescue<KS_LAPLACE, NR><<<grid, 256, 0, s>>>(a, rlist, rcount, u, umap); break;
    default: return cudaSuccess;
  }
  return cudaGetLastError();
}
cudaError_t launch_rescue(const TileArgs &a, int grid, const int *rlist, const int *rcount, double *u,
                          const int *umap, cudaStream_t s, int nr)
{
  return nr > 1 ? launch_rescue_t<RMAX>(a, grid, rlist, rcount, u, umap, s)
                : launch_rescue_t<1>(a, grid, rlist, rcount, u, umap, s);
}

template <int KT, int NR>
cudaError_t launch_tiles_t(const TileArgs &a, int grid, size_t smem, cudaStream_t s)
{
  // The attribute is per function and device; raise it to what this launch needs.
  static int attr_bytes[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64 || attr_bytes[dev] < (int)smem) {
    cudaError_t e = cudaFuncSetAttribute(split_tiles<KT, NR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64) attr_bytes[dev] = (int)smem;
  }
  split_tiles<KT, NR><<<grid, NTHREADS, smem, s>>>(a);
  return cudaGetLastError();
}

template <int NR>
cudaError_t launch_tiles_nr(const TileArgs &a, int grid, size_t smem, cudaStream_t s)
{
  switch (a.kt) {
    case KS_GAUSSIAN: return launch_tiles_t<KS_GAUSSIAN, NR>(a, grid, smem, s);
    case KS_GAUSSIAN_VAR_BANDWIDTH: return launch_tiles_t<KS_GAUSSIAN_VAR_BANDWIDTH, NR>(a, grid, smem, s);
    case KS_POLYNOMIAL: return launch_tiles_t<KS_POLYNOMIAL, NR>(a, grid, smem, s);
    case KS_LAPLACE: return launch_tiles_t<KS_LAPLACE, NR>(a, grid, smem, s);
    case KS_TANH: return launch_tiles_t<KS_TANH, NR>(a, grid, smem, s);
    case KS_QUARTIC: return launch_tiles_t<KS_QUARTIC, NR>(a, grid, smem, s);
    case KS_MULTIQUADRATIC: return launch_tiles_t<KS_MULTIQUADRATIC, NR>(a, grid, smem, s);
    default: return launch_tiles_t<KS_EPANECHNIKOV, NR>(a, grid, smem, s);
  }
}

// nr: weight columns of the sweep (1, or RMAX); the list form takes one.
cudaError_t launch_tiles(const TileArgs &a, int grid, size_t smem, cudaStream_t s, int nr = 1)
{
  if (a.kt == KS_LIST) return launch_tiles_t<KS_LIST, 1>(a, grid, smem, s);
  return nr > 1 ? launch_tiles_nr<RMAX>(a, grid, smem, s) : launch_tiles_nr<1>(a, grid, smem, s);
}

size_t smem_bytes(int kpad, int kt, int nr = 1)
{
  const SmemLayout L = smem_layout(kpad, kt, nr);
  return smem_fixed(L) + (L.tab_sh >= 0 ? ((size_t)LTAB << L.tab_sh) * 16 : 0);
}

}  // namespace split

// Test hook state (gsks_split_test_wait): per host thread.
thread_local long long tl_split_wait = 0;
thread_local int tl_split_stall = 0;

// ---------------------------------------------------------------------------
int enqueue_split(Ctx *c, const ks_t *ker, int m, int n, int k, double *u, const int *umap,
                  const double *XA, const double *XA2, const int *amap, int nxa,
                  const double *XB, const double *XB2, const int *bmap, int nxb,
                  const double *w, const int *wmap, const double *hi, const double *hj,
                  cudaStream_t s, bool stream_ordered_alloc, int nrhs)
{
  using namespace split;
  (void)XA2; (void)XB2;
  // several right-hand sides (u, w with nrhs interleaved columns, nrhs <= RMAX)
  // in one sweep: every kernel value times each weight column
  if (nrhs < 1 || nrhs > RMAX) return GSKS_ERR_ARG;
  const int NRK = nrhs > 1 ? RMAX : 1;   // weight columns of the kernel
  // padded k: a multiple of the MMA k-step (16) up to one chunk, of the chunk beyond
  const int kpad = k <= KCH ? (k + 15) / 16 * 16 : (k + KCH - 1) / KCH * KCH;
  if (kpad > 1024) return GSKS_ERR_TOO_LARGE;   // the exact head accumulation needs k <= 1024
  if (smem_bytes(kpad, ker->type, NRK) > SMEM_MAX) return GSKS_ERR_TOO_LARGE;
  const int ntm = (m + BM - 1) / BM, ntn = (n + BN - 1) / BN;
  const int sms = std::max(1, c->num_sms);
  // decomposition: the source tiles of a target tile split into nsc chunks of
  // chunk_tiles, one work item each, dealt round-robin to the CTAs.  The choice
  // minimises the slowest CTA's work, waves x (chunk + one tile of per-item
  // overhead), over up to 32 items per SM (measured as fast as the best of
  // fixed 4 / 8 / 16 / 32 items per SM on every workload tried, 2-7% faster
  // than a fixed 8 where the waves came out ragged)
  int nsc = 1, chunk_tiles = ntn;
  {
    const int cmax = (int)std::min<long long>(ntn, std::max<long long>(1, (32LL * sms + ntm - 1) / ntm));
    long long best = -1;
    for (int c = 1; c <= cmax; c++) {
      const int ch = (ntn + c - 1) / c;
      if ((ntn + ch - 1) / ch != c) continue;   // same chunks as a smaller c
      const long long waves = ((long long)ntm * c + sms - 1) / sms;
      const long long cost = waves * (ch + 1);
      if (best < 0 || cost < best) { best = cost; nsc = c; chunk_tiles = ch; }
    }
  }
  const int ldp = ntm * BM;

  // workspace: params | centre | bbox | A images | B images | partials
  auto al = [](size_t x) { return (x + 1023) & ~(size_t)1023; };
  const size_t o_params = 0;
  const size_t o_centre = al(sizeof(Params));
  const size_t o_bbox = o_centre + al((size_t)k * 8);
  const size_t o_a = o_bbox + al((size_t)2 * k * 8);
  const size_t o_b = o_a + al((size_t)ntm * tile_bytes(BM, kpad));
  const size_t o_p = o_b + al((size_t)ntn * tile_bytes(BN, kpad, smeta_pt(NRK)));
  // partial sums: [nsc][ldp], or with several columns [RMAX][nsc][groups][ldp]
  const size_t nparts = NRK > 1 ? (size_t)RMAX * nsc * EPI_GROUPS * ldp : (size_t)nsc * ldp;
  const size_t nskips = NRK > 1 ? (size_t)nsc * EPI_GROUPS * ldp : (size_t)nsc * ldp;
  // float-pair copies for cheap rechecks (kernels with rechecks; written only
  // when the call may flag pairs): of the pool when the targets and sources
  // share one whose points are no more than the gathered ones (indexed by
  // pool point), else of the gathered rows (indexed by position)
  const bool same_pool = XA == XB && nxa == nxb;
  const bool ff = kt_rescue(ker->type);
  const bool ffpos = !(same_pool && nxa >= 0 && (long long)nxa <= (long long)m + n);
  const long long ffa = ffpos ? m : nxa, ffb = ffpos ? n : (same_pool ? 0 : nxb);   // points per copy
  // row rescue (exponential kernels): skipped-group weights, row list, count
  const bool defer = kt_rescue(ker->type);
  const size_t o_ps = o_p + al(nparts * 8);
  const size_t o_rl = o_ps + (defer ? al(nskips * 4) : 0);
  const size_t o_rc = o_rl + (defer ? al((size_t)m * 4) : 0);
  const size_t o_ni = o_rc + (defer ? al(4) : 0);   // work counter
  const size_t o_xaf = o_ni + al(4);
  const size_t o_xbf = o_xaf + (ff ? al((size_t)ffa * k * sizeof(float2)) : 0);
  // anchored polynomial: source mean and weight sum (ybar | wsum | block
  // partials) and the rows' v0^p
  const bool anch = ker->type == KS_TANH || ker->type == KS_QUARTIC || ker->type == KS_EPANECHNIKOV ||
                    ker->type == KS_MULTIQUADRATIC ||
                    (ker->type == KS_POLYNOMIAL && ker->powe == rint(ker->powe) && ker->powe >= 1.0 && ker->powe <= 4.0);
  const int nwb = (n + ANCHOR_WPER - 1) / ANCHOR_WPER;   // blocks of the weight sum
  const size_t o_anc = o_xbf + (ff ? al((size_t)ffb * k * sizeof(float2)) : 0);
  // ybar[k] | wsum[RMAX] | wpart[nwb nrhs] | ybsq[k] | cpart[ANCHOR_SB 2 k]
  const size_t o_rowc = o_anc + (anch ? al(((size_t)2 * k + RMAX + (size_t)nwb * nrhs +
                                            (size_t)ANCHOR_SB * 2 * k) * 8) : 0);
  const size_t total = o_rowc + (anch ? al((size_t)m * 8) : 0);
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
    const int blocks = (int)std::max<long long>((k + 255) / 256,
                                                std::min<long long>(8LL * sms, std::max<long long>(1, (tot + 255) / 256)));
    bbox_kernel<<<blocks, 256, 2 * k * sizeof(long long), s>>>(m, n, k, XA, amap, nxa, XB, bmap, nxb,
                                                               err_word(c), bbox);
  }
  params_kernel<<<1, 1024, 0, s>>>(k, ker->type, ker->scal, ker->cons, ker->powe, tau, bbox, centre, P);
  double *ybar = anch ? (double *)(ws + o_anc) : nullptr;
  double *ybsq = anch ? ybar + k + RMAX + (size_t)nwb * nrhs : nullptr;   // after the weight-sum partials
  double *rowc = anch ? (double *)(ws + o_rowc) : nullptr;
  if (anch) {
    double *wpart = ybar + k + RMAX, *cpart = ybsq + k;
    anchor_coords<<<dim3((k + 31) / 32, ANCHOR_SB), 256, 0, s>>>(n, k, XB, bmap, nxb, err_word(c), cpart);
    anchor_weights<<<nwb, 256, 0, s>>>(n, w, wmap, nrhs, wpart);
    anchor_final<<<1, 256, 0, s>>>(n, k, nwb, nrhs, cpart, wpart, ybar, ybsq, ybar + k);
  }
  pack_kernel<<<ntm, BM, 0, s>>>(0, m, k, kpad, XA, amap, nxa, err_word(c), nullptr, nullptr, hi, ker->type,
                                 centre, P, ws + o_a, nullptr, nullptr, nullptr, ybar, rowc, 1, ybsq);
  pack_kernel<<<ntn, BN, 0, s>>>(1, n, k, kpad, XB, bmap, nxb, err_word(c), w, wmap, hj, ker->type, centre,
                                 P, ws + o_b, nullptr, nullptr, nullptr, nullptr, nullptr, nrhs);

  TileArgs a{};
  a.m = m; a.n = n; a.k = k; a.kpad = kpad; a.kt = ker->type;
  a.ntm = ntm; a.ntn = ntn; a.nsc = nsc; a.chunk_tiles = chunk_tiles;
  a.imgA = ws + o_a; a.imgB = ws + o_b;
  a.XA = XA; a.XB = XB; a.amap = amap; a.bmap = bmap; a.wmap = wmap; a.w = w;
  a.nxa = nxa; a.nxb = nxb;
  a.hi = hi; a.hj = hj;
  int ff_launches = 0;
  if (ff) {
    float2 *xaf = (float2 *)(ws + o_xaf), *xbf = ffb == 0 ? xaf : (float2 *)(ws + o_xbf);
    const long long na_c = ffa * k, nb_c = ffb * k;
    const int ga = (int)std::min<long long>(8LL * sms, (na_c + 255) / 256 + 1);
    const int gb = (int)std::min<long long>(8LL * sms, (nb_c + 255) / 256 + 1);
    pool_split<<<ga, 256, 0, s>>>(na_c, k, XA, ffpos ? amap : nullptr, nxa, xaf, P);
    ff_launches = 1;
    if (ffb) { pool_split<<<gb, 256, 0, s>>>(nb_c, k, XB, ffpos ? bmap : nullptr, nxb, xbf, P); ff_launches = 2; }
    a.XAf = xaf; a.XBf = xbf;
    a.ffpos = ffpos ? 1 : 0;
  }
  a.kp = make_kparams(ker, hi, hj);
  a.kp.coinc = coincidence_eps(k);
  a.P = P;
  a.partial = (double *)(ws + o_p);
  a.pskip = defer ? (float *)(ws + o_ps) : nullptr;
  a.next_item = (int *)(ws + o_ni);
  a.ldp = ldp;
  a.err = err_word(c);
  a.wait_limit = tl_split_wait > 0 ? tl_split_wait : WAIT_LIMIT;
  a.stall = tl_split_stall;
  a.nrhs = nrhs;
  const int grid = std::min(ntm * nsc, sms);
  int *rlist = defer ? (int *)(ws + o_rl) : nullptr, *rcount = defer ? (int *)(ws + o_rc) : nullptr;
  // diagnostics of this call (gsks_split_stats): rechecked pairs, rescued rows
  if (!c->stats.ensure(16)) {
    if (stream_ordered_alloc) cudaFreeAsync(ws, s);
    return GSKS_ERR_ALLOC;
  }
  a.nrecheck = (unsigned long long *)c->stats.p;
  cudaError_t e = cudaMemsetAsync(c->stats.p, 0, 16, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(a.next_item, 0, sizeof(int), s);
  if (e == cudaSuccess && defer) e = cudaMemsetAsync(rcount, 0, sizeof(int), s);
  if (e == cudaSuccess) e = launch_tiles(a, grid, smem_bytes(kpad, a.kt, NRK), s, NRK);
  if (e == cudaSuccess) {
    if (NRK > 1)
      split_reduce<RMAX><<<(m + 255) / 256, 256, 0, s>>>(m, nsc, ldp, a.partial, a.pskip, u, umap, rlist, rcount,
                                                         rowc, anch ? ybar + k : nullptr, nrhs);
    else
      split_reduce<1><<<(m + 255) / 256, 256, 0, s>>>(m, nsc, ldp, a.partial, a.pskip, u, umap, rlist, rcount, rowc,
                                                      anch ? ybar + k : nullptr, 1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && defer)
    e = cudaMemcpyAsync((uint8_t *)c->stats.p + 8, rcount, sizeof(int), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess && defer)
    e = launch_rescue(a, std::max(1, std::min(2 * sms, (m + 7) / 8)), rlist, rcount, u, umap, s, NRK);
  if (stream_ordered_alloc) cudaFreeAsync(ws, s);
  if (e != cudaSuccess) return cuda_status(e, "split launch");
  note_launches((defer ? 8 : 7) + ff_launches + (anch ? 3 : 0));
  return GSKS_OK;
}

// ---------------------------------------------------------------------------
namespace split {

// Deferred row rescue of the list form: a target row of a task whose skipped
// groups (values below 2^-96) could reach 2^-27 of its sum is listed, then
// recomputed over all of the task's sources; its chunk sums are replaced by
// the result (chunk 0) and zeros, so that the merge adds it as before.
__device__ __forceinline__ int task_of(const int *__restrict__ aoff, int ntask, int pos)
{
  int lo = 0, hi = ntask - 1;                    // last t with aoff[t] <= pos
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (aoff[mid] <= pos) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void list_rescue_mark(int ma, int ntask, const int *__restrict__ aoff,
                                 const SplitTaskGeo *__restrict__ tg, const double *__restrict__ partial,
                                 const float *__restrict__ pskip, int *__restrict__ rlist, int *__restrict__ rcount)
{
  const int pos = blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= ma) return;
  const SplitTaskGeo G = tg[task_of(aoff, ntask, pos)];
  const int r = pos - G.a0;
  double sum = 0.0;
  float b = 0.0f;
  for (int c = 0; c < G.nsc; c++) {
    sum += partial[G.pbase + (long long)c * G.m + r];
    b += pskip[G.pbase + (long long)c * G.m + r];
  }
  if (b > 0.0f && fabs(sum) < 0x1p-69 * (double)b) rlist[atomicAdd(rcount, 1)] = pos;
}

// Anchored polynomial tasks: each row's v0^p times the task's weight sum
// (FP64) goes into the row's first chunk partial, before the merge.
__global__ void list_anchor_add(int ma, int ntask, const int *__restrict__ aoff, const SplitTaskGeo *__restrict__ tg,
                                const TaskParam *__restrict__ tp, const double *__restrict__ rowc,
                                const double *__restrict__ wsum, double *__restrict__ partial)
{
  const int pos = blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= ma) return;
  const int t = task_of(aoff, ntask, pos);
  const SplitTaskGeo G = tg[t];
  if (!tp[t].anch || G.n <= 0 || G.m <= 0) return;
  partial[G.pbase + (pos - G.a0)] += rowc[pos] * wsum[t];
}

__global__ void __launch_bounds__(256) list_rescue(TileArgs a, int ntask, const int *__restrict__ aoff,
                                                   const SplitTaskGeo *__restrict__ tg,
                                                   const int *__restrict__ rlist, const int *__restrict__ rcount)
{
  __shared__ float4 tab[LTAB];
  laplace_table(tab, 0);
  __syncthreads();
  const LTab ltab{tab, 0};
  const int nr = *rcount, lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < nr; e += nw) {
    const int pos = rlist[e];
    const int t = task_of(aoff, ntask, pos);
    const SplitTaskGeo G = tg[t];
    const TaskParam &T = a.tp[t];
    double r = 0.0;
    for (int j = G.b0 + lane; j < G.b0 + G.n; j += 32) {
      double kv;
      switch (T.kp.type) {
        case KS_GAUSSIAN: kv = recheck<KS_GAUSSIAN, true>(a, T, ltab, pos, j); break;
        case KS_GAUSSIAN_VAR_BANDWIDTH: kv = recheck<KS_GAUSSIAN_VAR_BANDWIDTH, true>(a, T, ltab, pos, j); break;
        default: kv = recheck<KS_LAPLACE, true>(a, T, ltab, pos, j); break;
      }
      r += kv * wcol64(a, j, 0);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    if (lane == 0) {
      const int row = pos - G.a0;
      a.partial[G.pbase + row] = r;
      for (int c = 1; c < G.nsc; c++) a.partial[G.pbase + (long long)c * G.m + row] = 0.0;
    }
  }
}

}  // namespace split

// ---------------------------------------------------------------------------
// Split-precision form of dgsks_list.  Every task's targets and sources are
// packed into tiles of their own (tile images carry the task's centring and
// bandwidths); a work item is (task, target tile, up to chunk / BN source
// tiles), and every item writes the row sums of its chunk to
// partial[pbase[t] + sc * m_t + r], the layout the list merge reads.  One
// bounding box, hence one scale and one centre, covers all tasks, and the
// per-task flag thresholds come from it.
//
// split_list_plan builds the tile and item tables of a fixed set of lists on
// the device (and sizes the workspace); split_list_run evaluates them with the
// current coordinates and weights, launches only.
int split_list_plan(SplitListPlan &Pl, const KParams *kps, int ntask, int k, const int *hoff_a, const int *hoff_b,
                    const long long *pbase, int chunk, int nxa, int nxb, bool same_pool, cudaStream_t s)
{
  using namespace split;
  if (chunk % BN) return GSKS_ERR_ARG;
  const int kpad = k <= KCH ? (k + 15) / 16 * 16 : (k + KCH - 1) / KCH * KCH;
  if (kpad > 1024) return GSKS_ERR_TOO_LARGE;
  const int chunk_tiles = chunk / BN;

  // tiles and items on the host: counts per task, offsets, then every task's
  // entries filled in parallel (the same order as a serial pass: task, then
  // source chunk, then target tile)
  std::vector<int> ota(ntask + 1, 0), otb(ntask + 1, 0);
  std::vector<long long> oit(ntask + 1, 0);
  long long na = 0, nb = 0;
  for (int t = 0; t < ntask; t++) {
    const int m = hoff_a[t + 1] - hoff_a[t], n = hoff_b[t + 1] - hoff_b[t];
    const bool live = m > 0 && n > 0;
    const int ca = live ? (m + BM - 1) / BM : 0, cb = live ? (n + BN - 1) / BN : 0;
    if (live) { na += m; nb += n; }
    ota[t + 1] = ota[t] + ca;
    otb[t + 1] = otb[t] + cb;
    oit[t + 1] = oit[t] + (long long)ca * ((cb + chunk_tiles - 1) / chunk_tiles);
  }
  if (na > INT32_MAX || nb > INT32_MAX || oit[ntask] > INT32_MAX) return GSKS_ERR_TOO_LARGE;
  std::vector<int2> ta(ota[ntask]), tb(otb[ntask]);
  std::vector<int> ta_task(ota[ntask]), tb_task(otb[ntask]), tb_cols(otb[ntask]);
  std::vector<SplitItem> items(oit[ntask]);
  std::vector<int> cost(oit[ntask]);     // relative epilogue cost: source tiles, x3 for Laplace
#pragma omp parallel for schedule(dynamic, 64) if (ntask > 512)
  for (int t = 0; t < ntask; t++) {
    const int m = hoff_a[t + 1] - hoff_a[t], n = hoff_b[t + 1] - hoff_b[t];
    if (m <= 0 || n <= 0) continue;
    const int a_base = ota[t], b_base = otb[t];
    for (int i0 = 0; i0 < m; i0 += BM) {
      ta[a_base + i0 / BM] = make_int2(hoff_a[t] + i0, std::min(BM, m - i0));
      ta_task[a_base + i0 / BM] = t;
    }
    for (int j0 = 0; j0 < n; j0 += BN) {
      tb[b_base + j0 / BN] = make_int2(hoff_b[t] + j0, std::min(BN, n - j0));
      tb_task[b_base + j0 / BN] = t;
      tb_cols[b_base + j0 / BN] = std::min(BN, n - j0);
    }
    const int ntn = otb[t + 1] - b_base;
    // the Laplace evaluation dominates the epilogue
    const int wkt = kps[t].type == KS_LAPLACE ? 3 : 1;
    long long q = oit[t];
    for (int sc = 0; sc * chunk_tiles < ntn; sc++)
      for (int i0 = 0; i0 < m; i0 += BM, q++) {
        SplitItem it{};
        it.a_tile = a_base + i0 / BM;
        it.b0 = b_base + sc * chunk_tiles;
        it.b1 = b_base + std::min(ntn, (sc + 1) * chunk_tiles);
        it.task = t;
        it.out = pbase[t] + (long long)sc * m + i0;
        it.rows = std::min(BM, m - i0);
        items[q] = it;
        cost[q] = wkt * (it.b1 - it.b0);
      }
  }
  {
    // largest cost first, ties in build order: a counting sort over the few
    // distinct costs (bucket cmax - cost)
    int cmax = 0;
    for (const int c : cost) cmax = std::max(cmax, c);
    std::vector<size_t> start((size_t)cmax + 2, 0);
    for (const int c : cost) start[(size_t)(cmax - c) + 1]++;
    for (int b = 0; b <= cmax; b++) start[b + 1] += start[b];
    std::vector<SplitItem> sorted(items.size());
    for (size_t i = 0; i < items.size(); i++) sorted[start[cmax - cost[i]]++] = items[i];
    items.swap(sorted);
  }
  std::vector<SplitTaskGeo> tg(ntask);
  long long ptotal = 0;
  for (int t = 0; t < ntask; t++) {
    const int m = hoff_a[t + 1] - hoff_a[t], n = hoff_b[t + 1] - hoff_b[t];
    const int nsc = (m > 0 && n > 0) ? (n + chunk - 1) / chunk : 0;
    tg[t] = SplitTaskGeo{pbase[t], hoff_a[t], m, hoff_b[t], n, nsc, 0};
    ptotal = std::max(ptotal, pbase[t] + (long long)nsc * m);
  }

  auto al = [](size_t x) { return (x + 1023) & ~(size_t)1023; };
  Pl.ntask = ntask; Pl.k = k; Pl.kpad = kpad;
  Pl.ma = hoff_a[ntask]; Pl.mb = hoff_b[ntask];
  Pl.nxa = nxa; Pl.nxb = nxb; Pl.same_pool = same_pool;
  Pl.n_ta = (int)ta.size(); Pl.n_tb = (int)tb.size(); Pl.n_items = (int)items.size();
  Pl.o_params = 0;
  Pl.o_centre = al(sizeof(Params));
  Pl.o_bbox = Pl.o_centre + al((size_t)k * 8);
  Pl.o_ta = Pl.o_bbox + al((size_t)2 * k * 8);
  Pl.o_tat = Pl.o_ta + al(ta.size() * sizeof(int2));
  Pl.o_tb = Pl.o_tat + al(ta.size() * sizeof(int));
  Pl.o_tbt = Pl.o_tb + al(tb.size() * sizeof(int2));
  Pl.o_tbc = Pl.o_tbt + al(tb.size() * sizeof(int));
  Pl.o_items = Pl.o_tbc + al(tb.size() * sizeof(int));
  Pl.o_kps = Pl.o_items + al(items.size() * sizeof(SplitItem));
  Pl.o_tp = Pl.o_kps + al((size_t)ntask * sizeof(KParams));
  Pl.o_a = Pl.o_tp + al((size_t)ntask * sizeof(TaskParam));
  Pl.o_b = Pl.o_a + al(ta.size() * tile_bytes(BM, kpad));
  // float-pair copies of the pools for the rechecks (one when both sides share it)
  Pl.o_tg = Pl.o_b + al(tb.size() * tile_bytes(BN, kpad));
  Pl.o_aoff = Pl.o_tg + al((size_t)ntask * sizeof(SplitTaskGeo));
  Pl.o_pskip = Pl.o_aoff + al(((size_t)ntask + 1) * sizeof(int));
  Pl.o_rl = Pl.o_pskip + al((size_t)std::max(ptotal, 1LL) * sizeof(float));
  Pl.o_rc = Pl.o_rl + al((size_t)std::max(Pl.ma, 1) * sizeof(int));
  Pl.o_ni = Pl.o_rc + al(sizeof(int));
  Pl.o_xaf = Pl.o_ni + al(sizeof(int));
  Pl.o_xbf = Pl.o_xaf + al((size_t)nxa * k * sizeof(float2));
  // anchored polynomial tasks: per-task source means and weight sums, and the
  // rows' v0^p
  Pl.any_anch = false;
  for (int t = 0; t < ntask && !Pl.any_anch; t++)
    Pl.any_anch = (kps[t].type == KS_POLYNOMIAL && kps[t].pmode == POW_INT && kps[t].pint >= 1 && kps[t].pint <= 4) ||
                  kps[t].type == KS_TANH;
  Pl.o_ybar = Pl.o_xbf + (same_pool ? 0 : al((size_t)nxb * k * sizeof(float2)));
  Pl.o_wsum = Pl.o_ybar + (Pl.any_anch ? al((size_t)ntask * k * 8) : 0);
  Pl.o_rowc = Pl.o_wsum + (Pl.any_anch ? al((size_t)ntask * 8) : 0);
  // per-task boxes (2 k keys) and centres (k doubles)
  Pl.o_tbox = Pl.o_rowc + (Pl.any_anch ? al((size_t)std::max(Pl.ma, 1) * 8) : 0);
  Pl.o_tcen = Pl.o_tbox + al((size_t)ntask * 2 * k * sizeof(long long));
  const size_t total = Pl.o_tcen + al((size_t)ntask * k * sizeof(double));
  if (!Pl.ws.ensure(total)) return GSKS_ERR_ALLOC;
  uint8_t *ws = (uint8_t *)Pl.ws.p;
  auto up = [&](size_t off, const void *src, size_t bytes) {
    return bytes == 0 || cudaMemcpyAsync(ws + off, src, bytes, cudaMemcpyHostToDevice, s) == cudaSuccess;
  };
  if (!(up(Pl.o_ta, ta.data(), ta.size() * sizeof(int2)) &&
        up(Pl.o_tat, ta_task.data(), ta_task.size() * sizeof(int)) &&
        up(Pl.o_tb, tb.data(), tb.size() * sizeof(int2)) &&
        up(Pl.o_tbt, tb_task.data(), tb_task.size() * sizeof(int)) &&
        up(Pl.o_tbc, tb_cols.data(), tb_cols.size() * sizeof(int)) &&
        up(Pl.o_items, items.data(), items.size() * sizeof(SplitItem)) &&
        up(Pl.o_kps, kps, (size_t)ntask * sizeof(KParams)) &&
        up(Pl.o_tg, tg.data(), tg.size() * sizeof(SplitTaskGeo)) &&
        up(Pl.o_aoff, hoff_a, ((size_t)ntask + 1) * sizeof(int))))
    return cuda_status(cudaGetLastError(), "split list tables");
  // the host vectors above die here: the copies must have left them
  cudaError_t e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? GSKS_OK : cuda_status(e, "split list tables");
}

int split_list_run(const SplitListPlan &Pl, Ctx *c, const double *XA, const int *a_idx, const double *XB,
                   const int *b_idx, const double *w, const int *w_idx, double *partial, int *err, cudaStream_t s,
                   int *launches)
{
  using namespace split;
  if (Pl.n_items == 0) return GSKS_OK;
  const int k = Pl.k, kpad = Pl.kpad, ntask = Pl.ntask, nxa = Pl.nxa, nxb = Pl.nxb;
  uint8_t *ws = (uint8_t *)Pl.ws.p;
  Params *P = (Params *)(ws + Pl.o_params);
  double *centre = (double *)(ws + Pl.o_centre);
  long long *bbox = (long long *)(ws + Pl.o_bbox);
  TaskParam *tp = (TaskParam *)(ws + Pl.o_tp);
  const float tau = 5e-7f;
  const int sms = std::max(1, c->num_sms);
  const SplitTaskGeo *tg = (const SplitTaskGeo *)(ws + Pl.o_tg);
  long long *tbox = (long long *)(ws + Pl.o_tbox);
  double *tcen = (double *)(ws + Pl.o_tcen);
  bbox_init<<<1, 256, 0, s>>>(k, bbox);
  // every task's box (its targets and sources), folded into the global box
  list_box_kernel<<<ntask, 256, 0, s>>>(ntask, k, tg, XA, a_idx, nxa, XB, b_idx, nxb, err, tbox, bbox);
  params_kernel<<<1, 1024, 0, s>>>(k, KS_LIST, 0.0, 0.0, 0.0, tau, bbox, centre, P);
  task_params_kernel<<<(ntask + 127) / 128, 128, 0, s>>>(ntask, (const KParams *)(ws + Pl.o_kps), P, tau, tp, tbox,
                                                          tcen);
  double *ybar = Pl.any_anch ? (double *)(ws + Pl.o_ybar) : nullptr;
  double *wsum = Pl.any_anch ? (double *)(ws + Pl.o_wsum) : nullptr;
  double *rowc = Pl.any_anch ? (double *)(ws + Pl.o_rowc) : nullptr;
  if (Pl.any_anch)
    list_anchor<<<ntask, 256, 256 * sizeof(double), s>>>(ntask, k, tp, tg, XB, b_idx, nxb, w, w_idx, err, ybar, wsum);
  pack_kernel<<<Pl.n_ta, BM, 0, s>>>(0, 0, k, kpad, XA, a_idx, nxa, err, nullptr, nullptr, nullptr, KS_LIST,
                                     tcen, P, ws + Pl.o_a, (const int2 *)(ws + Pl.o_ta),
                                     (const int *)(ws + Pl.o_tat), tp, ybar, rowc);
  pack_kernel<<<Pl.n_tb, BN, 0, s>>>(1, 0, k, kpad, XB, b_idx, nxb, err, w, w_idx, nullptr, KS_LIST,
                                     tcen, P, ws + Pl.o_b, (const int2 *)(ws + Pl.o_tb),
                                     (const int *)(ws + Pl.o_tbt), tp, nullptr, nullptr);
  float2 *xaf = (float2 *)(ws + Pl.o_xaf), *xbf = Pl.same_pool ? xaf : (float2 *)(ws + Pl.o_xbf);
  {
    const long long na_c = (long long)nxa * k, nb_c = (long long)nxb * k;
    pool_split<<<(int)std::min<long long>(8LL * sms, (na_c + 255) / 256 + 1), 256, 0, s>>>(na_c, k, XA, nullptr, -1, xaf,
                                                                                        nullptr);
    if (!Pl.same_pool)
      pool_split<<<(int)std::min<long long>(8LL * sms, (nb_c + 255) / 256 + 1), 256, 0, s>>>(nb_c, k, XB, nullptr, -1,
                                                                                          xbf, nullptr);
  }
  TileArgs a{};
  a.k = k; a.kpad = kpad; a.kt = KS_LIST;
  a.XAf = xaf; a.XBf = xbf;
  a.imgA = ws + Pl.o_a; a.imgB = ws + Pl.o_b;
  a.XA = XA; a.XB = XB; a.amap = a_idx; a.bmap = b_idx; a.wmap = w_idx; a.w = w;
  a.nxa = nxa; a.nxb = nxb;
  a.P = P;
  a.partial = partial;
  a.pskip = (float *)(ws + Pl.o_pskip);
  a.next_item = (int *)(ws + Pl.o_ni);
  a.err = err;
  a.nrhs = 1;
  a.wait_limit = tl_split_wait > 0 ? tl_split_wait : WAIT_LIMIT;
  a.stall = tl_split_stall;
  a.tab = (const SplitItem *)(ws + Pl.o_items);
  a.ntab = Pl.n_items;
  a.tp = tp;
  a.btile_cols = (const int *)(ws + Pl.o_tbc);
  const int grid = std::min(Pl.n_items, sms);
  int *rlist = (int *)(ws + Pl.o_rl), *rcount = (int *)(ws + Pl.o_rc);
  const int *aoff = (const int *)(ws + Pl.o_aoff);
  cudaError_t e = cudaMemsetAsync(rcount, 0, sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(a.next_item, 0, sizeof(int), s);
  if (e == cudaSuccess) e = launch_tiles(a, grid, smem_bytes(kpad, a.kt), s);
  if (e == cudaSuccess && Pl.ma > 0 && Pl.any_anch)
    list_anchor_add<<<(Pl.ma + 255) / 256, 256, 0, s>>>(Pl.ma, ntask, aoff, tg, tp, rowc, wsum, partial);
  if (e == cudaSuccess && Pl.ma > 0) {
    list_rescue_mark<<<(Pl.ma + 255) / 256, 256, 0, s>>>(Pl.ma, ntask, aoff, tg, partial, a.pskip, rlist, rcount);
    list_rescue<<<std::max(1, std::min(2 * sms, (Pl.ma + 7) / 8)), 256, 0, s>>>(a, ntask, aoff, tg, rlist, rcount);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return cuda_status(e, "split list launch");
  *launches += (Pl.same_pool ? 10 : 11) + (Pl.any_anch ? 2 : 0);
  return GSKS_OK;
}

}  // namespace gsks

using namespace gsks;

// Diagnostics (gsks.h) of this thread's last single split-precision call.
extern "C" int gsks_split_stats(long long *rechecked_pairs, int *rescued_rows)
{
  Ctx *c = get_ctx();
  if (!c) return gsks_last_error();
  unsigned long long v[2] = {0, 0};
  if (c->stats.p) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(v, c->stats.p, 16, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_status(e, "gsks_split_stats");
  }
  if (rechecked_pairs) *rechecked_pairs = (long long)v[0];
  if (rescued_rows) *rescued_rows = (int)(v[1] & 0xffffffffu);
  return set_status(GSKS_OK, nullptr);
}

// Test hook (gsks.h): the wait limit and the producer stall of this thread's
// later split-precision calls.
extern "C" int gsks_split_test_wait(long long wait_cycles, int stall)
{
  tl_split_wait = wait_cycles > 0 ? wait_cycles : 0;
  tl_split_stall = stall ? 1 : 0;
  return set_status(GSKS_OK, nullptr);
}
