// gsks_sort.cu -- owner lists of the batched merge, built on the device.
//
// dgsks_list adds, for every u entry, the contributions of all target-list
// positions that name it, in ascending position order (a fixed order, so the
// result does not depend on scheduling).  The grouping is a stable LSD radix
// sort of the list's u indices with the positions as values: positions start
// ascending and every pass is stable, so they stay ascending within an entry.
// Each 8-bit pass is a per-tile digit histogram, one exclusive scan over all
// (digit, tile) counts and a stable scatter that ranks equal digits by warp
// match masks and per-warp counts.
#include "gsks.h"
#include "gsks_internal.cuh"
#include "gsks_host.h"

#include <algorithm>

namespace gsks {
namespace {

constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;   // elements per tile (one block)
constexpr int RS_BINS = 256;                     // 8-bit digits
constexpr int RS_WARPS = RS_THREADS / 32;

// keys = u_idx with out-of-range entries replaced by 0 (and flagged), vals = i.
__global__ void rs_init(int n, const int *__restrict__ u_idx, int nu, int *__restrict__ keys,
                        int *__restrict__ vals, int *err)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += blockDim.x * gridDim.x) {
    int key = u_idx[i];
    if (key < 0 || key >= nu) { atomicOr(err, DEVERR_MAP_RANGE); key = 0; }
    keys[i] = key;
    vals[i] = i;
  }
}

// Digit histogram of one tile, stored digit-major: hist[d * ntile + tile].
__global__ void __launch_bounds__(RS_THREADS) rs_hist(int n, const int *__restrict__ keys, int shift, int ntile,
                                                      int *__restrict__ hist)
{
  __shared__ int h[RS_BINS];
  for (int d = threadIdx.x; d < RS_BINS; d += RS_THREADS) h[d] = 0;
  __syncthreads();
  const int base = blockIdx.x * RS_TILE;
  for (int r = 0; r < RS_ITEMS; r++) {
    const int i = base + r * RS_THREADS + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & (RS_BINS - 1)], 1);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < RS_BINS; d += RS_THREADS) hist[(size_t)d * ntile + blockIdx.x] = h[d];
}

// Stable scatter of one tile: element i goes to offs[d * ntile + tile] plus the
// number of earlier elements of the tile with the same digit d.
__global__ void __launch_bounds__(RS_THREADS) rs_scatter(int n, const int *__restrict__ kin,
                                                         const int *__restrict__ vin, int *__restrict__ kout,
                                                         int *__restrict__ vout, int shift, int ntile,
                                                         const int *__restrict__ offs)
{
  __shared__ int run[RS_BINS];               // slot of the next element of each digit
  __shared__ int wcnt[RS_WARPS][RS_BINS];    // this round's count per warp and digit
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int d = threadIdx.x; d < RS_BINS; d += RS_THREADS) run[d] = offs[(size_t)d * ntile + blockIdx.x];
  const int base = blockIdx.x * RS_TILE;
  for (int r = 0; r < RS_ITEMS; r++) {
    for (int x = threadIdx.x; x < RS_WARPS * RS_BINS; x += RS_THREADS) (&wcnt[0][0])[x] = 0;
    __syncthreads();
    const int i = base + r * RS_THREADS + threadIdx.x;   // element order = (round, warp, lane)
    const bool valid = i < n;
    int key = 0, val = 0, d = -1;
    if (valid) { key = kin[i]; val = vin[i]; d = (key >> shift) & (RS_BINS - 1); }
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int lrank = __popc(peers & ((1u << lane) - 1u));
    if (valid && lane == __ffs(peers) - 1) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    int dst = 0;
    if (valid) {
      int before = 0;
      for (int w = 0; w < warp; w++) before += wcnt[w][d];
      dst = run[d] + before + lrank;
    }
    __syncthreads();                         // every read of run[] precedes its update
    if (valid) { kout[dst] = key; vout[dst] = val; }
    for (int dd = threadIdx.x; dd < RS_BINS; dd += RS_THREADS) {
      int tot = 0;
      for (int w = 0; w < RS_WARPS; w++) tot += wcnt[w][dd];
      run[dd] += tot;
    }
    __syncthreads();
  }
}

// ---- exclusive scan of int arrays ------------------------------------------
constexpr int SC_THREADS = 1024;
constexpr int SC_ITEMS = 4;
constexpr int SC_TILE = SC_THREADS * SC_ITEMS;

// Exclusive scan within tiles of SC_TILE elements; tile totals to sums (if any).
__global__ void __launch_bounds__(SC_THREADS) scan_tiles(int n, const int *__restrict__ in, int *__restrict__ out,
                                                         int *__restrict__ sums)
{
  __shared__ int wsum[SC_THREADS / 32];
  const int base = blockIdx.x * SC_TILE + threadIdx.x * SC_ITEMS;
  int v[SC_ITEMS], s = 0;
  for (int j = 0; j < SC_ITEMS; j++) { v[j] = base + j < n ? in[base + j] : 0; s += v[j]; }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = s;                                 // inclusive warp scan of the thread sums
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int t = lane < SC_THREADS / 32 ? wsum[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < SC_THREADS / 32) wsum[lane] = t;   // inclusive over warps
  }
  __syncthreads();
  int run = x - s + (warp > 0 ? wsum[warp - 1] : 0);
  for (int j = 0; j < SC_ITEMS; j++) {
    if (base + j < n) out[base + j] = run;
    run += v[j];
  }
  if (sums && threadIdx.x == SC_THREADS - 1) sums[blockIdx.x] = wsum[SC_THREADS / 32 - 1];
}

__global__ void scan_add(int n, int *__restrict__ out, const int *__restrict__ tile_off)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += tile_off[i / SC_TILE];
}

size_t scan_work_ints(int n)
{
  size_t w = 0;
  while (n > SC_TILE) {
    n = (n + SC_TILE - 1) / SC_TILE;
    w += 2 * (size_t)n;
  }
  return w + 1;
}

// out = exclusive scan of in (n elements); work holds scan_work_ints(n) ints.
void scan_exclusive(int n, const int *in, int *out, int *work, cudaStream_t s, int *launches)
{
  const int nt = (n + SC_TILE - 1) / SC_TILE;
  if (nt <= 1) {
    scan_tiles<<<1, SC_THREADS, 0, s>>>(n, in, out, nullptr);
    (*launches)++;
    return;
  }
  int *sums = work, *sums_off = work + nt;
  scan_tiles<<<nt, SC_THREADS, 0, s>>>(n, in, out, sums);
  scan_exclusive(nt, sums, sums_off, work + 2 * (size_t)nt, s, launches);
  scan_add<<<(n + 255) / 256, 256, 0, s>>>(n, out, sums_off);
  *launches += 2;
}

// Segment heads of the sorted keys: ent_u / own_off per distinct key, nent.
__global__ void seg_flags(int n, const int *__restrict__ keys, int *__restrict__ flag)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

__global__ void seg_emit(int n, const int *__restrict__ keys, const int *__restrict__ flag,
                         const int *__restrict__ idx, int *__restrict__ ent_u, int *__restrict__ own_off,
                         int *__restrict__ nent)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (flag[i]) { ent_u[idx[i]] = keys[i]; own_off[idx[i]] = i; }
  if (i == n - 1) {
    const int ne = idx[i] + flag[i];
    own_off[ne] = n;
    *nent = ne;
  }
}

}  // namespace

size_t owner_work_bytes(int na)
{
  const int ntile = (na + RS_TILE - 1) / RS_TILE;
  const int nh = std::max(RS_BINS * ntile, na);
  const size_t ints = 4 * (size_t)na + 2 * (size_t)nh + scan_work_ints(nh) + 64;
  return ints * sizeof(int);
}

int owner_lists(const int *u_idx, int na, int nu, void *work, int *own_pos, int *ent_u, int *own_off, int *nent,
                int *err, cudaStream_t s, int *launches)
{
  if (na <= 0) return GSKS_OK;
  const int ntile = (na + RS_TILE - 1) / RS_TILE;
  const int nh = std::max(RS_BINS * ntile, na);
  int *k0 = (int *)work, *v0 = k0 + na, *k1 = v0 + na, *v1 = k1 + na;
  int *hist = v1 + na, *offs = hist + nh, *swork = offs + nh;
  int bits = 1;
  while (bits < 31 && (1LL << bits) < (long long)nu) bits++;
  const int passes = (bits + 7) / 8;
  rs_init<<<std::min((na + 255) / 256, 4096), 256, 0, s>>>(na, u_idx, nu, k0, v0, err);
  (*launches)++;
  for (int p = 0; p < passes; p++) {
    rs_hist<<<ntile, RS_THREADS, 0, s>>>(na, k0, 8 * p, ntile, hist);
    scan_exclusive(RS_BINS * ntile, hist, offs, swork, s, launches);
    rs_scatter<<<ntile, RS_THREADS, 0, s>>>(na, k0, v0, k1, v1, 8 * p, ntile, offs);
    *launches += 2;
    std::swap(k0, k1);
    std::swap(v0, v1);
  }
  // k0 / v0: keys and positions sorted by key, positions ascending within a key
  cudaMemcpyAsync(own_pos, v0, (size_t)na * sizeof(int), cudaMemcpyDeviceToDevice, s);
  int *flag = hist, *idx = offs;           // both at least na long
  seg_flags<<<(na + 255) / 256, 256, 0, s>>>(na, k0, flag);
  scan_exclusive(na, flag, idx, swork, s, launches);
  seg_emit<<<(na + 255) / 256, 256, 0, s>>>(na, k0, flag, idx, ent_u, own_off, nent);
  *launches += 2;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GSKS_OK : cuda_status(e, "owner lists");
}

}  // namespace gsks
