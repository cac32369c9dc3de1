// gsks_host.h -- host-side context and helpers shared by the C-ABI units.
#pragma once

#include <cstddef>
#include <cuda_runtime.h>
#include "ks.h"
#include "gsks_internal.cuh"
#include <nvtx3/nvToolsExt.h>

namespace gsks {

// A named NVTX range around an entry point, for timeline profilers (Nsight
// Systems, ncu's NVTX filters); a push and a pop of a few nanoseconds when no
// tool is attached.
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

// Growable device / pinned host buffers owned by a per-thread context.
struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  bool ensure(size_t bytes);
  void release();
};
struct PinBuf {
  void *p = nullptr;
  size_t cap = 0;
  bool ensure(size_t bytes);
  void release();
};

// Per host thread, per device: stream, error flags, staging and workspace.
struct Ctx {
  int device = -1;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  DevBuf partial, err;
  DevBuf dA, dA2, dB, dB2, dw, du, dhi, dhj, dwork;
  DevBuf rmaps;                // per-rhs u and w maps of the multi-rhs calls
  DevBuf serr;                 // synchronous calls: [0] device error flags, [1] sgsks map-check flag
  DevBuf stats;                // the last split-precision call: rechecked pairs (u64), rescued rows (int)
  int *cur_err = nullptr;      // the error word kernels write (nullptr: err, the asynchronous calls')
  int host_direct = -1;        // the GPU reads pageable host memory (the host calls' gather), -1: not asked yet
  PinBuf hA, hA2, hB, hB2, hw, hu, hhi, hhj;
  ~Ctx();
};

// Device error word the kernels of the current call write.
inline int *err_word(Ctx *c) { return c->cur_err ? c->cur_err : (int *)c->err.p; }

// A synchronous call's own device error word: cleared on entry (stream
// ordered), made current for the call's kernels, read by finish() after the
// call's work is enqueued.  The asynchronous calls' flags in Ctx::err stay
// as they were.
struct SyncErrScope {
  Ctx *c;
  bool ok = false;
  explicit SyncErrScope(Ctx *ctx);
  ~SyncErrScope() { c->cur_err = nullptr; }
  // Waits for the stream; GSKS_ERR_TIMEOUT if a bounded wait gave up,
  // GSKS_ERR_MAP_RANGE for a map index out of range, else GSKS_OK.
  int finish();
};

// Packed, identity-mapped device copy of a host-pointer call.
struct Staged {
  const double *A = nullptr, *A2 = nullptr, *B = nullptr, *B2 = nullptr;
  const double *hi = nullptr, *hj = nullptr, *w = nullptr;
  double *u = nullptr;
};

Ctx *get_ctx();
int set_status(int s, const char *where);
int cuda_status(cudaError_t e, const char *where);
void note_launches(int n);
int effective_precision();
int check_kernel(ks_t *ker, int k);
bool is_device_pointer(const void *p);
KParams make_kparams(const ks_t *ker, const double *hi, const double *hj);
double coincidence_eps(int k);
int read_device_errors(Ctx *c);

int stage_host(Ctx *c, const ks_t *ker, int m, int n, int k,
               const double *u, const int *umap,
               const double *XA, const double *XA2, const int *amap,
               const double *XB, const double *XB2, const int *bmap,
               const double *w, const int *wmap, Staged &v, int nrhs = 1);
int unstage_host(Ctx *c, int m, double *u, const int *umap, int nrhs = 1);

int enqueue_fused(Ctx *c, const ks_t *ker, int m, int n, int k,
                  double *u, const int *umap,
                  const double *XA, const double *XA2, const int *amap, int nxa,
                  const double *XB, const double *XB2, const int *bmap, int nxb,
                  const double *w, const int *wmap, const double *hi, const double *hj,
                  int precision, cudaStream_t s, bool stream_ordered_alloc, int nrhs = 1);

// Split-precision form (gsks_split.cu).  nrhs <= 4 interleaved columns of u
// and w in one sweep; GSKS_ERR_TOO_LARGE when k or the shared memory of that
// sweep does not fit (the caller then sweeps once per column).
int enqueue_split(Ctx *c, const ks_t *ker, int m, int n, int k,
                  double *u, const int *umap,
                  const double *XA, const double *XA2, const int *amap, int nxa,
                  const double *XB, const double *XB2, const int *bmap, int nxb,
                  const double *w, const int *wmap, const double *hi, const double *hj,
                  cudaStream_t s, bool stream_ordered_alloc, int nrhs = 1);

// Split-precision form of dgsks_list (gsks_split.cu), planned once for a set
// of lists: row sums of every (task t, target position r, source chunk sc)
// into partial[pbase[t] + sc * m_t + r], chunk sources per chunk (a multiple
// of 128).  kps: ntask device-side descriptors; hoff_a / hoff_b: host
// offsets.  split_list_run takes device pointers and only launches kernels.
struct SplitListPlan {
  int ntask = 0, k = 0, kpad = 0, ma = 0, mb = 0, nxa = 0, nxb = 0;
  int n_ta = 0, n_tb = 0, n_items = 0;
  bool same_pool = false;
  DevBuf ws;
  size_t o_params = 0, o_centre = 0, o_bbox = 0, o_ta = 0, o_tat = 0, o_tb = 0, o_tbt = 0, o_tbc = 0;
  size_t o_items = 0, o_kps = 0, o_tp = 0, o_a = 0, o_b = 0, o_xaf = 0, o_xbf = 0;
  // deferred row rescue: task geometry, a-list offsets, skipped-group weights
  // (the partial layout), rescue list and its count
  size_t o_tg = 0, o_aoff = 0, o_pskip = 0, o_rl = 0, o_rc = 0;
  size_t o_ni = 0;   // work counter of the tile kernel
  // polynomial tasks summed around row anchors: per-task source means and
  // weight sums, the rows' v0^p
  bool any_anch = false;
  size_t o_ybar = 0, o_wsum = 0, o_rowc = 0;
  size_t o_tbox = 0, o_tcen = 0;   // per-task boxes and centres (each task's own frame)
};
int split_list_plan(SplitListPlan &P, const KParams *kps, int ntask, int k, const int *hoff_a, const int *hoff_b,
                    const long long *pbase, int chunk, int nxa, int nxb, bool same_pool, cudaStream_t s);
int split_list_run(const SplitListPlan &P, Ctx *c, const double *XA, const int *a_idx, const double *XB,
                   const int *b_idx, const double *w, const int *w_idx, double *partial, int *err, cudaStream_t s,
                   int *launches);

// Owner lists of the batched merge (gsks_sort.cu): u_idx holds na device
// indices in [0, nu) (others raise DEVERR_MAP_RANGE in *err).  Writes own_pos
// (na: the positions grouped by u entry, ascending within an entry), ent_u
// (the distinct entries, ascending), own_off (entry e owns own_pos[own_off[e]
// .. own_off[e+1])) and *nent, all on the device; work holds
// owner_work_bytes(na) bytes.
size_t owner_work_bytes(int na);
int owner_lists(const int *u_idx, int na, int nu, void *work, int *own_pos, int *ent_u, int *own_off, int *nent,
                int *err, cudaStream_t s, int *launches);

}  // namespace gsks
