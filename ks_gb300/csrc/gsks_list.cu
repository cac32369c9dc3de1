// gsks_list.cu -- dgsks_list: many kernel summations in one persistent launch.
//
// The reference batches with OpenMP: a greedy cost-balanced assignment of
// tasks to 68 worker queues, one dgsks call per task into a per-thread copy of
// u, and a serial merge (frame/omp_dgsks_list.cpp:297-420).  Here the whole
// list becomes one queue of work items (task, target tile, source chunk)
// sorted by cost, largest first, which a persistent kernel drains through an
// atomic counter (no waits).  Every item writes per-row partial sums; a merge
// kernel then adds, for each distinct u entry, the contributions of all list
// positions that name it in ascending position order -- the same order on
// every run, so the result is deterministic without floating-point atomics.
// With the split-precision form selected, the same partial layout is filled
// by the tensor-core kernel of gsks_split.cu (split_list_run) and merged by
// the same merge kernel.  A plan (gsks_list_plan_*) keeps the lists' tables
// on the device and replays its evaluation as a CUDA graph.
#include "gsks.h"
#include "gsks_internal.cuh"
#include "gsks_host.h"
#include "gsks_fp64_item.cuh"

#include <algorithm>
#include <cstring>
#include <map>
#include <numeric>
#include <vector>

namespace gsks {

struct ListItem {
  int task;
  int a0, rows;    // positions a0 .. a0+rows-1 of the target list
  int b0, cols;    // positions b0 .. b0+cols-1 of the source list
  int pad;
  long long out;   // partial offset of row 0
};

struct ListTask {
  long long pbase;  // partial offset of chunk 0, row 0
  int m, nsc;       // rows, source chunks (partial row stride is m)
};

namespace {

constexpr int LIST_CHUNK = 1024;  // sources per item

__global__ void __launch_bounds__(fp64cfg::NT, 2)
list_fp64_kernel(FusedArgs a, const KParams *__restrict__ kps, int per_task,
                 const ListItem *__restrict__ items, int nitems, int *counter,
                 double *__restrict__ partial)
{
  __shared__ Fp64Smem sm;
  __shared__ int s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= nitems) break;
    const ListItem d = items[it];
    const KParams kp = kps[per_task ? d.task : 0];
    double *out = partial + d.out;
    switch (kp.type) {
      case KS_GAUSSIAN: fp64_item<KS_GAUSSIAN>(a, kp, sm, d.a0, d.rows, d.b0, d.cols, out); break;
      case KS_POLYNOMIAL: fp64_item<KS_POLYNOMIAL>(a, kp, sm, d.a0, d.rows, d.b0, d.cols, out); break;
      case KS_LAPLACE: fp64_item<KS_LAPLACE>(a, kp, sm, d.a0, d.rows, d.b0, d.cols, out); break;
      case KS_GAUSSIAN_VAR_BANDWIDTH:
        fp64_item<KS_GAUSSIAN_VAR_BANDWIDTH>(a, kp, sm, d.a0, d.rows, d.b0, d.cols, out); break;
      case KS_TANH: fp64_item<KS_TANH>(a, kp, sm, d.a0, d.rows, d.b0, d.cols, out); break;
      case KS_QUARTIC: fp64_item<KS_QUARTIC>(a, kp, sm, d.a0, d.rows, d.b0, d.cols, out); break;
      case KS_MULTIQUADRATIC:
        fp64_item<KS_MULTIQUADRATIC>(a, kp, sm, d.a0, d.rows, d.b0, d.cols, out); break;
      default: fp64_item<KS_EPANECHNIKOV>(a, kp, sm, d.a0, d.rows, d.b0, d.cols, out); break;
    }
    __syncthreads();  // every thread has read s_item before thread 0 rewrites it
  }
}

// For each distinct u entry e: u[ent_u[e]] += sum over the list positions that
// name it (ascending) of the sum over that position's source chunks.
__global__ void list_merge(const int *__restrict__ nent, const int *__restrict__ ent_u,
                           const int *__restrict__ own_off, const int *__restrict__ own_pos, int ntask,
                           const int *__restrict__ a_off, const ListTask *__restrict__ tasks,
                           const double *__restrict__ partial, double *__restrict__ u)
{
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= *nent) return;
  double s = 0.0;
  for (int q = own_off[e]; q < own_off[e + 1]; q++) {
    const int pos = own_pos[q];
    int lo = 0, hi = ntask - 1;  // task t with a_off[t] <= pos < a_off[t+1]
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (a_off[mid] <= pos) lo = mid; else hi = mid - 1;
    }
    const ListTask t = tasks[lo];
    const int r = pos - a_off[lo];
    double ps = 0.0;
    for (int c = 0; c < t.nsc; c++) ps += partial[t.pbase + (long long)c * t.m + r];
    s += ps;
  }
  u[ent_u[e]] += s;
}

// Flags DEVERR_MAP_RANGE if an index lies outside [0, lim).
__global__ void check_range(int n, const int *__restrict__ idx, int lim, int *err)
{
  bool bad = false;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += blockDim.x * gridDim.x)
    bad |= (idx[i] < 0 || idx[i] >= lim);
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(err, DEVERR_MAP_RANGE);
}

template <typename T>
bool upload(DevBuf &b, const T *src, size_t n, cudaStream_t s)
{
  if (!b.ensure(std::max<size_t>(n, 1) * sizeof(T))) return false;
  return n == 0 || cudaMemcpyAsync(b.p, src, n * sizeof(T), cudaMemcpyHostToDevice, s) == cudaSuccess;
}

// A planned batched evaluation: the task lists' work tables, owner lists and
// workspace on the device.  list_plan_run evaluates it for given coordinates,
// norms, weights and u (device pointers), launches only, so that the same run
// can be captured into a CUDA graph and replayed.
struct ListPlan {
  int ntask = 0, k = 0, nu = 0, nxa = 0, nxb = 0, nw = 0, na = 0, nb = 0;
  bool split = false, any_norms = false, per_task = false, same_pool = false;
  long long pbase = 0;
  int nitems = 0;
  const int *a_idx = nullptr, *b_idx = nullptr, *w_idx = nullptr, *u_idx = nullptr;   // device
  DevBuf items, tasks, kps, counter, partial, ent_u, own_off, own_pos, sort_work, a_off, err;
  DevBuf l_a, l_b, l_w, l_u;            // device copies of host lists
  DevBuf XA2, XB2;                      // norms computed on the device
  std::vector<DevBuf> bandwidths;       // device copies of host bandwidth arrays
  SplitListPlan sp;
  // graph of the last run: replayed while the pointers and the stream stay the same
  cudaGraphExec_t gexec = nullptr;
  const void *gkey[7] = {};
  void release()
  {
    if (gexec) cudaGraphExecDestroy(gexec);
    gexec = nullptr;
    for (DevBuf *b : {&items, &tasks, &kps, &counter, &partial, &ent_u, &own_off, &own_pos, &sort_work, &a_off,
                      &err, &l_a, &l_b, &l_w, &l_u, &XA2, &XB2, &sp.ws})
      b->release();
    for (auto &b : bandwidths) b.release();
    bandwidths.clear();
  }
  ~ListPlan() { release(); }
};

// Builds the plan.  Lists (offsets included) are host or device arrays as
// `dev_lists` says; bandwidth arrays of the descriptors are host arrays when
// `host_bw` (then copied).  Checks the lists' index ranges on the device.
int list_plan_build(ListPlan &L, Ctx *c, ks_t *kernel, ks_t *kernels, int ntask, int k, int nu,
                    const int *a_off, const int *a_idx, const int *u_idx, const int *b_off, const int *b_idx,
                    const int *w_idx, int nxa, int nxb, int nw, bool dev_lists, bool host_bw, int prec,
                    bool same_pool, cudaStream_t s, int *launches)
{
  if (L.gexec) { cudaGraphExecDestroy(L.gexec); L.gexec = nullptr; }
  L.ntask = ntask; L.k = k; L.nu = nu; L.nxa = nxa; L.nxb = nxb; L.nw = nw;
  L.split = prec == GSKS_SPLIT_BF16X3;
  L.per_task = kernels != nullptr;
  L.same_pool = same_pool;
  if (!u_idx) u_idx = a_idx;
  if (!w_idx) w_idx = b_idx;

  // ---- offsets on the host ------------------------------------------------
  std::vector<int> hoff_a(ntask + 1), hoff_b(ntask + 1);
  if (dev_lists) {
    if (cudaMemcpy(hoff_a.data(), a_off, (ntask + 1) * sizeof(int), cudaMemcpyDeviceToHost) ||
        cudaMemcpy(hoff_b.data(), b_off, (ntask + 1) * sizeof(int), cudaMemcpyDeviceToHost))
      return cuda_status(cudaGetLastError(), "dgsks_list offsets");
  } else {
    memcpy(hoff_a.data(), a_off, (ntask + 1) * sizeof(int));
    memcpy(hoff_b.data(), b_off, (ntask + 1) * sizeof(int));
  }
  if (hoff_a[0] != 0 || hoff_b[0] != 0) return GSKS_ERR_LIST;
  for (int t = 0; t < ntask; t++)
    if (hoff_a[t + 1] < hoff_a[t] || hoff_b[t + 1] < hoff_b[t]) return GSKS_ERR_LIST;
  const int na = hoff_a[ntask], nb = hoff_b[ntask];
  L.na = na; L.nb = nb;

  // ---- kernel descriptors -------------------------------------------------
  for (auto &b : L.bandwidths) b.release();
  L.bandwidths.clear();
  L.bandwidths.reserve(4 * (size_t)(kernels ? ntask : 1));
  const int nk = kernels ? ntask : 1;
  std::vector<KParams> kps(nk);
  std::map<const double *, const double *> bw_dev;  // host bandwidth array -> device copy
  L.any_norms = false;
  for (int t = 0; t < nk; t++) {
    ks_t *kt = kernels ? &kernels[t] : kernel;
    int st = check_kernel(kt, k);
    if (st) return st;
    L.any_norms |= kt_uses_norms(kt->type);
    const double *hi = kt->hi, *hj = kt->hj;
    if (kt->type == KS_GAUSSIAN_VAR_BANDWIDTH && host_bw) {
      for (const double **hp : {&hi, &hj}) {
        const int len = (hp == &hi) ? nxa : nxb;
        auto f = bw_dev.find(*hp);
        if (f == bw_dev.end()) {
          L.bandwidths.emplace_back();
          if (!upload(L.bandwidths.back(), *hp, (size_t)len, s)) return GSKS_ERR_ALLOC;
          f = bw_dev.emplace(*hp, (const double *)L.bandwidths.back().p).first;
        }
        *hp = f->second;
      }
    }
    kps[t] = make_kparams(kt, hi, hj);
    kps[t].coinc = coincidence_eps(k);
  }

  // ---- lists on the device -----------------------------------------------
  if (dev_lists) {
    L.a_idx = a_idx; L.b_idx = b_idx; L.w_idx = w_idx; L.u_idx = u_idx;
  } else {
    if (!(upload(L.l_a, a_idx, (size_t)na, s) && upload(L.l_b, b_idx, (size_t)nb, s) &&
          upload(L.l_w, w_idx, (size_t)nb, s) && (u_idx == a_idx || upload(L.l_u, u_idx, (size_t)na, s))))
      return GSKS_ERR_ALLOC;
    L.a_idx = (const int *)L.l_a.p; L.b_idx = (const int *)L.l_b.p; L.w_idx = (const int *)L.l_w.p;
    L.u_idx = u_idx == a_idx ? L.a_idx : (const int *)L.l_u.p;
  }
  if (!L.err.ensure(sizeof(int)) || cudaMemsetAsync(L.err.p, 0, sizeof(int), s) != cudaSuccess)
    return GSKS_ERR_ALLOC;
  {
    int *err = (int *)L.err.p;
    auto chk = [&](const int *idx, int n, int lim) {
      if (n > 0) {
        check_range<<<std::min((n + 255) / 256, 4096), 256, 0, s>>>(n, idx, lim, err);
        (*launches)++;
      }
    };
    chk(L.a_idx, na, nxa); chk(L.b_idx, nb, nxb); chk(L.w_idx, nb, nw); chk(L.u_idx, na, nu);
    int flags = 0;
    if (cudaMemcpyAsync(&flags, err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return cuda_status(cudaGetLastError(), "dgsks_list checks");
    if (flags & DEVERR_MAP_RANGE) return GSKS_ERR_MAP_RANGE;
  }

  // ---- work items, largest first ----------------------------------------
  std::vector<ListTask> tasks(ntask);
  std::vector<ListItem> items;
  long long pbase = 0;
  for (int t = 0; t < ntask; t++) {
    const int m = hoff_a[t + 1] - hoff_a[t], n = hoff_b[t + 1] - hoff_b[t];
    const int nsc = (m > 0 && n > 0) ? (n + LIST_CHUNK - 1) / LIST_CHUNK : 0;
    tasks[t] = ListTask{pbase, m, nsc};
    if (L.split) { pbase += (long long)nsc * m; continue; }   // the split form plans its own items
    for (int sc = 0; sc < nsc; sc++)
      for (int i0 = 0; i0 < m; i0 += fp64cfg::BM) {
        ListItem it{};
        it.task = t; it.a0 = hoff_a[t] + i0; it.rows = std::min(fp64cfg::BM, m - i0);
        it.b0 = hoff_b[t] + sc * LIST_CHUNK; it.cols = std::min(LIST_CHUNK, n - sc * LIST_CHUNK);
        it.out = pbase + (long long)sc * m + i0;
        items.push_back(it);
      }
    pbase += (long long)nsc * m;
  }
  {
    // largest rows x cols first, ties in build order: a counting sort (the
    // products are bounded by the tile height times the source chunk)
    int cmax = 0;
    for (const ListItem &it : items) cmax = std::max(cmax, it.rows * it.cols);
    std::vector<size_t> start((size_t)cmax + 2, 0);
    for (const ListItem &it : items) start[(size_t)(cmax - it.rows * it.cols) + 1]++;
    for (int b = 0; b <= cmax; b++) start[b + 1] += start[b];
    std::vector<ListItem> sorted(items.size());
    for (const ListItem &it : items) sorted[start[cmax - it.rows * it.cols]++] = it;
    items.swap(sorted);
  }
  L.pbase = pbase;
  L.nitems = (int)items.size();
  bool ok = (L.split || upload(L.items, items.data(), items.size(), s)) &&
            upload(L.tasks, tasks.data(), tasks.size(), s) && upload(L.kps, kps.data(), kps.size(), s) &&
            upload(L.a_off, hoff_a.data(), (size_t)ntask + 1, s) &&
            L.partial.ensure(std::max<long long>(pbase, 1) * sizeof(double)) && L.counter.ensure(2 * sizeof(int)) &&
            L.own_pos.ensure(std::max(na, 1) * sizeof(int)) && L.ent_u.ensure(std::max(na, 1) * sizeof(int)) &&
            L.own_off.ensure((std::max(na, 1) + 1) * sizeof(int)) && L.sort_work.ensure(owner_work_bytes(na));
  if (ok && !L.split && L.any_norms)
    ok = L.XA2.ensure((size_t)std::max(nxa, 1) * 8) && L.XB2.ensure((size_t)std::max(nxb, 1) * 8);
  if (!ok) return GSKS_ERR_ALLOC;
  // owners of each u entry, ascending positions (device radix sort)
  if (na > 0) {
    const int st = owner_lists(L.u_idx, na, nu, L.sort_work.p, (int *)L.own_pos.p, (int *)L.ent_u.p,
                               (int *)L.own_off.p, (int *)L.counter.p + 1, (int *)L.err.p, s, launches);
    if (st) return st;
  }
  if (L.split) {
    std::vector<KParams> kpt(ntask);
    std::vector<long long> pb(ntask);
    for (int t = 0; t < ntask; t++) { kpt[t] = kps[kernels ? t : 0]; pb[t] = tasks[t].pbase; }
    const int st = split_list_plan(L.sp, kpt.data(), ntask, k, hoff_a.data(), hoff_b.data(), pb.data(), LIST_CHUNK,
                                   nxa, nxb, same_pool, s);
    if (st) return st;
  }
  // the host vectors above die here: every copy from them must have left
  cudaError_t e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? GSKS_OK : cuda_status(e, "dgsks_list plan");
}

// Enqueues one evaluation of the plan on s (no host synchronisation, no
// allocation).  XA2 / XB2 may be nullptr: the FP64 form then computes them.
int list_plan_run(ListPlan &L, Ctx *c, double *u, const double *XA, const double *XA2, const double *XB,
                  const double *XB2, const double *w, cudaStream_t s, int *launches)
{
  const int ntask = L.ntask, na = L.na;
  int *err = (int *)L.err.p;
  if (L.split) {
    const int st = split_list_run(L.sp, c, XA, L.a_idx, XB, L.b_idx, w, L.w_idx, (double *)L.partial.p, err, s,
                                  launches);
    if (st) return st;
  } else if (L.nitems > 0) {
    const double *dXA2 = nullptr, *dXB2 = nullptr;
    if (L.any_norms) {
      // caller-supplied norms are used as given; missing ones are computed on
      // the device (the list wrappers of frame/omp_dgsks_list.cpp:74-92)
      if (XA2) dXA2 = XA2;
      else { norms_launch(L.nxa, L.k, XA, (double *)L.XA2.p, s); (*launches)++; dXA2 = (const double *)L.XA2.p; }
      if (XB == XA && XB2 == XA2) dXB2 = dXA2;
      else if (XB2) dXB2 = XB2;
      else { norms_launch(L.nxb, L.k, XB, (double *)L.XB2.p, s); (*launches)++; dXB2 = (const double *)L.XB2.p; }
    }
    FusedArgs a{};
    a.k = L.k; a.XA = XA; a.XA2 = dXA2; a.amap = L.a_idx; a.XB = XB; a.XB2 = dXB2; a.bmap = L.b_idx;
    a.w = w; a.wmap = L.w_idx; a.nxa = L.nxa; a.nxb = L.nxb; a.err = err;
    cudaMemsetAsync(L.counter.p, 0, sizeof(int), s);
    const int grid = std::max(1, std::min<int>(L.nitems, c->num_sms * 2));
    list_fp64_kernel<<<grid, fp64cfg::NT, 0, s>>>(a, (const KParams *)L.kps.p, L.per_task ? 1 : 0,
                                                  (const ListItem *)L.items.p, L.nitems, (int *)L.counter.p,
                                                  (double *)L.partial.p);
    *launches += 2;
  }
  if (na > 0) {
    list_merge<<<(na + 127) / 128, 128, 0, s>>>((const int *)L.counter.p + 1, (const int *)L.ent_u.p,
                                                (const int *)L.own_off.p, (const int *)L.own_pos.p, ntask,
                                                (const int *)L.a_off.p, (const ListTask *)L.tasks.p,
                                                (const double *)L.partial.p, u);
    (*launches)++;
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GSKS_OK : cuda_status(e, "dgsks_list launch");
}

// Device-side state of the one-shot list path, per host thread.
struct ListBufs {
  ListPlan plan;
  DevBuf XA, XB, XA2, XB2, w, u;
  ~ListBufs()
  {
    for (DevBuf *b : {&XA, &XB, &XA2, &XB2, &w, &u}) b->release();
  }
};
thread_local ListBufs *tl_list = nullptr;
thread_local struct ListBufsOwner { ~ListBufsOwner() { delete tl_list; } } tl_list_owner;

}  // namespace

}  // namespace gsks

using namespace gsks;

extern "C" int dgsks_list(ks_t *kernel, ks_t *kernels, int ntask, int k,
                          double *u, int nu,
                          const int *a_off, const int *a_idx, const int *u_idx,
                          const int *b_off, const int *b_idx, const int *w_idx,
                          double *XA, double *XA2, int nxa,
                          double *XB, double *XB2, int nxb,
                          double *w, int nw)
{
  NvtxRange nvtx_("dgsks_list");
  note_launches(0);
  if (ntask < 0 || k < 0 || nu < 0 || nxa < 0 || nxb < 0 || nw < 0)
    return set_status(GSKS_ERR_ARG, "dgsks_list");
  if (ntask == 0 || k == 0) return set_status(GSKS_OK, nullptr);  // early return
  if (!a_off || !b_off || !a_idx || !b_idx || !u || !XA || !XB || !w || (!kernel && !kernels))
    return set_status(GSKS_ERR_ARG, "dgsks_list");

  Ctx *c = get_ctx();
  if (!c) return gsks_last_error();
  cudaStream_t s = c->stream;
  if (!tl_list) tl_list = new ListBufs;
  ListBufs &B = *tl_list;
  const bool dev = is_device_pointer(XA);
  const int prec = effective_precision();
  if (prec != GSKS_FP64 && prec != GSKS_SPLIT_BF16X3) return set_status(GSKS_ERR_PRECISION, "dgsks_list");

  int launches = 0;
  int st = list_plan_build(B.plan, c, kernel, kernels, ntask, k, nu, a_off, a_idx, u_idx, b_off, b_idx, w_idx, nxa,
                           nxb, nw, dev, !dev, prec, XA == XB && nxa == nxb, s, &launches);
  if (st) return set_status(st, "dgsks_list");

  // ---- coordinates, norms, weights, u on the device -----------------------
  const double *dXA = XA, *dXB = XB, *dXA2 = XA2, *dXB2 = XB2, *dw = w;
  double *du = u;
  if (!dev) {
    bool ok = upload(B.XA, XA, (size_t)nxa * k, s) && upload(B.w, w, (size_t)nw, s) && upload(B.u, u, (size_t)nu, s);
    dXA = (const double *)B.XA.p;
    if (ok && XB != XA) { ok = upload(B.XB, XB, (size_t)nxb * k, s); dXB = (const double *)B.XB.p; }
    else dXB = dXA;
    if (ok && XA2) { ok = upload(B.XA2, XA2, (size_t)nxa, s); dXA2 = (const double *)B.XA2.p; }
    if (ok && XB2) {
      if (XB2 == XA2 && XB == XA) dXB2 = dXA2;
      else { ok = upload(B.XB2, XB2, (size_t)nxb, s); dXB2 = (const double *)B.XB2.p; }
    }
    dw = (const double *)B.w.p; du = (double *)B.u.p;
    if (!ok) return set_status(GSKS_ERR_ALLOC, "dgsks_list upload");
  }
  st = list_plan_run(B.plan, c, du, dXA, dXA2, dXB, dXB2, dw, s, &launches);
  if (st) return set_status(st, "dgsks_list");
  // the flags first: host arrays keep their u when the evaluation failed
  int flags = 0;
  cudaError_t e = cudaMemcpyAsync(&flags, B.plan.err.p, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e, "dgsks_list");
  if (flags & DEVERR_MAP_RANGE) return set_status(GSKS_ERR_MAP_RANGE, "dgsks_list");
  if (flags & DEVERR_TIMEOUT) return set_status(GSKS_ERR_TIMEOUT, "dgsks_list");
  if (!dev) {
    e = cudaMemcpyAsync(u, du, (size_t)nu * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e, "dgsks_list copy back");
  }
  note_launches(launches);
  return set_status(GSKS_OK, nullptr);
}

// ---- planned evaluation (include/gsks.h) ----------------------------------
struct gsks_list_plan {
  ListPlan plan;
  int device = -1;
};

extern "C" int gsks_list_plan_create(gsks_list_plan **out, ks_t *kernel, ks_t *kernels, int ntask, int k, int nu,
                                     const int *a_off, const int *a_idx, const int *u_idx, const int *b_off,
                                     const int *b_idx, const int *w_idx, int nxa, int nxb, int nw, int precision,
                                     int same_pool)
{
  if (!out) return set_status(GSKS_ERR_ARG, "gsks_list_plan_create");
  *out = nullptr;
  if (ntask < 0 || k <= 0 || nu < 0 || nxa < 0 || nxb < 0 || nw < 0 || !a_off || !b_off || !a_idx || !b_idx ||
      (!kernel && !kernels))
    return set_status(GSKS_ERR_ARG, "gsks_list_plan_create");
  if (precision != GSKS_FP64 && precision != GSKS_SPLIT_BF16X3)
    return set_status(GSKS_ERR_PRECISION, "gsks_list_plan_create");
  Ctx *c = get_ctx();
  if (!c) return gsks_last_error();
  gsks_list_plan *p = new (std::nothrow) gsks_list_plan;
  if (!p) return set_status(GSKS_ERR_ALLOC, "gsks_list_plan_create");
  cudaGetDevice(&p->device);
  int launches = 0;
  bool bw_host = false;
  for (int t = 0; t < (kernels ? ntask : 1); t++) {
    const ks_t *kt = kernels ? &kernels[t] : kernel;
    if (kt->type == KS_GAUSSIAN_VAR_BANDWIDTH && kt->hi && !is_device_pointer(kt->hi)) bw_host = true;
  }
  const int st = list_plan_build(p->plan, c, kernel, kernels, ntask, k, nu, a_off, a_idx, u_idx, b_off, b_idx, w_idx,
                                 nxa, nxb, nw, is_device_pointer(a_idx), bw_host, precision, same_pool != 0, c->stream,
                                 &launches);
  if (st) { delete p; return set_status(st, "gsks_list_plan_create"); }
  *out = p;
  return set_status(GSKS_OK, nullptr);
}

extern "C" int gsks_list_plan_execute(gsks_list_plan *p, double *u, const double *XA, const double *XA2,
                                      const double *XB, const double *XB2, const double *w, void *stream)
{
  NvtxRange nvtx_("gsks_list_plan_execute");
  if (!p || !u || !XA || !XB || !w) return set_status(GSKS_ERR_ARG, "gsks_list_plan_execute");
  Ctx *c = get_ctx();
  if (!c) return gsks_last_error();
  ListPlan &L = p->plan;
  if (L.same_pool && XB != XA) return set_status(GSKS_ERR_ARG, "gsks_list_plan_execute: planned with XB = XA");
  cudaStream_t s = (cudaStream_t)stream;
  const void *key[7] = {u, XA, XA2, XB, XB2, w, stream};
  if (L.gexec && memcmp(key, L.gkey, sizeof(key)) == 0) {
    cudaError_t e = cudaGraphLaunch(L.gexec, s);
    note_launches(1);
    return e == cudaSuccess ? set_status(GSKS_OK, nullptr) : cuda_status(e, "gsks_list_plan_execute");
  }
  if (L.gexec) { cudaGraphExecDestroy(L.gexec); L.gexec = nullptr; }
  // capture the run on a stream of our own, then launch the graph on the caller's
  cudaStream_t cs = c->stream;
  int launches = 0;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_status(e, "gsks_list_plan_execute capture");
  const int st = list_plan_run(L, c, u, XA, XA2, XB, XB2, w, cs, &launches);
  e = cudaStreamEndCapture(cs, &g);
  if (st) { if (g) cudaGraphDestroy(g); return set_status(st, "gsks_list_plan_execute"); }
  if (e != cudaSuccess) return cuda_status(e, "gsks_list_plan_execute capture");
  e = cudaGraphInstantiate(&L.gexec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) { L.gexec = nullptr; return cuda_status(e, "gsks_list_plan_execute instantiate"); }
  memcpy(L.gkey, key, sizeof(key));
  e = cudaGraphLaunch(L.gexec, s);
  note_launches(launches);
  return e == cudaSuccess ? set_status(GSKS_OK, nullptr) : cuda_status(e, "gsks_list_plan_execute");
}

extern "C" int gsks_list_plan_errors(gsks_list_plan *p)
{
  if (!p) return -1;
  int flags = 0;
  if (cudaMemcpy(&flags, p->plan.err.p, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  if (flags) cudaMemset(p->plan.err.p, 0, sizeof(int));
  return flags;
}

extern "C" int gsks_list_plan_destroy(gsks_list_plan *p)
{
  delete p;
  return set_status(GSKS_OK, nullptr);
}
