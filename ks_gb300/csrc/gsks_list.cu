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
// by the tensor-core kernel of gsks_split.cu (enqueue_split_list) and merged
// by the same merge kernel.
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

// Device-side state of the list path, per host thread.
struct ListBufs {
  DevBuf items, tasks, kps, counter, partial, ent_u, own_off, own_pos, sort_work;
  DevBuf a_off, a_idx, b_idx, w_idx, u_idx;
  DevBuf XA, XB, XA2, XB2, w, u;
  std::vector<DevBuf> bandwidths;
  ~ListBufs()
  {
    for (DevBuf *b : {&items, &tasks, &kps, &counter, &partial, &ent_u, &own_off, &own_pos, &sort_work, &a_off,
                      &a_idx, &b_idx, &w_idx, &u_idx, &XA, &XB, &XA2, &XB2, &w, &u})
      b->release();
    for (auto &b : bandwidths) b.release();
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
  note_launches(0);
  if (ntask < 0 || k < 0 || nu < 0 || nxa < 0 || nxb < 0 || nw < 0)
    return set_status(GSKS_ERR_ARG, "dgsks_list");
  if (ntask == 0 || k == 0) return set_status(GSKS_OK, nullptr);  // early return
  if (!a_off || !b_off || !a_idx || !b_idx || !u || !XA || !XB || !w || (!kernel && !kernels))
    return set_status(GSKS_ERR_ARG, "dgsks_list");
  if (!u_idx) u_idx = a_idx;
  if (!w_idx) w_idx = b_idx;

  Ctx *c = get_ctx();
  if (!c) return gsks_last_error();
  cudaStream_t s = c->stream;
  if (!tl_list) tl_list = new ListBufs;
  ListBufs &L = *tl_list;
  const bool dev = is_device_pointer(XA);
  const int prec = effective_precision();
  if (prec != GSKS_FP64 && prec != GSKS_SPLIT_BF16X3) return set_status(GSKS_ERR_PRECISION, "dgsks_list");
  const bool split = prec == GSKS_SPLIT_BF16X3;

  // ---- offsets and lists on the host ------------------------------------
  std::vector<int> hoff_a(ntask + 1), hoff_b(ntask + 1);
  if (dev) {
    if (cudaMemcpy(hoff_a.data(), a_off, (ntask + 1) * sizeof(int), cudaMemcpyDeviceToHost) ||
        cudaMemcpy(hoff_b.data(), b_off, (ntask + 1) * sizeof(int), cudaMemcpyDeviceToHost))
      return cuda_status(cudaGetLastError(), "dgsks_list offsets");
  } else {
    memcpy(hoff_a.data(), a_off, (ntask + 1) * sizeof(int));
    memcpy(hoff_b.data(), b_off, (ntask + 1) * sizeof(int));
  }
  if (hoff_a[0] != 0 || hoff_b[0] != 0) return set_status(GSKS_ERR_LIST, "dgsks_list");
  for (int t = 0; t < ntask; t++)
    if (hoff_a[t + 1] < hoff_a[t] || hoff_b[t + 1] < hoff_b[t])
      return set_status(GSKS_ERR_LIST, "dgsks_list");
  const int na = hoff_a[ntask], nb = hoff_b[ntask];

  // ---- kernel descriptors -------------------------------------------------
  for (auto &b : L.bandwidths) b.release();
  L.bandwidths.clear();
  L.bandwidths.reserve(4 * (size_t)(kernels ? ntask : 1));
  const int nk = kernels ? ntask : 1;
  std::vector<KParams> kps(nk);
  std::map<const double *, const double *> bw_dev;  // host bandwidth array -> device copy
  bool any_norms = false;
  for (int t = 0; t < nk; t++) {
    ks_t *kt = kernels ? &kernels[t] : kernel;
    int st = check_kernel(kt, k);
    if (st) return set_status(st, "dgsks_list");
    any_norms |= kt_uses_norms(kt->type);
    const double *hi = kt->hi, *hj = kt->hj;
    if (kt->type == KS_GAUSSIAN_VAR_BANDWIDTH && !dev) {
      for (const double **hp : {&hi, &hj}) {
        const int len = (hp == &hi) ? nxa : nxb;
        auto f = bw_dev.find(*hp);
        if (f == bw_dev.end()) {
          L.bandwidths.emplace_back();
          if (!upload(L.bandwidths.back(), *hp, (size_t)len, s))
            return set_status(GSKS_ERR_ALLOC, "dgsks_list bandwidth");
          f = bw_dev.emplace(*hp, (const double *)L.bandwidths.back().p).first;
        }
        *hp = f->second;
      }
    }
    kps[t] = make_kparams(kt, hi, hj);
    kps[t].coinc = coincidence_eps(k);
  }

  // ---- work items, largest first ----------------------------------------
  std::vector<ListTask> tasks(ntask);
  std::vector<ListItem> items;
  long long pbase = 0;
  for (int t = 0; t < ntask; t++) {
    const int m = hoff_a[t + 1] - hoff_a[t], n = hoff_b[t + 1] - hoff_b[t];
    const int nsc = (m > 0 && n > 0) ? (n + LIST_CHUNK - 1) / LIST_CHUNK : 0;
    tasks[t] = ListTask{pbase, m, nsc};
    if (split) { pbase += (long long)nsc * m; continue; }   // the split form plans its own items
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
  std::stable_sort(items.begin(), items.end(), [](const ListItem &x, const ListItem &y) {
    return (long long)x.rows * x.cols > (long long)y.rows * y.cols;
  });

  // ---- device data --------------------------------------------------------
  const double *dXA = XA, *dXB = XB, *dXA2 = nullptr, *dXB2 = nullptr, *dw = w;
  double *du = u;
  const int *da_idx = a_idx, *db_idx = b_idx, *dw_idx = w_idx, *du_idx = u_idx;
  bool ok = true;
  if (!dev) {
    ok = upload(L.XA, XA, (size_t)nxa * k, s) && upload(L.w, w, (size_t)nw, s) &&
         upload(L.u, u, (size_t)nu, s) && upload(L.a_idx, a_idx, (size_t)na, s) &&
         upload(L.b_idx, b_idx, (size_t)nb, s) && upload(L.w_idx, w_idx, (size_t)nb, s) &&
         (u_idx == a_idx || upload(L.u_idx, u_idx, (size_t)na, s));
    dXA = (const double *)L.XA.p;
    if (ok && XB != XA) { ok = upload(L.XB, XB, (size_t)nxb * k, s); dXB = (const double *)L.XB.p; }
    else dXB = dXA;
    dw = (const double *)L.w.p; du = (double *)L.u.p;
    du_idx = u_idx == a_idx ? (const int *)L.a_idx.p : (const int *)L.u_idx.p;
    da_idx = (const int *)L.a_idx.p; db_idx = (const int *)L.b_idx.p; dw_idx = (const int *)L.w_idx.p;
  }
  if (!ok) return set_status(GSKS_ERR_ALLOC, "dgsks_list upload");
  int launches = 0;
  // ---- index ranges, checked on the device before any kernel reads through them
  {
    int *err = (int *)c->err.p;
    auto chk = [&](const int *idx, int n, int lim) {
      if (n > 0) {
        check_range<<<std::min((n + 255) / 256, 4096), 256, 0, s>>>(n, idx, lim, err);
        launches++;
      }
    };
    chk(da_idx, na, nxa); chk(db_idx, nb, nxb); chk(dw_idx, nb, nw); chk(du_idx, na, nu);
    if (read_device_errors(c) & DEVERR_MAP_RANGE) return set_status(GSKS_ERR_MAP_RANGE, "dgsks_list");
  }
  if (any_norms && !split) {   // the split form forms its own norms
    // caller-supplied norms are used as given; missing ones are computed on
    // the device (the list wrappers of frame/omp_dgsks_list.cpp:74-92)
    if (XA2) {
      if (dev) dXA2 = XA2;
      else if (upload(L.XA2, XA2, (size_t)nxa, s)) dXA2 = (const double *)L.XA2.p;
      else return set_status(GSKS_ERR_ALLOC, "dgsks_list norms");
    } else {
      if (!L.XA2.ensure((size_t)nxa * 8)) return set_status(GSKS_ERR_ALLOC, "dgsks_list norms");
      norms_launch(nxa, k, dXA, (double *)L.XA2.p, s); launches++;
      dXA2 = (const double *)L.XA2.p;
    }
    if (XB == XA && XB2 == XA2) {
      dXB2 = dXA2;
    } else if (XB2) {
      if (dev) dXB2 = XB2;
      else if (upload(L.XB2, XB2, (size_t)nxb, s)) dXB2 = (const double *)L.XB2.p;
      else return set_status(GSKS_ERR_ALLOC, "dgsks_list norms");
    } else {
      if (!L.XB2.ensure((size_t)nxb * 8)) return set_status(GSKS_ERR_ALLOC, "dgsks_list norms");
      norms_launch(nxb, k, dXB, (double *)L.XB2.p, s); launches++;
      dXB2 = (const double *)L.XB2.p;
    }
  }
  ok = (split || upload(L.items, items.data(), items.size(), s)) && upload(L.tasks, tasks.data(), tasks.size(), s) &&
       upload(L.kps, kps.data(), kps.size(), s) &&
       L.partial.ensure(std::max<long long>(pbase, 1) * sizeof(double)) && L.counter.ensure(2 * sizeof(int)) &&
       L.own_pos.ensure(std::max(na, 1) * sizeof(int)) && L.ent_u.ensure(std::max(na, 1) * sizeof(int)) &&
       L.own_off.ensure((std::max(na, 1) + 1) * sizeof(int)) && L.sort_work.ensure(owner_work_bytes(na));
  if (!ok) return set_status(GSKS_ERR_ALLOC, "dgsks_list plan");
  // owners of each u entry, ascending positions (device radix sort)
  int *d_nent = (int *)L.counter.p + 1;
  if (na > 0) {
    const int st = owner_lists(du_idx, na, nu, L.sort_work.p, (int *)L.own_pos.p, (int *)L.ent_u.p,
                               (int *)L.own_off.p, d_nent, (int *)c->err.p, s, &launches);
    if (st) return set_status(st, "dgsks_list owners");
  }
  if (!upload(L.a_off, hoff_a.data(), (size_t)ntask + 1, s)) return set_status(GSKS_ERR_ALLOC, "dgsks_list");
  const int *da_off = (const int *)L.a_off.p;

  FusedArgs a{};
  a.k = k; a.XA = dXA; a.XA2 = dXA2; a.amap = da_idx; a.XB = dXB; a.XB2 = dXB2; a.bmap = db_idx;
  a.w = dw; a.wmap = dw_idx; a.nxa = nxa; a.nxb = nxb; a.err = (int *)c->err.p;
  if (split) {
    std::vector<KParams> kpt(ntask);
    std::vector<long long> pb(ntask);
    for (int t = 0; t < ntask; t++) { kpt[t] = kps[kernels ? t : 0]; pb[t] = tasks[t].pbase; }
    const int st = enqueue_split_list(c, kpt.data(), ntask, k, hoff_a.data(), hoff_b.data(), pb.data(), LIST_CHUNK,
                                      dXA, da_idx, nxa, dXB, db_idx, nxb, dw, dw_idx, (double *)L.partial.p, s,
                                      &launches);
    if (st) return set_status(st, "dgsks_list split");
  } else if (!items.empty()) {
    cudaMemsetAsync(L.counter.p, 0, sizeof(int), s);
    const int grid = std::max(1, std::min<int>((int)items.size(), c->num_sms * 2));
    list_fp64_kernel<<<grid, fp64cfg::NT, 0, s>>>(a, (const KParams *)L.kps.p, kernels ? 1 : 0,
                                                  (const ListItem *)L.items.p, (int)items.size(),
                                                  (int *)L.counter.p, (double *)L.partial.p);
    launches++;
  }
  if (na > 0) {
    list_merge<<<(na + 127) / 128, 128, 0, s>>>(d_nent, (const int *)L.ent_u.p, (const int *)L.own_off.p,
                                                (const int *)L.own_pos.p, ntask, da_off,
                                                (const ListTask *)L.tasks.p, (const double *)L.partial.p, du);
    launches++;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e, "dgsks_list launch");
  if (!dev) {
    e = cudaMemcpyAsync(u, du, (size_t)nu * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return cuda_status(e, "dgsks_list copy back");
  }
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e, "dgsks_list");
  if (read_device_errors(c) & DEVERR_MAP_RANGE) return set_status(GSKS_ERR_MAP_RANGE, "dgsks_list");
  note_launches(launches);
  return set_status(GSKS_OK, nullptr);
}
