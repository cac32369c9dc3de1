/*
 * gsks.h -- GB300 extensions of the GSKS C ABI (libgsks.so).
 *
 * ks.h keeps the reference's interface unchanged.  This header adds what the
 * reference has no counterpart for, or reports through printf/exit:
 *   - status codes and gsks_last_error() (the reference prints and exits,
 *     frame/dgsks.c:465-467, frame/omp_dgsks_list.cpp:321-324,
 *     frame/ks_util.c:50-51);
 *   - a precision switch: plain FP64 or split-precision tensor-core form;
 *   - device-resident entry points taking device pointers and a CUDA stream;
 *   - dgsks_list, a flat C-ABI batched call over CSR task lists (the
 *     reference only has the C++ std::vector interface of
 *     include/omp_dgsks_list.hpp:48-115, which forwards here).
 *
 * All entry points are plain C: pointers, sizes and a stream handle passed as
 * void*.  They are thread-safe; every calling host thread gets its own CUDA
 * stream, staging buffers and workspace on the current device.
 */
#ifndef GSKS_GB300_GSKS_H
#define GSKS_GB300_GSKS_H

#include <stddef.h>
#include "ks.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status ------------------------------------------------------------ */
enum {
  GSKS_OK = 0,
  GSKS_ERR_ARG = 1,          /* negative size, NULL array that is needed      */
  GSKS_ERR_KERNEL_TYPE = 2,  /* ks_t.type outside ks_type                     */
  GSKS_ERR_BANDWIDTH = 3,    /* var-bandwidth Gaussian without hi/hj          */
  GSKS_ERR_LAPLACE_K = 4,    /* Laplace needs k > 2                           */
  GSKS_ERR_MAP_RANGE = 5,    /* a map index is negative or beyond the pool    */
  GSKS_ERR_CUDA = 6,         /* a CUDA runtime call failed                    */
  GSKS_ERR_ALLOC = 7,        /* host or device allocation failed              */
  GSKS_ERR_LIST = 8,         /* inconsistent task lists                       */
  GSKS_ERR_PRECISION = 9,    /* unknown precision, or form not built          */
  GSKS_ERR_NO_DEVICE = 10,   /* no CUDA device visible                        */
  GSKS_ERR_TOO_LARGE = 11,   /* a size beyond what the entry point supports   */
  GSKS_ERR_TIMEOUT = 12      /* a kernel's bounded wait gave up: u incomplete */
};

/* Status of the calling thread's most recent GSKS call. */
int gsks_last_error(void);
/* Static description of a status code. */
const char *gsks_error_string(int code);

/* ---- precision --------------------------------------------------------- */
enum {
  GSKS_FP64 = 0,        /* FP64 rank-k, FP64 kernel function and sums        */
  GSKS_SPLIT_BF16X3 = 1 /* split-precision tensor-core form.  (The name is
                           kept for compatibility: each coordinate is split
                           into three 16-bit slices, an integer head exact in
                           FP16 and two FP16 remainders, multiplied with
                           tcgen05 kind::f16 and FP32 accumulation.)  FP32
                           kernel function; FP64 norms, near-pair distances
                           and accumulation of u; <= 1e-6 relative error.   */
};

/* Precision used by dgsks()/dgsks_list() on the calling thread.  The
 * initial value comes from GSKS_PRECISION ("fp64" or "split"). */
int gsks_set_precision(int precision);
int gsks_get_precision(void);

/* dgsks() with a status return (same arguments as ks.h dgsks). */
int dgsks_status(ks_t *kernel, int m, int n, int k,
                 double *u, int *umap,
                 double *XA, double *XA2, int *amap,
                 double *XB, double *XB2, int *bmap,
                 double *w, int *wmap);

/* ---- device-resident entry points ------------------------------------- */
/* All arrays are device pointers on the current device; `stream` is a
 * cudaStream_t (NULL = the legacy default stream).  kernel->hi / hj must be
 * device pointers too.  The call is asynchronous with respect to the host:
 * it enqueues its kernels on `stream` and returns.  umap must not repeat an
 * index within one call (each target row owns its u entry).  XA2/XB2 may be
 * NULL for the inner-product kernels (polynomial, tanh).  Workspace is held
 * by the calling thread's context and reused across calls.
 * nxa / nxb: pool sizes used to range-check the maps on the device (pass -1
 * to skip the check). */
int gsks_dgsks_device(ks_t *kernel, int m, int n, int k,
                      double *u, const int *umap,
                      const double *XA, const double *XA2, const int *amap, int nxa,
                      const double *XB, const double *XB2, const int *bmap, int nxb,
                      const double *w, const int *wmap,
                      int precision, void *stream);

/* Several right-hand sides.  u and w hold nrhs interleaved columns, the layout
 * the reference's weighted sums use when built with KS_RHS = nrhs
 * (include/ks.h:46):
 *     u[umap[i]*nrhs + r] += sum_j K(XA[amap[i]], XB[bmap[j]]) w[wmap[j]*nrhs + r].
 * The FP64 form takes up to four right-hand sides in one pass, each kernel
 * value multiplied by every weight column.  Otherwise (the split form, or
 * nrhs > 4) right-hand side r is one evaluation with the maps umap*nrhs + r
 * and wmap*nrhs + r, and the kernel values are evaluated again for every r.
 * The host-pointer form stages the points once for all r.  dgsks_rhs: host or
 * device arrays, synchronous, as dgsks_status; gsks_dgsks_device_rhs: device
 * arrays on `stream`, as gsks_dgsks_device. */
int dgsks_rhs(ks_t *kernel, int m, int n, int k, int nrhs,
              double *u, int *umap,
              double *XA, double *XA2, int *amap,
              double *XB, double *XB2, int *bmap,
              double *w, int *wmap);
int gsks_dgsks_device_rhs(ks_t *kernel, int m, int n, int k, int nrhs,
                          double *u, const int *umap,
                          const double *XA, const double *XA2, const int *amap, int nxa,
                          const double *XB, const double *XB2, const int *bmap, int nxb,
                          const double *w, const int *wmap,
                          int precision, void *stream);

/* Single precision: dgsks on FP32 arrays (host or device, synchronous).  The
 * reference declares no such entry; its single-precision micro-kernels are
 * stubs.  The rows the maps name are converted to FP64 as they are gathered,
 * and XA2/XB2 are recomputed in FP64 from them (the arguments are accepted and
 * ignored).  The evaluation is dgsks's, in the precision of
 * gsks_set_precision(), and u[umap[i]] is written back rounded to FP32.  The
 * bandwidth vectors of the variable-bandwidth kernel stay FP64 (ks_t).
 * sgsks_status returns the status; sgsks is void like dgsks. */
int sgsks_status(ks_t *kernel, int m, int n, int k,
                 float *u, int *umap,
                 float *XA, float *XA2, int *amap,
                 float *XB, float *XB2, int *bmap,
                 float *w, int *wmap);
void sgsks(ks_t *kernel, int m, int n, int k,
           float *u, int *umap,
           float *XA, float *XA2, int *amap,
           float *XB, float *XB2, int *bmap,
           float *w, int *wmap);

/* gsks_dgsks_device() for callers that cannot let a library allocate device
 * memory -- e.g. a process whose device memory is reserved up front by its
 * own pool allocator, or a loop that may not allocate after start-up.  No
 * counterpart in the reference (its dgsks allocates host pack buffers on
 * every call).  FP64 form only, arguments as gsks_dgsks_device without the
 * precision and pool sizes (maps are not range-checked).  Its scratch is a
 * fixed 8 MiB array inside the library, so m may be at most 1048576
 * (GSKS_ERR_TOO_LARGE otherwise).  The first call on a device looks up that
 * array's device address; make it before any stream capture.  All calls on a
 * device share the array: calls that overlap on the GPU race, so serialise
 * them.  Allocates nothing: no cudaMalloc, cudaFree or allocating library
 * call, and no stream or context of its own; enqueues on `stream`. */
int gsks_dgsks_device_noalloc(ks_t *kernel, int m, int n, int k,
                              double *u, const int *umap,
                              const double *XA, const double *XA2, const int *amap,
                              const double *XB, const double *XB2, const int *bmap,
                              const double *w, const int *wmap, void *stream);

/* Squared norms X2[p] = sum_q X[p*k+q]^2 of N device-resident points. */
int gsks_norms_device(int N, int k, const double *X, double *X2, void *stream);

/* Number of kernels the last device call of this thread enqueued. */
int gsks_last_launch_count(void);

/* Waits for the device, then returns and clears the device-side error flags
 * of the calling thread's asynchronous calls (gsks_dgsks_device,
 * gsks_dgsks_device_rhs).  Bit 0: a map index outside [0, nxa/nxb) was
 * clamped and read as point 0.  Bit 1: a bounded wait inside the
 * split-precision kernel gave up (the kernel returned early and u is
 * incomplete).  The flags accumulate over calls until read.  The synchronous
 * calls (dgsks, dgsks_status, dgsks_rhs, sgsks) keep their own flags and
 * return GSKS_ERR_TIMEOUT instead.  Returns -1 if the flags could not be
 * read. */
int gsks_device_errors(void);

/* ---- calibration -------------------------------------------------------- */
/* Measured issue rate of one pipe of the current device, in operations per
 * second (an FMA counts as one operation): what = 0 FP64 FMA, 1 FP32 FMA,
 * 2 SFU ex2, 3 FP64 tensor-core FMA (DMMA, mma.sync m8n8k4).  Used for the
 * roofline fractions the benchmark reports; the reference has no
 * counterpart. */
int gsks_probe_peak(int what, double *ops_per_s);

/* ---- diagnostics -------------------------------------------------------- */
/* Counts of the calling thread's last single split-precision evaluation
 * (dgsks / gsks_dgsks_device with GSKS_SPLIT_BF16X3; not dgsks_list): the
 * pairs whose kernel value an error bound sent to a recheck from the pool
 * coordinates, and the target rows redone in full because all their values
 * lay below the FP32 range.  Waits for the device.  No counterpart in the
 * reference. */
int gsks_split_stats(long long *rechecked_pairs, int *rescued_rows);

/* Host-pointer calls (dgsks, dgsks_status, dgsks_ref, dgsks_rhs) gather the
 * rows their maps name before the kernels run.  Where the device reads
 * pageable host memory coherently (cudaDevAttrPageableMemoryAccess, as on
 * Grace-Blackwell), a kernel gathers them straight from the caller's arrays;
 * elsewhere, or with the environment variable GSKS_HOST_GATHER=cpu, the host
 * gathers them into pinned buffers and copies those.  Returns 1 for the
 * first, 0 for the second, on the calling thread's current device (negative:
 * no CUDA context). */
int gsks_host_gather_on_device(void);

/* Test hook of the split-precision form (no counterpart in the reference).
 * Sets, for the calling thread's later split-precision calls (dgsks,
 * dgsks_status, gsks_dgsks_device, dgsks_list, ...), the limit of the
 * kernel's bounded waits in clock cycles (wait_cycles <= 0: the library's
 * limit, about 2 s) and, with stall != 0, makes the bulk-copy role of every
 * CTA issue nothing.  The tensor-core and epilogue roles then wait for data
 * that never comes: each CTA's waits run out, it records the timeout, frees
 * its tensor memory and returns.  Synchronous calls return GSKS_ERR_TIMEOUT
 * (host u untouched); asynchronous ones set bit 1 of gsks_device_errors()
 * and leave u incomplete.  This exercises the failure path of the bounded
 * waits without faulting or hanging the GPU.  gsks_split_test_wait(0, 0)
 * restores normal operation. */
int gsks_split_test_wait(long long wait_cycles, int stall);

/* ---- batched evaluation ------------------------------------------------ */
/* dgsks_list: ntask independent kernel summations accumulated into one u.
 * Task t evaluates, for a in [a_off[t], a_off[t+1]) and b in [b_off[t], b_off[t+1]),
 *     u[u_idx[a]] += K(XA[a_idx[a]], XB[b_idx[b]]) * w[w_idx[b]]
 * Contributions of different tasks to the same u entry are summed in a fixed
 * order (deterministic).  kernels: NULL to use `kernel` for every task, or an
 * array of ntask descriptors (per-task kernel type and parameters).  u_idx
 * may be NULL (= a_idx) and w_idx may be NULL (= b_idx).  XA2/XB2 may be NULL,
 * in which case the norms are computed on the device.  Host or device arrays
 * (all of one kind).  nu/nxa/nxb/nw: sizes of u, the two pools and w. */
int dgsks_list(ks_t *kernel, ks_t *kernels, int ntask, int k,
               double *u, int nu,
               const int *a_off, const int *a_idx, const int *u_idx,
               const int *b_off, const int *b_idx, const int *w_idx,
               double *XA, double *XA2, int nxa,
               double *XB, double *XB2, int nxb,
               double *w, int nw);

/* ---- planned batched evaluation ----------------------------------------- */
/* A plan fixes the task lists, kernel descriptors, sizes and precision of a
 * dgsks_list and keeps their work tables (tile / item queues, the owner lists
 * of u, workspace) on the device.  gsks_list_plan_execute then evaluates it
 * for device-resident coordinates, norms (NULL: computed on the device),
 * weights and u, asynchronously on `stream` (a cudaStream_t).  The first
 * execute captures the evaluation into a CUDA graph; later executes with the
 * same pointers and stream replay the graph.  Lists given as device arrays and
 * device bandwidth arrays must stay valid while the plan exists (host arrays
 * are copied at creation).  same_pool != 0: executes pass XB == XA.  The
 * reference has no counterpart (its list driver plans on every call,
 * frame/omp_dgsks_list.cpp:297-359). */
typedef struct gsks_list_plan gsks_list_plan;
int gsks_list_plan_create(gsks_list_plan **plan, ks_t *kernel, ks_t *kernels, int ntask, int k, int nu,
                          const int *a_off, const int *a_idx, const int *u_idx,
                          const int *b_off, const int *b_idx, const int *w_idx,
                          int nxa, int nxb, int nw, int precision, int same_pool);
int gsks_list_plan_execute(gsks_list_plan *plan, double *u, const double *XA, const double *XA2,
                           const double *XB, const double *XB2, const double *w, void *stream);
/* Waits for the device, then returns and clears the plan's device-side error
 * flags (as gsks_device_errors); -1 if they could not be read. */
int gsks_list_plan_errors(gsks_list_plan *plan);
int gsks_list_plan_destroy(gsks_list_plan *plan);

#ifdef __cplusplus
}
#endif

#endif /* GSKS_GB300_GSKS_H */
