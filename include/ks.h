/*
 * ks.h -- public C surface of the GB300 GSKS library (libgsks.so).
 *
 * GSKS (general stride kernel summation) evaluates, for i in [0, m),
 *
 *     u[umap[i]] += sum_{j<n} K( XA[amap[i]*k : +k], XB[bmap[j]*k : +k] ) * w[wmap[j]]
 *
 * without ever storing the m x n kernel matrix.  This header keeps the
 * binary interface of the reference header include/ks.h (ChenhanYu/ks) so
 * that existing C callers relink unchanged:
 *   - the ks_type enumerators keep their values (include/ks.h:49-58),
 *   - struct kernel_s / ks_t keeps its field order and types (include/ks.h:60-71),
 *   - dgsks, dgsks_ref and ks_malloc_aligned keep their prototypes
 *     (include/ks.h:73-111).
 *
 * All arrays passed to dgsks()/dgsks_ref() are caller-owned.  They may be
 * ordinary host memory (the library stages them through pinned buffers and
 * runs on the current CUDA device) or CUDA device / managed memory (used in
 * place).  The calls are synchronous: u holds the result on return.
 *
 * Layouts (unchanged from the reference): XA is k-leading (point p occupies
 * XA[p*k .. p*k+k-1]); XA2[p] = sum_q XA[p*k+q]^2; u and w are rhs-leading
 * with KS_RHS == 1; the four maps are int32 indices.
 *
 * The reference reports errors with printf and exit(1).  This library never
 * exits: every entry point records a status that gsks_last_error() (see
 * gsks.h) returns, and prints nothing unless GSKS_VERBOSE is set.
 */
#ifndef GSKS_GB300_KS_H
#define GSKS_GB300_KS_H

#include <stdio.h>
#include <stdlib.h>
#include <math.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Number of right-hand sides carried by u and w (include/ks.h:46). */
#define KS_RHS 1
/* Worker count of the reference's batched scheduler (include/ks.h:47). */
#define KS_NUM_THREAD 68

/* Kernel functions; the values are part of the ABI (include/ks.h:49-58). */
typedef enum {
  KS_GAUSSIAN,                /* exp(scal * d2)                               */
  KS_POLYNOMIAL,              /* (scal * x.y + cons)^powe                     */
  KS_LAPLACE,                 /* scal * d2^powe, powe/scal set from k         */
  KS_GAUSSIAN_VAR_BANDWIDTH,  /* exp(-0.5 * d2 * hi[amap[i]] * hj[bmap[j]])   */
  KS_TANH,                    /* tanh(scal * x.y + cons)                      */
  KS_QUARTIC,                 /* d2 < 1 ? 15/16 (1 - d2)^2 : 0                */
  KS_MULTIQUADRATIC,          /* d2 + cons                                    */
  KS_EPANECHNIKOV             /* d2 < 1 ? 3/4 (1 - d2) : 0                    */
} ks_type;

/* Kernel descriptor (include/ks.h:60-71).  hi/hj are per-point bandwidth
 * factors indexed through amap/bmap (variable-bandwidth Gaussian only); h is
 * carried for layout compatibility and never read.  For KS_LAPLACE the
 * library overwrites powe and scal, exactly as the reference does
 * (frame/dgsks.c:445-447). */
struct kernel_s {
  ks_type type;
  double  powe;
  double  scal;
  double  cons;
  double *hi;
  double *hj;
  double *h;
};

typedef struct kernel_s ks_t;

/* Fused kernel summation on the GPU.  Replaces frame/dgsks.c:367-776.
 * Precision follows the GSKS_PRECISION environment variable
 * ("fp64" -- the default -- or "split"); see gsks.h for explicit control. */
void dgsks(
    ks_t   *kernel,
    int    m,
    int    n,
    int    k,
    double *u,
    int    *umap,
    double *XA,
    double *XA2,
    int    *amap,
    double *XB,
    double *XB2,
    int    *bmap,
    double *w,
    int    *wmap
    );

/* Unfused reference evaluation on the GPU (gather, rank-k, kernel function
 * and weighted sum as separate FP64 passes over a materialised kernel
 * block).  Same contract as frame/dgsks_ref.c:94-535; intended as an
 * independent cross-check of dgsks(). */
void dgsks_ref(
    ks_t   *kernel,
    int    m,
    int    n,
    int    k,
    double *u,
    int    *umap,
    double *XA,
    double *XA2,
    int    *amap,
    double *XB,
    double *XB2,
    int    *bmap,
    double *w,
    int    *wmap
    );

/* Host allocation of m*n elements of `size` bytes, 64-byte aligned
 * (frame/ks_util.c:34-55).  Returns NULL on failure instead of exiting. */
double *ks_malloc_aligned(
    int    m,
    int    n,
    int    size
    );

/* Flat-argument entry points used by ctypes callers
 * (frame/dgsks.c:783-826, frame/dgsks_ref.c:537-580).  Unlike the
 * reference wrappers, `cons` is forwarded into the descriptor. */
void dgsks_wrapper(
    int m, int n, int k,
    double *u, int *umap,
    double *XA, double *XA2, int *amap,
    double *XB, double *XB2, int *bmap,
    double *w, int *wmap,
    int type, double scal, double cons, double powe, double *h);

void dgsks_ref_wrapper(
    int m, int n, int k,
    double *u, int *umap,
    double *XA, double *XA2, int *amap,
    double *XB, double *XB2, int *bmap,
    double *w, int *wmap,
    int type, double scal, double cons, double powe, double *h);

#ifdef __cplusplus
}
#endif

#endif /* GSKS_GB300_KS_H */
