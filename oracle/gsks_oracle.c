/*
 * gsks_oracle.c -- CPU restatement of the reference GSKS algorithm.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or calls
 * this file; only the tests, __graft_entry__.smoke() and the cpu_baseline /
 * reference legs of bench.py load it, as the checker and as the timed CPU
 * baseline.
 *
 * What it restates (file:line in ChenhanYu/ks):
 *   oracle_dgsks_ref    frame/dgsks_ref.c:94-535  (per-element operation order
 *                       of the GEMM + kernel + GEMV reference, evaluated row by
 *                       row so that no m x n buffer is needed)
 *   oracle_setup        frame/dgsks_ref.c:121-173 and frame/dgsks.c:420-468
 *                       (kernel-type switch; Laplace overwrites powe and scal)
 *   oracle_rows         sampled rows of dgsks_ref with Neumaier-compensated
 *                       sums plus the conditioning sum  sum_j |K_ij w_j|
 *   oracle_dgsks_fused  frame/dgsks.c:367-776 (packed, blocked, fused
 *                       rank-k + kernel + weighted sum with 8x4 micro tiles,
 *                       OpenMP over target blocks) -- the timed CPU baseline
 *   oracle_norms        frame/omp_dgsks_list.cpp:74-92
 *   oracle_dgsks_list   frame/omp_dgsks_list.cpp:297-420 (every task adds into
 *                       u; contributions of different tasks sum)
 *
 * Parity of this restatement is pinned against the reference itself: the
 * tests compare it with oracle/_ref/libgsks_ref.so (compiled from the
 * reference sources by oracle/build_ref.sh) and with golden vectors that the
 * reference produced (tests/golden/).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "ks.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ---------------------------------------------------------------------- */
/* Kernel-type setup.  Returns the factor applied to the raw inner product
 * (dgsks_ref.c:121-173): -2 for distance kernels, +1 for inner-product
 * kernels; -0 (a NaN sentinel) for an illegal type.  Laplace overwrites
 * powe/scal in the caller's descriptor like the reference. */
double oracle_setup(ks_t *ker, int k)
{
  switch (ker->type) {
    case KS_GAUSSIAN:
    case KS_GAUSSIAN_VAR_BANDWIDTH:
    case KS_QUARTIC:
    case KS_MULTIQUADRATIC:
    case KS_EPANECHNIKOV:
      return -2.0;
    case KS_POLYNOMIAL:
    case KS_TANH:
      return 1.0;
    case KS_LAPLACE:
      ker->powe = 0.5 * (2.0 - (double)k);
      ker->scal = tgamma(0.5 * k + 1.0) /
                  ((double)k * (double)(k - 2) * pow(M_PI, 0.5 * k));
      return -2.0;
    default:
      return NAN;
  }
}

/* One kernel value from the raw inner product `dot` of target i and source
 * j, following the per-element operation order of dgsks_ref.c:253-420. */
static inline double oracle_pair(const ks_t *ker, double rks, double dot,
                                 double aa, double bb, double hi, double hj)
{
  double c = dot * rks;
  switch (ker->type) {
    case KS_GAUSSIAN:
      c += aa; c += bb; c *= ker->scal;
      return exp(c);
    case KS_GAUSSIAN_VAR_BANDWIDTH:
      c += aa; c += bb; c *= -0.5; c *= hi; c *= hj;
      return exp(c);
    case KS_POLYNOMIAL:
      c *= ker->scal; c += ker->cons;
      if (ker->powe == 2.0) return c * c;
      if (ker->powe == 4.0) { c = c * c; return c * c; }
      return pow(c, ker->powe);
    case KS_LAPLACE:
      c += aa; c += bb;
      if (c < 1E-15) c = 1.79E+308;
      return pow(c, ker->powe) * ker->scal;
    case KS_TANH:
      c *= ker->scal; c += ker->cons;
      return tanh(c);
    case KS_QUARTIC:
      c += aa; c += bb;
      if (c < 1.0) { c = 1.0 - c; return (15.0 / 16.0) * c * c; }
      return 0.0;
    case KS_MULTIQUADRATIC:
      c += aa; c += bb; c += ker->cons;
      return c;
    case KS_EPANECHNIKOV:
      c += aa; c += bb;
      if (c < 1.0) { c = 1.0 - c; return (3.0 / 4.0) * c; }
      return 0.0;
    default:
      return NAN;
  }
}

static inline int uses_norms(ks_type t)
{
  return !(t == KS_POLYNOMIAL || t == KS_TANH);
}

void oracle_set_threads(int nt)
{
#ifdef _OPENMP
  if (nt > 0) omp_set_num_threads(nt);
#else
  (void)nt;
#endif
}

int oracle_get_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ---------------------------------------------------------------------- */
/* dgsks_ref restated.  us[i] starts from u[umap[i]] (dgsks_ref.c:192-200),
 * accumulates sum_j K_ij w_j in source order (dgsks_ref.c:437-444), and is
 * written back with u[umap[i]] = us[i] in target order
 * (dgsks_ref.c:454-459), so duplicated umap entries keep the last
 * writer.  Returns 0, or -1 for an illegal kernel type. */
int oracle_dgsks_ref(ks_t *ker, int m, int n, int k,
                     double *u, const int *umap,
                     const double *XA, const double *XA2, const int *amap,
                     const double *XB, const double *XB2, const int *bmap,
                     const double *w, const int *wmap)
{
  double rks = oracle_setup(ker, k);
  if (isnan(rks)) return -1;
  if (m <= 0 || n <= 0) return 0;
  const int norms = uses_norms(ker->type);
  const int varbw = (ker->type == KS_GAUSSIAN_VAR_BANDWIDTH);
  double *us = (double *)malloc(sizeof(double) * (size_t)m);
  if (!us) return -2;
  for (int i = 0; i < m; i++) us[i] = u[umap[i]];

  #pragma omp parallel for schedule(dynamic, 4)
  for (int i = 0; i < m; i++) {
    const double *a = XA + (size_t)amap[i] * k;
    const double aa = norms ? XA2[amap[i]] : 0.0;
    const double hi = varbw ? ker->hi[amap[i]] : 0.0;
    double acc = us[i];
    for (int j = 0; j < n; j++) {
      const double *b = XB + (size_t)bmap[j] * k;
      double dot = 0.0;
      for (int p = 0; p < k; p++) dot += a[p] * b[p];
      const double bb = norms ? XB2[bmap[j]] : 0.0;
      const double hj = varbw ? ker->hj[bmap[j]] : 0.0;
      acc += oracle_pair(ker, rks, dot, aa, bb, hi, hj) * w[wmap[j]];
    }
    us[i] = acc;
  }
  for (int i = 0; i < m; i++) u[umap[i]] = us[i];
  free(us);
  return 0;
}

/* ---------------------------------------------------------------------- */
/* Sampled rows.  For each of the nrows target positions rows[r] (indices
 * into amap), sum_out[r] = sum_j K w (Neumaier-compensated, independent of
 * u) and abs_out[r] = sum_j |K w|, the denominator of the conditioned
 * relative error.  Used where an m x n reference evaluation is too large. */
int oracle_rows(ks_t *ker, int nrows, const int *rows, int n, int k,
                const double *XA, const double *XA2, const int *amap,
                const double *XB, const double *XB2, const int *bmap,
                const double *w, const int *wmap,
                double *sum_out, double *abs_out)
{
  double rks = oracle_setup(ker, k);
  if (isnan(rks)) return -1;
  const int norms = uses_norms(ker->type);
  const int varbw = (ker->type == KS_GAUSSIAN_VAR_BANDWIDTH);

  #pragma omp parallel for schedule(dynamic, 1)
  for (int r = 0; r < nrows; r++) {
    const int i = rows[r];
    const double *a = XA + (size_t)amap[i] * k;
    const double aa = norms ? XA2[amap[i]] : 0.0;
    const double hi = varbw ? ker->hi[amap[i]] : 0.0;
    double s = 0.0, comp = 0.0, sabs = 0.0;
    for (int j = 0; j < n; j++) {
      const double *b = XB + (size_t)bmap[j] * k;
      double dot = 0.0;
      for (int p = 0; p < k; p++) dot += a[p] * b[p];
      const double bb = norms ? XB2[bmap[j]] : 0.0;
      const double hj = varbw ? ker->hj[bmap[j]] : 0.0;
      const double t = oracle_pair(ker, rks, dot, aa, bb, hi, hj) * w[wmap[j]];
      const double ns = s + t;   /* Neumaier's variant of Kahan summation */
      comp += (fabs(s) >= fabs(t)) ? (s - ns) + t : (t - ns) + s;
      s = ns;
      sabs += fabs(t);
    }
    sum_out[r] = s + comp;
    abs_out[r] = sabs;
  }
  return 0;
}

/* ---------------------------------------------------------------------- */
/* Squared norms of N k-dimensional points (omp_dgsks_list.cpp:74-92). */
void oracle_norms(int N, int k, const double *X, double *X2)
{
  #pragma omp parallel for
  for (int i = 0; i < N; i++) {
    double t = 0.0;
    for (int p = 0; p < k; p++) t += X[(size_t)i * k + p] * X[(size_t)i * k + p];
    X2[i] = t;
  }
}

/* ---------------------------------------------------------------------- */
/* Fused, blocked CPU evaluation in the manner of dgsks.c:367-776: sources are
 * packed once into NR-interleaved panels (packB_kcxnc, dgsks.c:104-132),
 * each OpenMP thread packs MR-interleaved target panels (packA_kcxmc,
 * dgsks.c:70-95), and an MR x NR micro tile forms the rank-k product,
 * assembles the kernel and folds it into the packed u in registers.
 * Same results as oracle_dgsks_ref up to rounding order; this is the
 * timed CPU baseline. */
#define OR_MR 8
#define OR_NR 4
#define OR_MC 128

int oracle_dgsks_fused(ks_t *ker, int m, int n, int k,
                       double *u, const int *umap,
                       const double *XA, const double *XA2, const int *amap,
                       const double *XB, const double *XB2, const int *bmap,
                       const double *w, const int *wmap)
{
  double rks = oracle_setup(ker, k);
  if (isnan(rks)) return -1;
  if (m <= 0 || n <= 0 || k <= 0) return 0;
  const int norms = uses_norms(ker->type);
  const int varbw = (ker->type == KS_GAUSSIAN_VAR_BANDWIDTH);
  const int npan = (n + OR_NR - 1) / OR_NR;
  double *pB  = (double *)malloc(sizeof(double) * (size_t)npan * OR_NR * k);
  double *pB2 = (double *)malloc(sizeof(double) * (size_t)npan * OR_NR);
  double *pBh = (double *)malloc(sizeof(double) * (size_t)npan * OR_NR);
  double *pw  = (double *)malloc(sizeof(double) * (size_t)npan * OR_NR);
  double *us  = (double *)malloc(sizeof(double) * (size_t)m);
  if (!pB || !pB2 || !pBh || !pw || !us) {
    free(pB); free(pB2); free(pBh); free(pw); free(us);
    return -2;
  }

  /* Pack sources; tails padded with bmap[0] and zero weight (dgsks.c:122-124,155-157). */
  #pragma omp parallel for
  for (int jp = 0; jp < npan; jp++) {
    for (int jr = 0; jr < OR_NR; jr++) {
      const int j = jp * OR_NR + jr;
      const int src = (j < n) ? bmap[j] : bmap[0];
      for (int p = 0; p < k; p++)
        pB[((size_t)jp * k + p) * OR_NR + jr] = XB[(size_t)src * k + p];
      pB2[jp * OR_NR + jr] = norms ? XB2[src] : 0.0;
      pBh[jp * OR_NR + jr] = varbw ? ker->hj[src] : 0.0;
      pw[jp * OR_NR + jr]  = (j < n) ? w[wmap[j]] : 0.0;
    }
  }
  for (int i = 0; i < m; i++) us[i] = u[umap[i]];

  const int nblk = (m + OR_MC - 1) / OR_MC;
  #pragma omp parallel
  {
    double *pA  = (double *)malloc(sizeof(double) * (size_t)OR_MC * k);
    double pA2[OR_MC], pAh[OR_MC];
    #pragma omp for schedule(dynamic, 1)
    for (int blk = 0; blk < nblk; blk++) {
      const int i0 = blk * OR_MC;
      const int ib = (m - i0 < OR_MC) ? m - i0 : OR_MC;
      const int nip = (ib + OR_MR - 1) / OR_MR;
      for (int ip = 0; ip < nip; ip++) {
        for (int ir = 0; ir < OR_MR; ir++) {
          const int i = i0 + ip * OR_MR + ir;
          const int src = (i < i0 + ib) ? amap[i] : amap[i0];
          for (int p = 0; p < k; p++)
            pA[((size_t)ip * k + p) * OR_MR + ir] = XA[(size_t)src * k + p];
          pA2[ip * OR_MR + ir] = norms ? XA2[src] : 0.0;
          pAh[ip * OR_MR + ir] = varbw ? ker->hi[src] : 0.0;
        }
      }
      for (int ip = 0; ip < nip; ip++) {
        double uacc[OR_MR];
        for (int ir = 0; ir < OR_MR; ir++) uacc[ir] = 0.0;
        const double *a = pA + (size_t)ip * k * OR_MR;
        for (int jp = 0; jp < npan; jp++) {
          const double *b = pB + (size_t)jp * k * OR_NR;
          double c[OR_MR][OR_NR];
          for (int ir = 0; ir < OR_MR; ir++)
            for (int jr = 0; jr < OR_NR; jr++) c[ir][jr] = 0.0;
          for (int p = 0; p < k; p++)
            for (int ir = 0; ir < OR_MR; ir++)
              for (int jr = 0; jr < OR_NR; jr++)
                c[ir][jr] += a[p * OR_MR + ir] * b[p * OR_NR + jr];
          for (int ir = 0; ir < OR_MR; ir++) {
            double s = 0.0;
            for (int jr = 0; jr < OR_NR; jr++) {
              double kv = oracle_pair(ker, rks, c[ir][jr], pA2[ip * OR_MR + ir],
                                      pB2[jp * OR_NR + jr], pAh[ip * OR_MR + ir],
                                      pBh[jp * OR_NR + jr]);
              s += kv * pw[jp * OR_NR + jr];
            }
            uacc[ir] += s;
          }
        }
        for (int ir = 0; ir < OR_MR; ir++) {
          const int i = i0 + ip * OR_MR + ir;
          if (i < i0 + ib) us[i] += uacc[ir];
        }
      }
    }
    free(pA);
  }
  for (int i = 0; i < m; i++) u[umap[i]] = us[i];
  free(pB); free(pB2); free(pBh); free(pw); free(us);
  return 0;
}

/* ---------------------------------------------------------------------- */
/* Batched evaluation (omp_dgsks_list.cpp:297-420).  Task t uses
 * amap = a_idx[a_off[t] .. a_off[t+1]), umap = u_idx over the same range,
 * bmap = b_idx[b_off[t] .. b_off[t+1]) and wmap = w_idx over that range.
 * kers == NULL uses `ker` for every task; otherwise task t uses kers[t]
 * (the per-task descriptor extension of the GPU dgsks_list).  Every task
 * accumulates into u, so contributions of different tasks sum. */
int oracle_dgsks_list(ks_t *ker, ks_t *kers, int ntask, int k, double *u,
                      const int *a_off, const int *a_idx, const int *u_idx,
                      const int *b_off, const int *b_idx, const int *w_idx,
                      const double *XA, const double *XA2,
                      const double *XB, const double *XB2, const double *w)
{
  for (int t = 0; t < ntask; t++) {
    const int ma = a_off[t + 1] - a_off[t];
    const int nb = b_off[t + 1] - b_off[t];
    if (ma == 0 || nb == 0) continue;
    ks_t *kt = kers ? &kers[t] : ker;
    int rc = oracle_dgsks_ref(kt, ma, nb, k, u, u_idx + a_off[t],
                              XA, XA2, a_idx + a_off[t],
                              XB, XB2, b_idx + b_off[t],
                              w, w_idx + b_off[t]);
    if (rc) return rc;
  }
  return 0;
}

/* Multi-threaded batched evaluation (the timed CPU baseline of the batched
 * workload), after frame/omp_dgsks_list.cpp:297-420: the reference assigns
 * tasks greedily, largest cost first, to the least loaded of its threads and
 * runs one dgsks per task into a per-thread copy of u, then adds the copies.
 * Here the threads take the tasks in descending cost order from a shared
 * queue (the same balance without the ahead-of-time assignment), each task
 * runs oracle_dgsks_fused single-threaded into the thread's copy of u, and the
 * copies are added into u.  Arguments as oracle_dgsks_list; nu = size of u. */
static const int *g_cost_a, *g_cost_b;
static int cost_cmp(const void *x, const void *y)
{
  const int tx = *(const int *)x, ty = *(const int *)y;
  const long long cx = (long long)(g_cost_a[tx + 1] - g_cost_a[tx]) * (g_cost_b[tx + 1] - g_cost_b[tx]);
  const long long cy = (long long)(g_cost_a[ty + 1] - g_cost_a[ty]) * (g_cost_b[ty + 1] - g_cost_b[ty]);
  return cx < cy ? 1 : (cx > cy ? -1 : (tx - ty));
}

int oracle_dgsks_list_omp(ks_t *ker, ks_t *kers, int ntask, int k, double *u, int nu,
                          const int *a_off, const int *a_idx, const int *u_idx,
                          const int *b_off, const int *b_idx, const int *w_idx,
                          const double *XA, const double *XA2,
                          const double *XB, const double *XB2, const double *w)
{
  int *order = (int *)malloc(sizeof(int) * (size_t)(ntask > 0 ? ntask : 1));
  if (!order) return -2;
  for (int t = 0; t < ntask; t++) order[t] = t;
  g_cost_a = a_off; g_cost_b = b_off;
  qsort(order, (size_t)ntask, sizeof(int), cost_cmp);
  int nthr = 1;
#ifdef _OPENMP
  nthr = omp_get_max_threads();
#endif
  double *ucopy = (double *)calloc((size_t)nthr * (size_t)nu, sizeof(double));
  if (!ucopy) { free(order); return -2; }
  int rc = 0;
  #pragma omp parallel
  {
    int me = 0;
#ifdef _OPENMP
    me = omp_get_thread_num();
#endif
    double *um = ucopy + (size_t)me * nu;
    #pragma omp for schedule(dynamic, 1)
    for (int q = 0; q < ntask; q++) {
      const int t = order[q];
      const int ma = a_off[t + 1] - a_off[t], nb = b_off[t + 1] - b_off[t];
      if (ma == 0 || nb == 0) continue;
      ks_t kt = kers ? kers[t] : *ker;
      const int r = oracle_dgsks_fused(&kt, ma, nb, k, um, u_idx + a_off[t], XA, XA2, a_idx + a_off[t],
                                       XB, XB2, b_idx + b_off[t], w, w_idx + b_off[t]);
      if (r) {
        #pragma omp atomic write
        rc = r;
      }
    }
  }
  #pragma omp parallel for
  for (int e = 0; e < nu; e++)
    for (int q = 0; q < nthr; q++) u[e] += ucopy[(size_t)q * nu + e];
  free(ucopy);
  free(order);
  return rc;
}

