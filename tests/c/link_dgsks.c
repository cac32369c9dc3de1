/* A C caller written against ks.h alone, as existing GSKS users are: builds
 * with gcc, links libgsks.so, calls dgsks() and dgsks_ref() on host arrays
 * and prints u for the test to compare. */
#include <stdio.h>
#include <stdlib.h>
#include "ks.h"

int main(void)
{
  enum { N = 300, K = 9, M = 120, NS = 100 };
  double *X = ks_malloc_aligned(K, N, sizeof(double));
  double *X2 = ks_malloc_aligned(1, N, sizeof(double));
  double *w = ks_malloc_aligned(1, N, sizeof(double));
  double *u = ks_malloc_aligned(1, N, sizeof(double));
  double *uref = ks_malloc_aligned(1, N, sizeof(double));
  int amap[M], umap[M], bmap[NS], wmap[NS];
  unsigned s = 12345u;
  for (int i = 0; i < N * K; i++) { s = s * 1103515245u + 12345u; X[i] = (double)((s >> 8) % 1000) / 1000.0; }
  for (int i = 0; i < N; i++) {
    double t = 0.0;
    for (int p = 0; p < K; p++) t += X[i * K + p] * X[i * K + p];
    X2[i] = t; w[i] = (double)((i * 37) % 17) / 17.0 - 0.5; u[i] = uref[i] = 0.0;
  }
  for (int i = 0; i < M; i++) { amap[i] = (i * 7) % N; umap[i] = (i * 11) % N; }
  for (int j = 0; j < NS; j++) { bmap[j] = (j * 13 + 5) % N; wmap[j] = (j * 3 + 1) % N; }
  ks_t ker;
  ker.type = KS_GAUSSIAN; ker.scal = -0.5; ker.cons = 0.0; ker.powe = 1.0;
  ker.hi = ker.hj = ker.h = NULL;
  dgsks(&ker, M, NS, K, u, umap, X, X2, amap, X, X2, bmap, w, wmap);
  dgsks_ref(&ker, M, NS, K, uref, umap, X, X2, amap, X, X2, bmap, w, wmap);
  for (int i = 0; i < N; i++) printf("%.17g %.17g\n", u[i], uref[i]);
  free(X); free(X2); free(w); free(u); free(uref);
  return 0;
}
