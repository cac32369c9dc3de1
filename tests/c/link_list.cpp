// A C++ caller of the reference's batched interface (omp_dgsks_list.hpp),
// built with g++ against libgsks.so.  Runs the symmetric separated-u wrapper
// the reference's own list driver uses and prints u.
#include <cstdio>
#include <vector>
#include "ks.h"
#include "omp_dgsks_list.hpp"

int main()
{
  const int nx = 500, k = 6, ntask = 7;
  std::vector<double> X(nx * k), w(nx);
  unsigned s = 777u;
  for (auto &x : X) { s = s * 1664525u + 1013904223u; x = (double)((s >> 9) % 100) / 1000.0; }
  for (int i = 0; i < nx; i++) w[i] = 1.0 + 0.001 * (i % 13);
  std::vector<std::vector<int> > alist(ntask), blist(ntask), wlist(ntask), ulist(ntask);
  for (int t = 0; t < ntask; t++) {
    int na = 30 + 17 * t, nb = 25 + 11 * t;
    for (int i = 0; i < na; i++) { alist[t].push_back((i * 7 + t * 31) % nx); }
    for (int j = 0; j < nb; j++) { blist[t].push_back((j * 3 + t * 5) % nx); }
    wlist[t] = blist[t];
    ulist[t] = alist[t];
  }
  std::vector<double> u(nx, 0.0);
  ks_t ker;
  ker.type = KS_GAUSSIAN; ker.scal = -0.5; ker.cons = 0.0; ker.powe = 1.0;
  ker.hi = ker.hj = ker.h = nullptr;
  omp_dgsks_list_separated_u_symmetric(&ker, k, u, ulist, X.data(), nx, alist, blist, w.data(), wlist);
  for (int i = 0; i < nx; i++) std::printf("%.17g\n", u[i]);
  return 0;
}
