// A C++ caller of all five batched signatures of omp_dgsks_list.hpp, built
// with g++ against libgsks.so.  Reads its inputs from a binary file written by
// the test and writes u after each signature to another:
//   in:  int32 {nxa, nxb, k, ntask, nu, nw}; double {type, scal, cons, powe};
//        double XA[nxa*k], XB[nxb*k], w[nw], u0[nu];
//        int32 a_off[ntask+1], a_idx[na], u_idx[na], b_off[ntask+1], b_idx[nb], w_idx[nb]
//   out: double u[5][nu] in the order unsymmetric, symmetric,
//        separated_u_unsymmetric, separated_u_symmetric, omp_dgsks_list.
// The symmetric forms take XA for the sources; the unified-u forms take alist
// for ulist (frame/omp_dgsks_list.cpp:95-103,144-152).
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "ks.h"
#include "gsks.h"
#include "omp_dgsks_list.hpp"

typedef std::vector<std::vector<int> > Lists;

static bool rd(FILE *f, void *p, size_t bytes) { return fread(p, 1, bytes, f) == bytes; }

static Lists split(const std::vector<int> &off, const std::vector<int> &idx)
{
  Lists l(off.size() - 1);
  for (size_t t = 0; t + 1 < off.size(); t++) l[t].assign(idx.begin() + off[t], idx.begin() + off[t + 1]);
  return l;
}

int main(int argc, char **argv)
{
  if (argc != 3) return 2;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 3;
  int h[6];
  double kp[4];
  if (!rd(f, h, sizeof h) || !rd(f, kp, sizeof kp)) return 4;
  const int nxa = h[0], nxb = h[1], k = h[2], ntask = h[3], nu = h[4], nw = h[5];
  std::vector<double> XA((size_t)nxa * k), XB((size_t)nxb * k), w(nw), u0(nu);
  std::vector<int> a_off(ntask + 1), b_off(ntask + 1);
  bool ok = rd(f, XA.data(), XA.size() * 8) && rd(f, XB.data(), XB.size() * 8) && rd(f, w.data(), w.size() * 8) &&
            rd(f, u0.data(), u0.size() * 8) && rd(f, a_off.data(), a_off.size() * 4);
  if (!ok) return 5;
  std::vector<int> a_idx(a_off[ntask]), u_idx(a_off[ntask]);
  ok = rd(f, a_idx.data(), a_idx.size() * 4) && rd(f, u_idx.data(), u_idx.size() * 4) &&
       rd(f, b_off.data(), b_off.size() * 4);
  if (!ok) return 6;
  std::vector<int> b_idx(b_off[ntask]), w_idx(b_off[ntask]);
  ok = rd(f, b_idx.data(), b_idx.size() * 4) && rd(f, w_idx.data(), w_idx.size() * 4);
  fclose(f);
  if (!ok) return 7;

  Lists alist = split(a_off, a_idx), ulist = split(a_off, u_idx);
  Lists blist = split(b_off, b_idx), wlist = split(b_off, w_idx);
  // the core signature takes the squared norms from the caller
  std::vector<double> XA2(nxa), XB2(nxb);
  for (int i = 0; i < nxa; i++) {
    double s = 0.0;
    for (int p = 0; p < k; p++) s += XA[(size_t)i * k + p] * XA[(size_t)i * k + p];
    XA2[i] = s;
  }
  for (int i = 0; i < nxb; i++) {
    double s = 0.0;
    for (int p = 0; p < k; p++) s += XB[(size_t)i * k + p] * XB[(size_t)i * k + p];
    XB2[i] = s;
  }
  auto kernel = [&]() {   // a fresh descriptor per call: Laplace overwrites powe and scal
    ks_t ker;
    ker.type = (ks_type)(int)kp[0];
    ker.scal = kp[1]; ker.cons = kp[2]; ker.powe = kp[3];
    ker.hi = ker.hj = ker.h = nullptr;
    return ker;
  };
  FILE *o = fopen(argv[2], "wb");
  if (!o) return 8;
  for (int form = 0; form < 5; form++) {
    std::vector<double> u(u0);
    ks_t ker = kernel();
    switch (form) {
      case 0: omp_dgsks_list_unsymmetric(&ker, k, u, nxa, XA.data(), alist, nxb, XB.data(), blist, w.data(), wlist); break;
      case 1: omp_dgsks_list_symmetric(&ker, k, u, XA.data(), nxa, alist, blist, w.data(), wlist); break;
      case 2:
        omp_dgsks_list_separated_u_unsymmetric(&ker, k, u, ulist, nxa, XA.data(), alist, nxb, XB.data(), blist,
                                               w.data(), wlist);
        break;
      case 3: omp_dgsks_list_separated_u_symmetric(&ker, k, u, ulist, XA.data(), nxa, alist, blist, w.data(), wlist); break;
      default:
        omp_dgsks_list(&ker, k, u, ulist, XA.data(), XA2.data(), alist, XB.data(), XB2.data(), blist, w.data(),
                       wlist);
        break;
    }
    if (gsks_last_error() != GSKS_OK) { fclose(o); return 10 + form; }
    fwrite(u.data(), 8, u.size(), o);
  }
  fclose(o);
  return 0;
}
