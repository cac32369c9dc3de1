// omp_dgsks_list.cpp -- the reference's C++ batched interface over dgsks_list.
//
// Keeps the five signatures of include/omp_dgsks_list.hpp:48-115 and their
// semantics (frame/omp_dgsks_list.cpp:55-420): the wrappers differ only in
// which pool serves as sources, whether ulist is separate from alist, and in
// computing the squared norms themselves -- here dgsks_list computes missing
// norms on the device.  Each call flattens the std::vector lists into CSR
// arrays and makes one dgsks_list() call.
#include <vector>
#include "gsks.h"
#include "omp_dgsks_list.hpp"
#include "gsks_host.h"

namespace {

struct Csr {
  std::vector<int> off, idx;
  explicit Csr(const std::vector<std::vector<int> > &l)
  {
    off.resize(l.size() + 1, 0);
    size_t tot = 0;
    for (size_t t = 0; t < l.size(); t++) { off[t] = (int)tot; tot += l[t].size(); }
    off[l.size()] = (int)tot;
    idx.reserve(tot);
    for (const auto &v : l) idx.insert(idx.end(), v.begin(), v.end());
  }
};

int max_index(const std::vector<std::vector<int> > &l)
{
  int mx = -1;
  for (const auto &v : l) for (int x : v) mx = x > mx ? x : mx;
  return mx;
}

// Shared body.  nxa / nxb < 0: pool sizes unknown (the core omp_dgsks_list
// signature has none); they are taken from the largest index the lists name.
void run_list(ks_t *kernel, int k, std::vector<double> &u, std::vector<std::vector<int> > &ulist,
              double *XA, double *XA2, int nxa, std::vector<std::vector<int> > &alist,
              double *XB, double *XB2, int nxb, std::vector<std::vector<int> > &blist,
              double *w, std::vector<std::vector<int> > &wlist)
{
  if (alist.empty() || blist.empty()) return;  // frame/omp_dgsks_list.cpp:318
  if (alist.size() != blist.size() || blist.size() != wlist.size() || ulist.size() != alist.size()) {
    // frame/omp_dgsks_list.cpp:321-324 exits here; this library reports it.
    gsks::set_status(GSKS_ERR_LIST, "omp_dgsks_list");
    return;
  }
  Csr a(alist), b(blist), uu(ulist), ww(wlist);
  for (size_t t = 0; t < alist.size(); t++)
    if (ulist[t].size() != alist[t].size() || wlist[t].size() != blist[t].size()) {
      gsks::set_status(GSKS_ERR_LIST, "omp_dgsks_list");
      return;
    }
  if (nxa < 0) nxa = max_index(alist) + 1;
  if (nxb < 0) nxb = max_index(blist) + 1;
  if (XB == XA && nxb < nxa) nxb = nxa;
  if (XB == XA && nxa < nxb) nxa = nxb;
  const int nw = max_index(wlist) + 1;
  dgsks_list(kernel, nullptr, (int)alist.size(), k, u.data(), (int)u.size(),
             a.off.data(), a.idx.data(), uu.idx.data(), b.off.data(), b.idx.data(), ww.idx.data(),
             XA, XA2, nxa, XB, XB2, nxb, w, nw);
}

}  // namespace

void omp_dgsks_list_unsymmetric(ks_t *kernel, int k, std::vector<double> &u,
                                int nxa, double *XA, std::vector<std::vector<int> > &alist,
                                int nxb, double *XB, std::vector<std::vector<int> > &blist,
                                double *w, std::vector<std::vector<int> > &wlist)
{
  run_list(kernel, k, u, alist, XA, nullptr, nxa, alist, XB, nullptr, nxb, blist, w, wlist);
}

void omp_dgsks_list_symmetric(ks_t *kernel, int k, std::vector<double> &u,
                              double *XA, int nxa,
                              std::vector<std::vector<int> > &alist,
                              std::vector<std::vector<int> > &blist,
                              double *w, std::vector<std::vector<int> > &wlist)
{
  run_list(kernel, k, u, alist, XA, nullptr, nxa, alist, XA, nullptr, nxa, blist, w, wlist);
}

void omp_dgsks_list_separated_u_unsymmetric(ks_t *kernel, int k, std::vector<double> &u,
                                            std::vector<std::vector<int> > &ulist,
                                            int nxa, double *XA,
                                            std::vector<std::vector<int> > &alist,
                                            int nxb, double *XB,
                                            std::vector<std::vector<int> > &blist,
                                            double *w, std::vector<std::vector<int> > &wlist)
{
  run_list(kernel, k, u, ulist, XA, nullptr, nxa, alist, XB, nullptr, nxb, blist, w, wlist);
}

void omp_dgsks_list_separated_u_symmetric(ks_t *kernel, int k, std::vector<double> &u,
                                          std::vector<std::vector<int> > &ulist,
                                          double *XA, int nxa,
                                          std::vector<std::vector<int> > &alist,
                                          std::vector<std::vector<int> > &blist,
                                          double *w, std::vector<std::vector<int> > &wlist)
{
  run_list(kernel, k, u, ulist, XA, nullptr, nxa, alist, XA, nullptr, nxa, blist, w, wlist);
}

void omp_dgsks_list(ks_t *kernel, int k, std::vector<double> &u,
                    std::vector<std::vector<int> > &ulist,
                    double *XA, double *XA2, std::vector<std::vector<int> > &alist,
                    double *XB, double *XB2, std::vector<std::vector<int> > &blist,
                    double *w, std::vector<std::vector<int> > &wlist)
{
  run_list(kernel, k, u, ulist, XA, XA2, -1, alist, XB, XB2, -1, blist, w, wlist);
}
