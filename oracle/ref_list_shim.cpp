// ref_list_shim.cpp -- flat C entry into the reference's C++ batched driver.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build_ref.sh against the
// reference headers where they lie and linked with oracle/_ref/libgsks_ref.so,
// so that the golden-vector generator can call omp_dgsks_list
// (frame/omp_dgsks_list.cpp:297-420) without a C++ caller.  CSR lists:
// task t uses a_idx[a_off[t]..a_off[t+1]) for amap and umap, and
// b_idx[b_off[t]..b_off[t+1]) for bmap and wmap.
#include <vector>
extern "C" {
#include <ks.h>
}
#include <omp_dgsks_list.hpp>

extern "C" void ref_omp_dgsks_list_flat(ks_t *ker, int k, int nu, double *u,
                                        int ntask, const int *a_off, const int *a_idx,
                                        const int *b_off, const int *b_idx,
                                        double *XA, double *XA2, double *XB, double *XB2,
                                        double *w)
{
  std::vector<double> uv(u, u + nu);
  std::vector<std::vector<int>> al(ntask), bl(ntask);
  for (int t = 0; t < ntask; t++) {
    al[t].assign(a_idx + a_off[t], a_idx + a_off[t + 1]);
    bl[t].assign(b_idx + b_off[t], b_idx + b_off[t + 1]);
  }
  std::vector<std::vector<int>> ul = al, wl = bl;
  omp_dgsks_list(ker, k, uv, ul, XA, XA2, al, XB, XB2, bl, w, wl);
  for (int i = 0; i < nu; i++) u[i] = uv[i];
}
