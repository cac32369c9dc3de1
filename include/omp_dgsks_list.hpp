/*
 * omp_dgsks_list.hpp -- C++ batched interface of the GB300 GSKS library.
 *
 * Same five functions and signatures as the reference header
 * include/omp_dgsks_list.hpp:48-115 (ChenhanYu/ks), so C++ callers relink
 * unchanged.  The reference runs them on 68 OpenMP workers; here each call
 * becomes one dgsks_list() (gsks.h): one persistent GPU launch over all
 * tasks plus a deterministic merge into u.
 *
 * Semantics kept from the reference:
 *   - u[ulist[t][i]] += sum_j K(XA[alist[t][i]], XB[blist[t][j]]) w[wlist[t][j]]
 *     for every task t, contributions of different tasks summed;
 *   - the _unsymmetric / _symmetric / _separated_u_* wrappers compute the
 *     squared norms themselves (frame/omp_dgsks_list.cpp:55-294); the
 *     symmetric forms use XA as the source pool; the non-separated forms use
 *     alist as ulist;
 *   - empty alist or blist returns immediately (:318);
 *   - lists of different lengths are an error (:321-324), reported through
 *     gsks_last_error() as GSKS_ERR_LIST instead of exit(1).
 */
#ifndef GSKS_GB300_OMP_DGSKS_LIST_HPP
#define GSKS_GB300_OMP_DGSKS_LIST_HPP

#include <vector>
#include "ks.h"

void omp_dgsks_list_unsymmetric(
    ks_t *kernel, int k, std::vector<double> &u,
    int nxa, double *XA, std::vector<std::vector<int> > &alist,
    int nxb, double *XB, std::vector<std::vector<int> > &blist,
    double *w, std::vector<std::vector<int> > &wlist);

void omp_dgsks_list_symmetric(
    ks_t *kernel, int k, std::vector<double> &u,
    double *XA, int nxa,
    std::vector<std::vector<int> > &alist, std::vector<std::vector<int> > &blist,
    double *w, std::vector<std::vector<int> > &wlist);

void omp_dgsks_list_separated_u_unsymmetric(
    ks_t *kernel, int k, std::vector<double> &u, std::vector<std::vector<int> > &ulist,
    int nxa, double *XA, std::vector<std::vector<int> > &alist,
    int nxb, double *XB, std::vector<std::vector<int> > &blist,
    double *w, std::vector<std::vector<int> > &wlist);

void omp_dgsks_list_separated_u_symmetric(
    ks_t *kernel, int k, std::vector<double> &u, std::vector<std::vector<int> > &ulist,
    double *XA, int nxa,
    std::vector<std::vector<int> > &alist, std::vector<std::vector<int> > &blist,
    double *w, std::vector<std::vector<int> > &wlist);

void omp_dgsks_list(
    ks_t *kernel, int k, std::vector<double> &u, std::vector<std::vector<int> > &ulist,
    double *XA, double *XA2, std::vector<std::vector<int> > &alist,
    double *XB, double *XB2, std::vector<std::vector<int> > &blist,
    double *w, std::vector<std::vector<int> > &wlist);

#endif /* GSKS_GB300_OMP_DGSKS_LIST_HPP */
