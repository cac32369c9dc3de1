// gsks_internal.cuh -- shared definitions of the GB300 GSKS kernels.
//
// Device-side kernel functions (one per ks_type) and the argument blocks the
// host layer hands to the launchers in gsks_fp64.cu / gsks_split.cu /
// gsks_list.cu.
#pragma once

#include <cstdint>
#include <cstddef>
#include <cuda_runtime.h>
#include "ks.h"

namespace gsks {

// Device error flags (bit set), written by kernels that detect bad input.
enum : int {
  DEVERR_MAP_RANGE = 1,   // a map index outside [0, pool size)
  DEVERR_TIMEOUT = 2,     // a bounded wait gave up
};

// Kernel descriptor as the device sees it.  hi/hj are device pointers
// (variable-bandwidth Gaussian only), indexed by pool position.
struct KParams {
  int type;
  double scal, cons, powe;
  const double *hi, *hj;
  // Laplace only: an assembled d2 below coinc * (aa + bb) is rounding noise of
  // the |x|^2 - 2 x.y + |y|^2 form, i.e. the points coincide; it takes the
  // reference's coincident-point clamp (frame/dgsks_ref.c:343-345).
  double coinc;
  // Exponent class of powe (polynomial, Laplace): integer and half-integer
  // exponents up to 511 in magnitude are evaluated by binary powering (and one
  // square root) instead of the general pow().
  int pmode, pint;
  // scal, cons, powe rounded to FP32 (the split form's epilogue: FP64
  // instructions, conversions included, issue slowly on this GPU)
  float fscal, fcons, fpowe, fpad;
};

enum { POW_GENERAL = 0, POW_INT = 1, POW_HALF = 2 };

// x^e for 0 <= e <= 64 by binary powering: at most 2 log2(e) multiplies, a
// relative error of a few units in the last place.
__device__ __forceinline__ double pow_upos(double x, int e)
{
  double r = 1.0;
  for (;;) {
    if (e & 1) r *= x;
    e >>= 1;
    if (!e) break;
    x *= x;
  }
  return r;
}

// x^powe with the exponent class chosen on the host.
__device__ __forceinline__ double pow_class(double x, const KParams &kp)
{
  if (kp.pmode == POW_INT)
    return kp.pint >= 0 ? pow_upos(x, kp.pint) : 1.0 / pow_upos(x, -kp.pint);
  if (kp.pmode == POW_HALF) {
    const double r = sqrt(x);
    return kp.pint >= 0 ? pow_upos(x, kp.pint) * r : r / pow_upos(x, -kp.pint);
  }
  return pow(x, kp.powe);
}

// Everything one fused evaluation needs.  Maps may be nullptr, which means
// the identity (position i of the call is pool point i).
struct FusedArgs {
  int m, n, k;
  const double *XA, *XA2; const int *amap;
  const double *XB, *XB2; const int *bmap;
  const double *w; const int *wmap;
  KParams kp;
  int nxa, nxb;           // pool sizes for device range checks (-1: unchecked)
  // decomposition
  int ntm;                // number of target tiles
  int nsc;                // number of source chunks
  int chunk;              // sources per chunk (multiple of the source tile)
  double *partial;        // [nrhs][nsc][ldp] per-chunk row sums
  int ldp;
  int *err;               // device error flags
  int nrhs;               // right-hand sides interleaved in u and w (0 or 1: one)
  long long rstride;      // partial elements per right-hand side
};

// ---------------------------------------------------------------------------
// FP64 kernel functions.  `dot` is the raw inner product x.y; aa = |x|^2,
// bb = |y|^2.  The operation order follows the reference's dgsks_ref
// (frame/dgsks_ref.c:253-420); like the reference micro-kernels
// (micro_kernel/x86_64/haswell/sq2nrm_int_d8x6.h:65-79) the squared distance
// is clamped at zero before the Gaussian-type kernels.
template <int KT>
__device__ __forceinline__ double kfun64(double dot, double aa, double bb,
                                         double hi, double hj, const KParams &kp)
{
  if constexpr (KT == KS_GAUSSIAN) {
    double d2 = fmax(fma(-2.0, dot, aa) + bb, 0.0);
    return exp(d2 * kp.scal);
  } else if constexpr (KT == KS_GAUSSIAN_VAR_BANDWIDTH) {
    double d2 = fmax(fma(-2.0, dot, aa) + bb, 0.0);
    return exp(((d2 * -0.5) * hi) * hj);
  } else if constexpr (KT == KS_POLYNOMIAL) {
    double c = fma(dot, kp.scal, kp.cons);
    if (kp.powe == 2.0) return c * c;
    if (kp.powe == 4.0) { c = c * c; return c * c; }
    return pow_class(c, kp);
  } else if constexpr (KT == KS_LAPLACE) {
    double d2 = fma(-2.0, dot, aa) + bb;
    if (d2 < fmax(1e-15, kp.coinc * (aa + bb))) d2 = 1.79e308;
    return pow_class(d2, kp) * kp.scal;
  } else if constexpr (KT == KS_TANH) {
    return tanh(fma(dot, kp.scal, kp.cons));
  } else if constexpr (KT == KS_QUARTIC) {
    double d2 = fma(-2.0, dot, aa) + bb;
    if (d2 < 1.0) { double t = 1.0 - d2; return (15.0 / 16.0) * t * t; }
    return 0.0;
  } else if constexpr (KT == KS_MULTIQUADRATIC) {
    return (fma(-2.0, dot, aa) + bb) + kp.cons;
  } else {  // KS_EPANECHNIKOV
    double d2 = fma(-2.0, dot, aa) + bb;
    if (d2 < 1.0) return 0.75 * (1.0 - d2);
    return 0.0;
  }
}

__host__ __device__ constexpr bool kt_uses_norms(int kt)
{
  return !(kt == KS_POLYNOMIAL || kt == KS_TANH);
}

// ---------------------------------------------------------------------------
// Launchers (defined in gsks_fp64.cu).
struct Fp64Plan {
  int ntm, nsc, chunk, grid, ldp;
  size_t partial_elems;
};
Fp64Plan fp64_plan(int m, int n, int k, int num_sms);
int fp64_launch(const FusedArgs &a, const Fp64Plan &p, double *u, const int *umap,
                cudaStream_t s);
cudaError_t norms_launch(int N, int k, const double *X, double *X2, cudaStream_t s);

}  // namespace gsks
