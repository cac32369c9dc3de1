// gsks_split.cu -- split-precision tensor-core form (sm_103a).
#include "gsks.h"
#include "gsks_internal.cuh"
#include "gsks_host.h"

namespace gsks {

int enqueue_split(Ctx *, const ks_t *, int, int, int, double *, const int *,
                  const double *, const double *, const int *, int,
                  const double *, const double *, const int *, int,
                  const double *, const int *, const double *, const double *,
                  cudaStream_t, bool)
{
  return GSKS_ERR_PRECISION;
}

}  // namespace gsks
