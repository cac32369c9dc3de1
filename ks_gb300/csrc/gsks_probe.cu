// gsks_probe.cu -- device calibration: issue-rate probes for the roofline.
//
// The roofline of the plain form is set by the FP64 pipe, and that of the
// split form partly by the FP32 pipe and the SFU (ex2).  Their rates on a
// given part are measured here with independent dependency chains per thread
// (enough to cover pipe latency) on every SM, timed with CUDA events.  The
// result is in operations per second (one FMA = one operation).
#include "gsks.h"
#include "gsks_host.h"

namespace gsks {
namespace {

constexpr int CHAINS = 8;
// FP64: the operand pattern of the FP64 kernel's register tile, a 4 x 4 outer
// product c[i][j] += a[i] b[j] (16 independent chains, each operand reused
// four times); chains of fma(a, const, const) issue measurably slower.
__global__ void probe_dfma(int iters, double seed, double *sink)
{
  double a[4], b[4], c[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    a[i] = 0.999999 - 1e-7 * (i + threadIdx.x);
    b[i] = 1.000001 + 1e-7 * i;
#pragma unroll
    for (int j = 0; j < 4; j++) c[i][j] = seed + i - j;
  }
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) c[i][j] = fma(a[i], b[j], c[i][j]);
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) s += c[i][j];
  if (s == 12345.678) sink[0] = s;  // keeps the chains live
}

// FP64 tensor-core MMA (DMMA, mma.sync m8n8k4 f64): 256 FMA per warp and
// instruction; CHAINS independent accumulators per warp.
__global__ void probe_dmma(int iters, double seed, double *sink)
{
  double acc[CHAINS][2];
#pragma unroll
  for (int c = 0; c < CHAINS; c++) { acc[c][0] = seed + c; acc[c][1] = seed - c + threadIdx.x; }
  const double a = 0.999999 + 1e-9 * threadIdx.x, b = 1.0000001;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < CHAINS; c++)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                   : "+d"(acc[c][0]), "+d"(acc[c][1])
                   : "d"(a), "d"(b));
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < CHAINS; c++) s += acc[c][0] + acc[c][1];
  if (s == 12345.678) sink[0] = s;
}

__global__ void probe_ffma(int iters, float seed, float *sink)
{
  float a[CHAINS];
#pragma unroll
  for (int c = 0; c < CHAINS; c++) a[c] = seed + c + threadIdx.x;
  const float b = 0.9999f, d = 1e-7f;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < CHAINS; c++) a[c] = fmaf(a[c], b, d);
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < CHAINS; c++) s += a[c];
  if (s == 12345.678f) sink[0] = s;
}

__global__ void probe_ex2(int iters, float seed, float *sink)
{
  float a[CHAINS];
#pragma unroll
  for (int c = 0; c < CHAINS; c++) a[c] = -(seed + 0.001f * (c + threadIdx.x));
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < CHAINS; c++) {
      float r;
      asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a[c]));
      a[c] = -r;
    }
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < CHAINS; c++) s += a[c];
  if (s == 12345.678f) sink[0] = s;
}

}  // namespace
}  // namespace gsks

using namespace gsks;

// what: 0 = FP64 FMA, 1 = FP32 FMA, 2 = SFU ex2, 3 = FP64 tensor-core FMA
// (DMMA).  Writes operations/s (FMA counted once).
extern "C" int gsks_probe_peak(int what, double *ops_per_s)
{
  if (!ops_per_s || what < 0 || what > 3) return set_status(GSKS_ERR_ARG, "gsks_probe_peak");
  Ctx *c = get_ctx();
  if (!c) return gsks_last_error();
  const int threads = 256, blocks = c->num_sms * (what == 0 || what == 3 ? 4 : 8);
  const int iters = what == 0 ? 2048 : what == 3 ? 1024 : 65536;
  void *sink = nullptr;
  if (cudaMalloc(&sink, 64) != cudaSuccess) return set_status(GSKS_ERR_ALLOC, "gsks_probe_peak");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0); cudaEventCreate(&e1);
  float best_ms = 1e30f;
  for (int rep = 0; rep < 4; rep++) {
    cudaEventRecord(e0, c->stream);
    if (what == 0) probe_dfma<<<blocks, threads, 0, c->stream>>>(iters, 1.0, (double *)sink);
    else if (what == 3) probe_dmma<<<blocks, threads, 0, c->stream>>>(iters, 1.0, (double *)sink);
    else if (what == 1) probe_ffma<<<blocks, threads, 0, c->stream>>>(iters, 1.0f, (float *)sink);
    else probe_ex2<<<blocks, threads, 0, c->stream>>>(iters, 0.5f, (float *)sink);
    cudaEventRecord(e1, c->stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best_ms) best_ms = ms;  // rep 0 is a warm-up
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  cudaFree(sink);
  if (err != cudaSuccess) return cuda_status(err, "gsks_probe_peak");
  double ops = (double)blocks * threads * CHAINS * (double)iters;
  if (what == 0) ops = (double)blocks * threads * 64.0 * (double)iters;
  if (what == 3) ops = (double)blocks * (threads / 32) * CHAINS * 256.0 * (double)iters;
  *ops_per_s = ops / (best_ms * 1e-3);
  return set_status(GSKS_OK, nullptr);
}
