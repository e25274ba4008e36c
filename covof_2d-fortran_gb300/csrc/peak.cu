// peak.cu -- a self-measured FP64 rate of this GPU, the denominator of the
// VOF kernels' FP64 figures (the interface reconstruction is FP64 polygon
// clipping, not a memory stream).  Independent FMA chains in every warp
// slot, timed with CUDA events on the handle's stream.
#include "handle.cuh"

namespace covof {

namespace {

constexpr int kPeakChains = 8;

__global__ void __launch_bounds__(256) k_fp64_peak(int n, double seed, double* out) {
  double a[kPeakChains];
#pragma unroll
  for (int q = 0; q < kPeakChains; ++q) a[q] = seed + 1.0e-9 * (threadIdx.x + q);
  const double b = 0.9999999, c = 1.0e-7;
  for (int i = 0; i < n; ++i) {
#pragma unroll
    for (int q = 0; q < kPeakChains; ++q) a[q] = __fma_rn(a[q], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < kPeakChains; ++q) s += a[q];
  // keep the result alive (the value itself is never used)
  if (s == 12345.678) out[0] = s;
}

}  // namespace

}  // namespace covof

using namespace covof;
using namespace covof::host;

int covof_fp64_peak(covof_handle* h, double* gflops) {
  if (!h || !gflops) return COVOF_INVALID;
  CS(ensure_fields(h));
  const int n = 4096, blocks = 2 * h->sm_count, threads = 256;
  double* out = h->f_b;  // scratch, never written in practice
  k_fp64_peak<<<blocks, threads, 0, h->stream>>>(64, 1.0, out);  // warm-up
  CK(cudaEventRecord(h->ev0, h->stream));
  k_fp64_peak<<<blocks, threads, 0, h->stream>>>(n, 1.0, out);
  CK(cudaEventRecord(h->ev1, h->stream));
  CK(cudaGetLastError());
  CS(sync(h));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
  const double flops = 2.0 * (double)n * kPeakChains * (double)blocks * threads;
  *gflops = flops / (ms * 1.0e-3) / 1.0e9;
  return COVOF_OK;
}

COVOF_UNIT_HOOKS(peak)
