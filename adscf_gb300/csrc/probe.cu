// probe.cu -- bandwidth probe for the roofline denominators: copy bandwidth
// of a buffer pair small enough to stay resident in L2.  A measurement
// helper of the benchmark; it has no counterpart in the reference.
#include "internal.h"

namespace {

// Each thread copies its own float4 elements `reps` times in one launch, four
// loads in flight, loads cached in L2 only (ld.global.cg) so that the second
// and later passes read L2 rather than L1; one launch keeps launch gaps out
// of the figure.
__global__ void __launch_bounds__(512) k_copy16(const float4* __restrict__ a, float4* __restrict__ b, size_t n,
                                                int reps) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t i0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int r = 0; r < reps; ++r) {
    size_t i = i0;
    for (; i + 3 * stride < n; i += 4 * stride) {
      const float4 v0 = __ldcg(a + i), v1 = __ldcg(a + i + stride);
      const float4 v2 = __ldcg(a + i + 2 * stride), v3 = __ldcg(a + i + 3 * stride);
      __stcg(b + i, v0);
      __stcg(b + i + stride, v1);
      __stcg(b + i + 2 * stride, v2);
      __stcg(b + i + 3 * stride, v3);
    }
    for (; i < n; i += stride) __stcg(b + i, __ldcg(a + i));
  }
}

}  // namespace

extern "C" int adscf_probe_l2_copy(long long bytes, int reps, double* gbs) {
  ADSCF_RANGE("adscf_probe_l2_copy");
  if (bytes < (1 << 20) || bytes > (1LL << 28) || reps < 1 || !gbs) return ADSCF_E_ARG;
  const size_t n = (size_t)bytes / 16;
  float4 *a = nullptr, *b = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int dev = 0, nsm = 0, rc = ADSCF_OK;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return ADSCF_E_CUDA;
  if (cudaMalloc(&a, n * 16) != cudaSuccess || cudaMalloc(&b, n * 16) != cudaSuccess) {
    cudaFree(a);
    cudaGetLastError();
    return ADSCF_E_OOM;
  }
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_copy16, 512, 0) != cudaSuccess || occ < 1)
    occ = 1;
  const int grid = nsm * occ;
  float ms = 0.f;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess ||
      cudaMemsetAsync(a, 0, n * 16, s) != cudaSuccess) {
    rc = ADSCF_E_CUDA;
  } else {
    k_copy16<<<grid, 512, 0, s>>>(a, b, n, 2);   // both buffers into L2
    cudaEventRecord(e0, s);
    k_copy16<<<grid, 512, 0, s>>>(a, b, n, reps);
    cudaEventRecord(e1, s);
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
      rc = ADSCF_E_CUDA;
    else
      *gbs = 2.0 * (double)n * 16.0 * reps / (ms * 1e-3) / 1e9;   // bytes read + written
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  cudaFree(a);
  cudaFree(b);
  return rc;
}
