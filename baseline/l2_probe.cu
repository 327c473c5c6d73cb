// Read bandwidth of an L2-resident buffer: the ceiling of a kernel whose
// working set (BVH nodes, triangles) stays in the 129 MB L2, measured in the
// same run as that kernel.  A copy through torch is launch-bound at these
// sizes (a 32 MiB copy lasts a few microseconds), so the probe is one
// launch that sweeps the buffer `reps` times with 16-byte loads.
#include <cuda_runtime.h>

#include <cstdint>

__global__ void k_l2_read(const float4 *__restrict__ buf, uint32_t n, uint32_t reps, float *__restrict__ sink)
{
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t stride = gridDim.x * blockDim.x;
  float acc = 0.f;
  for (uint32_t r = 0; r < reps; ++r) {
    for (uint32_t i = tid; i < n; i += stride) {
      const float4 v = __ldcg(buf + i); // cached in L2 only: L1 holds none of it between sweeps
      acc += (v.x + v.y) + (v.z + v.w);
    }
  }
  sink[tid] = acc;
}

extern "C" {

// Average read bandwidth in GB/s of `reps` sweeps over `bytes` (a multiple of
// 16) of device memory at `buf`, after one warm-up sweep; `sink` holds
// blocks * 256 floats.  Returns a negative value on a CUDA error.
double l2_read_gbs(const void *buf, uint64_t bytes, uint32_t reps, uint32_t blocks, float *sink)
{
  const uint32_t n = uint32_t(bytes / 16);
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return -1.0;
  k_l2_read<<<blocks, 256>>>((const float4 *)buf, n, 1, sink);
  cudaEventRecord(e0);
  k_l2_read<<<blocks, 256>>>((const float4 *)buf, n, reps, sink);
  cudaEventRecord(e1);
  float ms = 0.f;
  const bool ok = cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess &&
      cudaGetLastError() == cudaSuccess;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ok && ms > 0.f ? double(n) * 16.0 * reps / (ms * 1e-3) / 1e9 : -1.0;
}

} // extern "C"
