// Scene tables built on the device at upload (scene_tables.cuh holds the
// arithmetic, shared with the host builders).
#include <string>

#include "scene_build.h"
#include "scene_tables.cuh"

namespace phc {
namespace {

// One thread per macro cell of the volume's majorant grid (grid-stride).
__global__ void __launch_bounds__(256) k_majorants(MajorantJob j, const float *__restrict__ vals,
    const float4 *__restrict__ tf, float *__restrict__ out)
{
  const uint32_t mx_n = j.macro_dims[0], my_n = j.macro_dims[1];
  const size_t n = size_t(mx_n) * my_n * j.macro_dims[2];
  auto alpha = [&](size_t t) { return __ldg(&tf[t].w); };
  for (size_t c = size_t(blockIdx.x) * blockDim.x + threadIdx.x; c < n; c += size_t(gridDim.x) * blockDim.x) {
    const uint32_t mx = uint32_t(c % mx_n), my = uint32_t((c / mx_n) % my_n), mz = uint32_t(c / (size_t(mx_n) * my_n));
    out[c] = majorant_cell(j, vals, alpha, mx, my, mz);
  }
}

} // namespace

std::string launch_majorants(const MajorantJob &job, const float *vals, const float4 *tf, float *out,
    cudaStream_t stream)
{
  const size_t n = size_t(job.macro_dims[0]) * job.macro_dims[1] * job.macro_dims[2];
  if (n == 0)
    return std::string();
  const unsigned blocks = unsigned(std::min<size_t>((n + 255) / 256, 152u * 16u));
  k_majorants<<<blocks, 256, 0, stream>>>(job, vals, tf, out);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? std::string() : std::string("majorant grid: ") + cudaGetErrorString(e);
}

} // namespace phc
