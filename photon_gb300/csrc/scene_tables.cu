// Scene tables built on the device at upload (scene_tables.cuh holds the
// arithmetic, shared with the host builders).
#include <algorithm>
#include <string>

#include "scene_build.h"
#include "scene_tables.cuh"
#include "bvh_gpu.h"

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

// The 8-bit code of one texel value: k where x is bit for bit dec[k], with
// the host packer's rounding (pack_texels_u8); flags any other value.
__device__ __forceinline__ uint32_t texel_code(float x, const float *tab, uint32_t &bad)
{
  const float y = __fmul_rn(x, 255.f);
  const bool in = y >= 0.f && y <= 255.f; // false for NaN
  const uint32_t k = in ? uint32_t(__fadd_rn(y, 0.5f)) : 0u;
  bad |= uint32_t(!in) | uint32_t(__float_as_uint(x) != __float_as_uint(tab[k]));
  return k;
}

// One thread per texel (grid-stride), the decode table in shared memory.
__global__ void __launch_bounds__(256) k_pack_texels_u8(const float4 *__restrict__ src, size_t n,
    const float *__restrict__ dec, uchar4 *__restrict__ dst, uint32_t *__restrict__ bad)
{
  __shared__ float tab[256];
  tab[threadIdx.x] = dec[threadIdx.x];
  __syncthreads();
  uint32_t b = 0;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    const float4 x = __ldcs(&src[i]);
    uchar4 q;
    q.x = uint8_t(texel_code(x.x, tab, b));
    q.y = uint8_t(texel_code(x.y, tab, b));
    q.z = uint8_t(texel_code(x.z, tab, b));
    q.w = uint8_t(texel_code(x.w, tab, b));
    dst[i] = q;
  }
  if (__any_sync(0xffffffffu, b != 0) && (threadIdx.x & 31) == 0)
    atomicOr(bad, 1u);
}

// ---------------------------------------------------------------- environment

// Texels of the environment map as the host builder stores them: RGB of the
// caller's array, non-finite and non-positive values as 0, w = 0.
__global__ void __launch_bounds__(256) k_env_texels(const float *__restrict__ rgb, size_t n, float4 *__restrict__ out)
{
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    float v[3];
    for (int c = 0; c < 3; ++c) {
      const float x = rgb[3 * i + c];
      v[c] = isfinite(x) && x > 0.f ? x : 0.f;
    }
    out[i] = make_float4(v[0], v[1], v[2], 0.f);
  }
}

// One thread per row: the running luminance sum in texel order (the
// reference's float order), normalised, and the row's weight sum * sin(theta);
// flags a row whose CDF is not non-decreasing.
__global__ void __launch_bounds__(128) k_env_rows(const float4 *__restrict__ px, uint32_t w, uint32_t h,
    const float *__restrict__ row_sin, float *__restrict__ cond, float *__restrict__ row_w, uint32_t *__restrict__ bad)
{
  const uint32_t y = blockIdx.x * blockDim.x + threadIdx.x;
  if (y >= h)
    return;
  float *c = cond + size_t(y) * (w + 1);
  const float4 *p = px + size_t(y) * w;
  c[0] = 0.f;
  float sum = 0.f;
  for (uint32_t x = 0; x < w; ++x) {
    const float4 t = p[x];
    sum += tbl_lum(t.x, t.y, t.z);
    c[x + 1] = sum;
  }
  if (sum > 0.f) {
    const float inv = 1.f / sum;
    for (uint32_t x = 0; x <= w; ++x)
      c[x] *= inv;
    c[w] = 1.f;
  } else {
    for (uint32_t x = 0; x <= w; ++x)
      c[x] = float(x) / float(w);
  }
  row_w[y] = sum * row_sin[y];
  bool ok = true;
  for (uint32_t x = 1; x <= w; ++x)
    ok = ok && c[x - 1] <= c[x];
  if (!ok)
    atomicOr(bad, 1u);
}

// The marginal CDF over the row weights, in row order, by one thread.
__global__ void k_env_marginal(const float *__restrict__ row_w, uint32_t h, float *__restrict__ marg,
    uint32_t *__restrict__ bad)
{
  if (blockIdx.x != 0 || threadIdx.x != 0)
    return;
  float total = 0.f;
  marg[0] = 0.f;
  for (uint32_t y = 0; y < h; ++y) {
    total += row_w[y];
    marg[y + 1] = total;
  }
  if (total > 0.f) {
    const float inv = 1.f / total;
    for (uint32_t y = 0; y <= h; ++y)
      marg[y] *= inv;
    marg[h] = 1.f;
  } else {
    for (uint32_t y = 0; y <= h; ++y)
      marg[y] = float(y) / float(h);
  }
  bool ok = true;
  for (uint32_t y = 1; y <= h; ++y)
    ok = ok && marg[y - 1] <= marg[y];
  if (!ok)
    atomicOr(bad, 2u);
}

// Guide entries: the marginal's (gm = 2^ENV_MGUIDE_BITS + 1) and every
// row's (gc = 2^ENV_CGUIDE_BITS + 1), one thread per entry.
__global__ void __launch_bounds__(256) k_env_guides(const float *__restrict__ marg, const float *__restrict__ cond,
    uint32_t w, uint32_t h, uint32_t *__restrict__ mguide, uint32_t *__restrict__ cguide)
{
  const uint32_t gm = (1u << ENV_MGUIDE_BITS) + 1, gc = (1u << ENV_CGUIDE_BITS) + 1;
  const size_t n = gm + size_t(h) * gc;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    if (i < gm) {
      const uint32_t k = uint32_t(i);
      mguide[k] = k + 1 == gm ? h - 1 : guide_le(marg, h, float(k) / float(1u << ENV_MGUIDE_BITS));
    } else {
      const uint32_t y = uint32_t((i - gm) / gc), k = uint32_t((i - gm) % gc);
      const float *c = cond + size_t(y) * (w + 1);
      cguide[i - gm] = k + 1 == gc ? w - 1 : guide_le(c, w, float(k) / float(1u << ENV_CGUIDE_BITS));
    }
  }
}

// ------------------------------------------------------------------- emitters

// Per triangle: 1 where its material may emit and its area is positive.
__global__ void __launch_bounds__(256) k_emissive_flags(const float4 *__restrict__ pos, const uint4 *__restrict__ vidx,
    const DevMaterial *__restrict__ mats, uint32_t tc, uint32_t *__restrict__ flag)
{
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < tc; t += gridDim.x * blockDim.x) {
    const uint4 v = vidx[t];
    uint32_t f = 0;
    if (tbl_may_emit(mats[v.w])) {
      const float4 a = pos[v.x], b = pos[v.y], c = pos[v.z];
      const float p0[3] = {a.x, a.y, a.z}, p1[3] = {b.x, b.y, b.z}, p2[3] = {c.x, c.y, c.z};
      f = tbl_tri_area(p0, p1, p2) > 0.f ? 1u : 0u;
    }
    flag[t] = f;
  }
}

// The flagged triangles' ids in triangle order: rank is the exclusive scan
// of the flags.
__global__ void __launch_bounds__(256) k_emissive_ids(const uint32_t *__restrict__ flag,
    const uint32_t *__restrict__ rank, uint32_t tc, uint32_t *__restrict__ ids)
{
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < tc; t += gridDim.x * blockDim.x)
    if (flag[t])
      ids[rank[t]] = t;
}

// Selection weight of each emitter (one thread per emitter).
__global__ void __launch_bounds__(256) k_emissive_weights(const float4 *__restrict__ pos,
    const uint4 *__restrict__ vidx, const DevMaterial *__restrict__ mats, const uint32_t *__restrict__ ids, uint32_t n,
    double *__restrict__ weight)
{
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint4 v = vidx[ids[i]];
    const float4 a = pos[v.x], b = pos[v.y], c = pos[v.z];
    const float p0[3] = {a.x, a.y, a.z}, p1[3] = {b.x, b.y, b.z}, p2[3] = {c.x, c.y, c.z};
    weight[i] = tbl_emit_weight(mats[v.w], tbl_tri_area(p0, p1, p2));
  }
}

// cdf[i] = prefix / total (the last entry 1) and the area density of each
// emitter's triangle; flags a CDF that is not non-decreasing.
__global__ void __launch_bounds__(256) k_emissive_cdf(const float4 *__restrict__ pos, const uint4 *__restrict__ vidx,
    const uint32_t *__restrict__ ids, uint32_t n, uint32_t tc, const double *__restrict__ weight,
    const double *__restrict__ prefix, double tw, float *__restrict__ cdf, float *__restrict__ pdf)
{
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    cdf[i] = i + 1 == n ? 1.f : float(prefix[i] / tw);
    const uint32_t t = ids[i];
    if (weight[i] > 0.0 && t < tc) {
      const uint4 v = vidx[t];
      const float4 a = pos[v.x], b = pos[v.y], c = pos[v.z];
      const float p0[3] = {a.x, a.y, a.z}, p1[3] = {b.x, b.y, b.z}, p2[3] = {c.x, c.y, c.z};
      pdf[t] = float(weight[i] / tw / double(tbl_tri_area(p0, p1, p2)));
    }
  }
}

// The emissive guide (2^EMISSIVE_GUIDE_BITS + 1 entries) and the check that
// the CDF is non-decreasing.
__global__ void __launch_bounds__(256) k_emissive_guide(const float *__restrict__ cdf, uint32_t n,
    uint32_t *__restrict__ guide, uint32_t *__restrict__ bad)
{
  const uint32_t G = 1u << EMISSIVE_GUIDE_BITS;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n + G + 1; i += gridDim.x * blockDim.x) {
    if (i <= G)
      guide[i] = i == G ? n - 1 : guide_gt(cdf, n, float(i) / float(G));
    else {
      const uint32_t j = i - G; // 1 .. n
      if (j < n && !(cdf[j - 1] <= cdf[j]))
        atomicOr(bad, 4u);
    }
  }
}

} // namespace

static unsigned grid_for(size_t n, unsigned block, unsigned per_sm)
{
  return unsigned(std::max<size_t>(1, std::min<size_t>((n + block - 1) / block, 152u * per_sm)));
}

std::string launch_env_tables(const EnvTablesJob &j, cudaStream_t s)
{
  const size_t n = size_t(j.w) * j.h;
  k_env_texels<<<grid_for(n, 256, 8), 256, 0, s>>>(j.rgb, n, j.pixels);
  k_env_rows<<<(j.h + 127) / 128, 128, 0, s>>>(j.pixels, j.w, j.h, j.row_sin, j.conditional, j.row_weight, j.bad);
  k_env_marginal<<<1, 1, 0, s>>>(j.row_weight, j.h, j.marginal, j.bad);
  const size_t g = (1u << ENV_MGUIDE_BITS) + 1 + size_t(j.h) * ((1u << ENV_CGUIDE_BITS) + 1);
  k_env_guides<<<grid_for(g, 256, 8), 256, 0, s>>>(j.marginal, j.conditional, j.w, j.h, j.mguide, j.cguide);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? std::string() : std::string("environment tables: ") + cudaGetErrorString(e);
}

std::string launch_emissive_ids(const EmissiveJob &j, cudaStream_t s)
{
  k_emissive_flags<<<grid_for(j.tc, 256, 8), 256, 0, s>>>(j.pos, j.vidx, j.mats, j.tc, j.flag);
  scan_u32(j.flag, j.rank, j.tc, j.count, j.scan_scratch, s);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? std::string() : std::string("emissive ids: ") + cudaGetErrorString(e);
}

std::string launch_emissive_weights(const EmissiveJob &j, cudaStream_t s)
{
  k_emissive_ids<<<grid_for(j.tc, 256, 8), 256, 0, s>>>(j.flag, j.rank, j.tc, j.ids);
  k_emissive_weights<<<grid_for(j.n, 256, 8), 256, 0, s>>>(j.pos, j.vidx, j.mats, j.ids, j.n, j.weight);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? std::string() : std::string("emissive weights: ") + cudaGetErrorString(e);
}

std::string launch_emissive_tables(const EmissiveJob &j, double total, cudaStream_t s)
{
  k_emissive_cdf<<<grid_for(j.n, 256, 8), 256, 0, s>>>(j.pos, j.vidx, j.ids, j.n, j.tc, j.weight, j.prefix, total,
      j.cdf, j.pdf);
  if (j.n > 1)
    k_emissive_guide<<<grid_for(j.n + (1u << EMISSIVE_GUIDE_BITS) + 1, 256, 8), 256, 0, s>>>(j.cdf, j.n, j.guide,
        j.bad);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? std::string() : std::string("emissive tables: ") + cudaGetErrorString(e);
}

std::string launch_pack_texels_u8(const float4 *src, size_t n, const float *dec, uchar4 *dst, uint32_t *bad,
    cudaStream_t stream)
{
  if (n == 0)
    return std::string();
  const unsigned blocks = unsigned(std::min<size_t>((n + 255) / 256, 152u * 8u));
  k_pack_texels_u8<<<blocks, 256, 0, stream>>>(src, n, dec, dst, bad);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? std::string() : std::string("texel packing: ") + cudaGetErrorString(e);
}

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
