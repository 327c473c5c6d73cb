// Level A of the C-ABI: the ray back-end (RayBackend::build_accel,
// trace_closest, trace_occluded; include/photon/pt/backend/ray_backend.h:44-54)
// on caller-owned device arrays.
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>

#include <cuda.h> // driver types only: cuCtxGetCurrent / cuCtxGetId are reached through the runtime

#include "../../include/photon_cuda.h"
#include "scene_build.h"
#include "traverse.cuh"
#include "tuning.h"

using namespace phc;

struct phc_accel {
  int device{0};
  int sm_count{0};
  cudaStream_t stream{nullptr};
  DeviceScene scene;
  uint64_t *counters{nullptr};
  uint64_t last_nodes{0}, last_tris{0};
  ~phc_accel()
  {
    if (counters)
      cudaFree(counters);
    if (stream)
      cudaStreamDestroy(stream);
  }
};

namespace {

thread_local std::string g_accel_error;

int fail(int code, const std::string &m)
{
  g_accel_error = m;
  return code;
}

constexpr uint32_t FULL = 0xffffffffu;

// One ray per thread; persistent warps take 32-ray batches.  INST: the
// accel holds instances (two-level traversal); full hit records then follow
// the reference's instanced back-end (photon_optix.cu:68-99, 161-187): the
// barycentrics as uv, the primitive's index within its object, the object's
// index as inst_id (the object count for the accel's own triangles).
template <int MODE, bool COUNT, bool INST = false> // MODE 0 full hit record, 1 compact, 2 occluded
__global__ void __launch_bounds__(128) k_level_a(DevScene sc, const float *__restrict__ orgs,
    const float *__restrict__ dirs, const float *__restrict__ tmins, const float *__restrict__ tmaxs, uint32_t n,
    void *out, uint32_t *fetch, unsigned long long *stats)
{
  TravCounters ctr{0u, 0u};
  for (;;) {
    uint32_t base = 0;
    if ((threadIdx.x & 31u) == 0)
      base = atomicAdd(fetch, 32u);
    base = __shfl_sync(FULL, base, 0);
    if (base >= n)
      break;
    const uint32_t i = base + (threadIdx.x & 31u);
    if (i >= n)
      continue;
    const size_t i3 = size_t(3) * i;
    const V3 o{orgs[i3], orgs[i3 + 1], orgs[i3 + 2]};
    const V3 d{dirs[i3], dirs[i3 + 1], dirs[i3 + 2]};
    const float t0 = tmins[i], t1 = tmaxs[i];
    uint32_t inst = INST_NONE;
    if (MODE == 2) {
      const RayHit h = INST ? trace_ray2<true, COUNT>(sc, o, d, t0, t1, &ctr, inst)
                            : trace_ray<true, COUNT>(sc, o, d, t0, t1, &ctr);
      static_cast<uint32_t *>(out)[i] = h.prim != 0xffffffffu ? 1u : 0u;
      continue;
    }
    const RayHit h = INST ? trace_ray2<false, COUNT>(sc, o, d, t0, t1, &ctr, inst)
                          : trace_ray<false, COUNT>(sc, o, d, t0, t1, &ctr);
    if (MODE == 1) {
      reinterpret_cast<float4 *>(out)[i] = make_float4(h.t, __uint_as_float(h.prim), h.u, h.v);
      continue;
    }
    // HitResult (ray_backend.h:15-29); like KokkosBackend only `hit` is written
    // for a miss, here the record is zeroed instead.
    float rec[22];
    for (int k = 0; k < 22; ++k)
      rec[k] = 0.f;
    uint32_t *urec = reinterpret_cast<uint32_t *>(rec);
    if (h.prim != 0xffffffffu) {
      const HitAttr a = hit_attributes(sc, o, d, h, inst);
      rec[0] = h.t;
      rec[1] = a.p.x;
      rec[2] = a.p.y;
      rec[3] = a.p.z;
      rec[4] = a.n.x;
      rec[5] = a.n.y;
      rec[6] = a.n.z;
      rec[7] = a.sn.x;
      rec[8] = a.sn.y;
      rec[9] = a.sn.z;
      rec[12] = h.u;
      rec[13] = h.v;
      urec[17] = h.prim;
      urec[20] = a.material_id;
      urec[21] = 1u; // hit = 1, has_interpolated_color = 0
      if (INST) {
        rec[10] = h.u; // no texture coordinates: uv = barycentrics
        rec[11] = h.v;
        if (inst != INST_NONE) {
          const uint4 info = __ldg(sc.inst_info + inst);
          urec[17] = h.prim - info.w;
          urec[19] = info.y;
        } else {
          urec[19] = sc.scene_object_id;
        }
      }
    }
    float *dst = static_cast<float *>(out) + size_t(i) * 22;
    for (int k = 0; k < 22; ++k)
      dst[k] = rec[k];
  }
  if (COUNT) {
    atomicAdd(&stats[0], (unsigned long long)ctr.nodes);
    atomicAdd(&stats[1], (unsigned long long)ctr.tris);
  }
}

template <int MODE>
int launch(phc_accel *a, const float *o, const float *d, const float *t0, const float *t1, uint32_t n, void *out,
    void *stream)
{
  if (!a)
    return fail(PHC_ERR_INVALID, "null accel");
  // the warps' 32-bit batch counter overshoots n by at most one batch per
  // warp of the grid, which stays far below 2^32 for n up to the limit
  if (n > PHC_TRACE_MAX_RAYS)
    return fail(PHC_ERR_LIMIT, "trace: n = " + std::to_string(n) + " rays exceeds the maximum of " +
        std::to_string(PHC_TRACE_MAX_RAYS) + " per call");
  if (n == 0)
    return PHC_OK;
  if (!o || !d || !t0 || !t1 || !out)
    return fail(PHC_ERR_INVALID, "null ray or output pointer");
  cudaError_t e = cudaSetDevice(a->device);
  if (e != cudaSuccess)
    return fail(PHC_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : a->stream;
  uint32_t *fetch = reinterpret_cast<uint32_t *>(a->counters + 2);
  e = cudaMemsetAsync(a->counters, 0, 4 * sizeof(uint64_t), s);
  if (e != cudaSuccess)
    return fail(PHC_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
  const int blocks = a->sm_count * 16;
  const bool count = tuning().count_traversal != 0;
  auto *st = reinterpret_cast<unsigned long long *>(a->counters);
  const bool inst = a->scene.dev.inst_count > 0;
  if (count && inst)
    k_level_a<MODE, true, true><<<blocks, 128, 0, s>>>(a->scene.dev, o, d, t0, t1, n, out, fetch, st);
  else if (count)
    k_level_a<MODE, true><<<blocks, 128, 0, s>>>(a->scene.dev, o, d, t0, t1, n, out, fetch, st);
  else if (inst)
    k_level_a<MODE, false, true><<<blocks, 128, 0, s>>>(a->scene.dev, o, d, t0, t1, n, out, fetch, st);
  else
    k_level_a<MODE, false><<<blocks, 128, 0, s>>>(a->scene.dev, o, d, t0, t1, n, out, fetch, st);
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(s);
  if (e != cudaSuccess)
    return fail(PHC_ERR_CUDA, std::string("trace: ") + cudaGetErrorString(e));
  uint64_t c[2] = {0, 0};
  if (count) {
    e = cudaMemcpy(c, a->counters, sizeof(c), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
      return fail(PHC_ERR_CUDA, std::string("trace counters: ") + cudaGetErrorString(e));
  }
  a->last_nodes = c[0];
  a->last_tris = c[1];
  return PHC_OK;
}

} // namespace

extern "C" {

int phc_accel_create(phc_accel **out, const float *positions, uint64_t vertex_count, const uint32_t *indices,
    uint64_t triangle_count, const float *normals, const uint32_t *material_ids)
{
  return phc_accel_create_instanced(out, positions, vertex_count, indices, triangle_count, normals, material_ids,
      nullptr, 0u, nullptr, 0u);
}

int phc_accel_create_instanced(phc_accel **out, const float *positions, uint64_t vertex_count,
    const uint32_t *indices, uint64_t triangle_count, const float *normals, const uint32_t *material_ids,
    const phc_object *objects, uint32_t object_count, const phc_instance *instances, uint32_t instance_count)
{
  static_assert(sizeof(phc_hit_result) == 88, "HitResult layout");
  if (!out)
    return fail(PHC_ERR_INVALID, "null output pointer");
  *out = nullptr;
  const bool instanced = object_count > 0 && instance_count > 0;
  if (instanced && (!objects || !instances))
    return fail(PHC_ERR_INVALID, "null objects or instances");
  if (!instanced && (!positions || !indices || vertex_count == 0 || triangle_count == 0))
    return fail(PHC_ERR_INVALID, "empty mesh");
  if ((vertex_count || triangle_count) && (!positions || !indices))
    return fail(PHC_ERR_INVALID, "null positions or indices");
  phc_accel *a = nullptr;
  try {
    a = new phc_accel();
    cudaGetDevice(&a->device);
    cudaDeviceGetAttribute(&a->sm_count, cudaDevAttrMultiProcessorCount, a->device);
    cudaError_t e = cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
      e = cudaMalloc(&a->counters, 4 * sizeof(uint64_t));
    if (e != cudaSuccess) {
      delete a;
      return fail(PHC_ERR_CUDA, std::string("accel: ") + cudaGetErrorString(e));
    }
    phc_scene_desc d{};
    d.positions = positions;
    d.vertex_count = vertex_count;
    d.indices = indices;
    d.triangle_count = triangle_count;
    d.normals = normals;
    d.material_ids = material_ids;
    d.material_id_count = material_ids ? triangle_count : 0;
    phc_pt_scene pt{};
    if (instanced) { // RayBackend::build_accel_instanced (optix_backend.cpp:659-722)
      pt.objects = objects;
      pt.object_count = object_count;
      pt.instances = instances;
      pt.instance_count = instance_count;
      d.pt = &pt;
    }
    HostScene hs;
    build_host_scene(d, hs);
    // Level A keeps the caller's material ids as given (no material table);
    // an object's triangles carry its material id (optix_backend.cpp:694-695)
    if (material_ids && triangle_count)
      for (uint64_t t = 0; t < triangle_count; ++t)
        hs.prim_vidx[4 * t + 3] = material_ids[t];
    for (size_t o = 0; o < hs.obj_prim_base.size(); ++o)
      for (uint32_t t = 0; t < hs.obj_prim_count[o]; ++t)
        hs.prim_vidx[4 * (size_t(hs.obj_prim_base[o]) + t) + 3] = objects[o].material_id;
    if (hs.bvh.max_depth >= 64) {
      delete a;
      return fail(PHC_ERR_LIMIT, "BVH deeper than the traversal stack (64 levels)");
    }
    const std::string err = a->scene.upload(hs, a->stream);
    if (!err.empty()) {
      delete a;
      return fail(PHC_ERR_CUDA, err);
    }
    if (a->scene.bvh_depth >= 64) {
      delete a;
      return fail(PHC_ERR_LIMIT, "BVH deeper than the traversal stack (64 levels)");
    }
  } catch (const std::bad_alloc &) {
    delete a;
    return fail(PHC_ERR_OOM, "host allocation failed");
  } catch (const std::exception &e) {
    delete a;
    return fail(PHC_ERR_INVALID, e.what());
  }
  *out = a;
  return PHC_OK;
}

void phc_accel_destroy(phc_accel *a) { delete a; }

int phc_trace_closest(phc_accel *a, const float *origins, const float *directions, const float *tmin,
    const float *tmax, uint32_t n, phc_hit_result *hits, void *stream)
{
  return launch<0>(a, origins, directions, tmin, tmax, n, hits, stream);
}

int phc_trace_closest_compact(phc_accel *a, const float *origins, const float *directions, const float *tmin,
    const float *tmax, uint32_t n, float *hits4, void *stream)
{
  return launch<1>(a, origins, directions, tmin, tmax, n, hits4, stream);
}

int phc_trace_occluded(phc_accel *a, const float *origins, const float *directions, const float *tmin,
    const float *tmax, uint32_t n, uint32_t *occluded, void *stream)
{
  return launch<2>(a, origins, directions, tmin, tmax, n, occluded, stream);
}

int phc_accel_counters(const phc_accel *a, uint64_t *node_visits, uint64_t *tri_tests)
{
  if (!a || !node_visits || !tri_tests)
    return fail(PHC_ERR_INVALID, "null argument");
  *node_visits = a->last_nodes;
  *tri_tests = a->last_tris;
  return PHC_OK;
}

int phc_accel_info(const phc_accel *a, uint64_t *node_bytes, uint64_t *tri_bytes, uint64_t *node_count)
{
  if (!a || !node_bytes || !tri_bytes || !node_count)
    return fail(PHC_ERR_INVALID, "null argument");
  *node_bytes = a->scene.node_bytes;
  *tri_bytes = a->scene.tri_bytes;
  *node_count = a->scene.dev.node_count;
  return PHC_OK;
}

const char *phc_accel_error(void) { return g_accel_error.c_str(); }

} // extern "C"

// ------------------------------------------- allocation-free closest-hit trace
//
// phc_trace_closest_compact_static runs the same traversal kernel as
// phc_trace_closest_compact, but the kernel's only scratch memory, the counter
// from which its persistent warps take 32-ray batches, lives in the
// file-scope array below instead of memory the accel allocated.  The array is
// part of the module image: every GPU that loads this library holds these
// 256 bytes until the process exits.  Host code must not use the array's name
// as a device address; it asks the runtime for the address once per device
// context (static_scratch).
#define PHC_STATIC_SCRATCH_WORDS 64
static __device__ __align__(256) uint32_t g_static_scratch[PHC_STATIC_SCRATCH_WORDS];

namespace {

// Identity of the CUDA context current on this thread: cuCtxGetId of
// cuCtxGetCurrent, both reached through the runtime's driver entry points
// (the library does not link the driver library itself).  Context ids are
// unique for the life of the process, so a context created after
// cudaDeviceReset, or a driver-API caller's own context, never matches an
// earlier one.  0 when the driver cannot say.
unsigned long long current_context_id()
{
  using GetCurrent = CUresult (*)(CUcontext *);
  using GetId = CUresult (*)(CUcontext, unsigned long long *);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
  });
  if (!get_current || !get_id)
    return 0;
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

// Device address of g_static_scratch in the context current on this thread
// (the caller has made the accel's device current).  The set-up looks it up
// with cudaGetSymbolAddress once per device context and caches it under the
// context's id; nullptr on failure, with err set.  Where the context has no
// id the address is looked up on every call.
uint32_t *static_scratch(std::string &err)
{
  struct Entry {
    unsigned long long ctx;
    uint32_t *ptr;
  };
  static std::mutex mu;
  static Entry cache[64] = {};
  static unsigned next = 0;
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(mu);
  if (ctx)
    for (const Entry &e : cache)
      if (e.ctx == ctx)
        return e.ptr;
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
  if (e != cudaSuccess) {
    err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
    return nullptr;
  }
  if (ctx) {
    cache[next] = Entry{ctx, static_cast<uint32_t *>(p)};
    next = (next + 1) % 64;
  }
  return static_cast<uint32_t *>(p);
}

} // namespace

extern "C" int phc_trace_closest_compact_static(phc_accel *a, const float *origins, const float *directions,
    const float *tmin, const float *tmax, uint32_t n, float *hits4, void *stream)
{
  if (!a)
    return fail(PHC_ERR_INVALID, "null accel");
  if (n > PHC_STATIC_MAX_RAYS)
    return fail(PHC_ERR_LIMIT, "phc_trace_closest_compact_static: n = " + std::to_string(n) +
        " rays exceeds the maximum of " + std::to_string(PHC_STATIC_MAX_RAYS) +
        " a call can take with its fixed scratch counter");
  if (n == 0)
    return PHC_OK;
  if (!origins || !directions || !tmin || !tmax || !hits4)
    return fail(PHC_ERR_INVALID, "null ray or output pointer");
  cudaError_t e = cudaSetDevice(a->device);
  if (e != cudaSuccess)
    return fail(PHC_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  std::string err;
  uint32_t *scratch = static_scratch(err);
  if (!scratch)
    return fail(PHC_ERR_CUDA, err);
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : a->stream;
  // the batch counter must start at zero; the array keeps the last call's value
  e = cudaMemsetAsync(scratch, 0, sizeof(uint32_t), s);
  if (e != cudaSuccess)
    return fail(PHC_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
  if (a->scene.dev.inst_count)
    k_level_a<1, false, true><<<a->sm_count * 16, 128, 0, s>>>(a->scene.dev, origins, directions, tmin, tmax, n,
        hits4, scratch, nullptr);
  else
    k_level_a<1, false><<<a->sm_count * 16, 128, 0, s>>>(a->scene.dev, origins, directions, tmin, tmax, n, hits4,
        scratch, nullptr);
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(s);
  if (e != cudaSuccess)
    return fail(PHC_ERR_CUDA, std::string("trace: ") + cudaGetErrorString(e));
  return PHC_OK;
}
