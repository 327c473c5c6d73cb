// libphoton_cuda.so: the renderer seam (Level B of include/photon_cuda.h).
//
// phc_renderer holds what photon::bridge::Renderer::Impl holds
// (src/photon/anari/RenderBridge.cpp:416-439): the device scene, the wavefront
// buffers of the path tracer, the accumulated frame and the sample counter
// that decorrelates successive render calls.  Calls run on the renderer's own
// CUDA stream and block until their device work is done.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <limits>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/photon_cuda.h"
#include "pt_math.cuh"
#include "scene_build.h"
#include "tuning.h"
#include "adjoint.h"
#include "wavefront.h"

using namespace phc;

namespace {

thread_local std::string g_error;

struct Buf {
  void *p{nullptr};
  size_t bytes{0};
  ~Buf() { release(); }
  void release()
  {
    if (p)
      cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  // (Re)allocates to at least n bytes; contents are not kept.
  cudaError_t ensure(size_t n)
  {
    if (n <= bytes && p)
      return cudaSuccess;
    release();
    const cudaError_t e = cudaMalloc(&p, n ? n : 16);
    if (e == cudaSuccess)
      bytes = n;
    else
      p = nullptr;
    return e;
  }
  template <class T> T *as() const { return static_cast<T *>(p); }
};

struct CudaError : std::runtime_error {
  cudaError_t code;
  CudaError(cudaError_t c, const char *what)
      : std::runtime_error(std::string(what) + ": " + cudaGetErrorString(c)), code(c)
  {
  }
};
inline void ck(cudaError_t e, const char *what)
{
  if (e != cudaSuccess)
    throw CudaError(e, what);
}
struct ApiError : std::runtime_error {
  int code;
  ApiError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

} // namespace

// The per-thread message of phc_global_error, for the other translation
// units of the C-ABI (the pbrt reader).
void phc::set_global_error(const std::string &msg) { g_error = msg; }

struct phc_renderer {
  int device{0};
  int sm_count{0};
  cudaStream_t stream{nullptr};
  std::string error;
  std::mutex mutex;

  DeviceScene scene;
  bool has_scene{false};
  bool atlas_textures{false}; // a material reads a pt-level atlas texture
  uint64_t scene_generation{0};

  // wavefront buffers
  size_t cap_paths{0};
  Buf st_o[2], st_d[2], st_tp[2], st_info[2], st_dist[2], hits, sh_a, sh_b, sh_c, hitq, missq, hitq_sorted;
  Buf vol_scatter, vol_rng, vol_q; // scenes with volumes: k_vol_scatter results per path, scattering queue
  size_t cap_vol{0};
  Buf hit_inst; // instance slot per hit (scenes with instances)
  Buf sort_bins; // per bounce iteration: material-sort counts and starts
  size_t cap_slots{0};
  Buf acc, acc_sq, acc_start, nsamp, aov_n, aov_a;
  Buf counters; // count, scount, fetch, wave, error
  Buf rc_buf, stats_buf, bg_buf;
  size_t bg_floats{0};
  // frame (RenderBridge.cpp:424-435)
  Buf f_color, f_normal, f_albedo, read_buf;
  uint32_t width{0}, height{0}, samples{0}, sample_counter{0};
  // graph of one wave
  cudaGraphExec_t graph{nullptr};
  uint64_t graph_key[8]{};
  // bumped whenever a buffer a recorded wave graph points to is reallocated
  uint64_t buf_gen{0};
  uint64_t graph_launches{0}; // kernels per replay of the wave graph
  // batched renders led by this renderer: job table, wave schedule, and the
  // job tags of the shadow queue
  Buf b_jobs, b_entries, b_wave_entry, b_wave_items, sh_job;
  // adjoint: constants, background, loss gradient, gradients, radiance
  Buf adj_rc, adj_bg, adj_dimg, adj_rad, adj_mat, adj_vol, adj_tex, adj_status, adj_pool;
  phc_render_stats last{};
  cudaEvent_t ev0{nullptr}, ev1{nullptr};

  ~phc_renderer()
  {
    if (graph)
      cudaGraphExecDestroy(graph);
    if (ev0)
      cudaEventDestroy(ev0);
    if (ev1)
      cudaEventDestroy(ev1);
    if (stream)
      cudaStreamDestroy(stream);
  }
};

namespace {

int set_error(phc_renderer *r, int code, const std::string &msg)
{
  if (r)
    r->error = msg;
  g_error = msg;
  return code;
}

template <class F> int guarded(phc_renderer *r, F &&f)
{
  try {
    f();
    if (r)
      r->error.clear();
    return PHC_OK;
  } catch (const ApiError &e) {
    return set_error(r, e.code, e.what());
  } catch (const CudaError &e) {
    return set_error(r, e.code == cudaErrorMemoryAllocation ? PHC_ERR_OOM : PHC_ERR_CUDA, e.what());
  } catch (const std::bad_alloc &) {
    return set_error(r, PHC_ERR_OOM, "host allocation failed");
  } catch (const std::length_error &e) {
    return set_error(r, PHC_ERR_LIMIT, e.what());
  } catch (const std::invalid_argument &e) {
    return set_error(r, PHC_ERR_INVALID, e.what());
  } catch (const std::out_of_range &e) {
    return set_error(r, PHC_ERR_INVALID, e.what());
  } catch (const std::exception &e) {
    return set_error(r, PHC_ERR_INVALID, e.what());
  }
}

inline V3 hv3(const float *p) { return V3{p[0], p[1], p[2]}; }
inline void put3(float *d, V3 v)
{
  d[0] = v.x;
  d[1] = v.y;
  d[2] = v.z;
}

// Camera of the render call: RenderBridge.cpp:872-891 with Camera::
// make_perspective / make_orthographic (include/photon/pt/camera.h:32-77), in
// float on the host with the reference's operation order.
void make_camera(const phc_camera &c, uint32_t w, uint32_t h, RenderConst &rc)
{
  const V3 position = hv3(c.position);
  V3 direction = normalize(hv3(c.direction));
  if (length(direction) == 0.f)
    direction = V3{0.f, 0.f, -1.f};
  V3 up = hv3(c.up);
  if (length(cross(direction, up)) < 1e-6f)
    up = std::fabs(direction.y) < 0.9f ? V3{0.f, 1.f, 0.f} : V3{1.f, 0.f, 0.f};
  const float aspect = c.aspect > 0.f ? c.aspect : float(w) / float(h);
  const V3 at = position + direction;
  V3 cw = normalize(position - at);
  V3 cu = normalize(cross(up, cw));
  V3 cv = cross(cw, cu);
  V3 horizontal, vertical, lower_left;
  float lens_radius = 0.f;
  if (c.orthographic) {
    horizontal = cu * (c.height * aspect);
    vertical = cv * c.height;
    lower_left = position - horizontal * 0.5f - vertical * 0.5f;
  } else {
    const float fovy_degrees = c.fovy * 180.f / 3.14159265358979f;
    const bool lens = c.aperture_radius > 0.f && c.focus_distance > 0.f;
    const float aperture = lens ? 2.f * c.aperture_radius : 0.f;
    const float focus = lens ? c.focus_distance : 1.f;
    const float theta = fovy_degrees * 3.1415926535f / 180.f;
    const float hh = std::tan(theta * 0.5f);
    const float vh = 2.f * hh;
    const float vw = aspect * vh;
    lens_radius = aperture * 0.5f;
    horizontal = cu * (vw * focus);
    vertical = cv * (vh * focus);
    lower_left = position - horizontal * 0.5f - vertical * 0.5f - cw * focus;
  }
  put3(rc.origin, position);
  put3(rc.lower_left, lower_left);
  put3(rc.horizontal, horizontal);
  put3(rc.vertical, vertical);
  put3(rc.cu, cu);
  put3(rc.cv, cv);
  put3(rc.cw, cw);
  rc.lens_radius = lens_radius;
  rc.ortho = c.orthographic ? 1 : 0;
  rc.clip_near = c.clip_near > 0.f ? c.clip_near : 0.f;
  rc.clip_far = c.clip_far < 1e30f ? c.clip_far : 1e30f;
  for (int i = 0; i < 4; ++i)
    rc.region[i] = c.image_region[i];
}

void check_device(phc_renderer *r) { ck(cudaSetDevice(r->device), "cudaSetDevice"); }

void ensure_path_state(phc_renderer *r, size_t n)
{
  r->buf_gen++;
  for (int b = 0; b < 2; ++b) {
    ck(r->st_o[b].ensure(n * 16), "alloc path state");
    ck(r->st_d[b].ensure(n * 16), "alloc path state");
    ck(r->st_tp[b].ensure(n * 16), "alloc path state");
    ck(r->st_info[b].ensure(n * 16), "alloc path state");
    ck(r->st_dist[b].ensure(n * 4), "alloc path state");
  }
  ck(r->hits.ensure(n * 16), "alloc hits");
  ck(r->hitq.ensure(n * 4), "alloc hit queue");
  ck(r->missq.ensure(n * 4), "alloc miss queue");
  ck(r->hitq_sorted.ensure(n * 4), "alloc sorted hit queue");
  ck(r->hit_inst.ensure(n * 4), "alloc hit instances");
  ck(r->sh_a.ensure(n * 16), "alloc shadow queue");
  ck(r->sh_b.ensure(n * 16), "alloc shadow queue");
  ck(r->sh_c.ensure(n * 16), "alloc shadow queue");
  r->cap_paths = n;
}

void ensure_paths(phc_renderer *r, size_t n)
{
  if (n > r->cap_paths)
    ensure_path_state(r, n);
  if (r->scene.dev.volume_count > 0 && r->cap_vol < r->cap_paths) {
    r->buf_gen++;
    ck(r->vol_scatter.ensure(r->cap_paths * 16), "alloc volume scattering");
    ck(r->vol_rng.ensure(r->cap_paths * 4), "alloc volume scattering");
    ck(r->vol_q.ensure(r->cap_paths * 4), "alloc volume scattering");
    r->cap_vol = r->cap_paths;
  }
}

void ensure_slots(phc_renderer *r, size_t n)
{
  if (n <= r->cap_slots)
    return;
  r->buf_gen++;
  ck(r->acc.ensure(n * 16), "alloc accumulators");
  ck(r->acc_sq.ensure(n * 16), "alloc accumulators");
  ck(r->acc_start.ensure(n * 16), "alloc accumulators");
  ck(r->nsamp.ensure(n * 4), "alloc accumulators");
  ck(r->aov_n.ensure(n * 16), "alloc accumulators");
  ck(r->aov_a.ensure(n * 16), "alloc accumulators");
  r->cap_slots = n;
}

// Counters, statistics and constants buffers of the wave kernels.
void ensure_wave_buffers(phc_renderer *r, int max_iter)
{
  const void *before[4] = {r->counters.p, r->stats_buf.p, r->rc_buf.p, r->sort_bins.p};
  ck(r->counters.ensure(wave_counter_alloc_bytes(max_iter)), "alloc counters");
  ck(r->stats_buf.ensure(8 * sizeof(uint64_t)), "alloc stats");
  ck(r->rc_buf.ensure(sizeof(RenderConst)), "alloc constants");
  ck(r->sort_bins.ensure(size_t(max_iter) * 2 * MAT_SORT_BINS * 4), "alloc sort bins");
  if (before[0] != r->counters.p || before[1] != r->stats_buf.p || before[2] != r->rc_buf.p ||
      before[3] != r->sort_bins.p)
    r->buf_gen++;
}

PathSoA path_soa(phc_renderer *r, int b)
{
  return PathSoA{r->st_o[b].as<float4>(), r->st_d[b].as<float4>(), r->st_tp[b].as<float4>(),
      r->st_info[b].as<uint4>(), r->st_dist[b].as<float>()};
}
Accum accum(phc_renderer *r)
{
  return Accum{r->acc.as<float4>(), r->acc_sq.as<float4>(), r->acc_start.as<float4>(), r->nsamp.as<uint32_t>(),
      r->aov_n.as<float4>(), r->aov_a.as<float4>()};
}
WaveCounters wave_counters(phc_renderer *r, int max_iter)
{
  uint32_t *c = r->counters.as<uint32_t>();
  WaveCounters wc;
  wc.count = c;
  wc.scount = c + (max_iter + 1);
  wc.hcount = c + (2 * max_iter + 1);
  wc.mcount = c + (3 * max_iter + 1);
  wc.fetch = c + (4 * max_iter + 1);
  wc.vfetch = c + (8 * max_iter + 1);
  wc.cfetch = c + (10 * max_iter + 1);
  wc.vcount = c + ((10 + SHADE_CLASSES) * max_iter + 1);
  wc.vqfetch = c + ((11 + SHADE_CLASSES) * max_iter + 1);
  wc.wave = c + wave_counter_words(max_iter);
  wc.error = c + wave_counter_words(max_iter) + 1;
  wc.dbg = c + wave_counter_words(max_iter) + 4;
  wc.trip_cap = uint32_t(tuning().wave_trip_cap);
  wc.vol_refill = uint32_t(tuning().vol_refill);
  wc.vol_passes = uint32_t(tuning().vol_passes);
  return wc;
}
// Bytes of the counters reset at the start of every wave (not wave / error).
size_t per_wave_counter_bytes(int max_iter) { return wave_counter_words(max_iter) * 4; }

// Per-kind kernel times of a render call (time_kernels mode): events around
// every launch of a wave, read after the wave.
struct KernelTimer {
  std::vector<cudaEvent_t> ev;
  std::vector<int> kind;
  size_t used{0};
  double ms[PHC_KERNEL_KINDS]{};
  uint64_t count[PHC_KERNEL_KINDS]{};
  ~KernelTimer()
  {
    for (cudaEvent_t e : ev)
      cudaEventDestroy(e);
  }
  void begin_wave() { used = 0; kind.clear(); }
  void mark(cudaStream_t s, int k)
  {
    if (used + 2 > ev.size()) {
      cudaEvent_t a, b;
      ck(cudaEventCreate(&a), "cudaEventCreate");
      ck(cudaEventCreate(&b), "cudaEventCreate");
      ev.push_back(a);
      ev.push_back(b);
    }
    kind.push_back(k);
    ck(cudaEventRecord(ev[used], s), "cudaEventRecord");
    used += 2;
  }
  void done(cudaStream_t s) { ck(cudaEventRecord(ev[used - 1], s), "cudaEventRecord"); }
  void end_wave(cudaStream_t s)
  {
    ck(cudaStreamSynchronize(s), "timed wave");
    for (size_t i = 0; i < kind.size(); ++i) {
      float t = 0.f;
      cudaEventElapsedTime(&t, ev[2 * i], ev[2 * i + 1]);
      ms[kind[i]] += t;
      count[kind[i]]++;
    }
  }
};

// One wave: counter reset, raygen, per iteration trace / shade / shadow, end.
// Returns the number of kernel launches.
// wave_paths: paths of one wave (lanes x pixels); the material sort and the
// class kernels are recorded only where an iteration can reach the sort
// threshold.
uint64_t record_wave(phc_renderer *r, cudaStream_t s, const LaunchCfg &cfg, const RenderConst *rc, uint32_t npix,
    size_t wave_paths, int max_iter, int adaptive, bool counting, KernelTimer *tm = nullptr)
{
  const WaveCounters wc = wave_counters(r, max_iter);
  ck(cudaMemsetAsync(wc.count, 0, per_wave_counter_bytes(max_iter), s), "reset counters");
  const DevScene sc = r->scene.dev;
  const Accum ac = accum(r);
  const ShadowSoA sh{r->sh_a.as<float4>(), r->sh_b.as<float4>(), r->sh_c.as<float4>()};
  uint64_t *stats = r->stats_buf.as<uint64_t>();
  auto timed = [&](int kind, auto &&launch) {
    if (tm)
      tm->mark(s, kind);
    launch();
    if (tm)
      tm->done(s);
  };
  // shading variants for this scene (shade_kernels.cu): the lean kernels
  // without volume / source / analytic-light code when the scene uses none,
  // misses and hits in separate kernels when no volume can scatter a miss
  const Tuning &tu = tuning();
  const bool full = (sc.features & (SCENE_VOLUMES | SCENE_SOURCES | SCENE_LIGHTS)) != 0 || !tu.shade_lean;
  const bool split = (sc.features & SCENE_VOLUMES) == 0 && tu.split_shade;
  HitQueues hq = split ? HitQueues{r->hitq.as<uint32_t>(), r->missq.as<uint32_t>()} : HitQueues{nullptr, nullptr};
  hq.inst = r->hit_inst.as<uint32_t>();
  // volume scenes: delta tracking in its own kernel ahead of the shading;
  // with split_volume a routing kernel then puts every path in the
  // scattering, hit or miss queue, each shaded by its own kernel
  const bool vol_pre = full && !split && sc.volume_count > 0 && r->cap_vol >= r->cap_paths && r->cap_vol > 0;
  const bool vsplit = vol_pre && tu.split_volume;
  if (vol_pre) {
    hq.vscatter = r->vol_scatter.as<float4>();
    hq.vrng = r->vol_rng.as<uint32_t>();
  }
  if (vsplit) {
    hq.hitq = r->hitq.as<uint32_t>();
    hq.missq = r->missq.as<uint32_t>();
    hq.vscatq = r->vol_q.as<uint32_t>();
  }
  // (volume scenes' hit queues stay unsorted: sorting them measured slower,
  // 238.6 against 239.9 Msamples/s on the 2M scene, and 238.6 when only the
  // bounces after the first are sorted, their shading 0.94 -> 1.02-1.04 s)
  // scenes whose materials all fall in one shading class run the same
  // shading code for every hit: sorting gains nothing there and the
  // shading's reads through the sorted order cost (box room 1503 against
  // 1813 Msamples/s)
  const bool sort = split && r->scene.shade_class_count > 1 && tu.sort_threshold > 0 &&
      wave_paths >= size_t(tu.sort_threshold);
  // lean scenes: the hit queue sorted by shading class, one kernel per class
  // (waves below class_threshold paths keep one lean hit kernel: the class
  // kernels' launches and tails cost more than they save on small waves)
  const bool classes = sort && !full && tu.shade_classes && wave_paths >= size_t(tu.class_threshold);
  const size_t bin_words = size_t(2) * MAT_SORT_BINS;
  if (sort) { // sort_bins sized by ensure_wave_buffers (no allocation while a graph is captured)
    hq.sorted = r->hitq_sorted.as<uint32_t>();
    hq.sort_threshold = uint32_t(tu.sort_threshold);
    hq.classes = classes ? 1u : 0u;
    ck(cudaMemsetAsync(r->sort_bins.p, 0, size_t(max_iter) * bin_words * 4, s), "reset sort bins");
  }
  uint64_t launches = 2;
  if (tm)
    tm->begin_wave();
  timed(0, [&] { launch_raygen(cfg, s, rc, sc, path_soa(r, 0), ac, wc); });
  for (int it = 0; it < max_iter; ++it) {
    const PathSoA in = path_soa(r, it & 1), out = path_soa(r, (it + 1) & 1);
    float4 *hits = r->hits.as<float4>();
    HitQueues hq_trace = hq;
    if (vsplit) // the tracking pre-pass writes the queues
      hq_trace.hitq = hq_trace.missq = nullptr;
    timed(1, [&] {
      launch_trace(cfg, s, sc, in, hits, wc, it, counting ? stats + 3 : nullptr, tu.trace_refill, hq_trace);
    });
    if (vsplit) {
      timed(5, [&] { launch_vol_scatter(cfg, s, rc, sc, in, hits, wc, it, hq, counting ? stats + 7 : nullptr); });
      timed(5, [&] { launch_vol_route(cfg, s, hits, wc, it, hq); });
      launches += 2;
    }
    if (sort) {
      timed(2, [&] {
        launch_material_sort(cfg, s, sc, hits, hq, wc, it, r->sort_bins.as<uint32_t>() + size_t(it) * bin_words);
      });
      launches += 3;
    }
    if (split) {
      HitQueues hqi = hq;
      if (classes) // the scatter leaves each bin's end in the upper half of the iteration's bins
        hqi.cls_end = r->sort_bins.as<uint32_t>() + size_t(it) * bin_words + MAT_SORT_BINS;
      timed(2, [&] { launch_shade(cfg, s, rc, sc, in, out, hits, sh, ac, wc, it, ShadeVariant{full, 1}, hqi); });
      if (classes) {
        for (uint32_t c = 1; c < SHADE_CLASSES; ++c)
          timed(2, [&] { launch_shade_class(cfg, s, rc, sc, in, out, hits, sh, ac, wc, it, c, hqi); });
        launches += SHADE_CLASSES - 1;
      }
      timed(2, [&] { launch_shade(cfg, s, rc, sc, in, out, hits, sh, ac, wc, it, ShadeVariant{full, 2}, hqi); });
      launches += 4;
    } else if (vsplit) {
      timed(2, [&] { launch_shade(cfg, s, rc, sc, in, out, hits, sh, ac, wc, it, ShadeVariant{full, 3}, hq); });
      timed(2, [&] { launch_shade(cfg, s, rc, sc, in, out, hits, sh, ac, wc, it, ShadeVariant{full, 1}, hq); });
      timed(2, [&] { launch_shade(cfg, s, rc, sc, in, out, hits, sh, ac, wc, it, ShadeVariant{full, 2}, hq); });
      launches += 3;
    } else {
      if (vol_pre) {
        timed(5, [&] { launch_vol_scatter(cfg, s, rc, sc, in, hits, wc, it, hq, counting ? stats + 7 : nullptr); });
        launches += 1;
      }
      timed(2, [&] { launch_shade(cfg, s, rc, sc, in, out, hits, sh, ac, wc, it, ShadeVariant{full, 0}, hq); });
      launches += 3;
    }
    timed(3, [&] { launch_shadow(cfg, s, rc, sc, sh, ac, wc, it, counting ? stats + 5 : nullptr, tu.trace_refill); });
    if (sc.volume_count > 0) {
      timed(6, [&] { launch_shadow_volume(cfg, s, rc, sc, sh, ac, wc, it, counting ? stats + 7 : nullptr); });
      launches += 1;
    }
  }
  timed(4, [&] { launch_wave_end(s, rc, ac, wc, npix, adaptive, max_iter, stats); });
  if (tm)
    tm->end_wave(s);
  return launches;
}

// The sticky error word of the wave kernels (WAVE_TRIP_CAP self-check) and
// the record of the failing warp.
void check_wave_error(uint32_t w, const WaveCounters &wc, cudaStream_t s)
{
  if (w == 0u)
    return;
  uint32_t d[WAVE_DBG_WORDS] = {};
  cudaMemcpyAsync(d, wc.dbg, sizeof(d), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  auto f = [&](int i) {
    float x;
    std::memcpy(&x, &d[i], 4);
    return std::to_string(x);
  };
  const uint32_t kind = w >> 16;
  if (kind == WAVE_ERR_VOLUME)
    throw ApiError(PHC_ERR_DEVICE, "a volume-tracking warp exceeded its loop-trip cap at bounce iteration " +
        std::to_string(w & 0xffffu));
  throw ApiError(PHC_ERR_DEVICE, std::string("a ") + (kind == WAVE_ERR_TRACE ? "closest-hit" : "shadow") +
          " traversal warp exceeded its loop-trip cap at bounce iteration " + std::to_string(w & 0xffffu) +
          " (queue " + std::to_string(d[0]) + ", fetched " + std::to_string(d[1]) + ", busy " +
          std::to_string(d[2]) + ", exhausted " + std::to_string(d[3]) + "; ray " + std::to_string(d[4]) + " o " +
          f(5) + " " + f(6) + " " + f(7) + " tmax " + f(8) + " d " + f(9) + " " + f(10) + " " + f(11) + " sp " +
          std::to_string(d[12]) + " base " + std::to_string(d[13]) + " hits " + std::to_string(d[14]) + " imask " +
          std::to_string(d[15]) + " steps " + std::to_string(d[16]) + " rays of the lane " + std::to_string(d[17]) + "; warp fetch trips " + std::to_string(d[18]) +
          " step trips " + std::to_string(d[19]) + " longest ray " + std::to_string(d[20]) + " steps (ray " +
          std::to_string(d[21]) + "); trips " + std::to_string(d[22]) + " active " + std::to_string(d[23]) + ")");
}

// What one render call of one renderer needs: its constants, sample lanes
// and wave count; prepared (buffers sized, accumulators zeroed) on stream s.
struct JobPlan {
  RenderConst rc{};
  uint32_t npix{0}, lanes{1}, waves{0};
  int max_iter{0};
  size_t slots{0};
  bool first{true};
};

void validate_call(phc_renderer *r, const phc_settings &st)
{
  if (st.width == 0 || st.height == 0)
    throw ApiError(PHC_ERR_INVALID, "invalid frame size");
  if (!r->has_scene)
    throw ApiError(PHC_ERR_NO_SCENE, "no scene");
  if (uint64_t(st.width) * st.height > (1ull << 28))
    throw ApiError(PHC_ERR_LIMIT, "frame larger than 2^28 pixels");
}

// The constants of one render call of a w x h frame (everything but the
// sample offset and lanes); a background image goes to `bg`.
RenderConst render_const(const phc_camera &cam, const phc_settings &st, Buf &bg, cudaStream_t s)
{
  const uint32_t w = st.width, h = st.height;
  const uint32_t npix = w * h;
  RenderConst rc{};
  make_camera(cam, w, h, rc);
  rc.w = w;
  rc.h = h;
  rc.npix = npix;
  rc.spp = std::max<uint32_t>(st.pixel_samples, 1);
  rc.max_depth = std::max<uint32_t>(st.max_depth, 1);
  rc.max_iter = rc.max_depth + 1u + 8u;
  std::memcpy(rc.bg, st.background, sizeof(rc.bg));
  // background image (RenderBridge.cpp:848-870)
  const size_t bg_n = size_t(st.background_width) * st.background_height * 4;
  if (st.background_image && bg_n > 0) {
    ck(bg.ensure(bg_n * 4), "alloc background");
    ck(cudaMemcpyAsync(bg.p, st.background_image, bg_n * 4, cudaMemcpyHostToDevice, s), "upload background");
    rc.bg_image = bg.as<float4>();
    rc.bg_w = st.background_width;
    rc.bg_h = st.background_height;
  }
  for (int i = 0; i < 3; ++i)
    rc.ambient[i] = st.ambient_color[i] * st.ambient_radiance;
  rc.adaptive = st.adaptive_sampling ? 1 : 0;
  rc.tp_clamp = st.throughput_clamp;
  rc.max_diffuse = st.max_diffuse_bounces;
  rc.max_glossy = st.max_glossy_bounces;
  rc.max_transmission = st.max_transmission_bounces;
  rc.max_volume = st.max_volume_bounces;
  rc.clamp_direct = 3.f * std::max(st.clamp_direct, 0.f);
  rc.clamp_indirect = 3.f * std::max(st.clamp_indirect, 0.f);
  return rc;
}

JobPlan prepare_job(phc_renderer *r, const phc_camera &cam, const phc_settings &st, bool reset, cudaStream_t s)
{
  validate_call(r, st);
  const uint32_t w = st.width, h = st.height;
  check_device(r);
  const uint32_t npix = w * h;
  if (w != r->width || h != r->height) {
    ck(r->f_color.ensure(size_t(npix) * 16), "alloc frame");
    ck(r->f_normal.ensure(size_t(npix) * 16), "alloc frame");
    ck(r->f_albedo.ensure(size_t(npix) * 16), "alloc frame");
    ck(r->read_buf.ensure(size_t(npix) * 16), "alloc frame");
    r->width = w;
    r->height = h;
    reset = true;
  }
  RenderConst rc = render_const(cam, st, r->bg_buf, s);
  rc.sample_offset = r->sample_counter;
  // samples of one pixel in flight: enough paths to fill the GPU, one when
  // adaptive sampling needs the samples in order
  const Tuning &tu = tuning();
  uint32_t lanes = 1;
  if (!rc.adaptive) {
    const uint64_t target = tu.wave_paths;
    lanes = uint32_t(std::min<uint64_t>(rc.spp, std::max<uint64_t>(1, (target + npix - 1) / npix)));
    lanes = std::min<uint32_t>(lanes, std::max<uint32_t>(1u, uint32_t((1ull << 28) / npix)));
  }
  rc.lanes = lanes;
  JobPlan p;
  p.npix = npix;
  p.lanes = lanes;
  p.max_iter = int(rc.max_iter);
  p.slots = size_t(lanes) * npix;
  p.waves = (rc.spp + lanes - 1) / lanes;
  p.first = reset || r->samples == 0;
  ensure_slots(r, p.slots);
  ensure_wave_buffers(r, p.max_iter);
  ck(cudaMemcpyAsync(r->rc_buf.p, &rc, sizeof(rc), cudaMemcpyHostToDevice, s), "upload constants");
  ck(cudaMemsetAsync(r->acc.p, 0, p.slots * 16, s), "reset accumulators");
  ck(cudaMemsetAsync(r->nsamp.p, 0, p.slots * 4, s), "reset accumulators");
  ck(cudaMemsetAsync(r->aov_a.p, 0, p.slots * 16, s), "reset accumulators");
  if (rc.adaptive)
    ck(cudaMemsetAsync(r->acc_sq.p, 0, p.slots * 16, s), "reset accumulators");
  p.rc = rc;
  return p;
}

Frame frame_of(phc_renderer *r)
{
  return Frame{r->f_color.as<float4>(), r->f_normal.as<float4>(), r->f_albedo.as<float4>()};
}

// After the device work: the bridge's sample bookkeeping (RenderBridge.cpp:920-927).
void commit_job(phc_renderer *r, const JobPlan &p)
{
  r->sample_counter += p.rc.spp;
  r->samples = p.first ? p.rc.spp : r->samples + p.rc.spp;
}

LaunchCfg launch_cfg(phc_renderer *r, size_t raygen_items)
{
  const Tuning &tu = tuning();
  LaunchCfg cfg;
  cfg.threads = 128;
  cfg.blocks_trace = r->sm_count * std::max(1, std::min(tu.trace_blocks_per_sm, max_active_blocks(0, 128)));
  cfg.blocks_shade = r->sm_count * std::max(1, std::min(tu.shade_blocks_per_sm, max_active_blocks(1, 128)));
  cfg.blocks_shade_lean = r->sm_count * std::max(1, std::min(tu.shade_blocks_per_sm, max_active_blocks(4, 128)));
  cfg.blocks_raygen = int(std::max<size_t>(1, std::min<size_t>((raygen_items + 255) / 256, size_t(r->sm_count) * 8)));
  return cfg;
}

void render_impl(phc_renderer *r, const phc_camera &cam, const phc_settings &st, bool reset)
{
  cudaStream_t s = r->stream;
  const JobPlan plan = prepare_job(r, cam, st, reset, s);
  const RenderConst &rc = plan.rc;
  const uint32_t npix = plan.npix, lanes = plan.lanes, waves = plan.waves;
  const int max_iter = plan.max_iter;
  const bool first = plan.first;
  const Tuning &tu = tuning();
  ensure_paths(r, plan.slots);
  ensure_wave_buffers(r, max_iter);
  ck(cudaMemsetAsync(r->stats_buf.p, 0, 8 * sizeof(uint64_t), s), "reset stats");
  const WaveCounters wc = wave_counters(r, max_iter);
  ck(cudaMemsetAsync(wc.wave, 0, 8, s), "reset wave");
  ck(cudaMemsetAsync(wc.dbg, 0, WAVE_DBG_WORDS * 4, s), "reset wave");
  const LaunchCfg cfg = launch_cfg(r, plan.slots);
  const bool counting = tu.count_traversal != 0;
  const RenderConst *drc = r->rc_buf.as<RenderConst>();

  ck(cudaEventRecord(r->ev0, s), "event");
  // everything the recorded launch sequence depends on
  const uint64_t key[8] = {uint64_t(npix) | (uint64_t(lanes) << 32),
      uint64_t(max_iter) | (uint64_t(rc.adaptive) << 32), r->scene_generation,
      uint64_t(counting) | (uint64_t(cfg.blocks_trace) << 8) | (uint64_t(cfg.blocks_shade) << 32),
      uint64_t(tu.trace_refill) | (uint64_t(tu.split_shade) << 8) | (uint64_t(tu.shade_lean) << 16) |
          (uint64_t(tu.shade_classes) << 23) | (uint64_t(tu.sort_threshold) << 24),
      r->buf_gen, uint64_t(tu.wave_trip_cap) | (uint64_t(tu.vol_refill) << 32) | (uint64_t(tu.vol_passes) << 40) |
          (uint64_t(tu.split_volume) << 60),
      uint64_t(tu.class_threshold)};
  uint64_t launches = 0;
  KernelTimer timer;
  if (tu.time_kernels) {
    for (uint32_t wv = 0; wv < waves; ++wv)
      launches += record_wave(r, s, cfg, drc, npix, plan.slots, max_iter, rc.adaptive, counting, &timer);
  } else if (tu.use_graph) {
    if (!r->graph || std::memcmp(key, r->graph_key, sizeof(key)) != 0) {
      if (r->graph) {
        cudaGraphExecDestroy(r->graph);
        r->graph = nullptr;
      }
      cudaGraph_t g = nullptr;
      ck(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
      try {
        r->graph_launches = record_wave(r, s, cfg, drc, npix, plan.slots, max_iter, rc.adaptive, counting);
      } catch (...) {
        cudaStreamEndCapture(s, &g);
        if (g)
          cudaGraphDestroy(g);
        cudaGetLastError(); // the failed capture's error is reported once, not left for later calls
        throw;
      }
      ck(cudaStreamEndCapture(s, &g), "end capture");
      const cudaError_t e = cudaGraphInstantiate(&r->graph, g, 0);
      cudaGraphDestroy(g);
      ck(e, "graph instantiate");
      std::memcpy(r->graph_key, key, sizeof(key));
    }
    for (uint32_t wv = 0; wv < waves; ++wv)
      ck(cudaGraphLaunch(r->graph, s), "graph launch");
    launches = uint64_t(waves) * r->graph_launches;
  } else {
    for (uint32_t wv = 0; wv < waves; ++wv)
      launches += record_wave(r, s, cfg, drc, npix, plan.slots, max_iter, rc.adaptive, counting);
  }
  const Frame fr = frame_of(r);
  if (tu.time_kernels)
    timer.mark(s, 4);
  launch_resolve(s, accum(r), fr, npix, lanes, float(rc.spp), first ? 1 : 0);
  if (tu.time_kernels) {
    timer.done(s);
    ck(cudaStreamSynchronize(s), "resolve");
    float t = 0.f;
    cudaEventElapsedTime(&t, timer.ev[timer.used - 2], timer.ev[timer.used - 1]);
    timer.ms[4] += t;
    timer.count[4]++;
  }
  launches += 1;
  ck(cudaGetLastError(), "kernel launch");
  ck(cudaEventRecord(r->ev1, s), "event");
  uint64_t stats[8];
  uint32_t err_word = 0;
  ck(cudaMemcpyAsync(stats, r->stats_buf.p, sizeof(stats), cudaMemcpyDeviceToHost, s), "read stats");
  ck(cudaMemcpyAsync(&err_word, wc.error, 4, cudaMemcpyDeviceToHost, s), "read error word");
  ck(cudaStreamSynchronize(s), "render");
  check_wave_error(err_word, wc, s);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, r->ev0, r->ev1);
  r->last.pixel_samples = stats[0];
  r->last.closest_rays = stats[1];
  r->last.shadow_rays = stats[2];
  r->last.node_visits = stats[3];
  r->last.tri_tests = stats[4];
  r->last.render_ms = ms;
  r->last.shadow_node_visits = stats[5];
  r->last.shadow_tri_tests = stats[6];
  r->last.kernel_launches = launches;
  r->last.volume_lookups = stats[7];
  for (int k = 0; k < PHC_KERNEL_KINDS; ++k) {
    r->last.kernel_ms[k] = timer.ms[k];
    r->last.kernel_count[k] = timer.count[k];
  }
  commit_job(r, plan);
}

// ---------------------------------------------------------------- batches
//
// Several renderers' render calls in one wavefront: every job keeps the
// sample lanes its own render would use (so its per-pixel sums and its image
// are bit-identical), and a batch wave packs at most one "chunk" (one plain
// wave: lanes samples of every pixel) per job, round-robin, until the wave
// holds batch_wave_paths paths.  One CUDA graph of one batch wave is
// replayed for all waves; the wave index selects the wave's table.
struct BatchPlan {
  std::vector<BatchJob> jobs;
  std::vector<BatchEntry> entries;
  std::vector<uint32_t> wave_entry, wave_items;
  uint32_t max_items{0};
  int max_iter{0};
  uint32_t features{0};
};

BatchPlan plan_batch(const std::vector<phc_renderer *> &rs, const std::vector<JobPlan> &plans, uint64_t cap)
{
  BatchPlan b;
  const size_t n = rs.size();
  std::vector<uint32_t> next(n, 0);
  for (size_t j = 0; j < n; ++j) {
    b.jobs.push_back(BatchJob{rs[j]->scene.dev, plans[j].rc, accum(rs[j])});
    b.max_iter = std::max(b.max_iter, plans[j].max_iter);
    b.features |= rs[j]->scene.dev.features;
  }
  size_t start = 0;
  b.wave_entry.push_back(0);
  for (;;) {
    uint64_t items = 0;
    bool any = false;
    for (size_t k = 0; k < n; ++k) {
      const size_t j = (start + k) % n;
      const JobPlan &p = plans[j];
      if (next[j] >= p.waves)
        continue;
      const uint32_t s0 = next[j] * p.lanes;
      const uint32_t ns = std::min(p.lanes, p.rc.spp - s0);
      const uint64_t paths = uint64_t(ns) * p.npix;
      if (items > 0 && items + paths > cap)
        continue;
      b.entries.push_back(BatchEntry{uint32_t(j), s0, ns, uint32_t(items)});
      items += paths;
      next[j]++;
      any = true;
    }
    if (!any)
      break;
    if (items > 0xffffffffull)
      throw ApiError(PHC_ERR_LIMIT, "batch wave larger than 2^32 paths");
    b.wave_entry.push_back(uint32_t(b.entries.size()));
    b.wave_items.push_back(uint32_t(items));
    b.max_items = std::max(b.max_items, uint32_t(items));
    start = (start + 1) % n;
  }
  return b;
}

void record_batch_wave(phc_renderer *lead, cudaStream_t s, const LaunchCfg &cfg, const BatchTable &bt, int max_iter,
    uint32_t features, uint32_t max_items)
{
  const Tuning &tu = tuning();
  const WaveCounters wc = wave_counters(lead, max_iter);
  ck(cudaMemsetAsync(wc.count, 0, per_wave_counter_bytes(max_iter), s), "reset counters");
  const ShadowSoA sh{lead->sh_a.as<float4>(), lead->sh_b.as<float4>(), lead->sh_c.as<float4>(),
      lead->sh_job.as<uint32_t>()};
  const bool full = (features & (SCENE_VOLUMES | SCENE_SOURCES | SCENE_LIGHTS)) != 0 || !tu.shade_lean;
  const bool split = (features & SCENE_VOLUMES) == 0 && tu.split_shade;
  HitQueues hq =
      split ? HitQueues{lead->hitq.as<uint32_t>(), lead->missq.as<uint32_t>()} : HitQueues{nullptr, nullptr};
  const bool sort = split && tu.sort_threshold > 0;
  // lean batches: the hit queue sorted by shading class, one kernel per class
  const bool classes = sort && !full && tu.shade_classes && max_items >= uint64_t(tu.class_threshold);
  const size_t bin_words = size_t(2) * MAT_SORT_BINS;
  if (sort) { // sort_bins sized by ensure_wave_buffers
    hq.sorted = lead->hitq_sorted.as<uint32_t>();
    hq.sort_threshold = uint32_t(tu.sort_threshold);
    hq.classes = classes ? 1u : 0u;
    ck(cudaMemsetAsync(lead->sort_bins.p, 0, size_t(max_iter) * bin_words * 4, s), "reset sort bins");
  }
  float4 *hits = lead->hits.as<float4>();
  launch_raygen_batch(cfg, s, bt, path_soa(lead, 0), wc);
  for (int it = 0; it < max_iter; ++it) {
    const PathSoA in = path_soa(lead, it & 1), out = path_soa(lead, (it + 1) & 1);
    launch_trace_batch(cfg, s, bt, in, hits, wc, it, tu.trace_refill, hq);
    if (sort)
      launch_material_sort_batch(cfg, s, bt, in.info, hits, hq, wc, it,
          lead->sort_bins.as<uint32_t>() + size_t(it) * bin_words);
    if (split) {
      HitQueues hqi = hq;
      if (classes) // the scatter leaves each bin's end in the upper half of the iteration's bins
        hqi.cls_end = lead->sort_bins.as<uint32_t>() + size_t(it) * bin_words + MAT_SORT_BINS;
      launch_shade_batch(cfg, s, bt, in, out, hits, sh, wc, it, ShadeVariant{full, 1}, hqi);
      if (classes)
        for (uint32_t c = 1; c < SHADE_CLASSES; ++c)
          launch_shade_class_batch(cfg, s, bt, in, out, hits, sh, wc, it, c, hqi);
      launch_shade_batch(cfg, s, bt, in, out, hits, sh, wc, it, ShadeVariant{full, 2}, hqi);
    } else {
      launch_shade_batch(cfg, s, bt, in, out, hits, sh, wc, it, ShadeVariant{full, 0}, hq);
    }
    launch_shadow_batch(cfg, s, bt, sh, wc, it, tu.trace_refill, (features & SCENE_VOLUMES) != 0);
  }
  launch_wave_end(s, nullptr, Accum{}, wc, 0, 0, max_iter, lead->stats_buf.as<uint64_t>());
}

template <class T> void upload_vec(Buf &b, const std::vector<T> &v, cudaStream_t s, const char *what)
{
  ck(b.ensure(std::max<size_t>(v.size(), 1) * sizeof(T)), what);
  if (!v.empty())
    ck(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s), what);
}

void render_batch_impl(const phc_job *jobs, uint32_t n, phc_render_stats *out_stats)
{
  std::vector<phc_renderer *> rs;
  std::vector<JobPlan> plans;
  std::vector<const phc_job *> batch_jobs;
  phc_renderer *lead = jobs[0].renderer;
  int device = lead->device;
  for (uint32_t i = 0; i < n; ++i) {
    const phc_job &jb = jobs[i];
    if (!jb.renderer || !jb.camera || !jb.settings)
      throw ApiError(PHC_ERR_INVALID, "batch job " + std::to_string(i) + ": null renderer, camera or settings");
    if (jb.renderer->device != device)
      throw ApiError(PHC_ERR_INVALID, "batch jobs must share one device");
    for (uint32_t k = 0; k < i; ++k)
      if (jobs[k].renderer == jb.renderer)
        throw ApiError(PHC_ERR_INVALID, "a renderer appears twice in the batch");
    validate_call(jb.renderer, *jb.settings);
  }
  if (n > MAX_BATCH_JOBS)
    throw ApiError(PHC_ERR_LIMIT, "more than 32768 jobs in one batch");
  check_device(lead);
  cudaStream_t s = lead->stream;
  // adaptive sampling needs the samples of a pixel in order, and the batched
  // kernels trace single-level scenes: such jobs run through their own
  // render path first
  for (uint32_t i = 0; i < n; ++i) {
    if (jobs[i].settings->adaptive_sampling || (jobs[i].renderer->has_scene && jobs[i].renderer->scene.dev.inst_count)) {
      render_impl(jobs[i].renderer, *jobs[i].camera, *jobs[i].settings, jobs[i].reset != 0);
      continue;
    }
    batch_jobs.push_back(&jobs[i]);
  }
  if (batch_jobs.empty())
    return;
  for (const phc_job *jb : batch_jobs) {
    rs.push_back(jb->renderer);
    plans.push_back(prepare_job(jb->renderer, *jb->camera, *jb->settings, jb->reset != 0, s));
  }
  const Tuning &tu = tuning();
  const BatchPlan bp = plan_batch(rs, plans, uint64_t(std::max<int64_t>(tu.batch_wave_paths, 1024)));
  upload_vec(lead->b_jobs, bp.jobs, s, "upload batch jobs");
  upload_vec(lead->b_entries, bp.entries, s, "upload batch entries");
  upload_vec(lead->b_wave_entry, bp.wave_entry, s, "upload batch waves");
  upload_vec(lead->b_wave_items, bp.wave_items, s, "upload batch waves");
  ensure_paths(lead, bp.max_items);
  ensure_wave_buffers(lead, bp.max_iter);
  ck(lead->sh_job.ensure(size_t(std::max<uint32_t>(bp.max_items, 1)) * 4), "alloc shadow jobs");
  ck(cudaMemsetAsync(lead->stats_buf.p, 0, 8 * sizeof(uint64_t), s), "reset stats");
  const WaveCounters wc = wave_counters(lead, bp.max_iter);
  ck(cudaMemsetAsync(wc.wave, 0, 8, s), "reset wave");
  ck(cudaMemsetAsync(wc.dbg, 0, WAVE_DBG_WORDS * 4, s), "reset wave");
  const BatchTable bt{lead->b_jobs.as<BatchJob>(), lead->b_entries.as<BatchEntry>(),
      lead->b_wave_entry.as<uint32_t>(), lead->b_wave_items.as<uint32_t>()};
  const LaunchCfg cfg = launch_cfg(lead, bp.max_items);
  const uint32_t waves = uint32_t(bp.wave_items.size());
  ck(cudaEventRecord(lead->ev0, s), "event");
  uint64_t launches = 0;
  if (tu.use_graph) {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    ck(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
    try {
      record_batch_wave(lead, s, cfg, bt, bp.max_iter, bp.features, bp.max_items);
    } catch (...) {
      cudaStreamEndCapture(s, &g);
      if (g)
        cudaGraphDestroy(g);
      cudaGetLastError();
      throw;
    }
    ck(cudaStreamEndCapture(s, &g), "end capture");
    size_t nodes = 0;
    cudaGraphGetNodes(g, nullptr, &nodes);
    const cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    ck(e, "graph instantiate");
    for (uint32_t wv = 0; wv < waves; ++wv) {
      const cudaError_t le = cudaGraphLaunch(ge, s);
      if (le != cudaSuccess) {
        cudaGraphExecDestroy(ge);
        ck(le, "graph launch");
      }
    }
    launches = uint64_t(waves) * (nodes > 0 ? nodes - 1 : 0); // minus the counter memset node
    ck(cudaStreamSynchronize(s), "batch");
    cudaGraphExecDestroy(ge);
  } else {
    for (uint32_t wv = 0; wv < waves; ++wv)
      record_batch_wave(lead, s, cfg, bt, bp.max_iter, bp.features, bp.max_items);
  }
  for (size_t j = 0; j < rs.size(); ++j)
    launch_resolve(s, accum(rs[j]), frame_of(rs[j]), plans[j].npix, plans[j].lanes, float(plans[j].rc.spp),
        plans[j].first ? 1 : 0);
  launches += rs.size();
  ck(cudaGetLastError(), "kernel launch");
  ck(cudaEventRecord(lead->ev1, s), "event");
  uint64_t stats[8];
  uint32_t err_word = 0;
  ck(cudaMemcpyAsync(stats, lead->stats_buf.p, sizeof(stats), cudaMemcpyDeviceToHost, s), "read stats");
  ck(cudaMemcpyAsync(&err_word, wc.error, 4, cudaMemcpyDeviceToHost, s), "read error word");
  ck(cudaStreamSynchronize(s), "batch");
  check_wave_error(err_word, wc, s);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, lead->ev0, lead->ev1);
  phc_render_stats st{};
  st.pixel_samples = stats[0];
  st.closest_rays = stats[1];
  st.shadow_rays = stats[2];
  st.render_ms = ms;
  st.kernel_launches = launches;
  for (size_t j = 0; j < rs.size(); ++j) {
    commit_job(rs[j], plans[j]);
    rs[j]->last = phc_render_stats{};
    rs[j]->last.pixel_samples = uint64_t(plans[j].npix) * plans[j].rc.spp;
    rs[j]->last.render_ms = ms;
  }
  lead->last = st;
  if (out_stats)
    *out_stats = st;
}

// ---------------------------------------------------------------- adjoint
// The adjoint's per-slot state beside the wavefront buffers: two path queues'
// extra fields (remainder, previous sample's pdf derivative and vertex), the
// shadow queue's extra fields and the collected radiance, carved from one
// allocation.
struct AdjQueues {
  AdjPathSoA path[2];
  AdjShadowSoA shadow;
  float4 *collected;
};
AdjQueues adj_queues(phc_renderer *r, size_t slots)
{
  const size_t f4 = slots * 16;
  const size_t per_path = 6 * f4, per_shadow = 5 * f4 + slots * 4 + 256;
  ck(r->adj_pool.ensure(2 * per_path + per_shadow + f4 + 1024), "alloc adjoint queues");
  char *p = r->adj_pool.as<char>();
  auto take = [&](size_t bytes) {
    char *q = p;
    p += (bytes + 255) & ~size_t(255);
    return q;
  };
  AdjQueues a;
  for (int b = 0; b < 2; ++b) {
    AdjPathSoA &s = a.path[b];
    s.p = path_soa(r, b);
    s.rem = reinterpret_cast<float4 *>(take(f4));
    s.g0 = reinterpret_cast<float4 *>(take(f4));
    s.g1 = reinterpret_cast<float4 *>(take(f4));
    s.v.q = reinterpret_cast<uint4 *>(take(f4));
    s.v.p = reinterpret_cast<float4 *>(take(f4));
    s.v.sn = reinterpret_cast<float4 *>(take(f4));
  }
  AdjShadowSoA &h = a.shadow;
  h.s = ShadowSoA{r->sh_a.as<float4>(), r->sh_b.as<float4>(), r->sh_c.as<float4>(), nullptr};
  h.next = reinterpret_cast<uint32_t *>(take(slots * 4));
  h.g0 = reinterpret_cast<float4 *>(take(f4));
  h.g1 = reinterpret_cast<float4 *>(take(f4));
  h.v.q = reinterpret_cast<uint4 *>(take(f4));
  h.v.p = reinterpret_cast<float4 *>(take(f4));
  h.v.sn = reinterpret_cast<float4 *>(take(f4));
  a.collected = reinterpret_cast<float4 *>(take(f4));
  return a;
}

void adjoint_impl(phc_renderer *r, const phc_camera &cam, const phc_settings &st, uint32_t sample_offset,
    const float *d_color, phc_adjoint_grads &g)
{
  validate_call(r, st);
  if (st.adaptive_sampling)
    throw ApiError(PHC_ERR_INVALID, "the adjoint takes every sample: adaptive sampling must be off");
  if (!g.materials)
    throw ApiError(PHC_ERR_INVALID, "null material gradient buffer");
  if (r->atlas_textures)
    throw ApiError(PHC_ERR_INVALID, "the adjoint does not differentiate atlas (pt-level) textures");
  if (r->scene.dev.inst_count)
    throw ApiError(PHC_ERR_INVALID, "the adjoint does not trace instanced geometry");
  const DevScene &sc = r->scene.dev;
  if (g.volumes && sc.volume_count > uint32_t(PHC_ADJ_MAX_VOLUMES))
    throw ApiError(PHC_ERR_LIMIT, "volume gradients for more than PHC_ADJ_MAX_VOLUMES volumes");
  check_device(r);
  cudaStream_t s = r->stream;
  const RenderConst base = render_const(cam, st, r->adj_bg, s);
  const uint32_t npix = base.npix, spp = base.spp;
  const int max_iter = int(base.max_iter);
  // both passes run over chunks of `chunk` samples, one sample per
  // accumulator slot (slot = sample-in-chunk * npix + pixel)
  const Tuning &tu = tuning();
  const uint64_t per_chunk = std::max<uint64_t>(uint64_t(tu.wave_paths), npix);
  const uint32_t chunk = uint32_t(std::min<uint64_t>(spp, std::max<uint64_t>(1, per_chunk / npix)));
  const size_t slots = size_t(chunk) * npix;
  ensure_slots(r, slots);
  ensure_paths(r, slots);
  ensure_wave_buffers(r, max_iter);
  const AdjQueues q = adj_queues(r, slots);
  const size_t nmat = size_t(sc.material_count) * ADJ_MATERIAL_PARAMS;
  const size_t nvol = size_t(std::min<uint32_t>(sc.volume_count, ADJ_MAX_VOLUMES)) * ADJ_VOLUME_PARAMS;
  const size_t ntex = g.texels ? size_t(r->scene.texel_count) : 0;
  ck(r->adj_rc.ensure(sizeof(RenderConst)), "alloc constants");
  ck(r->adj_dimg.ensure(size_t(npix) * 16), "alloc adjoint");
  ck(r->adj_rad.ensure(size_t(npix) * 12), "alloc adjoint");
  ck(r->adj_mat.ensure(nmat * 4), "alloc adjoint");
  ck(r->adj_vol.ensure(std::max<size_t>(nvol, 1) * 4), "alloc adjoint");
  if (ntex)
    ck(r->adj_tex.ensure(ntex * 16), "alloc adjoint");
  ck(r->adj_status.ensure(32), "alloc adjoint");
  ck(cudaEventRecord(r->ev0, s), "event");
  ck(cudaMemsetAsync(r->adj_status.p, 0, 32, s), "clear adjoint");
  ck(cudaMemcpyAsync(r->adj_dimg.p, d_color, size_t(npix) * 16, cudaMemcpyHostToDevice, s), "upload loss gradient");
  ck(cudaMemsetAsync(r->adj_rad.p, 0, size_t(npix) * 12, s), "clear adjoint");
  ck(cudaMemsetAsync(r->adj_mat.p, 0, nmat * 4, s), "clear adjoint");
  ck(cudaMemsetAsync(r->adj_vol.p, 0, std::max<size_t>(nvol, 1) * 4, s), "clear adjoint");
  if (ntex)
    ck(cudaMemsetAsync(r->adj_tex.p, 0, ntex * 16, s), "clear adjoint");
  const WaveCounters wc = wave_counters(r, max_iter);
  const LaunchCfg cfg = launch_cfg(r, slots);
  LaunchCfg acfg = cfg;
  acfg.blocks_shade = r->sm_count * adj_shade_max_active_blocks(128);
  const RenderConst *drc = r->adj_rc.as<RenderConst>();
  AdjointArgs a{};
  a.primal = r->acc.as<float4>();
  a.d_image = r->adj_dimg.as<float4>();
  a.collected = q.collected;
  a.radiance = g.color ? r->adj_rad.as<float>() : nullptr;
  a.mat_grads = r->adj_mat.as<float>();
  a.vol_grads = r->adj_vol.as<float>();
  a.texel_grads = ntex ? r->adj_tex.as<float4>() : nullptr;
  a.mismatches = r->adj_status.as<unsigned long long>();
  a.npix = npix;
  a.inv_spp = 1.f / float(spp);
  for (uint32_t s0 = 0; s0 < spp; s0 += chunk) {
    const uint32_t cnt = std::min(chunk, spp - s0);
    RenderConst rc = base;
    rc.spp = cnt;
    rc.lanes = cnt;
    rc.adaptive = 0;
    rc.sample_offset = sample_offset + s0;
    ck(cudaMemcpyAsync(r->adj_rc.p, &rc, sizeof(rc), cudaMemcpyHostToDevice, s), "upload constants");
    // pass 1: the forward wavefront, one sample per slot
    ck(cudaMemsetAsync(r->acc.p, 0, size_t(cnt) * npix * 16, s), "reset accumulators");
    ck(cudaMemsetAsync(r->nsamp.p, 0, size_t(cnt) * npix * 4, s), "reset accumulators");
    ck(cudaMemsetAsync(r->aov_a.p, 0, size_t(cnt) * npix * 16, s), "reset accumulators");
    ck(cudaMemsetAsync(wc.wave, 0, 8, s), "reset wave");
    record_wave(r, s, cfg, drc, npix, size_t(cnt) * npix, max_iter, 0, false);
    // pass 2: the replay, bounce by bounce
    ck(cudaMemsetAsync(wc.count, 0, per_wave_counter_bytes(max_iter), s), "reset counters");
    ck(cudaMemsetAsync(wc.wave, 0, 4, s), "reset wave");
    ck(cudaMemsetAsync(q.collected, 0, size_t(cnt) * npix * 16, s), "reset adjoint");
    launch_raygen(cfg, s, drc, sc, q.path[0].p, accum(r), wc);
    // the replay's hits sorted by material (tuning key adjoint_sort)
    HitQueues rq{nullptr, nullptr};
    const size_t bin_words = size_t(2) * MAT_SORT_BINS;
    if (tu.adjoint_sort && tu.sort_threshold > 0) {
      rq.hitq = r->hitq.as<uint32_t>();
      rq.missq = r->missq.as<uint32_t>();
      rq.sorted = r->hitq_sorted.as<uint32_t>();
      rq.sort_threshold = uint32_t(tu.sort_threshold);
      ck(cudaMemsetAsync(r->sort_bins.p, 0, size_t(max_iter) * bin_words * 4, s), "reset sort bins");
    }
    for (int it = 0; it < max_iter; ++it) {
      const AdjPathSoA &in = q.path[it & 1], &out = q.path[(it + 1) & 1];
      float4 *hits = r->hits.as<float4>();
      launch_trace(cfg, s, sc, in.p, hits, wc, it, nullptr, tu.trace_refill, rq);
      if (rq.hitq)
        launch_material_sort(cfg, s, sc, hits, rq, wc, it, r->sort_bins.as<uint32_t>() + size_t(it) * bin_words);
      launch_adj_shade(acfg, s, drc, sc, in, out, hits, q.shadow, wc, it, a, rq);
      launch_shadow_deferred(cfg, s, sc, q.shadow.s, wc, it, tu.trace_refill);
      launch_adj_resolve(acfg, s, drc, sc, q.shadow, out, wc, it, a);
    }
    launch_adj_finish(s, r->sm_count * 8, uint32_t(size_t(cnt) * npix), a);
    ck(cudaGetLastError(), "adjoint kernels");
  }
  ck(cudaEventRecord(r->ev1, s), "event");
  ck(cudaMemcpyAsync(g.materials, r->adj_mat.p, nmat * 4, cudaMemcpyDeviceToHost, s), "read gradients");
  if (g.volumes && nvol)
    ck(cudaMemcpyAsync(g.volumes, r->adj_vol.p, nvol * 4, cudaMemcpyDeviceToHost, s), "read gradients");
  if (ntex)
    ck(cudaMemcpyAsync(g.texels, r->adj_tex.p, ntex * 16, cudaMemcpyDeviceToHost, s), "read gradients");
  unsigned long long mism = 0;
  uint32_t err_word = 0;
  ck(cudaMemcpyAsync(&mism, r->adj_status.p, 8, cudaMemcpyDeviceToHost, s), "read status");
  ck(cudaMemcpyAsync(&err_word, wc.error, 4, cudaMemcpyDeviceToHost, s), "read error word");
  std::vector<float> rad;
  if (g.color) {
    rad.resize(size_t(npix) * 3);
    ck(cudaMemcpyAsync(rad.data(), r->adj_rad.p, rad.size() * 4, cudaMemcpyDeviceToHost, s), "read radiance");
  }
  ck(cudaStreamSynchronize(s), "adjoint");
  check_wave_error(err_word, wc, s);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, r->ev0, r->ev1);
  g.adjoint_ms = ms;
  g.replay_mismatches = mism;
  if (g.color)
    for (size_t p = 0; p < npix; ++p) {
      for (int c = 0; c < 3; ++c)
        g.color[4 * p + c] = rad[3 * p + c] / float(spp);
      g.color[4 * p + 3] = 0.f;
    }
}

int read_channel(phc_renderer *r, float *out, int channel)
{
  if (!r)
    return set_error(nullptr, PHC_ERR_INVALID, "null renderer");
  std::lock_guard<std::mutex> lock(r->mutex);
  if (!out)
    return set_error(r, PHC_ERR_INVALID, "null output buffer");
  if (r->samples == 0)
    return set_error(r, PHC_ERR_NO_FRAME, "no frame has been rendered");
  return guarded(r, [&] {
    check_device(r);
    const uint32_t npix = r->width * r->height;
    const Frame fr{r->f_color.as<float4>(), r->f_normal.as<float4>(), r->f_albedo.as<float4>()};
    launch_read(r->stream, fr, npix, 1.f / float(r->samples), channel, r->read_buf.as<float>());
    ck(cudaGetLastError(), "read kernel");
    const size_t n = size_t(npix) * (channel == 0 ? 4 : (channel == 1 ? 1 : 3));
    ck(cudaMemcpyAsync(out, r->read_buf.p, n * 4, cudaMemcpyDeviceToHost, r->stream), "read back");
    ck(cudaStreamSynchronize(r->stream), "read back");
  });
}

} // namespace

// ------------------------------------------------------------------ C-ABI
extern "C" {

int phc_abi_version(void) { return PHC_ABI_VERSION; }
const char *phc_global_error(void) { return g_error.c_str(); }

void phc_material_default(phc_material *m)
{
  if (!m)
    return;
  std::memset(m, 0, sizeof(*m));
  m->base_color[0] = m->base_color[1] = m->base_color[2] = 0.8f;
  m->opacity = 1.f;
  m->roughness = 1.f;
  m->ior = 1.5f;
  m->clearcoat_roughness = 0.03f;
  m->alpha_mode = 1;
  m->alpha_cutoff = 0.5f;
  m->emission_side = 2;
}
void phc_sampler_default(phc_sampler *s)
{
  if (!s)
    return;
  std::memset(s, 0, sizeof(*s));
  s->type = 1;
  s->linear = 1;
  s->size[0] = s->size[1] = s->size[2] = 1;
  for (int i = 0; i < 4; ++i)
    s->in_transform[5 * i] = s->out_transform[5 * i] = 1.f;
}
void phc_light_default(phc_light *l)
{
  if (!l)
    return;
  std::memset(l, 0, sizeof(*l));
  l->direction[2] = -1.f;
  l->color[0] = l->color[1] = l->color[2] = 1.f;
  l->intensity = 1.f;
  l->spot_angle = 3.14159265f;
}
void phc_volume_default(phc_volume *v)
{
  if (!v)
    return;
  std::memset(v, 0, sizeof(*v));
  v->world_to_local[0] = v->world_to_local[5] = v->world_to_local[10] = 1.f;
  v->spacing[0] = v->spacing[1] = v->spacing[2] = 1.f;
  v->dims[0] = v->dims[1] = v->dims[2] = 1;
  v->value_range[1] = 1.f;
  v->density_scale = 1.f;
  v->linear = 1;
}
void phc_camera_default(phc_camera *c)
{
  if (!c)
    return;
  std::memset(c, 0, sizeof(*c));
  c->direction[2] = -1.f;
  c->up[1] = 1.f;
  c->fovy = 1.0471976f;
  c->height = 1.f;
  c->aspect = 1.f;
  c->focus_distance = 1.f;
  c->image_region[2] = c->image_region[3] = 1.f;
  c->clip_far = std::numeric_limits<float>::infinity();
}
void phc_settings_default(phc_settings *s)
{
  if (!s)
    return;
  std::memset(s, 0, sizeof(*s));
  s->pixel_samples = 1;
  s->max_depth = 6;
  s->background[3] = 1.f;
  s->ambient_color[0] = s->ambient_color[1] = s->ambient_color[2] = 1.f;
  s->max_diffuse_bounces = s->max_glossy_bounces = s->max_transmission_bounces = s->max_volume_bounces = -1;
}
void phc_scene_desc_default(phc_scene_desc *d)
{
  if (d)
    std::memset(d, 0, sizeof(*d));
}

int phc_create(phc_renderer **out)
{
  if (!out)
    return set_error(nullptr, PHC_ERR_INVALID, "null output pointer");
  *out = nullptr;
  phc_renderer *r = nullptr;
  try {
    r = new phc_renderer();
  } catch (const std::bad_alloc &) {
    return set_error(nullptr, PHC_ERR_OOM, "host allocation failed");
  }
  const int rc = guarded(nullptr, [&] {
    int count = 0;
    ck(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
    if (count <= 0)
      throw ApiError(PHC_ERR_CUDA, "no CUDA device found");
    ck(cudaGetDevice(&r->device), "cudaGetDevice");
    ck(cudaDeviceGetAttribute(&r->sm_count, cudaDevAttrMultiProcessorCount, r->device), "device attribute");
    ck(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    ck(cudaEventCreate(&r->ev0), "cudaEventCreate");
    ck(cudaEventCreate(&r->ev1), "cudaEventCreate");
  });
  if (rc != PHC_OK) {
    delete r;
    return rc;
  }
  *out = r;
  return PHC_OK;
}

void phc_destroy(phc_renderer *r)
{
  if (!r)
    return;
  cudaSetDevice(r->device);
  if (r->stream)
    cudaStreamSynchronize(r->stream);
  delete r;
}

const char *phc_backend_name(const phc_renderer *) { return "cuda"; }

int phc_set_scene(phc_renderer *r, const phc_scene_desc *desc)
{
  if (!r)
    return set_error(nullptr, PHC_ERR_INVALID, "null renderer");
  std::lock_guard<std::mutex> lock(r->mutex);
  if (!desc)
    return set_error(r, PHC_ERR_INVALID, "null scene");
  return guarded(r, [&] {
    check_device(r);
    r->samples = 0;
    r->has_scene = false;
    HostScene hs;
    build_host_scene(*desc, hs);
    if (hs.bvh.max_depth >= 64)
      throw ApiError(PHC_ERR_LIMIT, "BVH deeper than the traversal stack (64 levels)");
    const std::string err = r->scene.upload(hs, r->stream);
    if (!err.empty())
      throw ApiError(err.find("out of memory") != std::string::npos ? PHC_ERR_OOM : PHC_ERR_CUDA, err);
    if (r->scene.bvh_depth >= 64) { // a GPU-built BVH8 is checked here
      r->scene.release();
      throw ApiError(PHC_ERR_LIMIT, "BVH deeper than the traversal stack (64 levels)");
    }
    r->atlas_textures = false;
    for (const DevMaterial &m : hs.materials)
      r->atlas_textures = r->atlas_textures || m.base_tex >= 0 || m.alpha_tex >= 0;
    r->has_scene = true;
    r->scene_generation++;
  });
}

int phc_render(phc_renderer *r, const phc_camera *camera, const phc_settings *settings, int reset)
{
  if (!r)
    return set_error(nullptr, PHC_ERR_INVALID, "null renderer");
  std::lock_guard<std::mutex> lock(r->mutex);
  if (!camera || !settings)
    return set_error(r, PHC_ERR_INVALID, "null camera or settings");
  return guarded(r, [&] { render_impl(r, *camera, *settings, reset != 0); });
}

int phc_render_batch(const phc_job *jobs, uint32_t n, phc_render_stats *batch_stats)
{
  if (!jobs || n == 0)
    return set_error(nullptr, PHC_ERR_INVALID, "empty batch");
  for (uint32_t i = 0; i < n; ++i)
    if (!jobs[i].renderer)
      return set_error(nullptr, PHC_ERR_INVALID, "batch job with a null renderer");
  // lock every renderer of the batch, in address order
  std::vector<phc_renderer *> order;
  for (uint32_t i = 0; i < n; ++i)
    order.push_back(jobs[i].renderer);
  std::sort(order.begin(), order.end());
  order.erase(std::unique(order.begin(), order.end()), order.end());
  for (phc_renderer *r : order)
    r->mutex.lock();
  const int rc = guarded(jobs[0].renderer, [&] { render_batch_impl(jobs, n, batch_stats); });
  for (phc_renderer *r : order)
    r->mutex.unlock();
  return rc;
}

int phc_adjoint(phc_renderer *r, const phc_camera *camera, const phc_settings *settings, uint32_t sample_offset,
    const float *d_color, phc_adjoint_grads *grads)
{
  if (!r)
    return set_error(nullptr, PHC_ERR_INVALID, "null renderer");
  std::lock_guard<std::mutex> lock(r->mutex);
  if (!camera || !settings || !d_color || !grads)
    return set_error(r, PHC_ERR_INVALID, "null camera, settings, loss gradient or gradient buffers");
  return guarded(r, [&] { adjoint_impl(r, *camera, *settings, sample_offset, d_color, *grads); });
}

int phc_adjoint_sizes(const phc_renderer *r, uint64_t *materials, uint64_t *volumes, uint64_t *texels)
{
  if (!r)
    return set_error(nullptr, PHC_ERR_INVALID, "null renderer");
  if (!r->has_scene)
    return set_error(nullptr, PHC_ERR_NO_SCENE, "no scene");
  if (materials)
    *materials = uint64_t(r->scene.dev.material_count) * PHC_ADJ_MATERIAL_PARAMS;
  if (volumes)
    *volumes = uint64_t(r->scene.dev.volume_count) * PHC_ADJ_VOLUME_PARAMS;
  if (texels)
    *texels = r->scene.texel_count * 4;
  return PHC_OK;
}

uint32_t phc_accumulated_samples(const phc_renderer *r) { return r ? r->samples : 0u; }

int phc_read_color(phc_renderer *r, float *rgba) { return read_channel(r, rgba, 0); }
int phc_read_depth(phc_renderer *r, float *depth) { return read_channel(r, depth, 1); }
int phc_read_normal(phc_renderer *r, float *xyz) { return read_channel(r, xyz, 2); }
int phc_read_albedo(phc_renderer *r, float *rgb) { return read_channel(r, rgb, 3); }

int phc_render_stats_get(const phc_renderer *r, phc_render_stats *out)
{
  if (!r || !out)
    return set_error(nullptr, PHC_ERR_INVALID, "null argument");
  *out = r->last;
  return PHC_OK;
}

int phc_scene_table(const phc_renderer *r, int32_t table, float *host_out, uint64_t capacity, uint64_t *count)
{
  if (!r || !count)
    return set_error(nullptr, PHC_ERR_INVALID, "null argument");
  if (table < PHC_TABLE_MAJORANTS || table > PHC_TABLE_PRIM_LIGHT_PDF)
    return set_error(nullptr, PHC_ERR_INVALID, "unknown scene table " + std::to_string(table));
  if (!r->has_scene)
    return set_error(nullptr, PHC_ERR_NO_SCENE, "no scene");
  const DevScene &d = r->scene.dev;
  const float *src[5] = {d.vol_majorants, d.env_marginal, d.env_conditional, d.emissive_cdf, d.prim_light_pdf};
  const uint64_t n = r->scene.table_floats[table];
  *count = n;
  if (!host_out || n == 0)
    return PHC_OK;
  if (capacity < n)
    return set_error(nullptr, PHC_ERR_LIMIT, "scene table: " + std::to_string(n) + " floats, capacity " +
        std::to_string(capacity));
  cudaError_t e = cudaSetDevice(r->device);
  if (e == cudaSuccess)
    e = cudaMemcpy(host_out, src[table], n * sizeof(float), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess)
    return set_error(nullptr, PHC_ERR_CUDA, std::string("scene table: ") + cudaGetErrorString(e));
  return PHC_OK;
}

const char *phc_last_error(const phc_renderer *r) { return r ? r->error.c_str() : g_error.c_str(); }

} // extern "C"
