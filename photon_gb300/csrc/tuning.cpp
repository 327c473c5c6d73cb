#include "tuning.h"

#include <cstdlib>
#include <cstring>
#include <mutex>

#include "../../include/photon_cuda.h"

namespace phc {

namespace {

std::once_flag g_once;
Tuning g_tuning;

struct Key {
  const char *name;
  const char *env;
  int64_t lo, hi;
  int64_t *wide;
  int *narrow;
};

// Every tunable with its environment override and admissible range.
const Key *keys(size_t &n)
{
  static Key k[] = {
      {"wave_paths", "PHC_TUNE_WAVE_PATHS", 1024, int64_t(1) << 28, &g_tuning.wave_paths, nullptr},
      {"trace_blocks_per_sm", "PHC_TUNE_TRACE_BLOCKS_PER_SM", 1, 32, nullptr, &g_tuning.trace_blocks_per_sm},
      {"shade_blocks_per_sm", "PHC_TUNE_SHADE_BLOCKS_PER_SM", 1, 32, nullptr, &g_tuning.shade_blocks_per_sm},
      {"use_graph", "PHC_TUNE_USE_GRAPH", 0, 1, nullptr, &g_tuning.use_graph},
      {"count_traversal", "PHC_TUNE_COUNT_TRAVERSAL", 0, 1, nullptr, &g_tuning.count_traversal},
      {"max_leaf", "PHC_TUNE_MAX_LEAF", 1, 3, nullptr, &g_tuning.max_leaf},
      {"time_kernels", "PHC_TUNE_TIME_KERNELS", 0, 1, nullptr, &g_tuning.time_kernels},
      {"trace_refill", "PHC_TUNE_TRACE_REFILL", 1, 32, nullptr, &g_tuning.trace_refill},
      {"vol_refill", "PHC_TUNE_VOL_REFILL", 1, 32, nullptr, &g_tuning.vol_refill},
      {"vol_passes", "PHC_TUNE_VOL_PASSES", 1, 1 << 16, nullptr, &g_tuning.vol_passes},
      {"split_shade", "PHC_TUNE_SPLIT_SHADE", 0, 1, nullptr, &g_tuning.split_shade},
      {"split_volume", "PHC_TUNE_SPLIT_VOLUME", 0, 1, nullptr, &g_tuning.split_volume},
      {"adjoint_sort", "PHC_TUNE_ADJOINT_SORT", 0, 1, nullptr, &g_tuning.adjoint_sort},
      {"class_threshold", "PHC_TUNE_CLASS_THRESHOLD", 0, int64_t(1) << 30, &g_tuning.class_threshold, nullptr},
      {"shade_lean", "PHC_TUNE_SHADE_LEAN", 0, 1, nullptr, &g_tuning.shade_lean},
      {"shade_classes", "PHC_TUNE_SHADE_CLASSES", 0, 1, nullptr, &g_tuning.shade_classes},
      {"batch_wave_paths", "PHC_TUNE_BATCH_WAVE_PATHS", 1024, int64_t(1) << 30, &g_tuning.batch_wave_paths, nullptr},
      {"sort_threshold", "PHC_TUNE_SORT_THRESHOLD", 0, int64_t(1) << 30, &g_tuning.sort_threshold, nullptr},
      {"gpu_bvh", "PHC_TUNE_GPU_BVH", 0, 1, nullptr, &g_tuning.gpu_bvh},
      {"gpu_max_leaf", "PHC_TUNE_GPU_MAX_LEAF", 1, 3, nullptr, &g_tuning.gpu_max_leaf},
      {"ploc_radius", "PHC_TUNE_PLOC_RADIUS", 2, 32, nullptr, &g_tuning.ploc_radius},
      {"collapse_tri_cost", "PHC_TUNE_COLLAPSE_TRI_COST", 0, 10000, nullptr, &g_tuning.collapse_tri_cost},
      {"gpu_tables", "PHC_TUNE_GPU_TABLES", 0, 1, nullptr, &g_tuning.gpu_tables},
      {"texels_u8", "PHC_TUNE_TEXELS_U8", 0, 1, nullptr, &g_tuning.texels_u8},
      {"wave_trip_cap", "PHC_TUNE_WAVE_TRIP_CAP", 1, int64_t(1) << 30, &g_tuning.wave_trip_cap, nullptr},
  };
  n = sizeof(k) / sizeof(k[0]);
  return k;
}

const Key *find(const char *name)
{
  size_t n;
  const Key *k = keys(n);
  for (size_t i = 0; i < n; ++i)
    if (!std::strcmp(k[i].name, name))
      return &k[i];
  return nullptr;
}

} // namespace

Tuning &tuning()
{
  std::call_once(g_once, [] {
    size_t n;
    const Key *k = keys(n);
    for (size_t i = 0; i < n; ++i) {
      const char *s = std::getenv(k[i].env);
      if (!s || !*s)
        continue;
      const int64_t v = std::strtoll(s, nullptr, 10);
      if (v < k[i].lo || v > k[i].hi)
        continue;
      if (k[i].wide)
        *k[i].wide = v;
      else
        *k[i].narrow = int(v);
    }
  });
  return g_tuning;
}

} // namespace phc

extern "C" {

// Sets one tuning parameter; returns PHC_ERR_INVALID for an unknown key or a
// value out of range.  Not synchronised with concurrent render calls.
int phc_tuning_set(const char *key, int64_t value)
{
  phc::tuning();
  if (!key)
    return PHC_ERR_INVALID;
  const phc::Key *k = phc::find(key);
  if (!k || value < k->lo || value > k->hi)
    return PHC_ERR_INVALID;
  if (k->wide)
    *k->wide = value;
  else
    *k->narrow = int(value);
  return PHC_OK;
}

int64_t phc_tuning_get(const char *key)
{
  phc::tuning();
  if (!key)
    return -1;
  const phc::Key *k = phc::find(key);
  if (!k)
    return -1;
  return k->wide ? *k->wide : int64_t(*k->narrow);
}

} // extern "C"
