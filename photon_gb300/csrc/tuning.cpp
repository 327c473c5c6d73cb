#include "tuning.h"

#include <cstdlib>
#include <cstring>
#include <mutex>

#include "../../include/photon_cuda.h"

namespace phc {

namespace {
std::once_flag g_once;
Tuning g_tuning;

int64_t env_or(const char *name, int64_t v)
{
  const char *s = std::getenv(name);
  return s && *s ? std::strtoll(s, nullptr, 10) : v;
}
} // namespace

Tuning &tuning()
{
  std::call_once(g_once, [] {
    Tuning &t = g_tuning;
    t.wave_paths = env_or("PHC_TUNE_WAVE_PATHS", t.wave_paths);
    t.trace_blocks_per_sm = int(env_or("PHC_TUNE_TRACE_BLOCKS_PER_SM", t.trace_blocks_per_sm));
    t.shade_blocks_per_sm = int(env_or("PHC_TUNE_SHADE_BLOCKS_PER_SM", t.shade_blocks_per_sm));
    t.use_graph = int(env_or("PHC_TUNE_USE_GRAPH", t.use_graph));
    t.count_traversal = int(env_or("PHC_TUNE_COUNT_TRAVERSAL", t.count_traversal));
    t.max_leaf = int(env_or("PHC_TUNE_MAX_LEAF", t.max_leaf));
    t.time_kernels = int(env_or("PHC_TUNE_TIME_KERNELS", t.time_kernels));
  });
  return g_tuning;
}

} // namespace phc

extern "C" {

// Sets one tuning parameter; returns PHC_ERR_INVALID for an unknown key or a
// value out of range.  Not synchronised with concurrent render calls.
int phc_tuning_set(const char *key, int64_t value)
{
  phc::Tuning &t = phc::tuning();
  if (!key)
    return PHC_ERR_INVALID;
  if (!std::strcmp(key, "wave_paths") && value >= 1024 && value <= (int64_t(1) << 28))
    t.wave_paths = value;
  else if (!std::strcmp(key, "trace_blocks_per_sm") && value >= 1 && value <= 32)
    t.trace_blocks_per_sm = int(value);
  else if (!std::strcmp(key, "shade_blocks_per_sm") && value >= 1 && value <= 32)
    t.shade_blocks_per_sm = int(value);
  else if (!std::strcmp(key, "use_graph") && (value == 0 || value == 1))
    t.use_graph = int(value);
  else if (!std::strcmp(key, "count_traversal") && (value == 0 || value == 1))
    t.count_traversal = int(value);
  else if (!std::strcmp(key, "max_leaf") && value >= 1 && value <= 3)
    t.max_leaf = int(value);
  else if (!std::strcmp(key, "time_kernels") && (value == 0 || value == 1))
    t.time_kernels = int(value);
  else
    return PHC_ERR_INVALID;
  return PHC_OK;
}

int64_t phc_tuning_get(const char *key)
{
  const phc::Tuning &t = phc::tuning();
  if (!key)
    return -1;
  if (!std::strcmp(key, "wave_paths"))
    return t.wave_paths;
  if (!std::strcmp(key, "trace_blocks_per_sm"))
    return t.trace_blocks_per_sm;
  if (!std::strcmp(key, "shade_blocks_per_sm"))
    return t.shade_blocks_per_sm;
  if (!std::strcmp(key, "use_graph"))
    return t.use_graph;
  if (!std::strcmp(key, "count_traversal"))
    return t.count_traversal;
  if (!std::strcmp(key, "max_leaf"))
    return t.max_leaf;
  if (!std::strcmp(key, "time_kernels"))
    return t.time_kernels;
  return -1;
}

} // extern "C"
