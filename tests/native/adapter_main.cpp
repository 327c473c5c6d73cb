// Link-and-run check of the reference-side adapters
// (photon_gb300/adapters/*.cpp) built against the reference's own headers:
// the RayBackend reports its name, and bridge::Renderer initializes (or,
// without a GPU, reports the library's error as the reference's bridge
// does: false plus a message).
#include <cstdio>
#include <memory>
#include <string>

#include "photon/anari/RenderBridge.h"
#include "photon/pt/backend/ray_backend.h"

namespace photon::pt {
std::unique_ptr<RayBackend> make_cuda_backend();
}

int main()
{
  auto backend = photon::pt::make_cuda_backend();
  std::printf("backend %s\n", backend->name());
  photon::bridge::Renderer r;
  std::string error;
  const bool ok = r.initialize(error);
  std::printf("initialize %d backend_name '%s' error '%s'\n", int(ok), r.backend_name().c_str(), error.c_str());
  float px[4];
  const bool read = r.read_color(px, error);
  std::printf("read before render %d error '%s'\n", int(read), error.c_str());
  return (ok || !error.empty()) && !read ? 0 : 1;
}
