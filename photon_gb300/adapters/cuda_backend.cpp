// Level A of the drop-in: a photon::pt::RayBackend (the reference's
// include/photon/pt/backend/ray_backend.h:44-54) over libphoton_cuda.so, for
// the reference to select as PHOTON_BACKEND=cuda beside kokkos / embree /
// optix.  This file belongs in the reference's tree
// (src/photon/pt/backend/cuda_backend.cpp), compiled with its headers and
// linked against libphoton_cuda.so; registration is one line in
// create_best_backend (src/photon/pt/backend/backend_factory.cpp:28-48):
//
//     if (std::strcmp(env, "cuda") == 0) return photon::pt::make_cuda_backend();
//
// With Kokkos-CUDA the views of RayBatch / HitBatch hold device memory, which
// the phc_trace_* calls take as they are (as the reference's OptiX back-end
// does, optix_backend.cpp:738-760); the scene arrays are mirrored to the host
// for the BVH build.  Errors become exceptions like the reference's back-ends
// (embree_backend.cpp:149-156); every call blocks until the traversal is done
// (kokkos_backend.cpp:60).
#include <cstddef>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <vector>

#include "photon/pt/backend/ray_backend.h"
#include "photon/pt/scene.h"
#include "photon_cuda.h"

namespace photon::pt {

// The 88-byte record both sides write: phc_trace_closest fills HitResult
// arrays directly, so every field must sit where the reference puts it.
static_assert(sizeof(HitResult) == sizeof(phc_hit_result), "HitResult size");
static_assert(offsetof(HitResult, t) == offsetof(phc_hit_result, t), "HitResult::t");
static_assert(offsetof(HitResult, position) == offsetof(phc_hit_result, position), "HitResult::position");
static_assert(offsetof(HitResult, normal) == offsetof(phc_hit_result, normal), "HitResult::normal");
static_assert(offsetof(HitResult, shading_normal) == offsetof(phc_hit_result, shading_normal),
    "HitResult::shading_normal");
static_assert(offsetof(HitResult, uv) == offsetof(phc_hit_result, uv), "HitResult::uv");
static_assert(offsetof(HitResult, bary) == offsetof(phc_hit_result, bary), "HitResult::bary");
static_assert(offsetof(HitResult, interpolated_color) == offsetof(phc_hit_result, interpolated_color),
    "HitResult::interpolated_color");
static_assert(offsetof(HitResult, prim_id) == offsetof(phc_hit_result, prim_id), "HitResult::prim_id");
static_assert(offsetof(HitResult, geom_id) == offsetof(phc_hit_result, geom_id), "HitResult::geom_id");
static_assert(offsetof(HitResult, inst_id) == offsetof(phc_hit_result, inst_id), "HitResult::inst_id");
static_assert(offsetof(HitResult, material_id) == offsetof(phc_hit_result, material_id), "HitResult::material_id");
static_assert(offsetof(HitResult, hit) == offsetof(phc_hit_result, hit), "HitResult::hit");
static_assert(offsetof(HitResult, has_interpolated_color) == offsetof(phc_hit_result, has_interpolated_color),
    "HitResult::has_interpolated_color");
static_assert(sizeof(Vec3) == 3 * sizeof(float), "RayBatch origins / directions are xyz float triples");

namespace {

[[noreturn]] void raise(const char *what)
{
  throw std::runtime_error(std::string("cuda back-end: ") + what + ": " + phc_accel_error());
}

struct CudaBackend final : RayBackend {
  phc_accel *accel = nullptr;

  ~CudaBackend() override { phc_accel_destroy(accel); }

  void build_accel(const Scene &scene) override { build(scene, nullptr); }

  void build_accel_instanced(const Scene &scene, const InstancedGeometry &instanced) override
  {
    build(scene, instanced.empty() ? nullptr : &instanced);
  }

  void trace_closest(const RayBatch &rays, HitBatch &hits) override
  {
    if (rays.count == 0)
      return;
    if (phc_trace_closest(accel, &rays.origins.data()->x, &rays.directions.data()->x, rays.tmin.data(),
            rays.tmax.data(), rays.count, reinterpret_cast<phc_hit_result *>(hits.hits.data()), nullptr) != PHC_OK)
      raise("trace_closest");
  }

  void trace_occluded(const RayBatch &rays, Kokkos::View<u32 *> occluded) override
  {
    if (rays.count == 0)
      return;
    if (phc_trace_occluded(accel, &rays.origins.data()->x, &rays.directions.data()->x, rays.tmin.data(),
            rays.tmax.data(), rays.count, occluded.data(), nullptr) != PHC_OK)
      raise("trace_occluded");
  }

  const char *name() const override { return "cuda"; }

 private:
  // The scene mesh (and, for build_accel_instanced, the objects and their
  // placements: ObjectMesh -> phc_object, Instance -> phc_instance with the
  // same column-major transform, scene.h:22-39).
  void build(const Scene &scene, const InstancedGeometry *ig)
  {
    const TriangleMesh &m = scene.mesh;
    auto pos = Kokkos::create_mirror_view_and_copy(Kokkos::HostSpace{}, m.positions);
    auto idx = Kokkos::create_mirror_view_and_copy(Kokkos::HostSpace{}, m.indices);
    auto nrm = Kokkos::create_mirror_view_and_copy(Kokkos::HostSpace{}, m.normals);
    auto mat = Kokkos::create_mirror_view_and_copy(Kokkos::HostSpace{}, m.material_ids);
    const uint64_t nv = pos.extent(0), nt = idx.extent(0) / 3;
    const float *normals = nrm.extent(0) >= nv && nv ? &nrm.data()->x : nullptr;
    const uint32_t *mids = mat.extent(0) >= nt && nt ? mat.data() : nullptr;
    std::vector<phc_object> objs;
    std::vector<phc_instance> insts;
    if (ig) {
      for (const ObjectMesh &o : ig->objects) {
        phc_object po{};
        po.positions = o.positions.data();
        po.vertex_count = o.positions.size() / 3;
        po.indices = reinterpret_cast<const uint32_t *>(o.indices.data());
        po.triangle_count = o.indices.size() / 3;
        po.normals = o.normals.size() >= o.positions.size() && !o.normals.empty() ? o.normals.data() : nullptr;
        po.material_id = o.material_id;
        objs.push_back(po);
      }
      for (const Instance &i : ig->instances) {
        phc_instance pi{};
        pi.object_id = i.object_id;
        static_assert(sizeof(pi.transform) == sizeof(i.transform), "instance transform");
        std::memcpy(pi.transform, i.transform, sizeof(pi.transform));
        insts.push_back(pi);
      }
    }
    phc_accel_destroy(accel);
    accel = nullptr;
    const int rc = ig ? phc_accel_create_instanced(&accel, nv ? &pos.data()->x : nullptr, nv, idx.data(), nt,
                            normals, mids, objs.data(), uint32_t(objs.size()), insts.data(), uint32_t(insts.size()))
                      : phc_accel_create(&accel, nv ? &pos.data()->x : nullptr, nv, idx.data(), nt, normals, mids);
    if (rc != PHC_OK)
      raise("build_accel");
  }
};

} // namespace

std::unique_ptr<RayBackend> make_cuda_backend() { return std::make_unique<CudaBackend>(); }

} // namespace photon::pt
