/*
 * photon_pbrt.h — pbrt-v4 scene reader of libphoton_cuda.so.
 *
 * One call stands in for the reference's two-step pbrt path
 * (app/photon_pbrt_render.cpp:103-139):
 *
 *   photon::pbrt::parse_pbrt_file(path, use_instancing)
 *       (include/photon/pbrt/pbrt_parser.h:8, src/photon/pbrt/pbrt_parser.cpp:272-640)
 *   photon::pbrt::convert_pbrt_scene(scene, base_dir)
 *       (include/photon/pbrt/pbrt_to_photon.h:15, src/photon/pbrt/pbrt_to_photon.cpp:58-503)
 *
 * and hands back the converted scene as the renderer's own scene
 * description: a phc_scene_desc whose `pt` part carries the path-tracer-level
 * materials, texture coordinates, atlas textures and environment rotation
 * (include/photon_cuda.h), plus the camera and render settings the reference's
 * renderer would use.  The same description drives phc_renderer_set_scene,
 * so a pbrt file renders on the GPU exactly as a scene built in memory.
 *
 * Supported input is the reference's: Integrator/Sampler/Film/Camera
 * parameters, Transform, LookAt, Scale, Rotate, ConcatTransform, Identity,
 * WorldBegin, AttributeBegin/End, MakeNamedMaterial/NamedMaterial
 * (diffuse, conductor, dielectric, coateddiffuse, diffusetransmission),
 * AreaLightSource, Shape trianglemesh/plymesh/sphere, Texture imagemap,
 * LightSource infinite, ObjectBegin/End/ObjectInstance and Include/Import,
 * with the reference's reading of each (for example Translate and
 * TransformBegin/End are read and ignored, as there).  Images: PFM (the
 * reference's own reader, image_loader.cpp:20-74); the stb_image formats are
 * not available (stb_image is not part of the reference), such textures are
 * skipped with a warning on stderr.  PLY: ASCII and binary little-endian
 * (ply_reader.cpp:62-251).
 */
#ifndef PHOTON_PBRT_H
#define PHOTON_PBRT_H

#include "photon_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct phc_pbrt_scene phc_pbrt_scene;

/* Overrides of photon_pbrt_render's command line (photon_pbrt_render.cpp:
   34-62, 120-123): a field > 0 replaces the file's value. */
typedef struct phc_pbrt_options {
  int32_t use_instancing; /* parse_pbrt_file's use_instancing: ObjectInstance
                             records instances without flattening them    */
  int32_t width;
  int32_t height;
  int32_t spp;
  int32_t max_depth;
} phc_pbrt_options;

/* Sizes of the parsed and converted scene. */
typedef struct phc_pbrt_info {
  uint64_t meshes;           /* PbrtScene::meshes (flattened instances included) */
  uint64_t named_materials;
  uint64_t textures;         /* Texture directives                            */
  uint64_t loaded_textures;  /* textures with pixels (the atlas)             */
  uint64_t object_defs;
  uint64_t object_instances;
  uint64_t triangles;        /* of the converted mesh                          */
  uint64_t emissive_triangles;
  uint32_t width, height, spp, max_depth;
  int32_t has_env_map;       /* an environment image was loaded               */
} phc_pbrt_info;

/* Parses and converts `path` (directory of `path` = base of relative file
   names).  options may be NULL.  On failure *out is NULL and
   phc_global_error() says why. */
int phc_pbrt_load(const char *path, const phc_pbrt_options *options, phc_pbrt_scene **out);
void phc_pbrt_free(phc_pbrt_scene *scene);
/* The converted scene; owned by `scene`, valid until phc_pbrt_free. */
int phc_pbrt_scene_desc(const phc_pbrt_scene *scene, const phc_scene_desc **desc);
/* Camera::make_perspective's inputs as a phc_camera (pbrt_to_photon.cpp:
   468-488): the renderer derives the same ray-generation camera from it. */
int phc_pbrt_camera(const phc_pbrt_scene *scene, phc_camera *camera);
/* PathTracer::params as photon_pbrt_render sets them (photon_pbrt_render.cpp:
   151-156): size, spp and depth from the file, the rest RenderParams'
   defaults (include/photon/pt/pathtracer.h:16-55). */
int phc_pbrt_settings(const phc_pbrt_scene *scene, phc_settings *settings);
int phc_pbrt_info_get(const phc_pbrt_scene *scene, phc_pbrt_info *info);

#ifdef __cplusplus
}
#endif

#endif
