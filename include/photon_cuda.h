/*
 * photon_cuda.h — C-ABI of libphoton_cuda.so, the GB300 (sm_103a) wavefront
 * path tracer that stands in for Photon's ray back-ends and path tracer.
 *
 * Two levels of drop-in, both from Photon (jar091/photon):
 *
 *   Level B, the renderer seam.  Each phc_* renderer call replaces one method
 *   of photon::bridge::Renderer (src/photon/anari/RenderBridge.h:175-214) with
 *   the same argument meaning: scene upload, render(frame) with progressive
 *   accumulation, and the colour / depth / normal / albedo channels the ANARI
 *   device maps (src/photon/anari/Frame.cpp:139-241).  The structs below are
 *   plain-old-data mirrors of bridge::SceneData, CameraData and RenderSettings
 *   (RenderBridge.h:21-170): pointers plus counts instead of std::vector.
 *
 *   Level A, the ray back-end.  phc_accel_* and phc_trace_* replace
 *   photon::pt::RayBackend::build_accel / trace_closest / trace_occluded
 *   (include/photon/pt/backend/ray_backend.h:44-54) on device pointers, the
 *   way the reference's OptiX back-end binds Kokkos::View::data()
 *   (src/photon/pt/backend/optix_backend.cpp:724-814).
 *
 * Conventions (reference: RenderBridge.cpp:83-110, 274-281):
 *   - every call returns PHC_OK (0) or a negative PHC_ERR_* code, and the
 *     message of the last failure is kept per object (phc_last_error) or per
 *     thread for calls without an object (phc_global_error);
 *   - the caller owns every host buffer it passes; set_scene copies the scene
 *     at call time; the library owns all device memory it allocates;
 *   - calls on one renderer are serialised by the caller (one at a time, from
 *     any thread) and block until their device work is done, as
 *     bridge::Renderer's methods do (RenderBridge.h:172-174).
 */
#ifndef PHOTON_CUDA_H
#define PHOTON_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PHC_ABI_VERSION 2

enum {
  PHC_OK = 0,
  PHC_ERR_INVALID = -1,    /* bad argument (null pointer, size 0, bad enum)   */
  PHC_ERR_CUDA = -2,       /* a CUDA runtime call failed                       */
  PHC_ERR_NO_SCENE = -3,   /* render before set_scene                          */
  PHC_ERR_NO_FRAME = -4,   /* read_* before any render (RenderBridge.cpp:1089) */
  PHC_ERR_OOM = -5,        /* device allocation failed                         */
  PHC_ERR_DEVICE = -6,     /* a kernel reported an error word (iteration cap,
                              queue overflow); the context stays usable        */
  PHC_ERR_LIMIT = -7       /* size beyond a documented maximum                 */
};

typedef struct phc_renderer phc_renderer;
typedef struct phc_accel phc_accel;

/* Mirrors bridge::ParamSourceData (RenderBridge.h:21-25). */
typedef struct phc_param_source {
  int32_t kind;  /* 0 constant, 1 vertex attribute, 2 sampler */
  int32_t index; /* attribute slot (0..3, 4 colour, 5 world position,
                    6 world normal) or sampler index */
} phc_param_source;

/* Mirrors bridge::MaterialData (RenderBridge.h:27-56); phc_material_default
   fills the reference's defaults. */
typedef struct phc_material {
  float base_color[3];
  float opacity;
  float metallic;
  float roughness; /* perceptual: the GGX alpha is its square (RenderBridge.cpp:330) */
  float ior;
  float transmission;
  float specular;  /* 0..1, becomes Disney specular 0.5*s (RenderBridge.cpp:334) */
  float emission[3];
  float clearcoat;
  float clearcoat_roughness;
  float sheen;
  phc_param_source base_color_src;
  phc_param_source opacity_src;
  phc_param_source metallic_src;
  phc_param_source roughness_src;
  phc_param_source emission_src;
  phc_param_source transmission_src;
  phc_param_source normal_src;
  int32_t alpha_mode; /* 0 blend, 1 opaque, 2 mask */
  float alpha_cutoff;
  int32_t base_color_alpha;
  int32_t thin_walled;
  int32_t emitter_only;
  int32_t hidden_to_camera;
  int32_t emission_side; /* 0 front, 1 back, 2 both */
} phc_material;

/* Mirrors bridge::SamplerData (RenderBridge.h:58-71). */
typedef struct phc_sampler {
  int32_t type; /* 0 image1D, 1 image2D, 2 image3D, 3 transform */
  int32_t in_attribute;
  int32_t linear;
  int32_t wrap[3]; /* 0 clampToEdge, 1 repeat, 2 mirrorRepeat */
  uint32_t size[3];
  float in_transform[16];  /* row-major */
  float in_offset[4];
  float out_transform[16]; /* row-major */
  float out_offset[4];
  const float *texels;     /* RGBA, texel_count texels (may be short: the
                              sampler then degrades to a transform, as in
                              RenderBridge.cpp:559-562) */
  uint64_t texel_count;
} phc_sampler;

/* Mirrors bridge::LightData (RenderBridge.h:73-85). */
typedef struct phc_light {
  int32_t type; /* 0 point, 1 directional, 2 spot */
  float position[3];
  float direction[3];
  float color[3];
  float intensity;
  float radius;
  float spot_angle;
  float spot_falloff;
} phc_light;

/* Mirrors bridge::EnvironmentData (RenderBridge.h:87-97). */
typedef struct phc_environment {
  int32_t present;
  int32_t visible;
  uint32_t width;
  uint32_t height;
  const float *pixels; /* RGB radiance, width*height*3, row 0 = bottom row */
  float world_to_map[9];
} phc_environment;

/* Mirrors bridge::VolumeData (RenderBridge.h:99-110). */
typedef struct phc_volume {
  float world_to_local[12]; /* row-major 3x4 */
  float origin[3];
  float spacing[3];
  uint32_t dims[3];
  const float *values; /* x fastest */
  uint64_t value_count;
  const float *transfer; /* RGBA entries */
  uint32_t transfer_count; /* number of RGBA entries */
  float value_range[2];
  float density_scale;
  int32_t linear;
} phc_volume;

/* Material at the path tracer's own level: the fields of
   photon::pt::Material (include/photon/pt/material.h:35-82) that scenes built
   without the bridge set, used as given (no bridge conversion: roughness is
   not squared, specular is not halved, flags are taken as they are).  The
   pbrt reader (pbrt_to_photon.cpp:98-170) produces these. */
typedef struct phc_pt_material {
  float base_color[3];
  float metallic;
  float roughness; /* as pt::Material::roughness */
  float ior;
  float transmission;
  float specular; /* as pt::Material::specular (0.5 = Fresnel of ior) */
  float clearcoat;
  float clearcoat_roughness;
  float sheen;
  float alpha;
  float emission[3];
  float emission_strength;
  int32_t flags;          /* pt MATERIAL_FLAG_* bits (material.h:28-32) */
  int32_t base_color_tex; /* texture of the list below, or -1 */
  int32_t alpha_tex;      /* texture of the list below (red channel), or -1 */
} phc_pt_material;

/* Texture of pt::TextureAtlas (include/photon/pt/texture.h:11-65): RGB,
   row 0 = the top row of the image (v = 1), sampled bilinearly with repeat
   wrapping. */
typedef struct phc_texture {
  uint32_t width;
  uint32_t height;
  const float *rgb; /* width*height*3 */
} phc_texture;

/* One object of instanced geometry (include/photon/pt/scene.h:22-28,
   ObjectMesh): a triangle mesh in its own space with one material. */
typedef struct phc_object {
  const float *positions;  /* xyz per vertex */
  uint64_t vertex_count;
  const uint32_t *indices; /* three per triangle */
  uint64_t triangle_count;
  const float *normals;    /* xyz per vertex, or NULL */
  uint32_t material_id;
} phc_object;

/* One placement of an object (scene.h:30-33, Instance). */
typedef struct phc_instance {
  uint32_t object_id;
  float transform[16]; /* object to world, column-major (pbrt order) */
} phc_instance;

/* Scene data that only a scene built at the path tracer's level carries
   (photon::pt::Scene, include/photon/pt/scene.h:40-70, as the pbrt reader
   fills it).  With it the renderer takes `materials` instead of
   phc_scene_desc::materials (same count, material_count) and ignores
   phc_scene_desc::samplers and attributes. */
typedef struct phc_pt_scene {
  const phc_pt_material *materials; /* phc_scene_desc::material_count of them */
  const float *texcoords;           /* uv per vertex, or NULL (uv = 0)        */
  const phc_texture *textures;
  uint32_t texture_count;
  int32_t env_map_to_world_given;   /* 1: env_map_to_world is the map-to-world
                                       rotation; 0: the transpose of
                                       phc_environment::world_to_map */
  float env_map_to_world[9];        /* row-major 3x3 */
  /* Instanced geometry (scene.h:35-39, InstancedGeometry), traced as a
     two-level BVH beside the scene's own triangles instead of being
     flattened into them.  Hits on instances report, as the reference's
     instanced back-end does (backend/optix/photon_optix.cu:68-99, 161-187),
     the object's material, object-space normals carried to world space by
     the inverse transpose of the instance transform, and the barycentrics
     as texture coordinates; instances are not light sources. */
  const phc_object *objects;
  uint32_t object_count;
  const phc_instance *instances;
  uint32_t instance_count;
} phc_pt_scene;

/* Mirrors bridge::SceneData (RenderBridge.h:112-126).  `pt` (may be NULL)
   adds the path-tracer-level data of phc_pt_scene. */
typedef struct phc_scene_desc {
  const float *positions; /* xyz per vertex */
  uint64_t vertex_count;
  const float *normals;   /* xyz per vertex or NULL */
  const float *attributes[5]; /* RGBA per vertex or NULL */
  const uint32_t *indices; /* three per triangle */
  uint64_t triangle_count;
  const uint32_t *material_ids; /* one per triangle, material_id_count of them */
  uint64_t material_id_count;
  const phc_material *materials;
  uint32_t material_count;
  const phc_sampler *samplers;
  uint32_t sampler_count;
  const phc_light *lights;
  uint32_t light_count;
  phc_environment environment;
  const phc_volume *volumes;
  uint32_t volume_count;
  const phc_pt_scene *pt;
} phc_scene_desc;

/* Mirrors bridge::CameraData (RenderBridge.h:128-144). */
typedef struct phc_camera {
  float position[3];
  float direction[3];
  float up[3];
  int32_t orthographic;
  float fovy; /* radians */
  float height;
  float aspect; /* <= 0: width / height */
  float aperture_radius;
  float focus_distance;
  float image_region[4];
  float clip_near;
  float clip_far; /* >= 1e30 or +inf: no far plane */
} phc_camera;

/* Mirrors bridge::RenderSettings (RenderBridge.h:146-170). */
typedef struct phc_settings {
  uint32_t width;
  uint32_t height;
  uint32_t pixel_samples;
  uint32_t max_depth;
  float background[4];
  const float *background_image; /* RGBA, rows from the bottom, or NULL */
  uint32_t background_width;
  uint32_t background_height;
  float ambient_color[3];
  float ambient_radiance;
  int32_t adaptive_sampling;
  float throughput_clamp;
  int32_t max_diffuse_bounces;
  int32_t max_glossy_bounces;
  int32_t max_transmission_bounces;
  int32_t max_volume_bounces;
  float clamp_direct;
  float clamp_indirect;
} phc_settings;

/* Counters of the last render call, read by phc_render_stats. */
#define PHC_KERNEL_KINDS 7
typedef struct phc_render_stats {
  uint64_t pixel_samples;   /* pixel-samples traced (adaptive: started ones)  */
  uint64_t closest_rays;    /* rays given to closest-hit traversal            */
  uint64_t shadow_rays;     /* rays given to any-hit traversal                */
  uint64_t node_visits;     /* BVH8 nodes visited by closest-hit rays (when
                               the "count_traversal" tuning key is 1)         */
  uint64_t tri_tests;       /* triangle tests of closest-hit rays (same)      */
  uint64_t shadow_node_visits; /* the same for the shadow (any-hit) rays      */
  uint64_t shadow_tri_tests;
  double render_ms;         /* device time of the render call                 */
  uint64_t kernel_launches; /* kernels launched by the call (graph nodes too) */
  /* Device time per kernel kind when the "time_kernels" tuning key is 1,
     else 0: raygen, closest-hit trace, shade (with the material sort), shadow
     (any hit), wave end + resolve, the volume-scattering pre-pass, the shadow
     transmittance of volume scenes. */
  double kernel_ms[PHC_KERNEL_KINDS];
  uint64_t kernel_count[PHC_KERNEL_KINDS];
  uint64_t volume_lookups;  /* density lookups of the volume-tracking kernels
                               (when "count_traversal" is 1)                   */
} phc_render_stats;

/* ------------------------------------------------------------------ defaults */
/* Fill the bridge's default values (RenderBridge.h:27-170). */
void phc_material_default(phc_material *m);
void phc_sampler_default(phc_sampler *s);
void phc_light_default(phc_light *l);
void phc_volume_default(phc_volume *v);
void phc_camera_default(phc_camera *c);
void phc_settings_default(phc_settings *s);
void phc_scene_desc_default(phc_scene_desc *d);

int phc_abi_version(void);
/* Message of the last failure on this thread for calls without an object. */
const char *phc_global_error(void);

/* ------------------------------------------------------- Level B (renderer) */
/* bridge::Renderer::Renderer + initialize (RenderBridge.cpp:1012-1034):
   selects the current CUDA device and creates the renderer's stream. */
int phc_create(phc_renderer **out);
/* bridge::Renderer::~Renderer (RenderBridge.cpp:949-965). */
void phc_destroy(phc_renderer *r);
/* bridge::Renderer::backend_name (RenderBridge.cpp:1036-1039): "cuda". */
const char *phc_backend_name(const phc_renderer *r);
/* bridge::Renderer::set_scene (RenderBridge.cpp:1046-1058, scene build
   441-826): uploads the scene, builds the BVH8 and the light tables.
   Drops the accumulated frame. */
int phc_set_scene(phc_renderer *r, const phc_scene_desc *scene);
/* bridge::Renderer::render (RenderBridge.cpp:1060-1075, 828-928): renders
   settings->pixel_samples more samples per pixel; reset != 0 drops the
   accumulated ones. */
int phc_render(phc_renderer *r, const phc_camera *camera, const phc_settings *settings, int reset);
/* bridge::Renderer::accumulated_samples (RenderBridge.cpp:1077-1080). */
uint32_t phc_accumulated_samples(const phc_renderer *r);
/* bridge::Renderer::read_color / read_depth / read_normal / read_albedo
   (RenderBridge.cpp:1082-1172): caller-owned host buffers of width*height
   RGBA / 1 / 3 / 3 floats, row 0 = bottom row; depth is +inf on a miss. */
int phc_read_color(phc_renderer *r, float *rgba);
int phc_read_depth(phc_renderer *r, float *depth);
int phc_read_normal(phc_renderer *r, float *xyz);
int phc_read_albedo(phc_renderer *r, float *rgb);
/* Counters of the last phc_render call. */
int phc_render_stats_get(const phc_renderer *r, phc_render_stats *out);
/* Scene tables the sampling reads, as built on the device at phc_set_scene
   (no reference counterpart; for checking them against the host builders of
   the same tables): the volumes' macro-cell majorant grids, the environment
   map's marginal and conditional CDFs, the emissive triangles' selection CDF
   and the per-primitive light pdf.  *count receives the table's length in
   floats; its floats are copied to host_out when host_out is not NULL and
   capacity (floats) holds them, else PHC_ERR_LIMIT. */
enum {
  PHC_TABLE_MAJORANTS = 0,
  PHC_TABLE_ENV_MARGINAL = 1,
  PHC_TABLE_ENV_CONDITIONAL = 2,
  PHC_TABLE_EMISSIVE_CDF = 3,
  PHC_TABLE_PRIM_LIGHT_PDF = 4
};
int phc_scene_table(const phc_renderer *r, int32_t table, float *host_out, uint64_t capacity, uint64_t *count);

/* One render call of a batch: the arguments of phc_render. */
typedef struct phc_job {
  phc_renderer *renderer;
  const phc_camera *camera;
  const phc_settings *settings;
  int32_t reset;
} phc_job;
/* Batched mode (no reference counterpart; the reference renders one frame
   per PathTracer::render call, pathtracer.cpp:564-1159): performs the n
   render calls -- distinct renderers with their own scenes, sizes, sample
   counts and depths, all on the current device -- in one wavefront whose
   queues carry a job tag, as one replayed CUDA graph.  Each renderer ends in
   exactly the state phc_render would leave it in, with the same image bit
   for bit.  Jobs with adaptive sampling run through phc_render's path.
   batch_stats (may be NULL) receives the counters of the whole batch. */
int phc_render_batch(const phc_job *jobs, uint32_t n, phc_render_stats *batch_stats);
/* Message of the last failed call on this renderer ("" when none). */
const char *phc_last_error(const phc_renderer *r);

/* ------------------------------------------------------------ adjoint */
/* Gradient layout.  Per material: base colour r, g, b, roughness (the
   bridge's perceptual roughness; GGX alpha = roughness^2), metallic,
   specTrans (transmission), sheen, clearcoat.  Per volume: density scale,
   albedo r, g, b (the transfer function's colour, taken as constant over the
   volume).  Per texel: the gradient of each of its four channels (r, g, b,
   a), for the texels of every sampler in the order of
   phc_scene_desc::samplers (sampler i's texels follow those of samplers
   0..i-1); a texel collects the gradient of every parameter its sampler
   feeds (base colour through channels r, g, b of the sampler's output;
   roughness, metallic and specTrans through output channel r). */
#define PHC_ADJ_MATERIAL_PARAMS 8
#define PHC_ADJ_VOLUME_PARAMS 4
#define PHC_ADJ_MAX_VOLUMES 4
typedef struct phc_adjoint_grads {
  float *materials; /* material_count * PHC_ADJ_MATERIAL_PARAMS (required)   */
  float *volumes;   /* volume_count * PHC_ADJ_VOLUME_PARAMS, or NULL          */
  float *texels;    /* 4 * total texel count, or NULL (no texel gradients)   */
  float *color;     /* width*height*4: the image of the pass's own samples
                       (RGB, alpha 0), or NULL                                */
  double adjoint_ms; /* out: device time of the call                          */
  uint64_t replay_mismatches; /* out: pixel samples whose replayed radiance
                       differed from the forward pass's (0 when the replay
                       walks every forward path)                               */
} phc_adjoint_grads;
/* No counterpart in the reference (it has no derivatives).  Path-replay
   backpropagation: gradients of a loss of the image I that phc_render would
   produce with these camera/settings from settings->pixel_samples samples
   starting at sample index sample_offset (a fresh renderer's first render
   uses sample_offset 0), given d_color = dLoss/dI (width*height RGBA floats
   in the phc_read_color layout; alpha is ignored).  The forward wavefront
   gives each pixel sample's radiance; each path is then traced again from
   its seed, so the memory does not grow with the depth.  Lobe
   selection, Russian roulette, MIS weights, clamps and stochastic
   transparency are held constant; visibility (edge) derivatives are not
   computed.  Parameters that come from attributes get no gradient; a base
   colour, roughness, metallic or specTrans read from an image sampler sends
   its gradient to that sampler's texels (through the sampler's output
   transform and the clamps of the material resolution).  Leaves
   the accumulated frame and the sample counter unchanged.  Every output
   buffer is host memory and is overwritten.  Volume gradients need
   volume_count <= PHC_ADJ_MAX_VOLUMES (else PHC_ERR_LIMIT). */
int phc_adjoint(phc_renderer *r, const phc_camera *camera, const phc_settings *settings, uint32_t sample_offset,
    const float *d_color, phc_adjoint_grads *grads);
/* Element counts of the scene's gradient buffers (any pointer may be NULL). */
int phc_adjoint_sizes(const phc_renderer *r, uint64_t *materials, uint64_t *volumes, uint64_t *texels);

/* -------------------------------------------------- Level A (ray back-end) */
/* Hit record of Level A, field for field photon::pt::HitResult
   (include/photon/pt/backend/ray_backend.h:15-29), 88 bytes. */
typedef struct phc_hit_result {
  float t;
  float position[3];
  float normal[3];
  float shading_normal[3];
  float uv[2];
  float bary[2];
  float interpolated_color[3];
  uint32_t prim_id;
  uint32_t geom_id;
  uint32_t inst_id;
  uint32_t material_id;
  uint8_t hit;
  uint8_t has_interpolated_color;
  uint8_t pad_[2];
} phc_hit_result;

/* RayBackend::build_accel (kokkos_backend.cpp:11-19): builds the BVH8 over
   an indexed triangle mesh given in host memory (positions xyz, indices,
   optional normals xyz and material ids). */
int phc_accel_create(phc_accel **out, const float *positions, uint64_t vertex_count, const uint32_t *indices,
    uint64_t triangle_count, const float *normals, const uint32_t *material_ids);
/* RayBackend::build_accel_instanced (ray_backend.h:47-49), as the reference's
   instanced back-end builds it (optix_backend.cpp:659-722): the mesh above
   (may be empty) plus objects placed by instances, traced as a two-level
   BVH8 without flattening.  Hit records of such an accel report, as that
   back-end does: the barycentrics as uv, prim_id within its object, inst_id
   = the object's index (object_count for the mesh's own triangles), the
   object's material id, normals carried to world space by the inverse
   transpose.  With no objects or instances it is phc_accel_create. */
int phc_accel_create_instanced(phc_accel **out, const float *positions, uint64_t vertex_count,
    const uint32_t *indices, uint64_t triangle_count, const float *normals, const uint32_t *material_ids,
    const phc_object *objects, uint32_t object_count, const phc_instance *instances, uint32_t instance_count);
void phc_accel_destroy(phc_accel *a);
/* Largest ray count one phc_trace_* call accepts (PHC_ERR_LIMIT above it). */
#define PHC_TRACE_MAX_RAYS 0x40000000u
/* RayBackend::trace_closest (kokkos_backend.cpp:21-61) on device pointers:
   origins/directions are xyz float triples (RayBatch, ray_backend.h:31-37),
   tmin/tmax one float each; a ray with !(tmax > tmin) misses.  Writes n
   phc_hit_result records.  stream is a cudaStream_t (NULL: the library's).
   Blocks until the trace is done; n above PHC_TRACE_MAX_RAYS is rejected
   with PHC_ERR_LIMIT. */
int phc_trace_closest(phc_accel *a, const float *origins, const float *directions, const float *tmin,
    const float *tmax, uint32_t n, phc_hit_result *hits, void *stream);
/* The same traversal with the compact 16-byte hit record the renderer uses:
   hits4[i] = (t, prim_id bits, u, v); prim_id = 0xffffffff on a miss. */
int phc_trace_closest_compact(phc_accel *a, const float *origins, const float *directions, const float *tmin,
    const float *tmax, uint32_t n, float *hits4, void *stream);
/* RayBackend::trace_occluded (kokkos_backend.cpp:63-86): occluded[i] = 1 when
   anything is hit in [tmin, tmax]. */
int phc_trace_occluded(phc_accel *a, const float *origins, const float *directions, const float *tmin,
    const float *tmax, uint32_t n, uint32_t *occluded, void *stream);
/* Node visits and triangle tests of the last trace call (counting build). */
int phc_accel_counters(const phc_accel *a, uint64_t *node_visits, uint64_t *tri_tests);
/* Size in bytes of the device BVH8 nodes, triangle records and node count. */
int phc_accel_info(const phc_accel *a, uint64_t *node_bytes, uint64_t *tri_bytes, uint64_t *node_count);
/* Message of the last failed phc_accel_* / phc_trace_* call on this thread. */
const char *phc_accel_error(void);

/* Largest ray count phc_trace_closest_compact_static accepts. */
#define PHC_STATIC_MAX_RAYS PHC_TRACE_MAX_RAYS
/* No counterpart in the reference: an allocation-free form of
   phc_trace_closest_compact, with the same arguments and the same results.
   It is for callers that must not allocate device memory while they trace:
   code holding a memory budget or pool that owns all device memory (a host
   application embedding the renderer), and hot loops where cudaMalloc /
   cudaFree would stall the device (they synchronise implicitly).  The
   traversal's only scratch, its 32-ray batch counter, sits in a 256-byte
   array compiled into the library, which every GPU that loads the library
   holds until the process exits; the accel, rays and hit buffer are the
   caller's as before.  The first call on a device looks the array's device
   address up (cudaGetSymbolAddress) and caches it per CUDA context (a
   context made after cudaDeviceReset gets its own lookup); that lookup must
   not run while a stream of the device is being captured, so make the first
   call before any stream capture starts.  Every call shares the one array
   and resets the counter itself: calls that overlap on the GPU (two
   streams, two threads) race and must be serialised by the caller.  n above
   PHC_STATIC_MAX_RAYS is rejected with PHC_ERR_LIMIT.  Each call blocks
   until its trace is done: it synchronises the stream before it returns,
   so no call can be captured into a CUDA graph. */
int phc_trace_closest_compact_static(phc_accel *a, const float *origins, const float *directions, const float *tmin,
    const float *tmax, uint32_t n, float *hits4, void *stream);

/* ------------------------------------------------------------ scheduling */
/* Launch parameters picked by the autotuner (photon_gb300/autotune.py; no
   reference counterpart, the reference has no tunables on this path).  Keys:
   "wave_paths" (paths in flight per wave: the queue capacity),
   "trace_blocks_per_sm", "shade_blocks_per_sm" (persistent grid sizes),
   "trace_refill" (a traversal warp takes new rays once this many lanes are
   idle), "split_shade" (0/1: hits and misses shaded by separate kernels),
   "split_volume" (0/1: in volume scenes the paths that scatter in a
   volume, reach their surface hit or escape go, after the tracking
   pre-pass, to separate queues, each shaded by its own kernel),
   "adjoint_sort" (0/1: the adjoint's replay shades the hits of each bounce
   sorted by material, hits before misses), "class_threshold" (waves of at
   least this many paths shade their hits with the shading-class kernels;
   smaller waves use one lean hit kernel),
   "shade_lean" (0/1: lean shading kernels for scenes without volumes /
   sources / lights), "sort_threshold" (sort the hit queue by material when it
   holds at least this many hits; 0: never), "max_leaf" (1..3, leaf size of the
   host-built BVH8, read at the next scene upload), "gpu_bvh" (0/1: build
   the BVH8 of single-level scenes on the GPU, read at the next scene
   upload), "gpu_max_leaf" (1..3, leaf size of the GPU-built BVH8, read at
   the next scene upload), "ploc_radius" (2..32: clusters the GPU build's
   clustering searches on each side, rounded up to 2, 4, 8, 16 or 32; read
   at the next scene upload), "collapse_tri_cost" (0..10000: a triangle
   test's cost in percent of a node visit, with which the GPU build chooses
   each wide node's children by the surface-area cost of the whole tree,
   default 30; 0: the largest subtrees are opened first; read at the next
   scene upload), "batch_wave_paths", "use_graph" (0/1),
   "count_traversal" (0/1: node / triangle / density-lookup counters),
   "time_kernels" (0/1), "shade_classes" (0/1: lean scenes sort the hit queue
   by shading class and shade each class with a kernel compiled for its
   lobes), "texels_u8" (0/1: keep samplers whose texels are all k / 255 as
   8-bit RGBA, read at the next scene upload), "gpu_tables" (0/1: build the
   volume majorant grids, the environment and emissive CDFs with their
   search guides, and the 8-bit texels on the GPU, equal to the host-built
   tables bit for bit; read at the next scene upload),
   "vol_refill" (a volume-tracking warp takes new rays once this many lanes
   are idle), "vol_passes" (volume tracking: at most this many macro-cell
   steps or lookups per lane and loop trip), "wave_trip_cap" (loop trips after which a persistent warp stops
   with PHC_ERR_DEVICE; a self-check).  Returns PHC_ERR_INVALID
   for an unknown key or out-of-range value; get returns -1 for an unknown
   key.  Settings are process-wide and read at the start of each call. */
int phc_tuning_set(const char *key, int64_t value);
int64_t phc_tuning_get(const char *key);

#ifdef __cplusplus
}
#endif

#endif /* PHOTON_CUDA_H */
