"""ctypes mirrors of the structs in include/photon_cuda.h.

The C structs themselves mirror photon::bridge::SceneData, CameraData and
RenderSettings (src/photon/anari/RenderBridge.h:21-170) with pointers and
counts in place of std::vector.  Field order and types here must match the
header exactly; tests/test_abi.py checks the sizes against the C compiler.
"""
import ctypes as C

f3 = C.c_float * 3
f4 = C.c_float * 4
f9 = C.c_float * 9
f12 = C.c_float * 12
f16 = C.c_float * 16
i3 = C.c_int32 * 3
u3 = C.c_uint32 * 3

PHC_OK = 0
ERROR_NAMES = {
    -1: "PHC_ERR_INVALID", -2: "PHC_ERR_CUDA", -3: "PHC_ERR_NO_SCENE",
    -4: "PHC_ERR_NO_FRAME", -5: "PHC_ERR_OOM", -6: "PHC_ERR_DEVICE",
    -7: "PHC_ERR_LIMIT",
}


class ParamSource(C.Structure):
    _fields_ = [("kind", C.c_int32), ("index", C.c_int32)]


class Material(C.Structure):
    _fields_ = [
        ("base_color", f3), ("opacity", C.c_float), ("metallic", C.c_float),
        ("roughness", C.c_float), ("ior", C.c_float), ("transmission", C.c_float),
        ("specular", C.c_float), ("emission", f3), ("clearcoat", C.c_float),
        ("clearcoat_roughness", C.c_float), ("sheen", C.c_float),
        ("base_color_src", ParamSource), ("opacity_src", ParamSource),
        ("metallic_src", ParamSource), ("roughness_src", ParamSource),
        ("emission_src", ParamSource), ("transmission_src", ParamSource),
        ("normal_src", ParamSource),
        ("alpha_mode", C.c_int32), ("alpha_cutoff", C.c_float),
        ("base_color_alpha", C.c_int32), ("thin_walled", C.c_int32),
        ("emitter_only", C.c_int32), ("hidden_to_camera", C.c_int32),
        ("emission_side", C.c_int32),
    ]


class Sampler(C.Structure):
    _fields_ = [
        ("type", C.c_int32), ("in_attribute", C.c_int32), ("linear", C.c_int32),
        ("wrap", i3), ("size", u3), ("in_transform", f16), ("in_offset", f4),
        ("out_transform", f16), ("out_offset", f4),
        ("texels", C.POINTER(C.c_float)), ("texel_count", C.c_uint64),
    ]


class Light(C.Structure):
    _fields_ = [
        ("type", C.c_int32), ("position", f3), ("direction", f3), ("color", f3),
        ("intensity", C.c_float), ("radius", C.c_float), ("spot_angle", C.c_float),
        ("spot_falloff", C.c_float),
    ]


class Environment(C.Structure):
    _fields_ = [
        ("present", C.c_int32), ("visible", C.c_int32), ("width", C.c_uint32),
        ("height", C.c_uint32), ("pixels", C.POINTER(C.c_float)), ("world_to_map", f9),
    ]


class Volume(C.Structure):
    _fields_ = [
        ("world_to_local", f12), ("origin", f3), ("spacing", f3), ("dims", u3),
        ("values", C.POINTER(C.c_float)), ("value_count", C.c_uint64),
        ("transfer", C.POINTER(C.c_float)), ("transfer_count", C.c_uint32),
        ("value_range", C.c_float * 2), ("density_scale", C.c_float), ("linear", C.c_int32),
    ]


class PtMaterial(C.Structure):
    _fields_ = [
        ("base_color", f3), ("metallic", C.c_float), ("roughness", C.c_float), ("ior", C.c_float),
        ("transmission", C.c_float), ("specular", C.c_float), ("clearcoat", C.c_float),
        ("clearcoat_roughness", C.c_float), ("sheen", C.c_float), ("alpha", C.c_float),
        ("emission", f3), ("emission_strength", C.c_float), ("flags", C.c_int32),
        ("base_color_tex", C.c_int32), ("alpha_tex", C.c_int32),
    ]


class Texture(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("rgb", C.POINTER(C.c_float))]


class Object(C.Structure):
    _fields_ = [
        ("positions", C.POINTER(C.c_float)), ("vertex_count", C.c_uint64),
        ("indices", C.POINTER(C.c_uint32)), ("triangle_count", C.c_uint64),
        ("normals", C.POINTER(C.c_float)), ("material_id", C.c_uint32),
    ]


class Instance(C.Structure):
    _fields_ = [("object_id", C.c_uint32), ("transform", C.c_float * 16)]


class PtScene(C.Structure):
    _fields_ = [
        ("materials", C.POINTER(PtMaterial)), ("texcoords", C.POINTER(C.c_float)),
        ("textures", C.POINTER(Texture)), ("texture_count", C.c_uint32),
        ("env_map_to_world_given", C.c_int32), ("env_map_to_world", f9),
        ("objects", C.POINTER(Object)), ("object_count", C.c_uint32),
        ("instances", C.POINTER(Instance)), ("instance_count", C.c_uint32),
    ]


class SceneDesc(C.Structure):
    _fields_ = [
        ("positions", C.POINTER(C.c_float)), ("vertex_count", C.c_uint64),
        ("normals", C.POINTER(C.c_float)),
        ("attributes", C.POINTER(C.c_float) * 5),
        ("indices", C.POINTER(C.c_uint32)), ("triangle_count", C.c_uint64),
        ("material_ids", C.POINTER(C.c_uint32)), ("material_id_count", C.c_uint64),
        ("materials", C.POINTER(Material)), ("material_count", C.c_uint32),
        ("samplers", C.POINTER(Sampler)), ("sampler_count", C.c_uint32),
        ("lights", C.POINTER(Light)), ("light_count", C.c_uint32),
        ("environment", Environment),
        ("volumes", C.POINTER(Volume)), ("volume_count", C.c_uint32),
        ("pt", C.POINTER(PtScene)),
    ]


class Camera(C.Structure):
    _fields_ = [
        ("position", f3), ("direction", f3), ("up", f3), ("orthographic", C.c_int32),
        ("fovy", C.c_float), ("height", C.c_float), ("aspect", C.c_float),
        ("aperture_radius", C.c_float), ("focus_distance", C.c_float),
        ("image_region", f4), ("clip_near", C.c_float), ("clip_far", C.c_float),
    ]


class Settings(C.Structure):
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32), ("pixel_samples", C.c_uint32),
        ("max_depth", C.c_uint32), ("background", f4),
        ("background_image", C.POINTER(C.c_float)),
        ("background_width", C.c_uint32), ("background_height", C.c_uint32),
        ("ambient_color", f3), ("ambient_radiance", C.c_float),
        ("adaptive_sampling", C.c_int32), ("throughput_clamp", C.c_float),
        ("max_diffuse_bounces", C.c_int32), ("max_glossy_bounces", C.c_int32),
        ("max_transmission_bounces", C.c_int32), ("max_volume_bounces", C.c_int32),
        ("clamp_direct", C.c_float), ("clamp_indirect", C.c_float),
    ]


# kernel kinds of RenderStats.kernel_ms (phc_render_stats)
KERNEL_KINDS = 7
KERNEL_KIND_NAMES = ("raygen", "trace_closest", "shade", "trace_shadow", "wave_end+resolve", "volume_scatter",
                     "shadow_transmittance")


class RenderStats(C.Structure):
    _fields_ = [
        ("pixel_samples", C.c_uint64), ("closest_rays", C.c_uint64),
        ("shadow_rays", C.c_uint64), ("node_visits", C.c_uint64),
        ("tri_tests", C.c_uint64), ("shadow_node_visits", C.c_uint64),
        ("shadow_tri_tests", C.c_uint64), ("render_ms", C.c_double),
        ("kernel_launches", C.c_uint64), ("kernel_ms", C.c_double * KERNEL_KINDS),
        ("kernel_count", C.c_uint64 * KERNEL_KINDS), ("volume_lookups", C.c_uint64),
    ]


ADJ_MATERIAL_PARAMS = 8
ADJ_VOLUME_PARAMS = 4
ADJ_MAX_VOLUMES = 4
# names of the per-material gradient entries, in buffer order
ADJ_MATERIAL_NAMES = ("base_r", "base_g", "base_b", "roughness", "metallic", "transmission", "sheen", "clearcoat")
ADJ_VOLUME_NAMES = ("density_scale", "albedo_r", "albedo_g", "albedo_b")


class AdjointGrads(C.Structure):
    _fields_ = [
        ("materials", C.c_void_p), ("volumes", C.c_void_p), ("texels", C.c_void_p),
        ("color", C.c_void_p), ("adjoint_ms", C.c_double), ("replay_mismatches", C.c_uint64),
    ]


class Job(C.Structure):
    _fields_ = [
        ("renderer", C.c_void_p), ("camera", C.POINTER(Camera)), ("settings", C.POINTER(Settings)),
        ("reset", C.c_int32),
    ]


class HitResult(C.Structure):
    _fields_ = [
        ("t", C.c_float), ("position", f3), ("normal", f3), ("shading_normal", f3),
        ("uv", C.c_float * 2), ("bary", C.c_float * 2), ("interpolated_color", f3),
        ("prim_id", C.c_uint32), ("geom_id", C.c_uint32), ("inst_id", C.c_uint32),
        ("material_id", C.c_uint32), ("hit", C.c_uint8),
        ("has_interpolated_color", C.c_uint8), ("pad_", C.c_uint8 * 2),
    ]


# numpy dtype of HitResult, for reading arrays of records.
def hit_dtype():
    import numpy as np
    return np.dtype([
        ("t", "<f4"), ("position", "<f4", 3), ("normal", "<f4", 3),
        ("shading_normal", "<f4", 3), ("uv", "<f4", 2), ("bary", "<f4", 2),
        ("interpolated_color", "<f4", 3), ("prim_id", "<u4"), ("geom_id", "<u4"),
        ("inst_id", "<u4"), ("material_id", "<u4"), ("hit", "u1"),
        ("has_interpolated_color", "u1"), ("pad_", "u1", 2),
    ])


def material_default():
    """bridge::MaterialData defaults (RenderBridge.h:27-56)."""
    m = Material()
    m.base_color[:] = (0.8, 0.8, 0.8)
    m.opacity = 1.0
    m.metallic = 0.0
    m.roughness = 1.0
    m.ior = 1.5
    m.transmission = 0.0
    m.specular = 0.0
    m.clearcoat = 0.0
    m.clearcoat_roughness = 0.03
    m.sheen = 0.0
    m.alpha_mode = 1
    m.alpha_cutoff = 0.5
    m.emission_side = 2
    return m


def sampler_default():
    """bridge::SamplerData defaults (RenderBridge.h:58-71)."""
    s = Sampler()
    s.type = 1
    s.in_attribute = 0
    s.linear = 1
    s.size[:] = (1, 1, 1)
    s.in_transform[:] = (1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1)
    s.out_transform[:] = (1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1)
    return s


def light_default():
    """bridge::LightData defaults (RenderBridge.h:73-85)."""
    l = Light()
    l.direction[:] = (0.0, 0.0, -1.0)
    l.color[:] = (1.0, 1.0, 1.0)
    l.intensity = 1.0
    l.spot_angle = 3.14159265
    return l


def volume_default():
    """bridge::VolumeData defaults (RenderBridge.h:99-110)."""
    v = Volume()
    v.world_to_local[:] = (1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0)
    v.spacing[:] = (1.0, 1.0, 1.0)
    v.dims[:] = (1, 1, 1)
    v.value_range[:] = (0.0, 1.0)
    v.density_scale = 1.0
    v.linear = 1
    return v


def camera_default():
    """bridge::CameraData defaults (RenderBridge.h:128-144)."""
    c = Camera()
    c.direction[:] = (0.0, 0.0, -1.0)
    c.up[:] = (0.0, 1.0, 0.0)
    c.fovy = 1.0471976
    c.height = 1.0
    c.aspect = 1.0
    c.focus_distance = 1.0
    c.image_region[:] = (0.0, 0.0, 1.0, 1.0)
    c.clip_far = float("inf")
    return c


def settings_default():
    """bridge::RenderSettings defaults (RenderBridge.h:146-170)."""
    s = Settings()
    s.pixel_samples = 1
    s.max_depth = 6
    s.background[:] = (0.0, 0.0, 0.0, 1.0)
    s.ambient_color[:] = (1.0, 1.0, 1.0)
    s.max_diffuse_bounces = -1
    s.max_glossy_bounces = -1
    s.max_transmission_bounces = -1
    s.max_volume_bounces = -1
    return s
