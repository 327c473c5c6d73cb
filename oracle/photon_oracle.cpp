// CPU restatement of Photon's path-tracing hot path — TEST INFRASTRUCTURE.
//
// This is the oracle the CUDA path is checked against where the reference
// sources are not available (the GPU host).  It restates, in plain scalar
// C++, the algorithm of:
//   - photon::bridge::Renderer's scene build, render and read-back
//     (src/photon/anari/RenderBridge.cpp:324-370, 386-410, 441-928, 1082-1172),
//   - PathTracer::build_light_tables and PathTracer::render
//     (src/photon/pt/pathtracer.cpp:20-391, 411-503, 564-1159),
//   - Bvh::build_cpu and intersect_mesh_bvh with the Möller–Trumbore test
//     (src/photon/pt/bvh/bvh.cpp:20-125, include/photon/pt/geom/mesh_intersector.h,
//     include/photon/pt/geom/triangle_intersect.h),
//   - the device functions of include/photon/pt/{disney_bsdf,light,
//     environment_map,tf_volume,sampler,camera,sampling,rng,math}.h and
//     src/photon/pt/environment_map.cpp.
// Every float expression keeps the reference's operation order, and the
// library is compiled with -ffp-contract=off, so on the same compiler and libm
// its results are bit-identical to the reference's (tests/test_oracle_pin.py
// checks that against the reference compiled from its own sources).
//
// Structure differs from the reference where results cannot change: each
// pixel runs its samples and bounce iterations to completion on one OpenMP
// thread (the reference sweeps all pixels per bounce), which is equivalent
// because no state is shared between pixels and every random stream is keyed
// by (pixel, sample, iteration) (pathtracer.cpp:31-34).  The bridge's scene
// data never carries TextureAtlas textures, mesh texture coordinates, vertex
// colours or area lights (RenderBridge.cpp:441-826), so those Scene fields are
// not restated.
#include "photon_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

namespace orc {

using f32 = float;

// The single-precision transcendental functions of the restatement.  By
// default they are the host C library's, which is what the reference calls
// (std::sin on a float, ...).  Built with -DORACLE_LIBM_DOUBLE each is
// evaluated in double precision and rounded to float instead: a different
// libm, correctly rounded almost everywhere, which the tests use to measure
// how much a libm difference alone moves per-sample results (the GPU's
// CUDA math functions are another such libm).
namespace lm {
#ifdef ORACLE_LIBM_DOUBLE
inline f32 sin(f32 x) { return f32(::sin(double(x))); }
inline f32 cos(f32 x) { return f32(::cos(double(x))); }
inline f32 tan(f32 x) { return f32(::tan(double(x))); }
inline f32 log(f32 x) { return f32(::log(double(x))); }
inline f32 pow(f32 x, f32 y) { return f32(::pow(double(x), double(y))); }
inline f32 acos(f32 x) { return f32(::acos(double(x))); }
inline f32 atan2(f32 y, f32 x) { return f32(::atan2(double(y), double(x))); }
#else
inline f32 sin(f32 x) { return std::sin(x); }
inline f32 cos(f32 x) { return std::cos(x); }
inline f32 tan(f32 x) { return std::tan(x); }
inline f32 log(f32 x) { return std::log(x); }
inline f32 pow(f32 x, f32 y) { return std::pow(x, y); }
inline f32 acos(f32 x) { return std::acos(x); }
inline f32 atan2(f32 y, f32 x) { return std::atan2(y, x); }
#endif
} // namespace lm
using u32 = uint32_t;
using i32 = int32_t;

// ----------------------------------------------------------------- math.h
struct V3 {
  f32 x{0.f}, y{0.f}, z{0.f};
  V3() = default;
  V3(f32 a, f32 b, f32 c) : x(a), y(b), z(c) {}
};
inline V3 operator+(const V3 &a, const V3 &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(const V3 &a, const V3 &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(const V3 &v) { return {-v.x, -v.y, -v.z}; }
inline V3 operator*(const V3 &a, f32 s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(f32 s, const V3 &a) { return a * s; }
inline V3 operator*(const V3 &a, const V3 &b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline f32 dot(const V3 &a, const V3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(const V3 &a, const V3 &b)
{
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline f32 length(const V3 &v) { return std::sqrt(dot(v, v)); }
inline V3 normalize(const V3 &v)
{
  const f32 len = length(v);
  return len > 0.f ? (v * (1.f / len)) : V3{};
}
inline V3 lerp(const V3 &a, const V3 &b, f32 t) { return a + (b - a) * t; }
inline V3 reflect(const V3 &I, const V3 &N) { return I - (2.f * dot(I, N)) * N; }
inline V3 refract(const V3 &I, const V3 &N, f32 eta)
{
  const f32 cosi = -dot(I, N);
  const f32 k = 1.f - eta * eta * (1.f - cosi * cosi);
  if (k < 0.f)
    return {};
  return eta * I + (eta * cosi - std::sqrt(k)) * N;
}
struct V4 {
  f32 x{0.f}, y{0.f}, z{0.f}, w{0.f};
  V4() = default;
  V4(f32 a, f32 b, f32 c, f32 d) : x(a), y(b), z(c), w(d) {}
  V4(const V3 &v, f32 d) : x(v.x), y(v.y), z(v.z), w(d) {}
  V3 xyz() const { return {x, y, z}; }
};
inline V4 operator+(const V4 &a, const V4 &b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
inline V4 operator*(const V4 &a, f32 s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
// math_vec4.h:33-39, row-major 4x4 times column vector
inline V4 mul_mat4(const f32 *m, const V4 &v)
{
  return {m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3] * v.w, m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7] * v.w,
      m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11] * v.w, m[12] * v.x + m[13] * v.y + m[14] * v.z + m[15] * v.w};
}
struct V2 {
  f32 x{0.f}, y{0.f};
};

constexpr f32 PI = 3.14159265358979323846f;
constexpr f32 INV_PI = 1.f / PI;
constexpr f32 TWO_PI = 2.f * PI;
constexpr f32 INV_TWO_PI = 1.f / TWO_PI;

inline f32 luminance(const V3 &c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

// ------------------------------------------------------------------ rng.h
// xorshift32, rng.h:9-30
struct Rng {
  u32 state;
  explicit Rng(u32 seed) : state(seed ? seed : 1u) {}
  u32 next_u32()
  {
    u32 x = state;
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    state = x;
    return x;
  }
  f32 next_f32() { return (next_u32() >> 8) * (1.0f / 16777216.0f); }
};

// pathtracer.cpp:20-34
inline u32 hash_u32(u32 x)
{
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}
inline Rng make_rng(u32 pixel, u32 sample, u32 dimension)
{
  return Rng(hash_u32(pixel + hash_u32(sample + hash_u32(dimension + 0x9e3779b9U))));
}

// ------------------------------------------------------------- sampling.h
inline f32 power_heuristic(f32 fPdf, f32 gPdf) // sampling.h:16-23 with nf = ng = 1
{
  const f32 f = 1 * fPdf;
  const f32 g = 1 * gPdf;
  const f32 f2 = f * f;
  const f32 g2 = g * g;
  return (f2 + g2) > 0.f ? f2 / (f2 + g2) : 0.f;
}
inline void onb(const V3 &n, V3 &t, V3 &b) // sampling.h:25-40
{
  if (n.z < -0.9999999f) {
    t = {0.f, -1.f, 0.f};
    b = {-1.f, 0.f, 0.f};
    return;
  }
  const f32 a = 1.f / (1.f + n.z);
  const f32 c = -n.x * n.y * a;
  t = {1.f - n.x * n.x * a, c, -n.x};
  b = {c, 1.f - n.y * n.y * a, -n.y};
  t = normalize(t);
  b = normalize(b);
}
inline V2 concentric_disk(Rng &rng) // sampling.h:53-76
{
  const f32 u = 2.f * rng.next_f32() - 1.f;
  const f32 v = 2.f * rng.next_f32() - 1.f;
  if (u == 0.f && v == 0.f)
    return {0.f, 0.f};
  f32 r, theta;
  const f32 au = std::fabs(u), av = std::fabs(v);
  if (au > av) {
    r = au;
    theta = (PI / 4.f) * (v / u);
  } else {
    r = av;
    theta = (PI / 2.f) - (PI / 4.f) * (u / v);
  }
  return {r * lm::cos(theta), r * lm::sin(theta)};
}
inline V3 cosine_hemisphere(const V3 &n, Rng &rng) // sampling.h:78-92 (direction only)
{
  V3 t, b;
  onb(n, t, b);
  const V2 d = concentric_disk(rng);
  const f32 z = std::sqrt(std::fmax(0.f, 1.f - d.x * d.x - d.y * d.y));
  V3 dir = d.x * t + d.y * b + z * n;
  return normalize(dir);
}
inline V3 uniform_sphere(Rng &rng) // sampling.h:94-100
{
  const f32 z = 1.f - 2.f * rng.next_f32();
  const f32 r = std::sqrt(std::fmax(0.f, 1.f - z * z));
  const f32 phi = TWO_PI * rng.next_f32();
  return {r * lm::cos(phi), r * lm::sin(phi), z};
}

// ------------------------------------------------------------- material.h
enum { K_CONST = 0, K_ATTR = 1, K_SAMPLER = 2 };
enum { A_BLEND = 0, A_OPAQUE = 1, A_MASK = 2 };
enum { F_EMITTER_ONLY = 1, F_HIDDEN = 2, F_EMIT_BOTH = 4, F_REFRACTIVE = 8, F_EMIT_BACK = 16 };
struct Src {
  i32 kind{K_CONST};
  i32 index{0};
};
struct Mat { // material.h:35-82 (the fields the bridge fills)
  V3 base_color{0.8f, 0.8f, 0.8f};
  f32 metallic{0.f}, roughness{0.5f}, ior{1.5f}, transmission{0.f}, specular{0.5f};
  f32 clearcoat{0.f}, clearcoat_roughness{0.03f}, sheen{0.f}, sheen_tint{0.5f}, specular_tint{0.f};
  f32 anisotropic{0.f};
  V3 emission{0.f, 0.f, 0.f};
  f32 emission_strength{0.f};
  f32 subsurface{0.f};
  V3 subsurface_color{1.f, 1.f, 1.f};
  f32 alpha{1.f};
  i32 thin{0};
  Src base_color_src, alpha_src, metallic_src, roughness_src, emission_src, transmission_src, normal_src;
  i32 alpha_mode{A_BLEND};
  f32 alpha_cutoff{0.5f};
  i32 flags{0};
  i32 base_color_alpha{0};
  i32 roughness_src_squared{0};
  i32 base_color_tex{-1}, alpha_tex{-1};
};
inline V3 mat_emission(const Mat &m) { return m.emission * m.emission_strength; }
inline bool may_emit(const Mat &m) // material.h:97-103 (no emission textures here)
{
  if (m.emission_strength <= 0.f)
    return false;
  return m.emission_src.kind != K_CONST || m.emission.x > 0.f || m.emission.y > 0.f || m.emission.z > 0.f;
}
// convert_material, RenderBridge.cpp:324-370
Mat convert_material(const phc_material &in)
{
  Mat m;
  m.base_color = {in.base_color[0], in.base_color[1], in.base_color[2]};
  m.metallic = in.metallic;
  m.roughness = in.roughness * in.roughness;
  m.ior = in.ior;
  m.transmission = in.transmission;
  m.specular = 0.5f * in.specular;
  m.clearcoat = in.clearcoat;
  m.clearcoat_roughness = in.clearcoat_roughness;
  m.sheen = in.sheen;
  m.emission = {in.emission[0], in.emission[1], in.emission[2]};
  m.emission_strength = 1.f;
  m.alpha = in.opacity;
  auto cs = [](const phc_param_source &s) {
    Src o;
    o.kind = s.kind == 1 ? K_ATTR : (s.kind == 2 ? K_SAMPLER : K_CONST);
    o.index = s.index;
    return o;
  };
  m.base_color_src = cs(in.base_color_src);
  m.alpha_src = cs(in.opacity_src);
  m.metallic_src = cs(in.metallic_src);
  m.roughness_src = cs(in.roughness_src);
  m.emission_src = cs(in.emission_src);
  m.transmission_src = cs(in.transmission_src);
  m.normal_src = cs(in.normal_src);
  m.roughness_src_squared = 1;
  m.base_color_alpha = in.base_color_alpha ? 1 : 0;
  if (m.alpha_src.kind != K_CONST)
    m.alpha = 1.f;
  m.alpha_mode = in.alpha_mode == 0 ? A_BLEND : (in.alpha_mode == 2 ? A_MASK : A_OPAQUE);
  m.alpha_cutoff = in.alpha_cutoff;
  m.thin = in.thin_walled ? 1 : 0;
  m.flags = F_REFRACTIVE;
  if (in.emitter_only)
    m.flags |= F_EMITTER_ONLY;
  if (in.hidden_to_camera)
    m.flags |= F_HIDDEN;
  if (in.emission_side == 2)
    m.flags |= F_EMIT_BOTH;
  else if (in.emission_side == 1)
    m.flags |= F_EMIT_BACK;
  return m;
}

// A pt::Material given at the path tracer's level (pbrt_to_photon.cpp:98-170):
// taken as it is, the other fields keep the Material{} defaults.
Mat pt_material(const phc_pt_material &in, u32 texture_count)
{
  Mat m;
  m.base_color = {in.base_color[0], in.base_color[1], in.base_color[2]};
  m.metallic = in.metallic;
  m.roughness = in.roughness;
  m.ior = in.ior;
  m.transmission = in.transmission;
  m.specular = in.specular;
  m.clearcoat = in.clearcoat;
  m.clearcoat_roughness = in.clearcoat_roughness;
  m.sheen = in.sheen;
  m.alpha = in.alpha;
  m.emission = {in.emission[0], in.emission[1], in.emission[2]};
  m.emission_strength = in.emission_strength;
  m.flags = in.flags & (F_EMITTER_ONLY | F_HIDDEN | F_EMIT_BOTH | F_REFRACTIVE | F_EMIT_BACK);
  m.base_color_tex = texture_count ? (in.base_color_tex < 0 ? -1 : in.base_color_tex) : -1;
  m.alpha_tex = texture_count ? (in.alpha_tex < 0 ? -1 : in.alpha_tex) : -1;
  return m;
}

// ----------------------------------------------------------- disney_bsdf.h
inline f32 saturate(f32 x) { return std::fmin(1.f, std::fmax(0.f, x)); }
inline f32 dielectric_f0(f32 ior)
{
  const f32 a = (1.f - ior) / (1.f + ior);
  return a * a;
}
inline V3 schlick(f32 c, const V3 &F0, const V3 &F90)
{
  const f32 m = 1.f - saturate(c);
  const f32 m2 = m * m;
  const f32 m5 = m2 * m2 * m;
  return F0 + (F90 - F0) * m5;
}
inline V3 schlick1(f32 c, const V3 &F0)
{
  const f32 m = 1.f - saturate(c);
  const f32 m2 = m * m;
  const f32 m5 = m2 * m2 * m;
  return F0 + (V3{1.f, 1.f, 1.f} - F0) * m5;
}
inline f32 fresnel_dielectric(f32 cos_i, f32 eta)
{
  cos_i = saturate(cos_i);
  const f32 sin2_t = eta * eta * (1.f - cos_i * cos_i);
  if (sin2_t >= 1.f)
    return 1.f;
  const f32 cos_t = std::sqrt(1.f - sin2_t);
  const f32 r_par = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
  const f32 r_perp = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
  return 0.5f * (r_par * r_par + r_perp * r_perp);
}
inline f32 D_ggx(f32 NoH, f32 a)
{
  const f32 a2 = a * a;
  const f32 d = NoH * NoH * (a2 - 1.f) + 1.f;
  return a2 / (PI * d * d);
}
inline f32 D_ggx_aniso(f32 NoH, f32 XoH, f32 YoH, f32 ax, f32 ay)
{
  const f32 d = (XoH * XoH) / (ax * ax) + (YoH * YoH) / (ay * ay) + NoH * NoH;
  return 1.f / (PI * ax * ay * d * d);
}
inline f32 G1(f32 NoV, f32 a)
{
  const f32 a2 = a * a;
  const f32 denom = NoV + std::sqrt(a2 + (1.f - a2) * NoV * NoV);
  if (denom <= 0.f)
    return 0.f;
  return (2.f * NoV) / denom;
}
inline f32 G2(f32 NoV, f32 NoL, f32 a) { return G1(NoV, a) * G1(NoL, a); }
inline f32 ggx_pdf_refl(f32 NoH, f32 VoH, f32 a)
{
  const f32 D = D_ggx(NoH, a);
  const f32 denom = 4.f * std::fmax(VoH, 1e-7f);
  return D * NoH / denom;
}
inline f32 spec_scale(const Mat &m) { return std::fmax(2.f * m.specular, 0.f); }
inline void spec_f0_f90(const Mat &m, V3 &F0, V3 &F90)
{
  const f32 scale = spec_scale(m);
  const f32 opaque = 1.f - saturate(m.transmission);
  const f32 f0d = std::fmin(dielectric_f0(m.ior) * scale, 1.f) * opaque;
  V3 F0d{f0d, f0d, f0d};
  if (m.specular_tint > 0.f) {
    const f32 lum = 0.2126f * m.base_color.x + 0.7152f * m.base_color.y + 0.0722f * m.base_color.z;
    const V3 tint = lum > 0.f ? m.base_color * (1.f / lum) : V3{1.f, 1.f, 1.f};
    F0d = lerp(F0d, tint * f0d, m.specular_tint);
  }
  F0 = lerp(F0d, m.base_color, m.metallic);
  const f32 f90d = std::fmin(scale, 1.f) * opaque;
  F90 = lerp(V3{f90d, f90d, f90d}, V3{1.f, 1.f, 1.f}, m.metallic);
}
inline f32 diffuse_scale(const Mat &m, f32 NoV)
{
  const f32 scale = spec_scale(m);
  const f32 f0d = std::fmin(dielectric_f0(m.ior) * scale, 1.f);
  const f32 f90d = std::fmin(scale, 1.f);
  const f32 c = 1.f - saturate(NoV);
  const f32 c2 = c * c;
  return 1.f - (f0d + (f90d - f0d) * c2 * c2 * c);
}
inline bool spec_is_delta(const Mat &m) { return m.roughness < 0.001f; }
inline void lobe_weights(const Mat &m, f32 NoV, f32 &wd, f32 &ws, f32 &wt, f32 &wc)
{
  const f32 opaque = 1.f - saturate(m.transmission);
  const f32 dielectric = 1.f - saturate(m.metallic);
  const f32 diffuse_energy = dielectric * opaque * diffuse_scale(m, NoV);
  const f32 base_lum = 0.2126f * m.base_color.x + 0.7152f * m.base_color.y + 0.0722f * m.base_color.z;
  wd = diffuse_energy > 0.f ? diffuse_energy * std::fmax(base_lum, 0.05f) : 0.f;
  if (m.sheen > 0.f && dielectric * opaque > 0.f)
    wd += 0.1f * m.sheen;
  V3 F0, F90;
  spec_f0_f90(m, F0, F90);
  const V3 F = schlick(NoV, F0, F90);
  const f32 spec = 0.2126f * F.x + 0.7152f * F.y + 0.0722f * F.z;
  ws = spec > 0.f ? std::fmax(spec, 0.05f) : 0.f;
  wt = saturate(m.transmission) * dielectric;
  wc = 0.f;
  if (m.clearcoat > 0.f) {
    const f32 c = 1.f - saturate(NoV);
    const f32 c2 = c * c;
    wc = std::fmax(m.clearcoat * 0.25f * (0.04f + 0.96f * c2 * c2 * c), 0.02f);
  }
}
inline V3 eval_diffuse(const Mat &m, f32 NoL, f32 NoV)
{
  const f32 w = (1.f - m.metallic) * (1.f - m.transmission) * diffuse_scale(m, NoV);
  if (w <= 0.f)
    return {0.f, 0.f, 0.f};
  if (m.subsurface > 0.f) {
    const V3 d = m.base_color * (w * INV_PI * NoL);
    const f32 Fd90 = 0.5f;
    const f32 c = 1.f - NoL;
    const f32 Fss = 1.f + (Fd90 - 1.f) * c * c * c * c * c;
    const f32 ss = 1.25f * (Fss * (1.f / (NoL + 0.001f) - 0.5f) + 0.5f);
    const V3 ssc = lerp(m.base_color, m.subsurface_color, m.subsurface);
    return lerp(d, ssc * (w * INV_PI * NoL * ss), m.subsurface);
  }
  return m.base_color * (w * INV_PI * NoL);
}
inline V3 eval_spec(const Mat &m, const V3 &wo, const V3 &wi, const V3 &n, f32 a)
{
  const f32 NoV = saturate(dot(n, wo));
  const f32 NoL = saturate(dot(n, wi));
  if (NoV <= 0.f || NoL <= 0.f)
    return {0.f, 0.f, 0.f};
  const V3 h = normalize(wi + wo);
  const f32 NoH = saturate(dot(n, h));
  const f32 VoH = saturate(dot(wo, h));
  V3 F0, F90;
  spec_f0_f90(m, F0, F90);
  const V3 F = schlick(VoH, F0, F90);
  f32 D, G;
  if (m.anisotropic > 0.f) {
    const f32 aspect = std::sqrt(1.f - 0.9f * m.anisotropic);
    const f32 ax = std::fmax(a / aspect, 0.001f);
    const f32 ay = std::fmax(a * aspect, 0.001f);
    V3 t, b;
    onb(n, t, b);
    D = D_ggx_aniso(NoH, dot(t, h), dot(b, h), ax, ay);
    G = G2(NoV, NoL, ax) * G2(NoV, NoL, ay);
    G = std::sqrt(G);
  } else {
    D = D_ggx(NoH, a);
    G = G2(NoV, NoL, a);
  }
  const f32 denom = 4.f * std::fmax(NoV, 1e-7f);
  return F * (D * G / denom);
}
inline V3 eval_sheen(const Mat &m, const V3 &wo, const V3 &wi, const V3 &n)
{
  if (m.sheen <= 0.f || m.metallic >= 1.f)
    return {0.f, 0.f, 0.f};
  const V3 h = normalize(wi + wo);
  const f32 HoL = std::fabs(dot(h, wi));
  const f32 lum = 0.2126f * m.base_color.x + 0.7152f * m.base_color.y + 0.0722f * m.base_color.z;
  const V3 tint = lum > 0.f ? m.base_color * (1.f / lum) : V3{1.f, 1.f, 1.f};
  const V3 c_sheen = lerp(V3{1.f, 1.f, 1.f}, tint, m.sheen_tint);
  const f32 c = 1.f - HoL;
  const f32 c2 = c * c;
  const f32 c5 = c2 * c2 * c;
  const f32 NoL = saturate(dot(n, wi));
  const f32 w = (1.f - m.metallic) * (1.f - m.transmission);
  return c_sheen * (m.sheen * c5 * w * NoL);
}
inline V3 eval_coat(const Mat &m, const V3 &wo, const V3 &wi, const V3 &n)
{
  if (m.clearcoat <= 0.f)
    return {0.f, 0.f, 0.f};
  const f32 NoV = saturate(dot(n, wo));
  const f32 NoL = saturate(dot(n, wi));
  if (NoV <= 0.f || NoL <= 0.f)
    return {0.f, 0.f, 0.f};
  const f32 a = std::fmax(m.clearcoat_roughness, 0.001f);
  const V3 h = normalize(wi + wo);
  const f32 NoH = saturate(dot(n, h));
  const f32 VoH = saturate(dot(wo, h));
  const f32 F0 = dielectric_f0(1.5f);
  const V3 F = schlick1(VoH, V3{F0, F0, F0});
  const f32 D = D_ggx(NoH, a);
  const f32 G = G2(NoV, NoL, a);
  const f32 denom = 4.f * std::fmax(NoV, 1e-7f);
  const f32 w = m.clearcoat * 0.25f;
  return F * (w * D * G / denom);
}
V3 bsdf_eval(const Mat &m, const V3 &wo, const V3 &wi, const V3 &n, const V3 &sn) // disney_bsdf.h:288-307
{
  if (dot(wo, n) <= 0.f || dot(wi, n) <= 0.f)
    return {0.f, 0.f, 0.f};
  const f32 NoL = saturate(dot(sn, wi));
  const f32 NoV = saturate(dot(sn, wo));
  if (NoL <= 0.f || NoV <= 0.f)
    return {0.f, 0.f, 0.f};
  const f32 a = std::fmax(m.roughness, 0.001f);
  V3 f = eval_diffuse(m, NoL, NoV);
  if (!spec_is_delta(m))
    f = f + eval_spec(m, wo, wi, sn, a);
  f = f + eval_sheen(m, wo, wi, sn);
  f = f + eval_coat(m, wo, wi, sn);
  return f;
}
f32 bsdf_pdf(const Mat &m, const V3 &wo, const V3 &wi, const V3 &n, const V3 &sn) // disney_bsdf.h:310-355
{
  if (dot(wo, n) <= 0.f || dot(wi, n) <= 0.f)
    return 0.f;
  const f32 NoL = saturate(dot(sn, wi));
  const f32 NoV = saturate(dot(sn, wo));
  if (NoL <= 0.f || NoV <= 0.f)
    return 0.f;
  const f32 a = std::fmax(m.roughness, 0.001f);
  f32 wd, ws, wt, wc;
  lobe_weights(m, NoV, wd, ws, wt, wc);
  const f32 sum = wd + ws + wt + wc;
  if (sum <= 0.f)
    return 0.f;
  const f32 pd = wd / sum, ps = ws / sum, pc = wc / sum;
  f32 pdf = 0.f;
  if (pd > 0.f)
    pdf += pd * (NoL * INV_PI);
  if (ps > 0.f && !spec_is_delta(m)) {
    const V3 h = normalize(wi + wo);
    pdf += ps * ggx_pdf_refl(saturate(dot(sn, h)), saturate(dot(wo, h)), a);
  }
  if (pc > 0.f) {
    const V3 h = normalize(wi + wo);
    pdf += pc * ggx_pdf_refl(saturate(dot(sn, h)), saturate(dot(wo, h)), std::fmax(m.clearcoat_roughness, 0.001f));
  }
  return std::fmax(pdf, 0.f);
}
inline V3 ggx_half(const V3 &n, f32 a, Rng &rng) // disney_bsdf.h:357-375
{
  V3 t, b;
  onb(n, t, b);
  const f32 r1 = rng.next_f32();
  const f32 r2 = rng.next_f32();
  const f32 a2 = a * a;
  const f32 ct = std::sqrt((1.f - r1) / (1.f + (a2 - 1.f) * r1));
  const f32 st = std::sqrt(std::fmax(0.f, 1.f - ct * ct));
  const f32 phi = 2.f * PI * r2;
  return normalize(t * (st * lm::cos(phi)) + b * (st * lm::sin(phi)) + n * ct);
}
struct BS {
  V3 wi, f;
  f32 pdf{0.f};
  bool spec{false}, diff{false};
};
BS bsdf_sample(const Mat &m, const V3 &wo, const V3 &n, const V3 &sn, Rng &rng) // disney_bsdf.h:381-521
{
  BS out;
  const bool front = dot(wo, n) > 0.f;
  if (!front && m.transmission <= 0.f)
    return out;
  const f32 rough = std::fmax(m.roughness, 0.001f);
  const f32 NoV = saturate(std::fabs(dot(sn, wo)));
  f32 wd, ws, wt, wc;
  f32 t_energy = 1.f;
  if (!front) {
    wd = 0.f;
    ws = 0.f;
    wt = 1.f;
    wc = 0.f;
  } else {
    lobe_weights(m, NoV, wd, ws, wt, wc);
    t_energy = wt;
  }
  const f32 sum = wd + ws + wt + wc;
  if (sum <= 0.f)
    return out;
  const f32 pd = wd / sum, ps = ws / sum, pt = wt / sum, pc = wc / sum;
  const f32 xi = rng.next_f32();
  if (xi < pd) {
    out.wi = cosine_hemisphere(sn, rng);
    out.diff = true;
    out.f = bsdf_eval(m, wo, out.wi, n, sn);
    out.pdf = bsdf_pdf(m, wo, out.wi, n, sn);
    return out;
  }
  if (xi < pd + ps) {
    if (spec_is_delta(m)) {
      out.wi = reflect(-wo, sn);
      if (dot(out.wi, n) <= 0.f)
        out.wi = reflect(-wo, n);
      if (dot(out.wi, n) <= 0.f)
        return BS{};
      V3 F0, F90;
      spec_f0_f90(m, F0, F90);
      out.f = schlick(saturate(dot(wo, sn)), F0, F90) * (1.f / ps);
      out.pdf = 1.f;
      out.spec = true;
      return out;
    }
    const V3 h = ggx_half(sn, rough, rng);
    out.wi = reflect(-wo, h);
    if (dot(out.wi, n) <= 0.f)
      return BS{};
    out.f = bsdf_eval(m, wo, out.wi, n, sn);
    out.pdf = bsdf_pdf(m, wo, out.wi, n, sn);
    return out;
  }
  if (xi < pd + ps + pt && m.transmission > 0.f) {
    const V3 nn = front ? n : n * -1.f;
    V3 snf = front ? sn : sn * -1.f;
    if (dot(snf, wo) <= 0.f)
      snf = nn;
    V3 h = snf;
    if (m.roughness >= 0.001f) {
      h = ggx_half(snf, rough, rng);
      if (dot(h, wo) <= 0.f)
        h = snf;
    }
    const bool refractive = (m.flags & F_REFRACTIVE) != 0 && m.thin == 0;
    const f32 ior = std::fmax(m.ior, 1.0001f);
    const f32 eta = refractive ? (front ? (1.f / ior) : ior) : 1.f;
    const f32 cos_i = saturate(dot(wo, h));
    f32 F;
    if (refractive) {
      F = fresnel_dielectric(cos_i, eta);
    } else {
      const f32 f0 = dielectric_f0(m.ior);
      F = f0 + (1.f - f0) * lm::pow(1.f - cos_i, 5.f);
    }
    const f32 lobe_weight = t_energy / pt;
    out.pdf = 1.f;
    out.spec = true;
    if (rng.next_f32() < F) {
      out.wi = reflect(-wo, h);
      if (dot(out.wi, nn) <= 0.f)
        out.wi = reflect(-wo, nn);
      if (dot(out.wi, nn) <= 0.f)
        return BS{};
      out.f = V3{1.f, 1.f, 1.f} * lobe_weight;
      return out;
    }
    if (refractive) {
      out.wi = normalize(refract(-wo, h, eta));
      if (dot(out.wi, nn) >= 0.f)
        out.wi = normalize(refract(-wo, snf, eta));
      if (dot(out.wi, nn) >= 0.f)
        return BS{};
    } else {
      out.wi = normalize(-wo);
    }
    out.f = m.base_color * lobe_weight;
    return out;
  }
  if (pc > 0.f) {
    const V3 h = ggx_half(sn, std::fmax(m.clearcoat_roughness, 0.001f), rng);
    out.wi = reflect(-wo, h);
    if (dot(out.wi, n) <= 0.f)
      return BS{};
    out.f = bsdf_eval(m, wo, out.wi, n, sn);
    out.pdf = bsdf_pdf(m, wo, out.wi, n, sn);
    return out;
  }
  return out;
}

// ----------------------------------------------------------------- lights
enum { L_POINT = 0, L_DIR = 1, L_SPOT = 2 };
struct Light { // light.h:19-35, fields the bridge fills (RenderBridge.cpp:573-592)
  i32 type{L_POINT};
  V3 position, direction{0.f, -1.f, 0.f}, color{1.f, 1.f, 1.f};
  f32 intensity{1.f}, spot_angle{0.5f}, spot_falloff{0.1f}, radius{0.f};
};
struct LS {
  V3 wi, Li;
  f32 pdf{0.f}, dist{0.f};
};
inline f32 clampf(f32 x, f32 a, f32 b) { return x < a ? a : (x > b ? b : x); }
inline V3 sphere_point(const Light &l, const V3 &p, Rng &rng) // light.h:52-61
{
  if (l.radius <= 0.f)
    return l.position;
  const V3 axis = normalize(l.position - p);
  V3 t, b;
  onb(axis, t, b);
  const V2 d = concentric_disk(rng);
  return l.position + (t * d.x + b * d.y) * l.radius;
}
LS sample_light(const Light &l, const V3 &p, Rng &rng) // light.h:66-142 (point, directional, spot)
{
  if (l.type == L_POINT) {
    const V3 center_to = l.position - p;
    const f32 cd2 = dot(center_to, center_to);
    const V3 to = sphere_point(l, p, rng) - p;
    const f32 dist = length(to);
    const V3 wi = dist > 0.f ? (to * (1.f / dist)) : V3{0.f, 1.f, 0.f};
    const f32 inv = cd2 > 0.f ? (1.f / cd2) : 0.f;
    return {wi, l.color * (l.intensity * inv), 1.f, dist};
  }
  if (l.type == L_DIR) {
    V3 wi = -normalize(l.direction);
    if (l.radius > 0.f) {
      const f32 cos_max = lm::cos(l.radius);
      const f32 ct = 1.f - rng.next_f32() * (1.f - cos_max);
      const f32 st = std::sqrt(std::fmax(0.f, 1.f - ct * ct));
      const f32 phi = TWO_PI * rng.next_f32();
      V3 t, b;
      onb(wi, t, b);
      wi = normalize(t * (st * lm::cos(phi)) + b * (st * lm::sin(phi)) + wi * ct);
    }
    return {wi, l.color * l.intensity, 1.f, 1e30f};
  }
  // spot
  const V3 center_to = l.position - p;
  const f32 cd2 = dot(center_to, center_to);
  const V3 to = sphere_point(l, p, rng) - p;
  const f32 dist = length(to);
  const V3 wi = dist > 0.f ? (to * (1.f / dist)) : V3{0.f, 1.f, 0.f};
  const V3 spot_dir = normalize(l.direction);
  const V3 from_light = -normalize(center_to);
  const f32 cos_angle = dot(from_light, spot_dir);
  const f32 cos_inner = lm::cos(std::fmax(l.spot_angle - l.spot_falloff, 0.f));
  const f32 cos_outer = lm::cos(l.spot_angle);
  f32 falloff = 0.f;
  if (cos_angle >= cos_inner)
    falloff = 1.f;
  else if (cos_angle <= cos_outer)
    falloff = 0.f;
  else {
    const f32 t = clampf((cos_angle - cos_outer) / (cos_inner - cos_outer), 0.f, 1.f);
    falloff = t * t * (3.f - 2.f * t);
  }
  const f32 inv = cd2 > 0.f ? (1.f / cd2) : 0.f;
  return {wi, l.color * (l.intensity * inv * falloff), 1.f, dist};
}

// -------------------------------------------------------- environment map
struct Env {
  u32 width{0}, height{0};
  std::vector<V3> pixels;       // (y, x)
  std::vector<f32> marginal;    // height + 1
  std::vector<f32> conditional; // height x (width + 1)
  f32 w2t[9]{1, 0, 0, 0, 1, 0, 0, 0, 1}, t2w[9]{1, 0, 0, 0, 1, 0, 0, 0, 1};
  f32 cond(u32 r, u32 c) const { return conditional[size_t(r) * (width + 1) + c]; }
  V3 to_tex(const V3 &d) const
  {
    return {w2t[0] * d.x + w2t[1] * d.y + w2t[2] * d.z, w2t[3] * d.x + w2t[4] * d.y + w2t[5] * d.z,
        w2t[6] * d.x + w2t[7] * d.y + w2t[8] * d.z};
  }
  V3 to_world(const V3 &d) const
  {
    return {t2w[0] * d.x + t2w[1] * d.y + t2w[2] * d.z, t2w[3] * d.x + t2w[4] * d.y + t2w[5] * d.z,
        t2w[6] * d.x + t2w[7] * d.y + t2w[8] * d.z};
  }
  static V2 dir_to_uv(const V3 &d) // environment_map.h:138-147
  {
    const V3 nd = normalize(d);
    const f32 phi = lm::atan2(nd.z, nd.x);
    const f32 y = clampf(nd.y, -1.f, 1.f);
    const f32 theta = lm::acos(y);
    return {(phi + PI) * INV_TWO_PI, theta * INV_PI};
  }
  static V3 uv_to_dir(const V2 &uv) // environment_map.h:149-155
  {
    const f32 phi = uv.x * TWO_PI - PI;
    const f32 theta = uv.y * PI;
    const f32 st = lm::sin(theta);
    return {st * lm::cos(phi), lm::cos(theta), st * lm::sin(phi)};
  }
  void texel(const V3 &direction, u32 &x, u32 &y, V2 &uv) const
  {
    uv = dir_to_uv(to_tex(direction));
    const f32 xf = uv.x * (f32)width;
    const f32 yf = uv.y * (f32)height;
    x = (u32)std::fmin((f32)(width - 1), std::fmax(0.f, xf));
    y = (u32)std::fmin((f32)(height - 1), std::fmax(0.f, yf));
  }
  V3 evaluate(const V3 &d) const // environment_map.h:40-54
  {
    if (width == 0 || height == 0)
      return {0.f, 0.f, 0.f};
    u32 x, y;
    V2 uv;
    texel(d, x, y, uv);
    return pixels[size_t(y) * width + x];
  }
  V3 sample(Rng &rng, f32 &pdf_out) const // environment_map.h:56-115
  {
    pdf_out = 0.f;
    if (width == 0 || height == 0)
      return {0.f, 1.f, 0.f};
    const f32 u1 = rng.next_f32();
    const f32 u2 = rng.next_f32();
    u32 lo = 0, hi = height;
    while (lo + 1 < hi) {
      const u32 mid = (lo + hi) / 2;
      if (marginal[mid] <= u2)
        lo = mid;
      else
        hi = mid;
    }
    const u32 row = lo;
    lo = 0;
    hi = width;
    while (lo + 1 < hi) {
      const u32 mid = (lo + hi) / 2;
      if (cond(row, mid) <= u1)
        lo = mid;
      else
        hi = mid;
    }
    const u32 col = lo;
    const f32 row_pdf = marginal[row + 1] - marginal[row];
    const f32 col_pdf = cond(row, col + 1) - cond(row, col);
    const f32 u = ((f32)col + rng.next_f32()) / (f32)width;
    const f32 v = ((f32)row + rng.next_f32()) / (f32)height;
    const V3 dir = to_world(uv_to_dir(V2{u, v}));
    const f32 theta = v * PI;
    const f32 denom = TWO_PI * PI * std::fmax(lm::sin(theta), 1e-6f);
    pdf_out = (row_pdf * col_pdf) * (f32)width * (f32)height / denom;
    return dir;
  }
  f32 pdf(const V3 &d) const // environment_map.h:117-136
  {
    if (width == 0 || height == 0)
      return 0.f;
    u32 x, y;
    V2 uv;
    texel(d, x, y, uv);
    const f32 row_pdf = marginal[y + 1] - marginal[y];
    const f32 col_pdf = cond(y, x + 1) - cond(y, x);
    const f32 theta = uv.y * PI;
    const f32 denom = TWO_PI * PI * std::fmax(lm::sin(theta), 1e-6f);
    return (row_pdf * col_pdf) * (f32)width * (f32)height / denom;
  }
  void build_cdf() // environment_map.cpp:8-65
  {
    marginal.assign(height + 1, 0.f);
    conditional.assign(size_t(height) * (width + 1), 0.f);
    std::vector<f32> row_w(height, 0.f);
    marginal[0] = 0.f;
    for (u32 y = 0; y < height; ++y) {
      f32 *c = &conditional[size_t(y) * (width + 1)];
      c[0] = 0.f;
      const f32 theta = ((f32)y + 0.5f) * (PI / (f32)height);
      const f32 st = lm::sin(theta);
      f32 sum = 0.f;
      for (u32 x = 0; x < width; ++x) {
        sum += luminance(pixels[size_t(y) * width + x]);
        c[x + 1] = sum;
      }
      if (sum > 0.f) {
        const f32 inv = 1.f / sum;
        for (u32 x = 0; x <= width; ++x)
          c[x] *= inv;
        c[width] = 1.f;
      } else {
        for (u32 x = 0; x <= width; ++x)
          c[x] = (f32)x / (f32)width;
      }
      row_w[y] = sum * st;
    }
    f32 total = 0.f;
    for (u32 y = 0; y < height; ++y) {
      total += row_w[y];
      marginal[y + 1] = total;
    }
    if (total > 0.f) {
      const f32 inv = 1.f / total;
      for (u32 y = 0; y <= height; ++y)
        marginal[y] *= inv;
      marginal[height] = 1.f;
    } else {
      for (u32 y = 0; y <= height; ++y)
        marginal[y] = (f32)y / (f32)height;
    }
  }
};

// ---------------------------------------------------------------- volumes
struct Vol { // tf_volume.h:14-33
  f32 w2l[12]{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  V3 origin, spacing{1.f, 1.f, 1.f};
  u32 dims[3]{1, 1, 1};
  u32 data_offset{0}, tf_offset{0}, tf_size{0};
  f32 value_lo{0.f}, value_hi{1.f}, density_scale{1.f}, majorant{0.f};
  u32 linear{1};
  u32 macro_offset{0};
  u32 macro_dims[3]{1, 1, 1};
};
struct VolSet {
  std::vector<Vol> vols;
  std::vector<f32> values;
  std::vector<V4> tf;
  std::vector<f32> majorants;

  static V3 lp(const Vol &v, const V3 &p)
  {
    const f32 *m = v.w2l;
    return {m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
        m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]};
  }
  static V3 lv(const Vol &v, const V3 &d)
  {
    const f32 *m = v.w2l;
    return {m[0] * d.x + m[1] * d.y + m[2] * d.z, m[4] * d.x + m[5] * d.y + m[6] * d.z,
        m[8] * d.x + m[9] * d.y + m[10] * d.z};
  }
  static bool clip(const Vol &v, const V3 &org, const V3 &dir, f32 &t0, f32 &t1) // tf_volume.h:58-82
  {
    const f32 o[3] = {org.x, org.y, org.z}, d[3] = {dir.x, dir.y, dir.z};
    const f32 lo[3] = {v.origin.x, v.origin.y, v.origin.z}, sp[3] = {v.spacing.x, v.spacing.y, v.spacing.z};
    for (int a = 0; a < 3; ++a) {
      const f32 hi = lo[a] + sp[a] * f32(v.dims[a] > 1 ? v.dims[a] - 1 : 1);
      if (d[a] == 0.f) {
        if (o[a] < lo[a] || o[a] > hi)
          return false;
        continue;
      }
      const f32 inv = 1.f / d[a];
      const f32 ta = (lo[a] - o[a]) * inv;
      const f32 tb = (hi - o[a]) * inv;
      const f32 tn = ta < tb ? ta : tb;
      const f32 tf = ta < tb ? tb : ta;
      t0 = tn > t0 ? tn : t0;
      t1 = tf < t1 ? tf : t1;
      if (t1 <= t0)
        return false;
    }
    return true;
  }
  f32 field(const Vol &v, const V3 &p) const // tf_volume.h:84-123
  {
    const f32 g[3] = {(p.x - v.origin.x) / v.spacing.x, (p.y - v.origin.y) / v.spacing.y,
        (p.z - v.origin.z) / v.spacing.z};
    int i0[3], i1[3];
    f32 fr[3];
    for (int a = 0; a < 3; ++a) {
      const int n = int(v.dims[a]);
      f32 x = g[a];
      x = x < 0.f ? 0.f : (x > f32(n - 1) ? f32(n - 1) : x);
      if (v.linear) {
        int i = int(x);
        if (i > n - 2)
          i = n - 2;
        if (i < 0)
          i = 0;
        i0[a] = i;
        i1[a] = i + 1 < n ? i + 1 : i;
        fr[a] = x - f32(i);
      } else {
        int i = int(x + 0.5f);
        i = i > n - 1 ? n - 1 : i;
        i0[a] = i1[a] = i;
        fr[a] = 0.f;
      }
    }
    const u32 sx = v.dims[0], sxy = v.dims[0] * v.dims[1], base = v.data_offset;
    auto at = [&](int x, int y, int z) { return values[base + u32(z) * sxy + u32(y) * sx + u32(x)]; };
    if (!v.linear)
      return at(i0[0], i0[1], i0[2]);
    const f32 c00 = at(i0[0], i0[1], i0[2]) * (1.f - fr[0]) + at(i1[0], i0[1], i0[2]) * fr[0];
    const f32 c10 = at(i0[0], i1[1], i0[2]) * (1.f - fr[0]) + at(i1[0], i1[1], i0[2]) * fr[0];
    const f32 c01 = at(i0[0], i0[1], i1[2]) * (1.f - fr[0]) + at(i1[0], i0[1], i1[2]) * fr[0];
    const f32 c11 = at(i0[0], i1[1], i1[2]) * (1.f - fr[0]) + at(i1[0], i1[1], i1[2]) * fr[0];
    const f32 c0 = c00 * (1.f - fr[1]) + c10 * fr[1];
    const f32 c1 = c01 * (1.f - fr[1]) + c11 * fr[1];
    return c0 * (1.f - fr[2]) + c1 * fr[2];
  }
  V4 classify(const Vol &v, const V3 &p) const // tf_volume.h:126-143
  {
    const f32 value = field(v, p);
    const f32 range = v.value_hi - v.value_lo;
    f32 x = range != 0.f ? (value - v.value_lo) / range : 0.f;
    x = x < 0.f ? 0.f : (x > 1.f ? 1.f : x);
    const f32 f = x * f32(v.tf_size - 1);
    u32 i = u32(f);
    if (i > v.tf_size - 2)
      i = v.tf_size >= 2 ? v.tf_size - 2 : 0;
    const f32 fr = v.tf_size >= 2 ? f - f32(i) : 0.f;
    const V4 a = tf[v.tf_offset + i];
    const V4 b = tf[v.tf_offset + (v.tf_size >= 2 ? i + 1 : i)];
    V4 c = a * (1.f - fr) + b * fr;
    c.w = c.w * v.density_scale;
    return c;
  }
  f32 track(const Vol &v, const V3 &org, const V3 &dir, f32 t0, f32 t1, Rng &rng, bool scatter, V3 &albedo,
      f32 &tr) const // tf_volume.h:150-232
  {
    const f32 o[3] = {org.x, org.y, org.z}, d[3] = {dir.x, dir.y, dir.z};
    const f32 lo[3] = {v.origin.x, v.origin.y, v.origin.z}, sp[3] = {v.spacing.x, v.spacing.y, v.spacing.z};
    int cell[3], step[3];
    f32 t_next[3], t_delta[3];
    for (int a = 0; a < 3; ++a) {
      const int m = int(v.macro_dims[a]);
      const f32 extent = sp[a] * f32(v.dims[a] > 1 ? v.dims[a] - 1 : 1);
      const f32 cpu = f32(m) / extent;
      const f32 g = (o[a] + d[a] * t0 - lo[a]) * cpu;
      int c = int(g);
      c = c < 0 ? 0 : (c > m - 1 ? m - 1 : c);
      cell[a] = c;
      const f32 speed = d[a] * cpu;
      if (speed > 0.f) {
        step[a] = 1;
        t_delta[a] = 1.f / speed;
        t_next[a] = t0 + (f32(c + 1) - g) * t_delta[a];
      } else if (speed < 0.f) {
        step[a] = -1;
        t_delta[a] = -1.f / speed;
        t_next[a] = t0 + (g - f32(c)) * t_delta[a];
      } else {
        step[a] = 0;
        t_delta[a] = 1e30f;
        t_next[a] = 1e30f;
      }
    }
    f32 t = t0;
    int lookups = 0;
    for (int visited = 0; visited < 4096; ++visited) {
      const int axis =
          t_next[0] < t_next[1] ? (t_next[0] < t_next[2] ? 0 : 2) : (t_next[1] < t_next[2] ? 1 : 2);
      const f32 t_exit = t_next[axis] < t1 ? t_next[axis] : t1;
      const f32 bound =
          majorants[v.macro_offset + (u32(cell[2]) * v.macro_dims[1] + u32(cell[1])) * v.macro_dims[0] + u32(cell[0])];
      if (bound > 0.f) {
        const f32 inv_bound = 1.f / bound;
        while (lookups < 8192) {
          t -= lm::log(1.f - rng.next_f32()) * inv_bound;
          if (t >= t_exit)
            break;
          ++lookups;
          const V4 c = classify(v, org + dir * t);
          if (scatter) {
            if (rng.next_f32() * bound < c.w) {
              albedo = c.xyz();
              return t;
            }
          } else {
            tr *= 1.f - c.w * inv_bound;
            if (tr < 0.05f) {
              if (!(tr > 0.f) || rng.next_f32() * 0.05f >= tr) {
                tr = 0.f;
                return -1.f;
              }
              tr = 0.05f;
            }
          }
        }
      }
      t = t_exit;
      if (t_exit >= t1 || lookups >= 8192)
        break;
      cell[axis] += step[axis];
      if (cell[axis] < 0 || cell[axis] >= int(v.macro_dims[axis]))
        break;
      t_next[axis] += t_delta[axis];
    }
    return -1.f;
  }
  f32 sample_scatter(const V3 &ro, const V3 &rd, f32 tmin, f32 tmax, Rng &rng, V3 &albedo) const
  {
    f32 t_event = -1.f, t_limit = tmax, unused = 1.f;
    for (size_t vi = 0; vi < vols.size(); ++vi) {
      const Vol &v = vols[vi];
      if (v.majorant <= 0.f || v.tf_size == 0)
        continue;
      const V3 org = lp(v, ro), dir = lv(v, rd);
      f32 t0 = tmin, t1 = t_limit;
      if (!clip(v, org, dir, t0, t1))
        continue;
      V3 ea;
      const f32 t = track(v, org, dir, t0, t1, rng, true, ea, unused);
      if (t >= 0.f) {
        t_event = t;
        t_limit = t;
        albedo = ea;
      }
    }
    return t_event;
  }
  f32 transmittance(const V3 &ro, const V3 &rd, f32 tmin, f32 tmax, Rng &rng) const
  {
    f32 tr = 1.f;
    V3 unused;
    for (size_t vi = 0; vi < vols.size(); ++vi) {
      const Vol &v = vols[vi];
      if (v.majorant <= 0.f || v.tf_size == 0)
        continue;
      const V3 org = lp(v, ro), dir = lv(v, rd);
      f32 t0 = tmin, t1 = tmax;
      if (!clip(v, org, dir, t0, t1))
        continue;
      track(v, org, dir, t0, t1, rng, false, unused, tr);
      if (tr <= 0.f)
        return 0.f;
    }
    return tr;
  }
};

// --------------------------------------------------------------- samplers
struct SInfo { // sampler.h:49-63
  i32 type{1}, in_attribute{0};
  u32 linear{1};
  i32 wrap[3]{0, 0, 0};
  u32 offset{0};
  u32 size[3]{1, 1, 1};
  f32 in_t[16], in_o[4], out_t[16], out_o[4];
};
inline i32 wrap_index(i32 i, i32 n, i32 mode) // sampler.h:73-82
{
  if (mode == 1)
    return ((i % n) + n) % n;
  if (mode == 2) {
    const i32 j = ((i % (2 * n)) + 2 * n) % (2 * n);
    return j < n ? j : 2 * n - 1 - j;
  }
  return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

// -------------------------------------------------------------------- BVH
struct Aabb {
  V3 lo{+1e30f, +1e30f, +1e30f}, hi{-1e30f, -1e30f, -1e30f};
  void extend(const V3 &p)
  {
    lo.x = lo.x < p.x ? lo.x : p.x;
    lo.y = lo.y < p.y ? lo.y : p.y;
    lo.z = lo.z < p.z ? lo.z : p.z;
    hi.x = hi.x > p.x ? hi.x : p.x;
    hi.y = hi.y > p.y ? hi.y : p.y;
    hi.z = hi.z > p.z ? hi.z : p.z;
  }
  void extend(const Aabb &b)
  {
    extend(b.lo);
    extend(b.hi);
  }
};
struct Node {
  Aabb b;
  u32 left{0}, right{0}, begin{0}, count{0}, leaf{0};
};
struct PrimRef {
  u32 id;
  Aabb b;
  V3 c;
};
struct Bvh { // bvh.cpp:20-125: median split on the largest centroid axis, leaves of <= 4
  std::vector<Node> nodes;
  std::vector<u32> prim_ids;
  u32 build_node(std::vector<PrimRef> &prims, u32 begin, u32 end)
  {
    const u32 id = u32(nodes.size());
    nodes.push_back({});
    Aabb b, cb;
    for (u32 i = begin; i < end; ++i) {
      b.extend(prims[i].b);
      cb.extend(prims[i].c);
    }
    nodes[id].b = b;
    const u32 pb = u32(prim_ids.size());
    nodes[id].count = end - begin;
    if (end - begin <= 4) {
      for (u32 i = begin; i < end; ++i)
        prim_ids.push_back(prims[i].id);
      nodes[id].begin = pb;
      nodes[id].leaf = 1;
      return id;
    }
    nodes[id].begin = begin;
    const V3 diag = cb.hi - cb.lo;
    int axis = diag.y > diag.x ? 1 : 0;
    if (diag.z > (axis == 0 ? diag.x : diag.y))
      axis = 2;
    const u32 mid = begin + (end - begin) / 2;
    auto key = [axis](const PrimRef &p) { return axis == 0 ? p.c.x : (axis == 1 ? p.c.y : p.c.z); };
    std::nth_element(prims.begin() + begin, prims.begin() + mid, prims.begin() + end,
        [&](const PrimRef &a, const PrimRef &c) { return key(a) < key(c); });
    const u32 l = build_node(prims, begin, mid);
    const u32 r = build_node(prims, mid, end);
    nodes[id].left = l;
    nodes[id].right = r;
    nodes[id].leaf = 0;
    return id;
  }
  void build(const std::vector<V3> &pos, const std::vector<u32> &idx)
  {
    const u32 n = u32(idx.size() / 3);
    std::vector<PrimRef> prims(n);
    for (u32 i = 0; i < n; ++i) {
      const V3 v0 = pos[idx[3 * i]], v1 = pos[idx[3 * i + 1]], v2 = pos[idx[3 * i + 2]];
      prims[i].id = i;
      prims[i].b = Aabb{};
      prims[i].b.extend(v0);
      prims[i].b.extend(v1);
      prims[i].b.extend(v2);
      prims[i].c = (v0 + v1 + v2) * (1.f / 3.f);
    }
    nodes.clear();
    prim_ids.clear();
    prim_ids.reserve(n);
    nodes.reserve(size_t(n) * 2);
    build_node(prims, 0, n);
  }
};

struct Mesh {
  std::vector<V3> pos, nrm;
  std::vector<u32> idx, mat_ids;
  Bvh bvh;
};

constexpr u32 NO_INST = 0xffffffffu;
struct Hit {
  bool hit{false};
  f32 t{0.f};
  u32 prim{0};
  f32 u{0.f}, v{0.f};
  u32 inst{NO_INST}; // instance of an instanced hit
};

// mesh_intersector.h:30-45
inline f32 entry_distance(const Aabb &b, const V3 &o, const V3 &inv, f32 tmin, f32 tmax)
{
  const f32 tx0 = (b.lo.x - o.x) * inv.x, tx1 = (b.hi.x - o.x) * inv.x;
  const f32 ty0 = (b.lo.y - o.y) * inv.y, ty1 = (b.hi.y - o.y) * inv.y;
  const f32 tz0 = (b.lo.z - o.z) * inv.z, tz1 = (b.hi.z - o.z) * inv.z;
  const f32 tn = std::fmax(std::fmax(std::fmin(tx0, tx1), std::fmin(ty0, ty1)), std::fmax(std::fmin(tz0, tz1), tmin));
  const f32 tf = std::fmin(std::fmin(std::fmax(tx0, tx1), std::fmax(ty0, ty1)), std::fmin(std::fmax(tz0, tz1), tmax));
  return tn <= tf ? tn : -1.f;
}
// triangle_intersect.h:18-52 (Möller–Trumbore)
inline bool tri_test(const V3 &o, const V3 &d, const V3 &v0, const V3 &v1, const V3 &v2, f32 tmin, f32 tmax,
    f32 &t, f32 &u, f32 &v)
{
  const V3 e1 = v1 - v0, e2 = v2 - v0;
  const V3 p = cross(d, e2);
  const f32 det = dot(e1, p);
  if (std::fabs(det) < 1e-30f)
    return false;
  const f32 inv_det = 1.f / det;
  const V3 tv = o - v0;
  u = dot(tv, p) * inv_det;
  if (u < 0.f || u > 1.f)
    return false;
  const V3 q = cross(tv, e1);
  v = dot(d, q) * inv_det;
  if (v < 0.f || (u + v) > 1.f)
    return false;
  t = dot(e2, q) * inv_det;
  if (t < tmin || t > tmax)
    return false;
  return true;
}
// mesh_intersector.h:57-128
Hit intersect(const Mesh &m, const V3 &o, const V3 &d, f32 tmin, f32 tmax, bool any_hit)
{
  Hit best;
  best.t = tmax;
  if (!(tmax > tmin) || m.bvh.nodes.empty())
    return best;
  auto inv1 = [](f32 x) { return 1.f / (std::fabs(x) > 1e-20f ? x : (x < 0.f ? -1e-20f : 1e-20f)); };
  const V3 inv{inv1(d.x), inv1(d.y), inv1(d.z)};
  u32 stack[64];
  int sp = 0;
  stack[sp++] = 0;
  while (sp > 0) {
    const Node &node = m.bvh.nodes[stack[--sp]];
    if (entry_distance(node.b, o, inv, tmin, best.t) < 0.f)
      continue;
    if (node.leaf) {
      for (u32 i = 0; i < node.count; ++i) {
        const u32 pid = m.bvh.prim_ids[node.begin + i];
        f32 t, u, v;
        if (!tri_test(o, d, m.pos[m.idx[3 * pid]], m.pos[m.idx[3 * pid + 1]], m.pos[m.idx[3 * pid + 2]], tmin,
                best.t, t, u, v))
          continue;
        best.t = t;
        best.prim = pid;
        best.hit = true;
        best.u = u;
        best.v = v;
        if (any_hit)
          return best;
      }
    } else if (sp + 2 <= 64) {
      const f32 dl = entry_distance(m.bvh.nodes[node.left].b, o, inv, tmin, best.t);
      const f32 dr = entry_distance(m.bvh.nodes[node.right].b, o, inv, tmin, best.t);
      if (dl >= 0.f && dr >= 0.f) {
        if (dl < dr) {
          stack[sp++] = node.right;
          stack[sp++] = node.left;
        } else {
          stack[sp++] = node.left;
          stack[sp++] = node.right;
        }
      } else if (dl >= 0.f) {
        stack[sp++] = node.left;
      } else if (dr >= 0.f) {
        stack[sp++] = node.right;
      }
    }
  }
  return best;
}

// Hit attributes, mesh_intersector.h:129-178 (no texcoords / vertex colours)
struct HitAttr {
  V3 p, n, sn;
  u32 material_id{0};
};
HitAttr hit_attributes(const Mesh &m, const V3 &o, const V3 &d, const Hit &h)
{
  HitAttr a;
  const u32 i0 = m.idx[3 * h.prim], i1 = m.idx[3 * h.prim + 1], i2 = m.idx[3 * h.prim + 2];
  const V3 v0 = m.pos[i0], v1 = m.pos[i1], v2 = m.pos[i2];
  a.p = o + d * h.t;
  const V3 nn = normalize(cross(v1 - v0, v2 - v0));
  a.n = nn;
  a.sn = nn;
  const f32 w0 = 1.f - h.u - h.v, w1 = h.u, w2 = h.v;
  if (!m.nrm.empty()) {
    a.sn = normalize(m.nrm[i0] * w0 + m.nrm[i1] * w1 + m.nrm[i2] * w2);
    if (dot(a.sn, nn) < 0.f)
      a.sn = a.sn * -1.f;
  }
  if (!m.mat_ids.empty())
    a.material_id = m.mat_ids[h.prim];
  return a;
}

// Instanced geometry (scene.h:18-39) as the reference's instanced back-end
// traces it (optix_backend.cpp:502-590, photon_optix.cu:68-99 and 161-187):
// the ray is carried into the object's space by the instance's
// world-to-object rows, the object's own BVH is intersected there (t keeps
// its meaning: the direction is not renormalised), and the hit's normals go
// back through the inverse transpose of the instance transform.
struct Obj {
  Mesh mesh;
  u32 material{0};
};
struct Inst {
  u32 obj{0};
  f32 w2o[12]; // rows of the world-to-object 3x4 matrix
  Aabb box;    // world bounds (padded)
};
inline V3 xf_point(const f32 *m, const V3 &p)
{
  return {m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
      m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]};
}
inline V3 xf_dir(const f32 *m, const V3 &d)
{
  return {m[0] * d.x + m[1] * d.y + m[2] * d.z, m[4] * d.x + m[5] * d.y + m[6] * d.z,
      m[8] * d.x + m[9] * d.y + m[10] * d.z};
}
// n' = M^T n for the world-to-object rows M: the inverse transpose of the
// object-to-world transform
inline V3 xf_normal(const f32 *m, const V3 &n)
{
  return {m[0] * n.x + m[4] * n.y + m[8] * n.z, m[1] * n.x + m[5] * n.y + m[9] * n.z,
      m[2] * n.x + m[6] * n.y + m[10] * n.z};
}

// ----------------------------------------------------------------- camera
struct Cam { // camera.h:11-160
  V3 origin, lower_left, horizontal, vertical, u, v, w;
  f32 lens_radius{0.f}, focus_dist{1.f};
  bool ortho{false};
  f32 clip_near{0.f}, clip_far{1e30f};

  static Cam perspective(const V3 &from, const V3 &at, const V3 &vup, f32 vfov, f32 aspect, f32 aperture, f32 focus)
  {
    const f32 theta = vfov * 3.1415926535f / 180.f;
    const f32 h = lm::tan(theta * 0.5f);
    const f32 vh = 2.f * h;
    const f32 vw = aspect * vh;
    Cam c;
    c.origin = from;
    c.w = normalize(from - at);
    c.u = normalize(cross(vup, c.w));
    c.v = cross(c.w, c.u);
    c.focus_dist = focus;
    c.lens_radius = aperture * 0.5f;
    c.ortho = false;
    c.horizontal = c.u * (vw * focus);
    c.vertical = c.v * (vh * focus);
    c.lower_left = c.origin - c.horizontal * 0.5f - c.vertical * 0.5f - c.w * focus;
    return c;
  }
  static Cam orthographic(const V3 &from, const V3 &at, const V3 &vup, f32 height, f32 aspect)
  {
    Cam c;
    c.origin = from;
    c.w = normalize(from - at);
    c.u = normalize(cross(vup, c.w));
    c.v = cross(c.w, c.u);
    c.focus_dist = 1.f;
    c.lens_radius = 0.f;
    c.ortho = true;
    c.horizontal = c.u * (height * aspect);
    c.vertical = c.v * height;
    c.lower_left = c.origin - c.horizontal * 0.5f - c.vertical * 0.5f;
    return c;
  }
  void clip_range(const V3 &dir, f32 &tn, f32 &tf) const
  {
    tn = 0.f;
    tf = 1e30f;
    if (clip_near <= 0.f && clip_far >= 1e30f)
      return;
    const f32 ca = dot(dir, w * -1.f);
    if (ca <= 1e-6f) {
      tn = 1.f;
      tf = 0.f;
      return;
    }
    if (clip_near > 0.f)
      tn = clip_near / ca;
    if (clip_far < 1e30f)
      tf = clip_far / ca;
  }
  void ray(f32 s, f32 t, Rng &rng, V3 &ro, V3 &rd) const
  {
    if (ortho) {
      ro = lower_left + horizontal * s + vertical * t;
      rd = -w;
      return;
    }
    if (lens_radius <= 0.f) {
      ro = origin;
      rd = normalize(lower_left + horizontal * s + vertical * t - origin);
      return;
    }
    V2 rdisk = concentric_disk(rng);
    rdisk = V2{rdisk.x * lens_radius, rdisk.y * lens_radius};
    const V3 offset = u * rdisk.x + v * rdisk.y;
    const V3 target = lower_left + horizontal * s + vertical * t;
    ro = origin + offset;
    rd = normalize(target - origin - offset);
  }
};

// ------------------------------------------------------------------ scene
struct Scene {
  Mesh mesh;
  std::vector<Mat> mats;
  // attributes: offset per slot into attr_values (RenderBridge.cpp:489-511)
  std::vector<V4> attr_values;
  i32 attr_offset[5]{-1, -1, -1, -1, -1};
  std::vector<SInfo> samplers;
  std::vector<V4> texels;
  // pt::TextureAtlas (texture.h:19-23): texel offset, width, height per texture
  std::vector<u32> atlas_off, atlas_w, atlas_h;
  std::vector<V3> atlas_px;
  std::vector<V2> uv;   // mesh.texcoords, empty: none
  std::vector<Light> lights;
  bool has_env{false}, env_visible{true};
  Env env;
  VolSet vols;
  std::vector<u32> emissive_ids;
  std::vector<f32> emissive_cdf, prim_light_pdf;
  u32 strategy_count{0};
  f32 eps{1e-3f};
  std::vector<Obj> objs; // instanced geometry
  std::vector<Inst> insts;
};

// Closest (or any) hit over the scene's triangles and every instance.
Hit intersect_scene(const Scene &sc, const V3 &o, const V3 &d, f32 tmin, f32 tmax, bool any_hit)
{
  Hit best = intersect(sc.mesh, o, d, tmin, tmax, any_hit);
  if (sc.insts.empty() || (any_hit && best.hit))
    return best;
  auto inv1 = [](f32 x) { return 1.f / (std::fabs(x) > 1e-20f ? x : (x < 0.f ? -1e-20f : 1e-20f)); };
  const V3 inv{inv1(d.x), inv1(d.y), inv1(d.z)};
  for (u32 i = 0; i < u32(sc.insts.size()); ++i) {
    const Inst &in = sc.insts[i];
    if (entry_distance(in.box, o, inv, tmin, best.t) < 0.f)
      continue;
    Hit h = intersect(sc.objs[in.obj].mesh, xf_point(in.w2o, o), xf_dir(in.w2o, d), tmin, best.t, any_hit);
    if (!h.hit)
      continue;
    h.inst = i;
    best = h;
    if (any_hit)
      return best;
  }
  return best;
}

// Hit attributes; an instanced hit's in object space, its normals carried to
// world space and normalised (photon_optix.cu:68-99, 183-186).
HitAttr hit_attributes_scene(const Scene &sc, const V3 &o, const V3 &d, const Hit &h)
{
  if (h.inst == NO_INST)
    return hit_attributes(sc.mesh, o, d, h);
  const Inst &in = sc.insts[h.inst];
  const Obj &ob = sc.objs[in.obj];
  HitAttr a = hit_attributes(ob.mesh, o, d, h);
  a.n = normalize(xf_normal(in.w2o, a.n));
  a.sn = normalize(xf_normal(in.w2o, a.sn));
  a.material_id = ob.material;
  return a;
}

struct Params {
  u32 w, h, spp, max_depth, sample_offset;
  V3 bg_color;
  f32 bg_alpha;
  std::vector<V4> bg_image; // (bh, bw)
  u32 bg_w{0}, bg_h{0};
  V3 ambient;
  bool adaptive;
  f32 tp_clamp;
  int max_diffuse, max_glossy, max_transmission, max_volume;
  f32 clamp_direct, clamp_indirect;
  bool bottom_up;
  f32 region[4];
};

// fetch_attribute / eval_source / apply_normal_map / resolve_material,
// pathtracer.cpp:97-247
struct Query {
  u32 prim{0}, material_id{0};
  f32 b1{0.f}, b2{0.f};
  V3 p, sn;
  u32 inst{NO_INST};
};
V4 fetch_attribute(const Scene &sc, i32 slot, const Query &q)
{
  if (slot == 5)
    return {q.p, 1.f};
  if (slot == 6)
    return {q.sn, 1.f};
  if (!(slot >= 0 && slot < 5 && sc.attr_offset[slot] >= 0) || q.inst != NO_INST) // instances carry none
    return {0.f, 0.f, 0.f, 1.f};
  const u32 base = u32(sc.attr_offset[slot]);
  const V4 a0 = sc.attr_values[base + sc.mesh.idx[q.prim * 3 + 0]];
  const V4 a1 = sc.attr_values[base + sc.mesh.idx[q.prim * 3 + 1]];
  const V4 a2 = sc.attr_values[base + sc.mesh.idx[q.prim * 3 + 2]];
  return a0 * (1.f - q.b1 - q.b2) + a1 * q.b1 + a2 * q.b2;
}
V4 sampler_sample(const Scene &sc, i32 id, const V4 &attr) // sampler.h:84-134
{
  if (id < 0 || u32(id) >= sc.samplers.size())
    return {0.f, 0.f, 0.f, 1.f};
  const SInfo &si = sc.samplers[u32(id)];
  V4 c = mul_mat4(si.in_t, attr);
  c.x += si.in_o[0];
  c.y += si.in_o[1];
  c.z += si.in_o[2];
  c.w += si.in_o[3];
  V4 result = c;
  if (si.type != 3) {
    const int dims = si.type == 0 ? 1 : (si.type == 1 ? 2 : 3);
    const f32 coord[3] = {c.x, c.y, c.z};
    i32 i0[3] = {0, 0, 0}, i1[3] = {0, 0, 0};
    f32 frac[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < dims; ++d) {
      const i32 n = i32(si.size[d]);
      f32 x = coord[d];
      if (!(x > -1e6f && x < 1e6f))
        x = 0.f;
      if (si.linear) {
        const f32 f = x * f32(n) - 0.5f;
        const f32 fl = std::floor(f);
        frac[d] = f - fl;
        i0[d] = wrap_index(i32(fl), n, si.wrap[d]);
        i1[d] = wrap_index(i32(fl) + 1, n, si.wrap[d]);
      } else {
        i0[d] = wrap_index(i32(std::floor(x * f32(n))), n, si.wrap[d]);
        i1[d] = i0[d];
      }
    }
    const u32 sx = si.size[0], sxy = si.size[0] * si.size[1], base = si.offset;
    V4 acc{0.f, 0.f, 0.f, 0.f};
    const int nz = dims > 2 ? 2 : 1, ny = dims > 1 ? 2 : 1;
    for (int kz = 0; kz < nz; ++kz) {
      const f32 wz = dims > 2 ? (kz ? frac[2] : 1.f - frac[2]) : 1.f;
      const u32 z = u32(kz ? i1[2] : i0[2]);
      for (int ky = 0; ky < ny; ++ky) {
        const f32 wy = dims > 1 ? (ky ? frac[1] : 1.f - frac[1]) : 1.f;
        const u32 y = u32(ky ? i1[1] : i0[1]);
        const V4 a = sc.texels[base + z * sxy + y * sx + u32(i0[0])];
        const V4 b = sc.texels[base + z * sxy + y * sx + u32(i1[0])];
        acc = acc + (a * (1.f - frac[0]) + b * frac[0]) * (wy * wz);
      }
    }
    result = acc;
  }
  V4 out = mul_mat4(si.out_t, result);
  out.x += si.out_o[0];
  out.y += si.out_o[1];
  out.z += si.out_o[2];
  out.w += si.out_o[3];
  return out;
}
V4 eval_source(const Scene &sc, const Src &src, const Query &q)
{
  if (src.kind == K_ATTR)
    return fetch_attribute(sc, src.index, q);
  if (src.index < 0 || u32(src.index) >= sc.samplers.size())
    return {0.f, 0.f, 0.f, 1.f};
  const i32 slot = sc.samplers[u32(src.index)].in_attribute;
  return sampler_sample(sc, src.index, fetch_attribute(sc, slot, q));
}
V3 apply_normal_map(const Scene &sc, const Src &src, const Query &q, const V3 &sn)
{
  const V4 c = eval_source(sc, src, q);
  const V3 nm{2.f * c.x - 1.f, 2.f * c.y - 1.f, 2.f * c.z - 1.f};
  i32 slot = src.index;
  if (src.kind != K_ATTR) {
    if (src.index < 0 || u32(src.index) >= sc.samplers.size())
      return sn;
    slot = sc.samplers[u32(src.index)].in_attribute;
  }
  Query corner = q;
  corner.b1 = 0.f;
  corner.b2 = 0.f;
  const V4 a0 = fetch_attribute(sc, slot, corner);
  corner.b1 = 1.f;
  const V4 a1 = fetch_attribute(sc, slot, corner);
  corner.b1 = 0.f;
  corner.b2 = 1.f;
  const V4 a2 = fetch_attribute(sc, slot, corner);
  const f32 du1 = a1.x - a0.x, dv1 = a1.y - a0.y, du2 = a2.x - a0.x, dv2 = a2.y - a0.y;
  const f32 det = du1 * dv2 - du2 * dv1;
  if (!(std::fabs(det) > 1e-20f))
    return sn;
  const V3 p0 = sc.mesh.pos[sc.mesh.idx[q.prim * 3 + 0]];
  const V3 e1 = sc.mesh.pos[sc.mesh.idx[q.prim * 3 + 1]] - p0;
  const V3 e2 = sc.mesh.pos[sc.mesh.idx[q.prim * 3 + 2]] - p0;
  V3 t = (e1 * dv2 - e2 * dv1) * (1.f / det);
  V3 b = (e2 * du1 - e1 * du2) * (1.f / det);
  t = t - sn * dot(sn, t);
  b = b - sn * dot(sn, b);
  if (!(dot(t, t) > 0.f) || !(dot(b, b) > 0.f))
    return sn;
  const V3 n = normalize(t) * nm.x + normalize(b) * nm.y + sn * nm.z;
  return dot(n, n) > 0.f ? normalize(n) : sn;
}
inline f32 clamp01(f32 x) { return x < 0.f ? 0.f : (x > 1.f ? 1.f : x); }
// TextureAtlas::sample, texture.h:25-64
V3 atlas_sample(const Scene &sc, i32 tex_id, f32 u, f32 v)
{
  if (tex_id < 0 || u32(tex_id) >= sc.atlas_w.size())
    return {1.f, 1.f, 1.f};
  const u32 w = sc.atlas_w[u32(tex_id)], h = sc.atlas_h[u32(tex_id)];
  if (w == 0 || h == 0)
    return {1.f, 1.f, 1.f};
  u = u - std::floor(u);
  v = 1.f - (v - std::floor(v));
  const f32 fx = u * f32(w) - 0.5f, fy = v * f32(h) - 0.5f;
  const i32 ix = i32(std::floor(fx)), iy = i32(std::floor(fy));
  const f32 tx = fx - std::floor(fx), ty = fy - std::floor(fy);
  auto wrap = [](i32 i, u32 sz) -> u32 {
    const i32 n = i32(sz);
    return u32(((i % n) + n) % n);
  };
  const u32 x0 = wrap(ix, w), x1 = wrap(ix + 1, w), y0 = wrap(iy, h), y1 = wrap(iy + 1, h);
  const u32 base = sc.atlas_off[u32(tex_id)];
  const V3 c00 = sc.atlas_px[base + y0 * w + x0], c10 = sc.atlas_px[base + y0 * w + x1];
  const V3 c01 = sc.atlas_px[base + y1 * w + x0], c11 = sc.atlas_px[base + y1 * w + x1];
  const V3 top = c00 * (1.f - tx) + c10 * tx;
  const V3 bot = c01 * (1.f - tx) + c11 * tx;
  return top * (1.f - ty) + bot * ty;
}

// the hit's uv (mesh_intersector.h:146-163)
V2 hit_uv(const Scene &sc, const Query &q)
{
  if (sc.uv.empty())
    return {0.f, 0.f};
  const u32 i0 = sc.mesh.idx[3 * q.prim], i1 = sc.mesh.idx[3 * q.prim + 1], i2 = sc.mesh.idx[3 * q.prim + 2];
  const f32 w0 = 1.f - q.b1 - q.b2, w1 = q.b1, w2 = q.b2;
  const V2 a = sc.uv[i0], b = sc.uv[i1], c = sc.uv[i2];
  return {a.x * w0 + b.x * w1 + c.x * w2, a.y * w0 + b.y * w1 + c.y * w2};
}

Mat resolve_material(const Scene &sc, const Query &q, f32 &alpha)
{
  Mat m = sc.mats[q.material_id];
  alpha = m.alpha;
  const bool has_textures = !sc.atlas_w.empty(); // pathtracer.cpp:190-199
  if (has_textures && (m.alpha_tex >= 0 || m.base_color_tex >= 0)) {
    const V2 uv = q.inst != NO_INST ? V2{q.b1, q.b2} : hit_uv(sc, q); // an instance's uv: its barycentrics
    if (m.alpha_tex >= 0)
      alpha = atlas_sample(sc, m.alpha_tex, uv.x, uv.y).x;
    if (m.base_color_tex >= 0)
      m.base_color = atlas_sample(sc, m.base_color_tex, uv.x, uv.y);
  }
  if (m.base_color_src.kind != K_CONST) {
    const V4 c = eval_source(sc, m.base_color_src, q);
    m.base_color = {std::fmax(c.x, 0.f), std::fmax(c.y, 0.f), std::fmax(c.z, 0.f)};
    if (m.base_color_alpha)
      alpha *= c.w;
  }
  if (m.alpha_src.kind != K_CONST)
    alpha *= eval_source(sc, m.alpha_src, q).x;
  if (m.metallic_src.kind != K_CONST)
    m.metallic = eval_source(sc, m.metallic_src, q).x;
  if (m.roughness_src.kind != K_CONST) {
    const f32 r = clamp01(eval_source(sc, m.roughness_src, q).x);
    m.roughness = m.roughness_src_squared ? r * r : r;
  }
  if (m.transmission_src.kind != K_CONST)
    m.transmission = eval_source(sc, m.transmission_src, q).x;
  if (m.emission_src.kind != K_CONST) {
    const V4 e = eval_source(sc, m.emission_src, q);
    m.emission = {std::fmax(e.x, 0.f), std::fmax(e.y, 0.f), std::fmax(e.z, 0.f)};
  }
  m.metallic = clamp01(m.metallic);
  m.roughness = clamp01(m.roughness);
  m.transmission = clamp01(m.transmission);
  if (m.alpha_mode == A_OPAQUE)
    alpha = 1.f;
  else if (m.alpha_mode == A_MASK)
    alpha = alpha >= m.alpha_cutoff ? 1.f : 0.f;
  else
    alpha = clamp01(alpha);
  return m;
}
inline bool emits_on_side(const Mat &m, bool front)
{
  if (m.flags & F_EMIT_BOTH)
    return true;
  const bool back_only = (m.flags & F_EMIT_BACK) != 0;
  return front ? !back_only : back_only;
}

struct DS {
  V3 wi, radiance;
  f32 pdf{0.f}, dist{0.f};
  bool mis{false}, valid{false};
};
DS sample_direct(const Scene &sc, const V3 &p, Rng &rng) // pathtracer.cpp:270-367
{
  DS ds;
  if (sc.strategy_count == 0)
    return ds;
  const f32 pick_pdf = 1.f / f32(sc.strategy_count);
  u32 pick = u32(rng.next_f32() * f32(sc.strategy_count));
  if (pick >= sc.strategy_count)
    pick = sc.strategy_count - 1;
  const u32 light_count = u32(sc.lights.size());
  const u32 emissive_count = u32(sc.emissive_cdf.size());
  if (pick < light_count) {
    const LS ls = sample_light(sc.lights[pick], p, rng);
    if (!(ls.pdf > 0.f))
      return ds;
    ds.wi = ls.wi;
    ds.radiance = ls.Li;
    ds.pdf = ls.pdf * pick_pdf;
    ds.dist = ls.dist;
    ds.mis = false;
    ds.valid = true;
    return ds;
  }
  if (emissive_count > 0 && pick == light_count) {
    const f32 xi = rng.next_f32();
    u32 lo = 0, hi = emissive_count - 1;
    while (lo < hi) {
      const u32 mid = (lo + hi) / 2;
      if (sc.emissive_cdf[mid] <= xi)
        lo = mid + 1;
      else
        hi = mid;
    }
    const u32 prim = sc.emissive_ids[lo];
    const f32 pdf_area = sc.prim_light_pdf[prim];
    if (!(pdf_area > 0.f))
      return ds;
    const V3 v0 = sc.mesh.pos[sc.mesh.idx[prim * 3 + 0]];
    const V3 v1 = sc.mesh.pos[sc.mesh.idx[prim * 3 + 1]];
    const V3 v2 = sc.mesh.pos[sc.mesh.idx[prim * 3 + 2]];
    const f32 su = std::sqrt(rng.next_f32());
    const f32 r2 = rng.next_f32();
    const f32 b0 = 1.f - su;
    const f32 b1 = r2 * su;
    const f32 b2 = 1.f - b0 - b1;
    const V3 lp = v0 * b0 + v1 * b1 + v2 * b2;
    const V3 to = lp - p;
    const f32 d2 = dot(to, to);
    if (!(d2 > 0.f))
      return ds;
    const f32 dist = std::sqrt(d2);
    const V3 wi = to * (1.f / dist);
    const V3 ln = normalize(cross(v1 - v0, v2 - v0));
    const f32 cos_light = -dot(wi, ln);
    if (std::fabs(cos_light) < 1e-6f)
      return ds;
    Query q;
    q.prim = prim;
    q.material_id = sc.mesh.mat_ids[prim];
    q.b1 = b1;
    q.b2 = b2;
    q.p = lp;
    q.sn = ln;
    f32 alpha = 1.f;
    const Mat em = resolve_material(sc, q, alpha);
    if (!emits_on_side(em, cos_light > 0.f))
      return ds;
    ds.wi = wi;
    ds.radiance = mat_emission(em) * alpha;
    ds.pdf = pdf_area * d2 / std::fabs(cos_light) * pick_pdf;
    ds.dist = dist;
    ds.mis = true;
    ds.valid = true;
    return ds;
  }
  if (sc.has_env) {
    f32 env_pdf = 0.f;
    const V3 wi = sc.env.sample(rng, env_pdf);
    if (!(env_pdf > 0.f))
      return ds;
    ds.wi = wi;
    ds.radiance = sc.env.evaluate(wi);
    ds.pdf = env_pdf * pick_pdf;
    ds.dist = 1e30f;
    ds.mis = true;
    ds.valid = true;
  }
  return ds;
}

inline V3 clamp_contrib(const V3 &c, int light_bounce, f32 direct_sum, f32 indirect_sum)
{
  const f32 limit = light_bounce > 0 ? indirect_sum : direct_sum;
  if (!(limit > 0.f))
    return c;
  const f32 sum = std::fabs(c.x) + std::fabs(c.y) + std::fabs(c.z);
  return sum > limit ? c * (limit / sum) : c;
}
inline bool count_bounce(u32 &kinds, u32 shift, int limit)
{
  u32 count = (kinds >> shift) & 0x7fu;
  if (count < 0x7fu)
    ++count;
  kinds = (kinds & ~(0x7fu << shift)) | (count << shift);
  return limit >= 0 && int(count) > limit;
}
constexpr u32 EMISSION_ONLY = 0x80000000u;

V4 background_image(const Params &pr, f32 s, f32 t) // pathtracer.cpp:370-389
{
  const int h = int(pr.bg_h), w = int(pr.bg_w);
  const f32 fx = s * f32(w) - 0.5f;
  const f32 fy = t * f32(h) - 0.5f;
  const f32 flx = std::floor(fx), fly = std::floor(fy);
  const f32 tx = fx - flx, ty = fy - fly;
  auto ci = [](int i, int n) { return i < 0 ? 0 : (i >= n ? n - 1 : i); };
  const int x0 = ci(int(flx), w), x1 = ci(int(flx) + 1, w), y0 = ci(int(fly), h), y1 = ci(int(fly) + 1, h);
  auto im = [&](int y, int x) { return pr.bg_image[size_t(y) * w + x]; };
  const V4 a = im(y0, x0) * (1.f - tx) + im(y0, x1) * tx;
  const V4 b = im(y1, x0) * (1.f - tx) + im(y1, x1) * tx;
  return a * (1.f - ty) + b * ty;
}

// Per-pixel accumulators, pathtracer.h:76-130.
struct PixelState {
  V3 accum, accum_sq;
  f32 accum_alpha{0.f};
  u32 samples{0};
  V3 aov_albedo, aov_normal;
  f32 aov_depth{1e30f};
  u32 aov_written{0};
  V3 sample_start; // accum when the pixel's last active sample began
};

// One sample of one pixel through the bounce loop: pt_init_sample, then per
// iteration trace_closest + pt_shade + trace_occluded + pt_nee_accum_pack,
// then pt_update_variance (pathtracer.cpp:691-1139).
void render_pixel_sample(const Scene &sc, const Cam &cam, const Params &pr, u32 idx, u32 s, PixelState &px)
{
  const u32 w = pr.w, h = pr.h;
  const u32 sample_index = s + pr.sample_offset;
  const u32 max_depth = pr.max_depth > 0 ? pr.max_depth : 1u;
  const u32 max_iterations = max_depth + 1u + 8u;
  const bool has_volumes = !sc.vols.vols.empty();
  const f32 eps = sc.eps;
  const u32 x = idx % w, y = idx / w;

  if (s == 0u) {
    px = PixelState{};
  }
  bool gated = false;
  if (pr.adaptive && s >= 16u) {
    const u32 ns = px.samples;
    if (ns >= 16u) {
      const V3 mean = px.accum * (1.f / f32(ns));
      const V3 sq = px.accum_sq * (1.f / f32(ns));
      const V3 var = sq - V3{mean.x * mean.x, mean.y * mean.y, mean.z * mean.z};
      const f32 max_var = std::fmax(var.x, std::fmax(var.y, var.z));
      const f32 lum = std::fmax(0.2126f * mean.x + 0.7152f * mean.y + 0.0722f * mean.z, 1e-4f);
      if (max_var / (lum * lum) < 0.01f)
        gated = true;
    }
  }
  if (!gated) {
    Rng rng = make_rng(idx, sample_index, 0u);
    f32 u = (f32(x) + rng.next_f32()) / f32(w);
    f32 v = (f32(y) + rng.next_f32()) / f32(h);
    if (!pr.bottom_up)
      v = 1.f - v;
    u = pr.region[0] + (pr.region[2] - pr.region[0]) * u;
    v = pr.region[1] + (pr.region[3] - pr.region[1]) * v;
    V3 ro, rd;
    cam.ray(u, v, rng, ro, rd);
    f32 tmin, tmax;
    cam.clip_range(rd, tmin, tmax);
    V3 tp{1.f, 1.f, 1.f};
    bool active = true;
    f32 prev_pdf = -1.f;
    u32 depth = 0u;
    bool primary = true;
    f32 path_dist = 0.f;
    u32 kinds = 0u;
    px.sample_start = px.accum;
    px.samples += 1u;

    for (u32 it = 0; it < max_iterations && active; ++it) {
      // trace_closest (kokkos_backend.cpp:21-61)
      const Hit hr = intersect_scene(sc, ro, rd, tmin, tmax, false);
      V3 nee_contrib;
      bool nee_active = false;
      V3 sh_o, sh_d;
      f32 sh_tmin = 1.f, sh_tmax = 0.f;
      const bool emission_only = (kinds & EMISSION_ONLY) != 0u;
      Rng r = make_rng(idx, sample_index, 1u + it);

      // ---- pt_shade (pathtracer.cpp:765-1090)
      [&] {
        if (has_volumes) {
          V3 albedo{0.f, 0.f, 0.f};
          const f32 t_end = hr.hit ? hr.t : tmax;
          const f32 t_sc = sc.vols.sample_scatter(ro, rd, tmin, t_end, r, albedo);
          if (t_sc >= 0.f) {
            const V3 p = ro + rd * t_sc;
            if (primary) {
              primary = false;
              px.accum_alpha = px.accum_alpha + 1.f;
              if (px.aov_written == 0u) {
                px.aov_written = 1u;
                px.aov_depth = path_dist + t_sc;
                px.aov_normal = -rd;
                px.aov_albedo = albedo;
              }
            }
            if (depth >= max_depth || emission_only) {
              active = false;
              return;
            }
            const V3 tpa = tp * albedo;
            const f32 phase = 0.25f * INV_PI;
            const DS ds = sample_direct(sc, p, r);
            if (ds.valid) {
              const f32 w_mis = ds.mis ? power_heuristic(ds.pdf, phase) : 1.f;
              nee_contrib = clamp_contrib(
                  tpa * ds.radiance * (phase * w_mis / ds.pdf), int(depth), pr.clamp_direct, pr.clamp_indirect);
              nee_active = true;
              sh_o = p;
              sh_d = ds.wi;
              sh_tmin = 0.f;
              sh_tmax = ds.dist < 1e29f ? ds.dist * (1.f - 1e-4f) : 1e30f;
            }
            V3 tp_next = tpa;
            if (depth >= 2) {
              const f32 max_tp = std::fmax(tpa.x, std::fmax(tpa.y, tpa.z));
              const f32 survive = std::fmin(std::fmax(max_tp, 0.05f), 0.95f);
              if (r.next_f32() >= survive) {
                active = false;
                return;
              }
              tp_next = tpa * (1.f / survive);
            }
            tp = tp_next;
            prev_pdf = phase;
            depth = depth + 1u;
            if (count_bounce(kinds, 24u, pr.max_volume))
              kinds |= EMISSION_ONLY;
            ro = p;
            rd = uniform_sphere(r);
            tmin = 0.f;
            tmax = 1e30f;
            return;
          }
        }
        if (!hr.hit) {
          V3 L{0.f, 0.f, 0.f};
          if (primary) {
            if (sc.has_env && sc.env_visible) {
              L = sc.env.evaluate(rd);
              px.accum_alpha = px.accum_alpha + 1.f;
            } else if (pr.bg_w > 0 && pr.bg_h > 0) {
              const f32 bs = (f32(x) + 0.5f) / f32(w);
              const f32 bt = (f32(y) + 0.5f) / f32(h);
              const V4 bg = background_image(pr, bs, pr.bottom_up ? bt : 1.f - bt);
              L = bg.xyz() * bg.w;
              px.accum_alpha = px.accum_alpha + bg.w;
            } else {
              L = pr.bg_color * pr.bg_alpha;
              px.accum_alpha = px.accum_alpha + pr.bg_alpha;
            }
          } else {
            L = pr.ambient;
            if (sc.has_env) {
              f32 w_mis = 1.f;
              if (prev_pdf > 0.f) {
                const f32 light_pdf = sc.env.pdf(rd) / f32(sc.strategy_count);
                w_mis = power_heuristic(prev_pdf, light_pdf);
              }
              L = L + sc.env.evaluate(rd) * w_mis;
            }
          }
          V3 from_miss = tp * L;
          if (!primary || (sc.has_env && sc.env_visible))
            from_miss = clamp_contrib(from_miss, int(depth) - 1, pr.clamp_direct, pr.clamp_indirect);
          px.accum = px.accum + from_miss;
          active = false;
          return;
        }
        const HitAttr ha = hit_attributes_scene(sc, ro, rd, hr);
        const V3 p = ha.p;
        const V3 wo = -rd;
        V3 hit_sn = ha.sn;
        if (!(dot(hit_sn, hit_sn) > 0.25f))
          hit_sn = ha.n;
        else if (dot(hit_sn, ha.n) < 0.f)
          hit_sn = hit_sn * -1.f;
        Query q;
        q.prim = hr.prim;
        q.inst = hr.inst;
        q.material_id = ha.material_id;
        q.b1 = hr.u;
        q.b2 = hr.v;
        q.p = p;
        q.sn = hit_sn;
        f32 alpha_val = 1.f;
        const Mat mat = resolve_material(sc, q, alpha_val);
        const bool hidden = (mat.flags & F_HIDDEN) != 0 && primary;
        if (hidden || (alpha_val < 1.f && r.next_f32() >= alpha_val)) {
          ro = p;
          tmin = eps;
          tmax = 1e30f;
          path_dist = path_dist + hr.t;
          if (primary) {
            f32 tn, tf;
            cam.clip_range(rd, tn, tf);
            if (tf < 1e30f) {
              tmax = tf - path_dist;
              if (tmax < eps) {
                tmin = 1.f;
                tmax = 0.f;
              }
            }
          }
          prev_pdf = -1.f;
          return;
        }
        V3 n = ha.n;
        V3 sn = hit_sn;
        const bool front = dot(n, wo) >= 0.f;
        const bool transmissive = mat.transmission > 0.f;
        if (!transmissive && !front) {
          n = n * -1.f;
          sn = sn * -1.f;
        }
        if (mat.normal_src.kind != K_CONST)
          sn = apply_normal_map(sc, mat.normal_src, q, sn);
        if (primary) {
          primary = false;
          px.accum_alpha = px.accum_alpha + 1.f;
          if (px.aov_written == 0u) {
            px.aov_written = 1u;
            px.aov_depth = path_dist + hr.t;
            px.aov_normal = normalize(sn);
            px.aov_albedo = mat.base_color;
          }
        }
        if (may_emit(mat) && emits_on_side(mat, front)) {
          f32 w_mis = 1.f;
          if (prev_pdf > 0.f && !sc.emissive_cdf.empty()) {
            const f32 pdf_area = hr.inst == NO_INST ? sc.prim_light_pdf[hr.prim] : 0.f; // instances are no lights
            const f32 cos_light = std::fabs(dot(ha.n, wo));
            if (pdf_area > 0.f && cos_light > 0.f) {
              const f32 light_pdf = pdf_area * hr.t * hr.t / cos_light / f32(sc.strategy_count);
              w_mis = power_heuristic(prev_pdf, light_pdf);
            }
          }
          px.accum = px.accum
              + clamp_contrib(tp * mat_emission(mat) * w_mis, int(depth) - 1, pr.clamp_direct, pr.clamp_indirect);
        }
        if ((mat.flags & F_EMITTER_ONLY) != 0 || depth >= max_depth || emission_only) {
          active = false;
          return;
        }
        {
          const DS ds = sample_direct(sc, p, r);
          if (ds.valid) {
            const V3 f = bsdf_eval(mat, wo, ds.wi, n, sn);
            if (f.x > 0.f || f.y > 0.f || f.z > 0.f) {
              f32 w_mis = 1.f;
              if (ds.mis)
                w_mis = power_heuristic(ds.pdf, bsdf_pdf(mat, wo, ds.wi, n, sn));
              nee_contrib = clamp_contrib(
                  tp * f * ds.radiance * (w_mis / ds.pdf), int(depth), pr.clamp_direct, pr.clamp_indirect);
              nee_active = true;
              const V3 so = p + n * eps;
              sh_o = so;
              sh_tmin = 0.f;
              if (ds.dist < 1e29f) {
                const V3 to_light = p + ds.wi * ds.dist - so;
                const f32 sd = length(to_light);
                sh_d = sd > 0.f ? to_light * (1.f / sd) : ds.wi;
                sh_tmax = sd * (1.f - 1e-3f);
              } else {
                sh_d = ds.wi;
                sh_tmax = 1e30f;
              }
            }
          }
        }
        const BS bs = bsdf_sample(mat, wo, n, sn, r);
        if (bs.pdf <= 0.f || (bs.f.x <= 0.f && bs.f.y <= 0.f && bs.f.z <= 0.f)) {
          active = false;
          return;
        }
        V3 tpn = tp * (bs.f * (1.f / bs.pdf));
        if (depth >= 2) {
          const f32 max_tp = std::fmax(tpn.x, std::fmax(tpn.y, tpn.z));
          const f32 survive = std::fmin(std::fmax(max_tp, 0.05f), 0.95f);
          if (r.next_f32() >= survive) {
            active = false;
            return;
          }
          tpn = tpn * (1.f / survive);
        }
        if (pr.tp_clamp > 0.f) {
          const f32 mx = std::fmax(tpn.x, std::fmax(tpn.y, tpn.z));
          if (mx > pr.tp_clamp)
            tpn = tpn * (pr.tp_clamp / mx);
        }
        if (!(tpn.x == tpn.x && tpn.y == tpn.y && tpn.z == tpn.z)) {
          active = false;
          return;
        }
        tp = tpn;
        prev_pdf = bs.spec ? -1.f : bs.pdf;
        depth = depth + 1u;
        const V3 wi = normalize(bs.wi);
        const f32 side = dot(wi, ha.n) < 0.f ? -1.f : 1.f;
        const bool through = (dot(wi, ha.n) < 0.f) != (dot(wo, ha.n) < 0.f);
        const bool exceeded = through ? count_bounce(kinds, 16u, pr.max_transmission)
                                      : (bs.diff ? count_bounce(kinds, 0u, pr.max_diffuse)
                                                 : count_bounce(kinds, 8u, pr.max_glossy));
        if (exceeded)
          kinds |= EMISSION_ONLY;
        ro = p + ha.n * (side * eps);
        rd = wi;
        tmin = 0.f;
        tmax = 1e30f;
      }();

      // ---- trace_occluded + pt_nee_accum_pack (pathtracer.cpp:1092-1123)
      if (nee_active) {
        const Hit occ = intersect_scene(sc, sh_o, sh_d, sh_tmin, sh_tmax, true);
        if (!occ.hit) {
          V3 contrib = nee_contrib;
          if (has_volumes) {
            Rng rs = make_rng(idx, sample_index, 0x10000u + it);
            contrib = contrib * sc.vols.transmittance(sh_o, sh_d, sh_tmin, sh_tmax, rs);
          }
          if (contrib.x == contrib.x && contrib.y == contrib.y && contrib.z == contrib.z)
            px.accum = px.accum + contrib;
        }
      }
      if (!active)
        break;
    }
  }
  // pt_update_variance (pathtracer.cpp:1129-1139)
  if (pr.adaptive) {
    const V3 sv = px.accum - px.sample_start;
    px.accum_sq = px.accum_sq + V3{sv.x * sv.x, sv.y * sv.y, sv.z * sv.z};
  }
}

} // namespace orc

// -------------------------------------------------------------- renderer
namespace {
using namespace orc;

thread_local std::string g_error;

struct Renderer {
  bool has_scene{false};
  Scene sc;
  std::string error;
  // accumulated frame (RenderBridge.cpp:424-435)
  u32 width{0}, height{0}, samples{0}, sample_counter{0};
  std::vector<V3> acc_color, first_normal, first_albedo;
  std::vector<f32> acc_alpha, first_depth;
  std::vector<PixelState> px;
};

inline V3 v3(const float *p) { return {p[0], p[1], p[2]}; }

// Renderer::Impl::build_scene, RenderBridge.cpp:441-826, plus
// PathTracer::build_light_tables, pathtracer.cpp:411-503.
void build_scene(Scene &s, const phc_scene_desc &in)
{
  s = Scene{};
  size_t vc = in.vertex_count, tc = in.triangle_count;
  const bool empty = tc == 0 || vc == 0;
  if (empty) {
    vc = 3;
    tc = 1;
  }
  Aabb bounds;
  s.mesh.pos.resize(vc);
  for (size_t i = 0; i < vc; ++i) {
    s.mesh.pos[i] = empty ? V3{0.f, 0.f, 0.f} : v3(&in.positions[3 * i]);
    bounds.extend(s.mesh.pos[i]);
  }
  s.mesh.idx.resize(tc * 3);
  for (size_t i = 0; i < tc * 3; ++i)
    s.mesh.idx[i] = empty ? u32(i) : in.indices[i];
  const u32 material_count = u32(std::max<size_t>(in.material_count, 1));
  s.mesh.mat_ids.resize(tc);
  for (size_t i = 0; i < tc; ++i) {
    const u32 id = (!empty && in.material_ids && i < in.material_id_count) ? in.material_ids[i] : 0u;
    s.mesh.mat_ids[i] = id < material_count ? id : 0u;
  }
  if (!empty && in.normals) {
    s.mesh.nrm.resize(vc);
    for (size_t i = 0; i < vc; ++i)
      s.mesh.nrm[i] = v3(&in.normals[3 * i]);
  }
  const phc_pt_scene *pt = in.pt;
  size_t total = 0;
  for (int slot = 0; slot < 5; ++slot)
    if (!pt && !empty && in.attributes[slot]) {
      s.attr_offset[slot] = int(total);
      total += vc;
    }
  s.attr_values.resize(total);
  for (int slot = 0; slot < 5; ++slot) {
    if (s.attr_offset[slot] < 0)
      continue;
    const float *src = in.attributes[slot];
    for (size_t i = 0; i < vc; ++i)
      s.attr_values[size_t(s.attr_offset[slot]) + i] = V4{src[4 * i], src[4 * i + 1], src[4 * i + 2], src[4 * i + 3]};
  }
  if (pt) { // a scene at the path tracer's level: materials, atlas and uv as given
    for (u32 i = 0; i < in.material_count; ++i)
      s.mats.push_back(pt_material(pt->materials[i], pt->texture_count));
    if (!empty && pt->texcoords)
      for (size_t i = 0; i < vc; ++i)
        s.uv.push_back(V2{pt->texcoords[2 * i], pt->texcoords[2 * i + 1]});
    u32 off = 0;
    for (u32 i = 0; i < pt->texture_count; ++i) {
      const phc_texture &t = pt->textures[i];
      s.atlas_off.push_back(off);
      s.atlas_w.push_back(t.width);
      s.atlas_h.push_back(t.height);
      for (size_t k = 0; k < size_t(t.width) * t.height; ++k)
        s.atlas_px.push_back(V3{t.rgb[3 * k], t.rgb[3 * k + 1], t.rgb[3 * k + 2]});
      off += t.width * t.height;
    }
  } else {
    for (u32 i = 0; i < in.material_count; ++i)
      s.mats.push_back(convert_material(in.materials[i]));
  }
  if (s.mats.empty())
    s.mats.push_back(Mat{});
  // samplers (RenderBridge.cpp:527-571)
  size_t offset = 0;
  for (u32 i = 0; !pt && i < in.sampler_count; ++i) {
    const phc_sampler &sd = in.samplers[i];
    SInfo si;
    si.type = sd.type == 0 ? 0 : (sd.type == 2 ? 2 : (sd.type == 3 ? 3 : 1));
    si.in_attribute = sd.in_attribute;
    si.linear = sd.linear ? 1u : 0u;
    for (int d = 0; d < 3; ++d) {
      si.wrap[d] = sd.wrap[d] == 1 ? 1 : (sd.wrap[d] == 2 ? 2 : 0);
      si.size[d] = std::max<uint32_t>(sd.size[d], 1);
    }
    si.offset = u32(offset);
    std::memcpy(si.in_t, sd.in_transform, sizeof(si.in_t));
    std::memcpy(si.in_o, sd.in_offset, sizeof(si.in_o));
    std::memcpy(si.out_t, sd.out_transform, sizeof(si.out_t));
    std::memcpy(si.out_o, sd.out_offset, sizeof(si.out_o));
    const size_t n = sd.texels ? size_t(sd.texel_count) : 0;
    const size_t expected = size_t(si.size[0]) * si.size[1] * si.size[2];
    if (si.type != 3 && n < expected)
      si.type = 3;
    for (size_t t = 0; t < n; ++t)
      s.texels.push_back(V4{sd.texels[4 * t], sd.texels[4 * t + 1], sd.texels[4 * t + 2], sd.texels[4 * t + 3]});
    offset += n;
    s.samplers.push_back(si);
  }
  for (u32 i = 0; i < in.light_count; ++i) {
    const phc_light &ld = in.lights[i];
    Light l;
    l.type = ld.type == 1 ? L_DIR : (ld.type == 2 ? L_SPOT : L_POINT);
    l.position = v3(ld.position);
    l.direction = v3(ld.direction);
    l.color = v3(ld.color);
    l.intensity = ld.intensity;
    l.radius = ld.radius;
    l.spot_angle = ld.spot_angle;
    l.spot_falloff = ld.spot_falloff;
    s.lights.push_back(l);
  }
  const phc_environment &env = in.environment;
  if (env.present && env.width > 0 && env.height > 0 && env.pixels) {
    s.env.width = env.width;
    s.env.height = env.height;
    s.env.pixels.resize(size_t(env.width) * env.height);
    auto finite = [](float v) { return std::isfinite(v) && v > 0.f ? v : 0.f; };
    for (size_t k = 0; k < s.env.pixels.size(); ++k) {
      const float *p = &env.pixels[k * 3];
      s.env.pixels[k] = V3{finite(p[0]), finite(p[1]), finite(p[2])};
    }
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        s.env.w2t[r * 3 + c] = env.world_to_map[r * 3 + c];
        s.env.t2w[c * 3 + r] = env.world_to_map[r * 3 + c];
      }
    if (pt && pt->env_map_to_world_given) // pbrt_to_photon.cpp:455-466
      std::memcpy(s.env.t2w, pt->env_map_to_world, sizeof(s.env.t2w));
    s.env.build_cdf();
    s.has_env = true;
    s.env_visible = env.visible != 0;
  }
  // instanced geometry: objects in their own space, each with its BVH; per
  // placement the world-to-object rows (inverted in double, then rounded)
  // and padded world bounds
  if (pt && pt->instance_count && pt->object_count) {
    const u32 nm = u32(s.mats.size());
    for (u32 o = 0; o < pt->object_count; ++o) {
      const phc_object &ob = pt->objects[o];
      Obj obj;
      if (ob.triangle_count && ob.vertex_count) {
        for (size_t v = 0; v < ob.vertex_count; ++v) {
          obj.mesh.pos.push_back(v3(&ob.positions[3 * v]));
          if (ob.normals)
            obj.mesh.nrm.push_back(v3(&ob.normals[3 * v]));
        }
        obj.mesh.idx.assign(ob.indices, ob.indices + 3 * ob.triangle_count);
        obj.mesh.bvh.build(obj.mesh.pos, obj.mesh.idx);
      }
      obj.material = ob.material_id < nm ? ob.material_id : 0u;
      s.objs.push_back(std::move(obj));
    }
    for (u32 i = 0; i < pt->instance_count; ++i) {
      const phc_instance &in = pt->instances[i];
      if (in.object_id >= pt->object_count || s.objs[in.object_id].mesh.idx.empty())
        continue;
      double m[3][4];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c)
          m[r][c] = double(in.transform[c * 4 + r]);
      const double det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
          m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) + m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
      if (!(std::fabs(det) > 1e-30) || !std::isfinite(det))
        continue;
      const double id = 1.0 / det;
      double inv[3][3];
      inv[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) * id;
      inv[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * id;
      inv[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
      inv[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) * id;
      inv[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
      inv[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * id;
      inv[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) * id;
      inv[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * id;
      inv[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
      Inst it;
      it.obj = in.object_id;
      for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c)
          it.w2o[r * 4 + c] = f32(inv[r][c]);
        it.w2o[r * 4 + 3] = f32(-(inv[r][0] * m[0][3] + inv[r][1] * m[1][3] + inv[r][2] * m[2][3]));
      }
      const Mesh &om = s.objs[in.object_id].mesh;
      double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300}, ext = 0.0;
      for (const V3 &p : om.pos)
        for (int r = 0; r < 3; ++r) {
          const double w = m[r][0] * p.x + m[r][1] * p.y + m[r][2] * p.z + m[r][3];
          lo[r] = std::min(lo[r], w);
          hi[r] = std::max(hi[r], w);
        }
      for (int r = 0; r < 3; ++r)
        ext = std::max(ext, std::max(std::fabs(lo[r]), std::fabs(hi[r])));
      const double pad = 1e-5 * ext + 1e-30;
      it.box.lo = V3{f32(lo[0] - pad), f32(lo[1] - pad), f32(lo[2] - pad)};
      it.box.hi = V3{f32(hi[0] + pad), f32(hi[1] + pad), f32(hi[2] + pad)};
      s.insts.push_back(it);
    }
  }
  // volumes with macro-cell majorants (RenderBridge.cpp:622-778)
  size_t value_offset = 0, tf_offset = 0;
  for (u32 i = 0; i < in.volume_count; ++i) {
    const phc_volume &vd = in.volumes[i];
    Vol v;
    std::memcpy(v.w2l, vd.world_to_local, sizeof(v.w2l));
    v.origin = v3(vd.origin);
    v.spacing = v3(vd.spacing);
    for (int d = 0; d < 3; ++d)
      v.dims[d] = std::max<uint32_t>(vd.dims[d], 1);
    v.data_offset = u32(value_offset);
    v.tf_offset = u32(tf_offset);
    const size_t table = vd.transfer ? vd.transfer_count : 0;
    v.tf_size = u32(table);
    v.value_lo = vd.value_range[0];
    v.value_hi = vd.value_range[1];
    v.density_scale = vd.density_scale;
    v.linear = vd.linear ? 1u : 0u;
    f32 max_opacity = 0.f;
    for (size_t t = 0; t < table; ++t) {
      const V4 c{vd.transfer[4 * t], vd.transfer[4 * t + 1], vd.transfer[4 * t + 2], vd.transfer[4 * t + 3]};
      s.vols.tf.push_back(c);
      max_opacity = std::max(max_opacity, c.w);
    }
    v.majorant = max_opacity * vd.density_scale;
    const size_t nvals = vd.values ? size_t(vd.value_count) : 0;
    const bool complete = nvals >= size_t(v.dims[0]) * v.dims[1] * v.dims[2];
    if (!complete)
      v.majorant = 0.f;
    v.macro_offset = u32(s.vols.majorants.size());
    u32 sub[3] = {0, 0, 0};
    for (int d = 0; d < 3; ++d) {
      const u32 cells = v.dims[d] > 1 ? v.dims[d] - 1 : 1;
      if (cells <= 32) {
        sub[d] = std::min<u32>(std::max<u32>((32 + cells - 1) / cells, 1), 16);
        v.macro_dims[d] = cells * sub[d];
      } else {
        v.macro_dims[d] = std::min<u32>(std::max<u32>((v.dims[d] + 2) / 4, 1), 128);
      }
    }
    const f32 range = vd.value_range[1] - vd.value_range[0];
    const bool refined = sub[0] > 0 && sub[1] > 0 && sub[2] > 0;
    if (!refined)
      for (int d = 0; d < 3; ++d)
        if (sub[d] > 0)
          v.macro_dims[d] = std::min<u32>(std::max<u32>((v.dims[d] + 2) / 4, 1), 128);
    const float *vals = vd.values;
    auto node = [&](u32 x, u32 y, u32 z) {
      x = std::min(x, v.dims[0] - 1);
      y = std::min(y, v.dims[1] - 1);
      z = std::min(z, v.dims[2] - 1);
      return vals[(size_t(z) * v.dims[1] + y) * v.dims[0] + x];
    };
    auto interp = [&](f32 gx, f32 gy, f32 gz) {
      const u32 x = u32(gx), y = u32(gy), z = u32(gz);
      const f32 fx = gx - f32(x), fy = gy - f32(y), fz = gz - f32(z);
      const f32 c00 = node(x, y, z) * (1.f - fx) + node(x + 1, y, z) * fx;
      const f32 c10 = node(x, y + 1, z) * (1.f - fx) + node(x + 1, y + 1, z) * fx;
      const f32 c01 = node(x, y, z + 1) * (1.f - fx) + node(x + 1, y, z + 1) * fx;
      const f32 c11 = node(x, y + 1, z + 1) * (1.f - fx) + node(x + 1, y + 1, z + 1) * fx;
      return (c00 * (1.f - fy) + c10 * fy) * (1.f - fz) + (c01 * (1.f - fy) + c11 * fy) * fz;
    };
    for (u32 mz = 0; mz < v.macro_dims[2]; ++mz)
      for (u32 my = 0; my < v.macro_dims[1]; ++my)
        for (u32 mx = 0; mx < v.macro_dims[0]; ++mx) {
          f32 bound = 0.f;
          if (complete && table > 0) {
            const u32 m[3] = {mx, my, mz};
            f32 vmin = std::numeric_limits<f32>::max(), vmax = -std::numeric_limits<f32>::max();
            if (refined) {
              for (int corner = 0; corner < 8; ++corner) {
                f32 g[3];
                for (int d = 0; d < 3; ++d)
                  g[d] = f32(m[d] + ((corner >> d) & 1)) / f32(sub[d]);
                const f32 value = interp(g[0], g[1], g[2]);
                vmin = std::min(vmin, value);
                vmax = std::max(vmax, value);
              }
            } else {
              u32 first[3], last[3];
              for (int d = 0; d < 3; ++d) {
                const f32 cells = f32(v.dims[d] > 1 ? v.dims[d] - 1 : 1);
                const f32 lo = f32(m[d]) / f32(v.macro_dims[d]) * cells;
                const f32 hi = f32(m[d] + 1) / f32(v.macro_dims[d]) * cells;
                first[d] = u32(std::max(std::floor(lo) - 1.f, 0.f));
                last[d] = std::min<u32>(u32(std::ceil(hi)) + 1, v.dims[d] - 1);
              }
              for (u32 z = first[2]; z <= last[2]; ++z)
                for (u32 y = first[1]; y <= last[1]; ++y)
                  for (u32 x = first[0]; x <= last[0]; ++x) {
                    const f32 value = vals[(size_t(z) * v.dims[1] + y) * v.dims[0] + x];
                    vmin = std::min(vmin, value);
                    vmax = std::max(vmax, value);
                  }
            }
            auto tpos = [&](f32 value) {
              f32 x = range != 0.f ? (value - vd.value_range[0]) / range : 0.f;
              x = std::min(std::max(x, 0.f), 1.f);
              return x * f32(table - 1);
            };
            const size_t i0 = size_t(std::floor(tpos(vmin)));
            const size_t i1 = std::min(size_t(std::ceil(tpos(vmax))), table - 1);
            for (size_t t = i0; t <= i1; ++t)
              bound = std::max(bound, vd.transfer[4 * t + 3]);
            if (!(vmin <= vmax))
              bound = max_opacity;
          }
          s.vols.majorants.push_back(bound * vd.density_scale * 1.01f);
        }
    for (size_t k = 0; k < nvals; ++k)
      s.vols.values.push_back(vals[k]);
    value_offset += nvals;
    tf_offset += table;
    s.vols.vols.push_back(v);
  }
  // emissive triangles (RenderBridge.cpp:780-813) and their CDF
  // (pathtracer.cpp:439-487)
  std::vector<u32> ids;
  std::vector<f32> areas;
  if (!empty) {
    for (size_t t = 0; t < tc; ++t) {
      const u32 mid = (in.material_ids && t < in.material_id_count && in.material_ids[t] < material_count)
          ? in.material_ids[t]
          : 0u;
      if (!may_emit(s.mats[mid]))
        continue;
      const V3 p0 = v3(&in.positions[3 * size_t(in.indices[3 * t + 0])]);
      const V3 p1 = v3(&in.positions[3 * size_t(in.indices[3 * t + 1])]);
      const V3 p2 = v3(&in.positions[3 * size_t(in.indices[3 * t + 2])]);
      const f32 area = 0.5f * length(cross(p1 - p0, p2 - p0));
      if (!(area > 0.f))
        continue;
      ids.push_back(u32(t));
      areas.push_back(area);
    }
  }
  if (!ids.empty()) {
    const u32 n = u32(ids.size());
    std::vector<double> weights(n, 0.0);
    double total_w = 0.0;
    for (u32 i = 0; i < n; ++i) {
      const Mat &m = s.mats[s.mesh.mat_ids[ids[i]]];
      const bool constant = m.emission_src.kind == K_CONST;
      const f32 power = constant ? luminance(mat_emission(m)) : m.emission_strength;
      weights[i] = double(areas[i]) * double(power > 1e-6f ? power : 1e-6f);
      if (!(areas[i] > 0.f))
        weights[i] = 0.0;
      total_w += weights[i];
    }
    if (total_w > 0.0) {
      s.emissive_ids = ids;
      s.emissive_cdf.assign(n, 0.f);
      s.prim_light_pdf.assign(tc, 0.f);
      double running = 0.0;
      for (u32 i = 0; i < n; ++i) {
        running += weights[i];
        s.emissive_cdf[i] = f32(running / total_w);
        if (weights[i] > 0.0 && ids[i] < tc)
          s.prim_light_pdf[ids[i]] = f32(weights[i] / total_w / double(areas[i]));
      }
      s.emissive_cdf[n - 1] = 1.f;
    }
  }
  s.eps = 1e-3f;
  if (!empty && bounds.hi.x >= bounds.lo.x) {
    const f32 e = 1e-4f * length(bounds.hi - bounds.lo);
    s.eps = std::min(std::max(e, 1e-6f), 1e-2f);
  }
  s.strategy_count =
      u32(s.lights.size()) + (s.emissive_cdf.empty() ? 0u : 1u) + (s.has_env ? 1u : 0u);
  s.mesh.bvh.build(s.mesh.pos, s.mesh.idx);
}

Cam make_camera(const phc_camera &camera, u32 w, u32 h) // RenderBridge.cpp:872-891
{
  const V3 position = v3(camera.position);
  V3 direction = normalize(v3(camera.direction));
  if (length(direction) == 0.f)
    direction = V3{0.f, 0.f, -1.f};
  V3 up = v3(camera.up);
  if (length(cross(direction, up)) < 1e-6f)
    up = std::fabs(direction.y) < 0.9f ? V3{0.f, 1.f, 0.f} : V3{1.f, 0.f, 0.f};
  const f32 aspect = camera.aspect > 0.f ? camera.aspect : f32(w) / f32(h);
  Cam cam;
  if (camera.orthographic) {
    cam = Cam::orthographic(position, position + direction, up, camera.height, aspect);
  } else {
    const f32 fovy_degrees = camera.fovy * 180.f / 3.14159265358979f;
    const bool lens = camera.aperture_radius > 0.f && camera.focus_distance > 0.f;
    cam = Cam::perspective(position, position + direction, up, fovy_degrees, aspect,
        lens ? 2.f * camera.aperture_radius : 0.f, lens ? camera.focus_distance : 1.f);
  }
  cam.clip_near = camera.clip_near > 0.f ? camera.clip_near : 0.f;
  cam.clip_far = camera.clip_far < 1e30f ? camera.clip_far : 1e30f;
  return cam;
}

Params make_params(const phc_camera &camera, const phc_settings &st, u32 sample_offset)
{
  Params p;
  p.w = st.width;
  p.h = st.height;
  p.spp = std::max<u32>(st.pixel_samples, 1);
  p.max_depth = std::max<u32>(st.max_depth, 1);
  p.sample_offset = sample_offset;
  p.bg_color = v3(st.background);
  p.bg_alpha = st.background[3];
  if (st.background_image && st.background_width > 0 && st.background_height > 0) {
    p.bg_w = st.background_width;
    p.bg_h = st.background_height;
    p.bg_image.resize(size_t(p.bg_w) * p.bg_h);
    for (size_t k = 0; k < p.bg_image.size(); ++k) {
      const float *q = &st.background_image[4 * k];
      p.bg_image[k] = V4{q[0], q[1], q[2], q[3]};
    }
  }
  p.ambient = v3(st.ambient_color) * st.ambient_radiance;
  p.adaptive = st.adaptive_sampling != 0;
  p.tp_clamp = st.throughput_clamp;
  p.max_diffuse = st.max_diffuse_bounces;
  p.max_glossy = st.max_glossy_bounces;
  p.max_transmission = st.max_transmission_bounces;
  p.max_volume = st.max_volume_bounces;
  p.clamp_direct = 3.f * std::max(st.clamp_direct, 0.f);
  p.clamp_indirect = 3.f * std::max(st.clamp_indirect, 0.f);
  p.bottom_up = true;
  for (int i = 0; i < 4; ++i)
    p.region[i] = camera.image_region[i];
  return p;
}

int fail(Renderer *r, const std::string &m)
{
  if (r)
    r->error = m;
  g_error = m;
  return PHC_ERR_INVALID;
}

} // namespace

extern "C" {

const char *orc_global_error(void) { return g_error.c_str(); }
void *orc_renderer_create(void) { return new Renderer(); }
void orc_renderer_destroy(void *h) { delete static_cast<Renderer *>(h); }
const char *orc_last_error(void *h) { return static_cast<Renderer *>(h)->error.c_str(); }

int orc_set_scene(void *h, const phc_scene_desc *desc)
{
  auto *r = static_cast<Renderer *>(h);
  if (!desc)
    return fail(r, "null scene");
  try {
    build_scene(r->sc, *desc);
  } catch (const std::exception &e) {
    return fail(r, e.what());
  }
  r->has_scene = true;
  r->samples = 0;
  return PHC_OK;
}

int orc_render(void *h, const phc_camera *camera, const phc_settings *settings, int reset_in)
{
  auto *r = static_cast<Renderer *>(h);
  if (!camera || !settings)
    return fail(r, "null argument");
  const u32 w = settings->width, hh = settings->height;
  if (w == 0 || hh == 0)
    return fail(r, "invalid frame size");
  if (!r->has_scene)
    return fail(r, "no scene");
  bool reset = reset_in != 0;
  const size_t n = size_t(w) * hh;
  if (w != r->width || hh != r->height) {
    r->acc_color.assign(n, V3{});
    r->acc_alpha.assign(n, 0.f);
    r->first_depth.assign(n, 0.f);
    r->first_normal.assign(n, V3{});
    r->first_albedo.assign(n, V3{});
    r->width = w;
    r->height = hh;
    reset = true;
  }
  const Cam cam = make_camera(*camera, w, hh);
  const Params pr = make_params(*camera, *settings, r->sample_counter);
  r->px.resize(n);
  const Scene &sc = r->sc;
  auto &pxs = r->px;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < int64_t(n); ++i)
    for (u32 s = 0; s < pr.spp; ++s)
      render_pixel_sample(sc, cam, pr, u32(i), s, pxs[size_t(i)]);
  // pt_resolve + accumulate_frame (pathtracer.cpp:1143-1155, RenderBridge.cpp:386-410)
  const f32 weight = f32(pr.spp);
  const bool first = reset || r->samples == 0;
  for (size_t i = 0; i < n; ++i) {
    const PixelState &p = pxs[i];
    const f32 inv = p.samples > 0 ? (1.f / f32(p.samples)) : 0.f;
    const V3 color = p.accum * inv;
    const f32 alpha = p.accum_alpha * inv;
    if (first) {
      r->acc_color[i] = color * weight;
      r->acc_alpha[i] = alpha * weight;
      r->first_depth[i] = p.aov_depth;
      r->first_normal[i] = p.aov_normal;
      r->first_albedo[i] = p.aov_albedo;
    } else {
      r->acc_color[i] = r->acc_color[i] + color * weight;
      r->acc_alpha[i] = r->acc_alpha[i] + alpha * weight;
    }
  }
  r->sample_counter += pr.spp;
  r->samples = first ? pr.spp : r->samples + pr.spp;
  return PHC_OK;
}

uint32_t orc_accumulated_samples(void *h) { return static_cast<Renderer *>(h)->samples; }

int orc_read_color(void *h, float *out) // RenderBridge.cpp:1082-1107
{
  auto *r = static_cast<Renderer *>(h);
  if (!out)
    return fail(r, "null buffer");
  if (r->samples == 0)
    return fail(r, "no frame has been rendered");
  const float inv = 1.f / float(r->samples);
  for (size_t i = 0; i < r->acc_color.size(); ++i) {
    out[4 * i + 0] = r->acc_color[i].x * inv;
    out[4 * i + 1] = r->acc_color[i].y * inv;
    out[4 * i + 2] = r->acc_color[i].z * inv;
    const float a = r->acc_alpha[i] * inv;
    out[4 * i + 3] = a < 0.f ? 0.f : (a > 1.f ? 1.f : a);
  }
  return PHC_OK;
}
int orc_read_depth(void *h, float *out)
{
  auto *r = static_cast<Renderer *>(h);
  if (!out)
    return fail(r, "null buffer");
  if (r->samples == 0)
    return fail(r, "no frame has been rendered");
  for (size_t i = 0; i < r->first_depth.size(); ++i) {
    const float d = r->first_depth[i];
    out[i] = d < 1e29f ? d : std::numeric_limits<float>::infinity();
  }
  return PHC_OK;
}
static int read_v3(Renderer *r, const std::vector<V3> &v, float *out)
{
  if (!out)
    return fail(r, "null buffer");
  if (r->samples == 0)
    return fail(r, "no frame has been rendered");
  for (size_t i = 0; i < v.size(); ++i) {
    out[3 * i] = v[i].x;
    out[3 * i + 1] = v[i].y;
    out[3 * i + 2] = v[i].z;
  }
  return PHC_OK;
}
int orc_read_normal(void *h, float *out)
{
  auto *r = static_cast<Renderer *>(h);
  return read_v3(r, r->first_normal, out);
}
int orc_read_albedo(void *h, float *out)
{
  auto *r = static_cast<Renderer *>(h);
  return read_v3(r, r->first_albedo, out);
}

int orc_render_sample(void *h, const phc_camera *camera, const phc_settings *settings, uint32_t sample_index,
    float *rgb_out)
{
  auto *r = static_cast<Renderer *>(h);
  if (!r->has_scene)
    return fail(r, "no scene");
  const u32 w = settings->width, hh = settings->height;
  const Cam cam = make_camera(*camera, w, hh);
  Params pr = make_params(*camera, *settings, sample_index);
  pr.spp = 1;
  pr.adaptive = false;
  const size_t n = size_t(w) * hh;
  const Scene &sc = r->sc;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < int64_t(n); ++i) {
    PixelState p;
    render_pixel_sample(sc, cam, pr, u32(i), 0, p);
    rgb_out[3 * i] = p.accum.x;
    rgb_out[3 * i + 1] = p.accum.y;
    rgb_out[3 * i + 2] = p.accum.z;
  }
  return PHC_OK;
}

int orc_trace(const float *positions, uint64_t vertex_count, const uint32_t *indices, uint64_t triangle_count,
    const float *normals, const uint32_t *material_ids, const float *orgs, const float *dirs, const float *tmin,
    const float *tmax, uint32_t n, int any_hit, phc_hit_result *hits, uint32_t *occluded)
{
  Mesh m;
  m.pos.resize(vertex_count);
  for (uint64_t i = 0; i < vertex_count; ++i)
    m.pos[i] = v3(&positions[3 * i]);
  m.idx.assign(indices, indices + 3 * triangle_count);
  if (normals) {
    m.nrm.resize(vertex_count);
    for (uint64_t i = 0; i < vertex_count; ++i)
      m.nrm[i] = v3(&normals[3 * i]);
  }
  if (material_ids)
    m.mat_ids.assign(material_ids, material_ids + triangle_count);
  m.bvh.build(m.pos, m.idx);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < int64_t(n); ++i) {
    const V3 o = v3(&orgs[3 * i]), d = v3(&dirs[3 * i]);
    const Hit hh = intersect(m, o, d, tmin[i], tmax[i], any_hit != 0);
    if (any_hit) {
      occluded[i] = hh.hit ? 1u : 0u;
      continue;
    }
    phc_hit_result &out = hits[i];
    std::memset(&out, 0, sizeof(out));
    out.hit = hh.hit ? 1 : 0;
    if (!hh.hit)
      continue;
    const HitAttr a = hit_attributes(m, o, d, hh);
    out.t = hh.t;
    out.position[0] = a.p.x; out.position[1] = a.p.y; out.position[2] = a.p.z;
    out.normal[0] = a.n.x; out.normal[1] = a.n.y; out.normal[2] = a.n.z;
    out.shading_normal[0] = a.sn.x; out.shading_normal[1] = a.sn.y; out.shading_normal[2] = a.sn.z;
    out.bary[0] = hh.u;
    out.bary[1] = hh.v;
    out.prim_id = hh.prim;
    out.material_id = a.material_id;
  }
  return PHC_OK;
}

int orc_bsdf_probe(const phc_material *pm, const float *n_geo, const float *n_shade, const float *wo, const float *wi,
    const uint32_t *seeds, uint32_t n, float *out, float *out2)
{
  Mat m;
  m.base_color = v3(pm->base_color);
  m.metallic = pm->metallic;
  m.roughness = pm->roughness * pm->roughness;
  m.ior = pm->ior;
  m.transmission = pm->transmission;
  m.specular = 0.5f * pm->specular;
  m.clearcoat = pm->clearcoat;
  m.clearcoat_roughness = pm->clearcoat_roughness;
  m.sheen = pm->sheen;
  m.thin = pm->thin_walled ? 1 : 0;
  m.flags = F_REFRACTIVE;
  for (uint32_t i = 0; i < n; ++i) {
    const V3 ng = v3(&n_geo[3 * i]), ns = v3(&n_shade[3 * i]), o = v3(&wo[3 * i]), w = v3(&wi[3 * i]);
    const V3 f = bsdf_eval(m, o, w, ng, ns);
    const f32 pdf = bsdf_pdf(m, o, w, ng, ns);
    Rng rng(seeds[i]);
    const BS s = bsdf_sample(m, o, ng, ns, rng);
    float *r = out + 8 * i;
    r[0] = f.x; r[1] = f.y; r[2] = f.z; r[3] = pdf;
    r[4] = s.wi.x; r[5] = s.wi.y; r[6] = s.wi.z; r[7] = s.pdf;
    float *r2 = out2 + 4 * i;
    r2[0] = s.f.x; r2[1] = s.f.y; r2[2] = s.f.z;
    r2[3] = float((s.spec ? 1 : 0) | (s.diff ? 2 : 0));
  }
  return PHC_OK;
}

} // extern "C"

// FP64 CPU adjoint (test infrastructure): see the file's own header.
#include "adjoint_fp64.inc"
