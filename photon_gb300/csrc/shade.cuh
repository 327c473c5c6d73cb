// Device shading functions of the wavefront path tracer.
//
// These restate, for the GPU, the device functions the reference's pt_shade
// kernel calls, with the reference's float operation order (the translation
// unit is compiled with --fmad=false):
//   Disney BSDF           include/photon/pt/disney_bsdf.h:21-521
//   lights (point/dir/spot) include/photon/pt/light.h:66-142
//   environment map       include/photon/pt/environment_map.h:40-155
//   TF volumes            include/photon/pt/tf_volume.h:43-283 (volume_track.cuh)
//   samplers/attributes   include/photon/pt/sampler.h:73-134,
//                         src/photon/pt/pathtracer.cpp:111-247
//   light selection       src/photon/pt/pathtracer.cpp:270-367
// Read-only scene data goes through the read-only data (texture/L1) path
// with __ldg.  The functions are inlined into the kernels (each has one or
// two call sites per kernel variant): calls under the shading kernels'
// register caps cost register saves and spills (measured: 12% more
// instructions, 10% slower shading when the BSDF, material and light
// functions were called).
#pragma once

#include "cdf_search.cuh"
#include "pt_math.cuh"
#include "scene_types.h"
#include "traverse.cuh"
#include "volume_track.cuh"

namespace phc {

// ------------------------------------------------------------- material
struct Mat {
  V3 base_color;
  float metallic, roughness, ior, transmission, specular, clearcoat, clearcoat_roughness, sheen;
  V3 emission;
  float emission_strength;
  int32_t flags, thin;
};

__device__ __forceinline__ bool may_emit(const DevMaterial &m)
{
  if (m.emission_strength <= 0.f)
    return false;
  return m.src_kind[SRC_EMIT] != 0 || m.emission[0] > 0.f || m.emission[1] > 0.f || m.emission[2] > 0.f;
}
__device__ __forceinline__ V3 mat_emission(const Mat &m) { return m.emission * m.emission_strength; }
__device__ __forceinline__ bool emits_on_side(int32_t flags, bool front)
{
  if (flags & MF_EMIT_BOTH)
    return true;
  const bool back_only = (flags & MF_EMIT_BACK) != 0;
  return front ? !back_only : back_only;
}

// ------------------------------------------------------------ Disney BSDF
__device__ __forceinline__ float dielectric_f0(float ior)
{
  const float a = (1.f - ior) / (1.f + ior);
  return a * a;
}
__device__ __forceinline__ V3 schlick(float c, V3 F0, V3 F90)
{
  const float m = 1.f - saturate(c);
  const float m2 = m * m;
  const float m5 = m2 * m2 * m;
  return F0 + (F90 - F0) * m5;
}
__device__ __forceinline__ float fresnel_dielectric(float cos_i, float eta)
{
  cos_i = saturate(cos_i);
  const float sin2_t = eta * eta * (1.f - cos_i * cos_i);
  if (sin2_t >= 1.f)
    return 1.f;
  const float cos_t = sqrtf(1.f - sin2_t);
  const float r_par = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
  const float r_perp = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
  return 0.5f * (r_par * r_par + r_perp * r_perp);
}
__device__ __forceinline__ float D_ggx(float NoH, float a)
{
  const float a2 = a * a;
  const float d = NoH * NoH * (a2 - 1.f) + 1.f;
  return a2 / (PI * d * d);
}
__device__ __forceinline__ float G1(float NoV, float a)
{
  const float a2 = a * a;
  const float denom = NoV + sqrtf(a2 + (1.f - a2) * NoV * NoV);
  if (denom <= 0.f)
    return 0.f;
  return (2.f * NoV) / denom;
}
__device__ __forceinline__ float G2(float NoV, float NoL, float a) { return G1(NoV, a) * G1(NoL, a); }
__device__ __forceinline__ float ggx_pdf_refl(float NoH, float VoH, float a)
{
  const float D = D_ggx(NoH, a);
  const float denom = 4.f * fmaxf(VoH, 1e-7f);
  return D * NoH / denom;
}
__device__ __forceinline__ float spec_scale(const Mat &m) { return fmaxf(2.f * m.specular, 0.f); }
// specular_tint is 0 and anisotropic is 0 for every material of the seam.
__device__ __forceinline__ void spec_f0_f90(const Mat &m, V3 &F0, V3 &F90)
{
  const float scale = spec_scale(m);
  const float opaque = 1.f - saturate(m.transmission);
  const float f0d = fminf(dielectric_f0(m.ior) * scale, 1.f) * opaque;
  F0 = lerp(V3{f0d, f0d, f0d}, m.base_color, m.metallic);
  const float f90d = fminf(scale, 1.f) * opaque;
  F90 = lerp(V3{f90d, f90d, f90d}, V3{1.f, 1.f, 1.f}, m.metallic);
}
__device__ __forceinline__ float diffuse_scale(const Mat &m, float NoV)
{
  const float scale = spec_scale(m);
  const float f0d = fminf(dielectric_f0(m.ior) * scale, 1.f);
  const float f90d = fminf(scale, 1.f);
  const float c = 1.f - saturate(NoV);
  const float c2 = c * c;
  return 1.f - (f0d + (f90d - f0d) * c2 * c2 * c);
}
__device__ __forceinline__ bool spec_is_delta(const Mat &m) { return m.roughness < 0.001f; }
// LOBES (an LB_* mask, scene_types.h): the lobes the material can have; a
// lobe outside it has weight exactly +0 (material_lobes proves it on the
// host), so its code is left out without changing a result.
template <uint32_t LOBES = LB_ALL>
__device__ __forceinline__ void lobe_weights(const Mat &m, float NoV, float &wd, float &ws, float &wt, float &wc)
{
  const float opaque = 1.f - saturate(m.transmission);
  const float dielectric = 1.f - saturate(m.metallic);
  wd = 0.f;
  if (LOBES & LB_DIFF) {
    const float diffuse_energy = dielectric * opaque * diffuse_scale(m, NoV);
    const float base_lum = lum(m.base_color);
    wd = diffuse_energy > 0.f ? diffuse_energy * fmaxf(base_lum, 0.05f) : 0.f;
    if (m.sheen > 0.f && dielectric * opaque > 0.f)
      wd += 0.1f * m.sheen;
  }
  ws = 0.f;
  if (LOBES & LB_SPEC) {
    V3 F0, F90;
    spec_f0_f90(m, F0, F90);
    const V3 F = schlick(NoV, F0, F90);
    const float spec = lum(F);
    ws = spec > 0.f ? fmaxf(spec, 0.05f) : 0.f;
  }
  wt = (LOBES & LB_TRANS) ? saturate(m.transmission) * dielectric : 0.f;
  wc = 0.f;
  if ((LOBES & LB_COAT) && m.clearcoat > 0.f) {
    const float c = 1.f - saturate(NoV);
    const float c2 = c * c;
    wc = fmaxf(m.clearcoat * 0.25f * (0.04f + 0.96f * c2 * c2 * c), 0.02f);
  }
}
__device__ __forceinline__ V3 eval_diffuse(const Mat &m, float NoL, float NoV)
{
  const float w = (1.f - m.metallic) * (1.f - m.transmission) * diffuse_scale(m, NoV);
  if (w <= 0.f)
    return V3{0.f, 0.f, 0.f};
  return m.base_color * (w * INV_PI * NoL);
}
__device__ __forceinline__ V3 eval_spec(const Mat &m, V3 wo, V3 wi, V3 n, float a)
{
  const float NoV = saturate(dot(n, wo));
  const float NoL = saturate(dot(n, wi));
  if (NoV <= 0.f || NoL <= 0.f)
    return V3{0.f, 0.f, 0.f};
  const V3 h = normalize(wi + wo);
  const float NoH = saturate(dot(n, h));
  const float VoH = saturate(dot(wo, h));
  V3 F0, F90;
  spec_f0_f90(m, F0, F90);
  const V3 F = schlick(VoH, F0, F90);
  const float D = D_ggx(NoH, a);
  const float G = G2(NoV, NoL, a);
  const float denom = 4.f * fmaxf(NoV, 1e-7f);
  return F * (D * G / denom);
}
__device__ __forceinline__ V3 eval_sheen(const Mat &m, V3 wo, V3 wi, V3 n)
{
  if (m.sheen <= 0.f || m.metallic >= 1.f)
    return V3{0.f, 0.f, 0.f};
  const V3 h = normalize(wi + wo);
  const float HoL = fabsf(dot(h, wi));
  const float l = lum(m.base_color);
  const V3 tint = l > 0.f ? m.base_color * (1.f / l) : V3{1.f, 1.f, 1.f};
  const V3 c_sheen = lerp(V3{1.f, 1.f, 1.f}, tint, 0.5f);
  const float c = 1.f - HoL;
  const float c2 = c * c;
  const float c5 = c2 * c2 * c;
  const float NoL = saturate(dot(n, wi));
  const float w = (1.f - m.metallic) * (1.f - m.transmission);
  return c_sheen * (m.sheen * c5 * w * NoL);
}
__device__ __forceinline__ V3 eval_coat(const Mat &m, V3 wo, V3 wi, V3 n)
{
  if (m.clearcoat <= 0.f)
    return V3{0.f, 0.f, 0.f};
  const float NoV = saturate(dot(n, wo));
  const float NoL = saturate(dot(n, wi));
  if (NoV <= 0.f || NoL <= 0.f)
    return V3{0.f, 0.f, 0.f};
  const float a = fmaxf(m.clearcoat_roughness, 0.001f);
  const V3 h = normalize(wi + wo);
  const float NoH = saturate(dot(n, h));
  const float VoH = saturate(dot(wo, h));
  const float F0 = dielectric_f0(1.5f);
  const float c = 1.f - saturate(VoH);
  const float c2 = c * c;
  const float c5 = c2 * c2 * c;
  const V3 F = V3{F0, F0, F0} + (V3{1.f, 1.f, 1.f} - V3{F0, F0, F0}) * c5;
  const float D = D_ggx(NoH, a);
  const float G = G2(NoV, NoL, a);
  const float denom = 4.f * fmaxf(NoV, 1e-7f);
  const float w = m.clearcoat * 0.25f;
  return F * (w * D * G / denom);
}
// The lobes outside LOBES evaluate to exactly +0 (eval_diffuse, eval_spec
// with F0 = F90 = 0, eval_sheen, eval_coat return +0 vectors for them), and
// f + (+0) = f: leaving them out returns the same f.
template <uint32_t LOBES = LB_ALL>
static __device__ __forceinline__ V3 bsdf_eval(const Mat &m, V3 wo, V3 wi, V3 n, V3 sn)
{
  if (dot(wo, n) <= 0.f || dot(wi, n) <= 0.f)
    return V3{0.f, 0.f, 0.f};
  const float NoL = saturate(dot(sn, wi));
  const float NoV = saturate(dot(sn, wo));
  if (NoL <= 0.f || NoV <= 0.f)
    return V3{0.f, 0.f, 0.f};
  const float a = fmaxf(m.roughness, 0.001f);
  V3 f = (LOBES & LB_DIFF) ? eval_diffuse(m, NoL, NoV) : V3{0.f, 0.f, 0.f};
  if ((LOBES & LB_SPEC) && !spec_is_delta(m))
    f = f + eval_spec(m, wo, wi, sn, a);
  if (LOBES & LB_SHEEN)
    f = f + eval_sheen(m, wo, wi, sn);
  if (LOBES & LB_COAT)
    f = f + eval_coat(m, wo, wi, sn);
  return f;
}
template <uint32_t LOBES = LB_ALL>
static __device__ __forceinline__ float bsdf_pdf(const Mat &m, V3 wo, V3 wi, V3 n, V3 sn)
{
  if (dot(wo, n) <= 0.f || dot(wi, n) <= 0.f)
    return 0.f;
  const float NoL = saturate(dot(sn, wi));
  const float NoV = saturate(dot(sn, wo));
  if (NoL <= 0.f || NoV <= 0.f)
    return 0.f;
  const float a = fmaxf(m.roughness, 0.001f);
  float wd, ws, wt, wc;
  lobe_weights<LOBES>(m, NoV, wd, ws, wt, wc);
  const float sum = wd + ws + wt + wc;
  if (sum <= 0.f)
    return 0.f;
  const float pd = wd / sum, ps = ws / sum, pc = wc / sum;
  float pdf = 0.f;
  if ((LOBES & LB_DIFF) && pd > 0.f)
    pdf += pd * (NoL * INV_PI);
  if ((LOBES & LB_SPEC) && ps > 0.f && !spec_is_delta(m)) {
    const V3 h = normalize(wi + wo);
    pdf += ps * ggx_pdf_refl(saturate(dot(sn, h)), saturate(dot(wo, h)), a);
  }
  if ((LOBES & LB_COAT) && pc > 0.f) {
    const V3 h = normalize(wi + wo);
    pdf += pc * ggx_pdf_refl(saturate(dot(sn, h)), saturate(dot(wo, h)), fmaxf(m.clearcoat_roughness, 0.001f));
  }
  return fmaxf(pdf, 0.f);
}
__device__ __forceinline__ V3 ggx_half(V3 n, float a, Rng &rng)
{
  V3 t, b;
  onb(n, t, b);
  const float r1 = rng.next();
  const float r2 = rng.next();
  const float a2 = a * a;
  const float ct = sqrtf((1.f - r1) / (1.f + (a2 - 1.f) * r1));
  const float st = sqrtf(fmaxf(0.f, 1.f - ct * ct));
  const float phi = 2.f * PI * r2;
  float sp, cp;
  m_sincos(phi, sp, cp);
  return normalize(t * (st * cp) + b * (st * sp) + n * ct);
}
// Sampled lobe: 1 diffuse, 2 GGX reflection, 3 smooth (delta) specular,
// 4 dielectric reflection, 5 dielectric transmission, 6 clearcoat.  noh > 0:
// the dielectric lobes went through a GGX-sampled microfacet normal h, with
// noh = dot(n, h) (the derivative code needs its density).
enum : int { LOBE_NONE = 0, LOBE_DIFFUSE, LOBE_GLOSSY, LOBE_SPEC_DELTA, LOBE_TRANS_REFL, LOBE_TRANS, LOBE_COAT };
struct BSample {
  V3 wi, f;
  float pdf;
  bool spec, diff;
  int lobe;
  float noh;
};
// A lobe outside LOBES has probability exactly 0, so its branch is never
// taken (xi >= 0, and the sums of the selection thresholds are unchanged by
// +0 terms); leaving it out returns the same sample.
template <uint32_t LOBES = LB_ALL>
static __device__ __forceinline__ BSample bsdf_sample(const Mat &m, V3 wo, V3 n, V3 sn, Rng &rng)
{
  BSample out{V3{0.f, 0.f, 0.f}, V3{0.f, 0.f, 0.f}, 0.f, false, false, LOBE_NONE, 0.f};
  const BSample none = out;
  const bool front = dot(wo, n) > 0.f;
  if (!front && m.transmission <= 0.f)
    return out;
  const float rough = fmaxf(m.roughness, 0.001f);
  const float NoV = saturate(fabsf(dot(sn, wo)));
  float wd, ws, wt, wc, t_energy = 1.f;
  if (!front) {
    wd = 0.f;
    ws = 0.f;
    wt = 1.f;
    wc = 0.f;
  } else {
    lobe_weights<LOBES>(m, NoV, wd, ws, wt, wc);
    t_energy = wt;
  }
  const float sum = wd + ws + wt + wc;
  if (sum <= 0.f)
    return out;
  const float pd = wd / sum, ps = ws / sum, pt = wt / sum, pc = wc / sum;
  const float xi = rng.next();
  if ((LOBES & LB_DIFF) && xi < pd) {
    out.wi = cosine_hemisphere(sn, rng);
    out.diff = true;
    out.lobe = LOBE_DIFFUSE;
    out.f = bsdf_eval<LOBES>(m, wo, out.wi, n, sn);
    out.pdf = bsdf_pdf<LOBES>(m, wo, out.wi, n, sn);
    return out;
  }
  if ((LOBES & LB_SPEC) && xi < pd + ps) {
    if (spec_is_delta(m)) {
      out.wi = reflect(-wo, sn);
      if (dot(out.wi, n) <= 0.f)
        out.wi = reflect(-wo, n);
      if (dot(out.wi, n) <= 0.f)
        return none;
      V3 F0, F90;
      spec_f0_f90(m, F0, F90);
      out.f = schlick(saturate(dot(wo, sn)), F0, F90) * (1.f / ps);
      out.pdf = 1.f;
      out.spec = true;
      out.lobe = LOBE_SPEC_DELTA;
      return out;
    }
    const V3 h = ggx_half(sn, rough, rng);
    out.wi = reflect(-wo, h);
    if (dot(out.wi, n) <= 0.f)
      return none;
    out.f = bsdf_eval<LOBES>(m, wo, out.wi, n, sn);
    out.pdf = bsdf_pdf<LOBES>(m, wo, out.wi, n, sn);
    out.lobe = LOBE_GLOSSY;
    return out;
  }
  if ((LOBES & LB_TRANS) && xi < pd + ps + pt && m.transmission > 0.f) {
    const V3 nn = front ? n : n * -1.f;
    V3 snf = front ? sn : sn * -1.f;
    if (dot(snf, wo) <= 0.f)
      snf = nn;
    V3 h = snf;
    if (m.roughness >= 0.001f) {
      h = ggx_half(snf, rough, rng);
      if (dot(h, wo) <= 0.f)
        h = snf;
      else
        out.noh = dot(snf, h);
    }
    const bool refractive = (m.flags & MF_REFRACTIVE) != 0 && m.thin == 0;
    const float ior = fmaxf(m.ior, 1.0001f);
    const float eta = refractive ? (front ? (1.f / ior) : ior) : 1.f;
    const float cos_i = saturate(dot(wo, h));
    float F;
    if (refractive) {
      F = fresnel_dielectric(cos_i, eta);
    } else {
      const float f0 = dielectric_f0(m.ior);
      F = f0 + (1.f - f0) * m_pow(1.f - cos_i, 5.f);
    }
    const float lobe_weight = t_energy / pt;
    out.pdf = 1.f;
    out.spec = true;
    if (rng.next() < F) {
      out.wi = reflect(-wo, h);
      if (dot(out.wi, nn) <= 0.f) {
        out.wi = reflect(-wo, nn);
        out.noh = 0.f;
      }
      if (dot(out.wi, nn) <= 0.f)
        return none;
      out.f = V3{1.f, 1.f, 1.f} * lobe_weight;
      out.lobe = LOBE_TRANS_REFL;
      return out;
    }
    if (refractive) {
      out.wi = normalize(refract(-wo, h, eta));
      if (dot(out.wi, nn) >= 0.f) {
        out.wi = normalize(refract(-wo, snf, eta));
        out.noh = 0.f;
      }
      if (dot(out.wi, nn) >= 0.f)
        return none;
    } else {
      out.wi = normalize(-wo);
      out.noh = 0.f;
    }
    out.f = m.base_color * lobe_weight;
    out.lobe = LOBE_TRANS;
    return out;
  }
  if ((LOBES & LB_COAT) && pc > 0.f) {
    const V3 h = ggx_half(sn, fmaxf(m.clearcoat_roughness, 0.001f), rng);
    out.wi = reflect(-wo, h);
    if (dot(out.wi, n) <= 0.f)
      return none;
    out.f = bsdf_eval<LOBES>(m, wo, out.wi, n, sn);
    out.pdf = bsdf_pdf<LOBES>(m, wo, out.wi, n, sn);
    out.lobe = LOBE_COAT;
    return out;
  }
  return out;
}

// ------------------------------------------------- attributes and samplers
struct Query {
  uint32_t prim;
  uint4 vidx;
  float b1, b2;
  V3 p, sn;
  uint32_t inst = INST_NONE; // instance slot of an instanced hit
};
__device__ __forceinline__ float4 fetch_attribute(const DevScene &sc, int32_t slot, const Query &q)
{
  if (slot == 5)
    return f4(q.p, 1.f);
  if (slot == 6)
    return f4(q.sn, 1.f);
  if (!(slot >= 0 && slot < 5 && sc.attr_offset[slot] >= 0) || q.inst != INST_NONE) // instances carry no attributes
    return make_float4(0.f, 0.f, 0.f, 1.f);
  const uint32_t base = uint32_t(sc.attr_offset[slot]);
  const float4 a0 = __ldg(sc.attr_values + base + q.vidx.x);
  const float4 a1 = __ldg(sc.attr_values + base + q.vidx.y);
  const float4 a2 = __ldg(sc.attr_values + base + q.vidx.z);
  return add4(add4(mul4(a0, 1.f - q.b1 - q.b2), mul4(a1, q.b1)), mul4(a2, q.b2));
}
__device__ __forceinline__ int32_t wrap_index(int32_t i, int32_t n, int32_t mode)
{
  if (mode == 1)
    return ((i % n) + n) % n;
  if (mode == 2) {
    const int32_t j = ((i % (2 * n)) + 2 * n) % (2 * n);
    return j < n ? j : 2 * n - 1 - j;
  }
  return i < 0 ? 0 : (i >= n ? n - 1 : i);
}
// One texel of an image sampler (index within the sampler's texels): fp32
// RGBA, or 8-bit RGBA decoded through the table of the 256 floats k / 255,
// which returns the caller's original floats bit for bit.
__device__ __forceinline__ float4 sampler_texel(const DevScene &sc, const DevSampler &si, uint32_t i)
{
  if (si.u8) {
    const uchar4 t = __ldg(sc.texels_u8 + si.offset + i);
    return make_float4(__ldg(sc.u8_decode + t.x), __ldg(sc.u8_decode + t.y), __ldg(sc.u8_decode + t.z),
        __ldg(sc.u8_decode + t.w));
  }
  return __ldg(sc.texels + si.offset + i);
}
static __device__ __forceinline__ float4 sampler_sample(const DevScene &sc, int32_t id, float4 attr)
{
  if (id < 0 || uint32_t(id) >= sc.sampler_count)
    return make_float4(0.f, 0.f, 0.f, 1.f);
  const DevSampler &si = sc.samplers[uint32_t(id)];
  float4 c = mat4_mul(si.in_t, attr);
  c.x += si.in_o[0];
  c.y += si.in_o[1];
  c.z += si.in_o[2];
  c.w += si.in_o[3];
  float4 result = c;
  if (si.type != 3) {
    const int dims = si.type == 0 ? 1 : (si.type == 1 ? 2 : 3);
    const float coord[3] = {c.x, c.y, c.z};
    int32_t i0[3] = {0, 0, 0}, i1[3] = {0, 0, 0};
    float frac[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < dims; ++d) {
      const int32_t n = int32_t(si.size[d]);
      float x = coord[d];
      if (!(x > -1e6f && x < 1e6f))
        x = 0.f;
      if (si.linear) {
        const float f = x * float(n) - 0.5f;
        const float fl = floorf(f);
        frac[d] = f - fl;
        i0[d] = wrap_index(int32_t(fl), n, si.wrap[d]);
        i1[d] = wrap_index(int32_t(fl) + 1, n, si.wrap[d]);
      } else {
        i0[d] = wrap_index(int32_t(floorf(x * float(n))), n, si.wrap[d]);
        i1[d] = i0[d];
      }
    }
    const uint32_t sx = si.size[0], sxy = si.size[0] * si.size[1];
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    const int nz = dims > 2 ? 2 : 1, ny = dims > 1 ? 2 : 1;
    for (int kz = 0; kz < nz; ++kz) {
      const float wz = dims > 2 ? (kz ? frac[2] : 1.f - frac[2]) : 1.f;
      const uint32_t z = uint32_t(kz ? i1[2] : i0[2]);
      for (int ky = 0; ky < ny; ++ky) {
        const float wy = dims > 1 ? (ky ? frac[1] : 1.f - frac[1]) : 1.f;
        const uint32_t y = uint32_t(ky ? i1[1] : i0[1]);
        const float4 a = sampler_texel(sc, si, z * sxy + y * sx + uint32_t(i0[0]));
        const float4 b = sampler_texel(sc, si, z * sxy + y * sx + uint32_t(i1[0]));
        acc = add4(acc, mul4(add4(mul4(a, 1.f - frac[0]), mul4(b, frac[0])), wy * wz));
      }
    }
    result = acc;
  }
  float4 out = mat4_mul(si.out_t, result);
  out.x += si.out_o[0];
  out.y += si.out_o[1];
  out.z += si.out_o[2];
  out.w += si.out_o[3];
  return out;
}
__device__ __forceinline__ float4 eval_source(const DevScene &sc, int32_t kind, int32_t index, const Query &q)
{
  if (kind == 1)
    return fetch_attribute(sc, index, q);
  if (index < 0 || uint32_t(index) >= sc.sampler_count)
    return make_float4(0.f, 0.f, 0.f, 1.f);
  const int32_t slot = sc.samplers[uint32_t(index)].in_attribute;
  return sampler_sample(sc, index, fetch_attribute(sc, slot, q));
}
static __device__ __forceinline__ V3 apply_normal_map(const DevScene &sc, int32_t kind, int32_t index, const Query &q, V3 sn)
{
  const float4 c = eval_source(sc, kind, index, q);
  const V3 nm{2.f * c.x - 1.f, 2.f * c.y - 1.f, 2.f * c.z - 1.f};
  int32_t slot = index;
  if (kind != 1) {
    if (index < 0 || uint32_t(index) >= sc.sampler_count)
      return sn;
    slot = sc.samplers[uint32_t(index)].in_attribute;
  }
  Query corner = q;
  corner.b1 = 0.f;
  corner.b2 = 0.f;
  const float4 a0 = fetch_attribute(sc, slot, corner);
  corner.b1 = 1.f;
  const float4 a1 = fetch_attribute(sc, slot, corner);
  corner.b1 = 0.f;
  corner.b2 = 1.f;
  const float4 a2 = fetch_attribute(sc, slot, corner);
  const float du1 = a1.x - a0.x, dv1 = a1.y - a0.y, du2 = a2.x - a0.x, dv2 = a2.y - a0.y;
  const float det = du1 * dv2 - du2 * dv1;
  if (!(fabsf(det) > 1e-20f))
    return sn;
  const float4 *g = sc.prim_geo + 3 * size_t(q.prim);
  const V3 e1 = v3(__ldg(g + 1)), e2 = v3(__ldg(g + 2));
  V3 t = (e1 * dv2 - e2 * dv1) * (1.f / det);
  V3 b = (e2 * du1 - e1 * du2) * (1.f / det);
  t = t - sn * dot(sn, t);
  b = b - sn * dot(sn, b);
  if (!(dot(t, t) > 0.f) || !(dot(b, b) > 0.f))
    return sn;
  const V3 n = normalize(t) * nm.x + normalize(b) * nm.y + sn * nm.z;
  return dot(n, n) > 0.f ? normalize(n) : sn;
}
// TextureAtlas::sample (include/photon/pt/texture.h:25-64): bilinear with
// repeat wrapping, v = 1 at row 0; white for an id that is not a texture.
__device__ __forceinline__ V3 atlas_sample(const DevScene &sc, int32_t tex, float u, float v)
{
  if (tex < 0 || uint32_t(tex) >= sc.sampler_count)
    return V3{1.f, 1.f, 1.f};
  const DevSampler &si = sc.samplers[uint32_t(tex)];
  const uint32_t w = si.size[0], h = si.size[1];
  if (si.type != 4 || w == 0u || h == 0u)
    return V3{1.f, 1.f, 1.f};
  u = u - floorf(u);
  v = 1.f - (v - floorf(v));
  const float fx = u * float(w) - 0.5f, fy = v * float(h) - 0.5f;
  const int32_t ix = int32_t(floorf(fx)), iy = int32_t(floorf(fy));
  const float tx = fx - floorf(fx), ty = fy - floorf(fy);
  const int32_t sw = int32_t(w), sh = int32_t(h);
  const uint32_t x0 = uint32_t(((ix % sw) + sw) % sw), x1 = uint32_t((((ix + 1) % sw) + sw) % sw);
  const uint32_t y0 = uint32_t(((iy % sh) + sh) % sh), y1 = uint32_t((((iy + 1) % sh) + sh) % sh);
  const float4 *px = sc.texels + si.offset;
  const float4 c00 = __ldg(px + y0 * w + x0), c10 = __ldg(px + y0 * w + x1);
  const float4 c01 = __ldg(px + y1 * w + x0), c11 = __ldg(px + y1 * w + x1);
  const V3 top = v3(c00) * (1.f - tx) + v3(c10) * tx;
  const V3 bot = v3(c01) * (1.f - tx) + v3(c11) * tx;
  return top * (1.f - ty) + bot * ty;
}

// resolve_material, pathtracer.cpp:188-247.  Atlas textures (pt-level
// scenes) read the hit's uv from attribute slot 0.
// SRC = false: the scene has no attribute / sampler / atlas sources, the
// constants are the parameters (the source branches are not compiled).
template <bool SRC>
static __device__ __forceinline__ Mat resolve_material(const DevScene &sc, const DevMaterial &dm, const Query &q, float &alpha)
{
  Mat m;
  m.base_color = V3{dm.base_color[0], dm.base_color[1], dm.base_color[2]};
  m.metallic = dm.metallic;
  m.roughness = dm.roughness;
  m.ior = dm.ior;
  m.transmission = dm.transmission;
  m.specular = dm.specular;
  m.clearcoat = dm.clearcoat;
  m.clearcoat_roughness = dm.clearcoat_roughness;
  m.sheen = dm.sheen;
  m.emission = V3{dm.emission[0], dm.emission[1], dm.emission[2]};
  m.emission_strength = dm.emission_strength;
  m.flags = dm.flags;
  m.thin = dm.thin;
  alpha = dm.alpha;
  if (SRC && (dm.alpha_tex >= 0 || dm.base_tex >= 0)) {
    // an instance's uv is its barycentrics (photon_optix.cu:88-90)
    const float4 uv = q.inst != INST_NONE ? make_float4(q.b1, q.b2, 0.f, 1.f) : fetch_attribute(sc, 0, q);
    if (dm.alpha_tex >= 0)
      alpha = atlas_sample(sc, dm.alpha_tex, uv.x, uv.y).x;
    if (dm.base_tex >= 0)
      m.base_color = atlas_sample(sc, dm.base_tex, uv.x, uv.y);
  }
  if (SRC && dm.src_kind[SRC_BASE] != 0) {
    const float4 c = eval_source(sc, dm.src_kind[SRC_BASE], dm.src_index[SRC_BASE], q);
    m.base_color = V3{fmaxf(c.x, 0.f), fmaxf(c.y, 0.f), fmaxf(c.z, 0.f)};
    if (dm.base_color_alpha)
      alpha *= c.w;
  }
  if (SRC && dm.src_kind[SRC_ALPHA] != 0)
    alpha *= eval_source(sc, dm.src_kind[SRC_ALPHA], dm.src_index[SRC_ALPHA], q).x;
  if (SRC && dm.src_kind[SRC_METAL] != 0)
    m.metallic = eval_source(sc, dm.src_kind[SRC_METAL], dm.src_index[SRC_METAL], q).x;
  if (SRC && dm.src_kind[SRC_ROUGH] != 0) {
    const float r = clamp01(eval_source(sc, dm.src_kind[SRC_ROUGH], dm.src_index[SRC_ROUGH], q).x);
    m.roughness = r * r;
  }
  if (SRC && dm.src_kind[SRC_TRANS] != 0)
    m.transmission = eval_source(sc, dm.src_kind[SRC_TRANS], dm.src_index[SRC_TRANS], q).x;
  if (SRC && dm.src_kind[SRC_EMIT] != 0) {
    const float4 e = eval_source(sc, dm.src_kind[SRC_EMIT], dm.src_index[SRC_EMIT], q);
    m.emission = V3{fmaxf(e.x, 0.f), fmaxf(e.y, 0.f), fmaxf(e.z, 0.f)};
  }
  m.metallic = clamp01(m.metallic);
  m.roughness = clamp01(m.roughness);
  m.transmission = clamp01(m.transmission);
  if (dm.alpha_mode == 1)
    alpha = 1.f;
  else if (dm.alpha_mode == 2)
    alpha = alpha >= dm.alpha_cutoff ? 1.f : 0.f;
  else
    alpha = clamp01(alpha);
  return m;
}

// ------------------------------------------------------------- env map
__device__ __forceinline__ V3 mat3_mul(const float *m, V3 d)
{
  return V3{m[0] * d.x + m[1] * d.y + m[2] * d.z, m[3] * d.x + m[4] * d.y + m[5] * d.z,
      m[6] * d.x + m[7] * d.y + m[8] * d.z};
}
__device__ __forceinline__ void env_texel(const DevScene &sc, V3 dir, uint32_t &x, uint32_t &y, float &v)
{
  const V3 nd = normalize(mat3_mul(sc.env_w2t, dir));
  const float phi = m_atan2(nd.z, nd.x);
  const float yy = fminf(fmaxf(nd.y, -1.f), 1.f);
  const float theta = m_acos(yy);
  const float u = (phi + PI) * INV_TWO_PI;
  v = theta * INV_PI;
  const float xf = u * float(sc.env_w);
  const float yf = v * float(sc.env_h);
  x = uint32_t(fminf(float(sc.env_w - 1), fmaxf(0.f, xf)));
  y = uint32_t(fminf(float(sc.env_h - 1), fmaxf(0.f, yf)));
}
__device__ __forceinline__ V3 env_eval(const DevScene &sc, V3 dir)
{
  uint32_t x, y;
  float v;
  env_texel(sc, dir, x, y, v);
  return v3(__ldg(sc.env_pixels + size_t(y) * sc.env_w + x));
}
// The pdf of a texel found by env_texel (EnvironmentMap::pdf,
// environment_map.h:117-136).
__device__ __forceinline__ float env_texel_pdf(const DevScene &sc, uint32_t x, uint32_t y, float v)
{
  const float row_pdf = __ldg(sc.env_marginal + y + 1) - __ldg(sc.env_marginal + y);
  const float *c = sc.env_conditional + size_t(y) * (sc.env_w + 1);
  const float col_pdf = __ldg(c + x + 1) - __ldg(c + x);
  const float theta = v * PI;
  const float denom = TWO_PI * PI * fmaxf(m_sin(theta), 1e-6f);
  return (row_pdf * col_pdf) * float(sc.env_w) * float(sc.env_h) / denom;
}
__device__ __forceinline__ float env_pdf(const DevScene &sc, V3 dir)
{
  uint32_t x, y;
  float v;
  env_texel(sc, dir, x, y, v);
  return env_texel_pdf(sc, x, y, v);
}
// Radiance and, with want_pdf, pdf of one direction (the direction -> texel
// mapping is evaluated once for both).
__device__ __forceinline__ V3 env_eval_pdf(const DevScene &sc, V3 dir, bool want_pdf, float &pdf)
{
  uint32_t x, y;
  float v;
  env_texel(sc, dir, x, y, v);
  pdf = want_pdf ? env_texel_pdf(sc, x, y, v) : 0.f;
  return v3(__ldg(sc.env_pixels + size_t(y) * sc.env_w + x));
}
static __device__ __forceinline__ V3 env_sample(const DevScene &sc, Rng &rng, float &pdf_out)
{
  const float u1 = rng.next();
  const float u2 = rng.next();
  const uint32_t row = cdf_search_le(sc.env_marginal, sc.env_h, sc.env_mguide, ENV_MGUIDE_BITS, u2);
  const float *c = sc.env_conditional + size_t(row) * (sc.env_w + 1);
  const uint32_t col = cdf_search_le(c, sc.env_w,
      sc.env_cguide ? sc.env_cguide + size_t(row) * ((1u << ENV_CGUIDE_BITS) + 1) : nullptr, ENV_CGUIDE_BITS, u1);
  const float row_pdf = __ldg(sc.env_marginal + row + 1) - __ldg(sc.env_marginal + row);
  const float col_pdf = __ldg(c + col + 1) - __ldg(c + col);
  const float u = (float(col) + rng.next()) / float(sc.env_w);
  const float v = (float(row) + rng.next()) / float(sc.env_h);
  const float phi = u * TWO_PI - PI;
  const float theta = v * PI;
  float st, ct, sp, cp;
  m_sincos(theta, st, ct);
  m_sincos(phi, sp, cp);
  const V3 d = mat3_mul(sc.env_t2w, V3{st * cp, ct, st * sp});
  // the pdf's sin(theta) (the same angle: v * PI again)
  const float denom = TWO_PI * PI * fmaxf(st, 1e-6f);
  pdf_out = (row_pdf * col_pdf) * float(sc.env_w) * float(sc.env_h) / denom;
  return d;
}

// --------------------------------------------------------------- lights
struct LightSample {
  V3 wi, Li;
  float pdf, dist;
};
__device__ __forceinline__ V3 sphere_point(const DevLight &l, V3 p, Rng &rng)
{
  const V3 pos{l.position[0], l.position[1], l.position[2]};
  if (l.radius <= 0.f)
    return pos;
  const V3 axis = normalize(pos - p);
  V3 t, b;
  onb(axis, t, b);
  float dx, dy;
  concentric_disk(rng, dx, dy);
  return pos + (t * dx + b * dy) * l.radius;
}
static __device__ __forceinline__ LightSample sample_light(const DevLight &l, V3 p, Rng &rng)
{
  const V3 color{l.color[0], l.color[1], l.color[2]};
  const V3 pos{l.position[0], l.position[1], l.position[2]};
  const V3 dirv{l.direction[0], l.direction[1], l.direction[2]};
  if (l.type == 1) {
    V3 wi = -normalize(dirv);
    if (l.radius > 0.f) {
      const float cos_max = m_cos(l.radius);
      const float ct = 1.f - rng.next() * (1.f - cos_max);
      const float st = sqrtf(fmaxf(0.f, 1.f - ct * ct));
      const float phi = TWO_PI * rng.next();
      V3 t, b;
      onb(wi, t, b);
      float sp, cp;
      m_sincos(phi, sp, cp);
      wi = normalize(t * (st * cp) + b * (st * sp) + wi * ct);
    }
    return LightSample{wi, color * l.intensity, 1.f, 1e30f};
  }
  const V3 center_to = pos - p;
  const float cd2 = dot(center_to, center_to);
  const V3 to = sphere_point(l, p, rng) - p;
  const float dist = length(to);
  const V3 wi = dist > 0.f ? (to * (1.f / dist)) : V3{0.f, 1.f, 0.f};
  const float inv = cd2 > 0.f ? (1.f / cd2) : 0.f;
  if (l.type == 2) {
    const V3 spot_dir = normalize(dirv);
    const V3 from_light = -normalize(center_to);
    const float ca = dot(from_light, spot_dir);
    const float ci = m_cos(fmaxf(l.spot_angle - l.spot_falloff, 0.f));
    const float co = m_cos(l.spot_angle);
    float falloff = 0.f;
    if (ca >= ci)
      falloff = 1.f;
    else if (ca <= co)
      falloff = 0.f;
    else {
      float t = (ca - co) / (ci - co);
      t = t < 0.f ? 0.f : (t > 1.f ? 1.f : t);
      falloff = t * t * (3.f - 2.f * t);
    }
    return LightSample{wi, color * (l.intensity * inv * falloff), 1.f, dist};
  }
  return LightSample{wi, color * (l.intensity * inv), 1.f, dist};
}

struct DirectSample {
  V3 wi, radiance;
  float pdf, dist;
  bool mis, valid;
};
// sample_direct, pathtracer.cpp:270-367
// FULL = false: no analytic lights and no material sources in the scene.
template <bool FULL>
static __device__ __forceinline__ DirectSample sample_direct(const DevScene &sc, V3 p, Rng &rng)
{
  DirectSample ds{V3{0.f, 0.f, 0.f}, V3{0.f, 0.f, 0.f}, 0.f, 0.f, false, false};
  if (sc.strategy_count == 0)
    return ds;
  const float pick_pdf = 1.f / float(sc.strategy_count);
  uint32_t pick = uint32_t(rng.next() * float(sc.strategy_count));
  if (pick >= sc.strategy_count)
    pick = sc.strategy_count - 1;
  if (FULL && pick < sc.light_count) {
    const LightSample ls = sample_light(sc.lights[pick], p, rng);
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
  if (sc.emissive_count > 0 && pick == sc.light_count) {
    const float xi = rng.next();
    const uint32_t lo = cdf_search_gt(sc.emissive_cdf, sc.emissive_count, sc.emissive_guide, EMISSIVE_GUIDE_BITS, xi);
    const uint32_t prim = __ldg(sc.emissive_ids + lo);
    const float pdf_area = __ldg(sc.prim_light_pdf + prim);
    if (!(pdf_area > 0.f))
      return ds;
    const float4 *g = sc.prim_geo + 3 * size_t(prim);
    const V3 v0 = v3(__ldg(g)), e1 = v3(__ldg(g + 1)), e2 = v3(__ldg(g + 2));
    const uint4 vidx = __ldg(sc.prim_vidx + prim);
    // v1 and v2 as loaded by the reference (vertex positions, not v0 + e)
    const V3 v1 = v3(__ldg(sc.positions + vidx.y));
    const V3 v2 = v3(__ldg(sc.positions + vidx.z));
    const float su = sqrtf(rng.next());
    const float r2 = rng.next();
    const float b0 = 1.f - su;
    const float b1 = r2 * su;
    const float b2 = 1.f - b0 - b1;
    const V3 lp = v0 * b0 + v1 * b1 + v2 * b2;
    const V3 to = lp - p;
    const float d2 = dot(to, to);
    if (!(d2 > 0.f))
      return ds;
    const float dist = sqrtf(d2);
    const V3 wi = to * (1.f / dist);
    const V3 ln = normalize(cross(e1, e2));
    const float cos_light = -dot(wi, ln);
    if (fabsf(cos_light) < 1e-6f)
      return ds;
    Query q;
    q.prim = prim;
    q.vidx = vidx;
    q.b1 = b1;
    q.b2 = b2;
    q.p = lp;
    q.sn = ln;
    float alpha = 1.f;
    const DevMaterial &dm = sc.materials[vidx.w];
    const Mat em = resolve_material<FULL>(sc, dm, q, alpha);
    if (!emits_on_side(em.flags, cos_light > 0.f))
      return ds;
    ds.wi = wi;
    ds.radiance = mat_emission(em) * alpha;
    ds.pdf = pdf_area * d2 / fabsf(cos_light) * pick_pdf;
    ds.dist = dist;
    ds.mis = true;
    ds.valid = true;
    return ds;
  }
  if (sc.has_env) {
    float env_p = 0.f;
    const V3 wi = env_sample(sc, rng, env_p);
    if (!(env_p > 0.f))
      return ds;
    ds.wi = wi;
    ds.radiance = env_eval(sc, wi);
    ds.pdf = env_p * pick_pdf;
    ds.dist = 1e30f;
    ds.mis = true;
    ds.valid = true;
  }
  return ds;
}

} // namespace phc
