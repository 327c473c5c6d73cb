// Path-replay adjoint (no reference counterpart: the reference has no
// derivatives).  Gradients of an image loss with respect to the Disney
// parameters of the materials (base colour, roughness, metallic, specTrans,
// sheen, clearcoat), the texels of the image samplers those parameters are
// read from (base colour, roughness, metallic, specTrans), and the
// extinction scale and albedo of homogeneous volumes.
//
// Path replay backpropagation (Vicini, Speierer and Jakob, "Path Replay
// Backpropagation", SIGGRAPH 2021), on the wavefront.  Pass 1 is the
// wavefront renderer itself, run with one pixel sample per accumulator slot:
// it leaves the radiance L of every pixel sample.  Pass 2 replays every path
// from its seed (same reference RNG streams, same shading code, so the same
// path) bounce by bounce with the renderer's queues: k_trace, k_adj_shade,
// k_shadow (deferred) and k_adj_resolve per bounce.  Each path carries the
// radiance it has yet to collect; every contribution is subtracted as it is
// collected, and each weight w the path picks up adds
//   delta . (radiance collected after w) * d log w / d theta,
// so the memory is one state per path whatever its depth.
//
// The derivative is that of the renderer's own expected image.  The sampled
// BSDF weight is f / pu with the direction drawn from the sampler's true
// density pt (pt != pu: see pdf_pair_d), so d log w = d log f - d log pu +
// d log pt; delta lobes give d log of their weight; the power-heuristic MIS
// weights contribute 2 (1 - w) d log pu (BSDF side, at the previous vertex)
// and -2 (1 - w) d log pu (light side); a rough dielectric sample adds the
// score of its GGX microfacet normal.  Lobe choice and Russian roulette
// probabilities cancel from the estimator (their weights divide by them).
// d f / d theta and the pdfs' derivatives come from forward-mode dual numbers
// (dual.cuh) over the 8 material parameters.  Clamps and stochastic
// transparency are held constant; visibility (edge) terms are not computed.
// Medium: the majorants scale with the density scale, so the derivative of a
// tracked segment's log weight is the score of its Poisson process of
// tentative collisions, (collisions - majorant optical depth) / scale, for
// delta and ratio tracking alike; a real scattering event multiplies the path
// by the albedo.
//
// Material gradients gather in a per-thread cache of the current material,
// then in block shared memory, then one global atomic per block and
// parameter; volume gradients in shared memory; texel gradients go to
// global memory with warp-aggregated atomics (lanes adding to the same texel
// channel combine first, warp_add).
#include "adjoint.h"
#include "dual.cuh"
#include "wave_common.cuh"

namespace phc {
namespace {

constexpr int NP = ADJ_MATERIAL_PARAMS; // base r, g, b, roughness, metallic, specTrans, sheen, clearcoat
using D = Dual<NP>;
constexpr int MAX_SMEM_MATERIALS = 64;
constexpr int MAX_VOLUMES = ADJ_MAX_VOLUMES;

struct D3 {
  D x, y, z;
};
__device__ __forceinline__ D3 d3(V3 v) { return D3{dconst<NP>(v.x), dconst<NP>(v.y), dconst<NP>(v.z)}; }
__device__ __forceinline__ D3 operator+(const D3 &a, const D3 &b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 operator*(const D3 &a, const D &s) { return D3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ D dlum(const D3 &c) { return c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f; }
// lerp(a, b, t) = a + (b - a) * t
__device__ __forceinline__ D dlerp(const D &a, const D &b, const D &t) { return a + (b - a) * t; }

// Material with the differentiable parameters as duals.
struct MatD {
  D3 base;
  D metallic, rough, trans, sheen, coat;
  float ior, specular, coat_rough;
};

// d/d(bridge roughness r) of the GGX alpha = r^2 is 2 r.
__device__ __forceinline__ MatD make_matd(const Mat &m)
{
  MatD d;
  d.base = D3{dvar<NP>(m.base_color.x, 0), dvar<NP>(m.base_color.y, 1), dvar<NP>(m.base_color.z, 2)};
  d.rough = dconst<NP>(m.roughness);
  d.rough.d[3] = 2.f * sqrtf(fmaxf(m.roughness, 0.f));
  d.metallic = dvar<NP>(m.metallic, 4);
  d.trans = dvar<NP>(m.transmission, 5);
  d.sheen = dvar<NP>(m.sheen, 6);
  d.coat = dvar<NP>(m.clearcoat, 7);
  d.ior = m.ior;
  d.specular = m.specular;
  d.coat_rough = m.clearcoat_roughness;
  return d;
}

__device__ __forceinline__ float f0_of(float ior)
{
  const float a = (1.f - ior) / (1.f + ior);
  return a * a;
}
__device__ __forceinline__ void spec_f0_f90_d(const MatD &m, D3 &F0, D3 &F90)
{
  const float scale = fmaxf(2.f * m.specular, 0.f);
  const D opaque = 1.f - dsat(m.trans);
  const D f0d = opaque * fminf(f0_of(m.ior) * scale, 1.f);
  F0 = D3{dlerp(f0d, m.base.x, m.metallic), dlerp(f0d, m.base.y, m.metallic), dlerp(f0d, m.base.z, m.metallic)};
  const D f90d = opaque * fminf(scale, 1.f);
  const D one = dconst<NP>(1.f);
  const D f90 = dlerp(f90d, one, m.metallic);
  F90 = D3{f90, f90, f90};
}
__device__ __forceinline__ D3 schlick_d(float c, const D3 &F0, const D3 &F90)
{
  const float k = 1.f - fminf(1.f, fmaxf(0.f, c));
  const float k2 = k * k;
  const float k5 = k2 * k2 * k;
  return D3{F0.x + (F90.x - F0.x) * k5, F0.y + (F90.y - F0.y) * k5, F0.z + (F90.z - F0.z) * k5};
}
__device__ __forceinline__ float diffuse_scale_f(const MatD &m, float NoV)
{
  const float scale = fmaxf(2.f * m.specular, 0.f);
  const float f0d = fminf(f0_of(m.ior) * scale, 1.f);
  const float f90d = fminf(scale, 1.f);
  const float c = 1.f - fminf(1.f, fmaxf(0.f, NoV));
  const float c2 = c * c;
  return 1.f - (f0d + (f90d - f0d) * c2 * c2 * c);
}
__device__ __forceinline__ D D_ggx_d(float NoH, const D &a)
{
  const D a2 = a * a;
  const D d = (a2 - 1.f) * (NoH * NoH) + 1.f;
  return a2 / (d * d * PI);
}
__device__ __forceinline__ D G1_d(float NoV, const D &a)
{
  const D a2 = a * a;
  const D denom = dsqrt(a2 + (1.f - a2) * (NoV * NoV)) + NoV;
  if (denom.v <= 0.f)
    return dconst<NP>(0.f);
  return (2.f * NoV) / denom;
}
__device__ __forceinline__ float D_ggx_f(float NoH, float a)
{
  const float a2 = a * a;
  const float d = NoH * NoH * (a2 - 1.f) + 1.f;
  return a2 / (PI * d * d);
}
__device__ __forceinline__ float G1_f(float NoV, float a)
{
  const float a2 = a * a;
  const float denom = NoV + sqrtf(a2 + (1.f - a2) * NoV * NoV);
  return denom <= 0.f ? 0.f : (2.f * NoV) / denom;
}

// Disney BSDF times cosine (disney_bsdf.h:288-307) with dual parameters.
__device__ __noinline__ D3 bsdf_eval_d(const MatD &m, V3 wo, V3 wi, V3 n, V3 sn)
{
  const D3 zero = d3(V3{0.f, 0.f, 0.f});
  if (dot(wo, n) <= 0.f || dot(wi, n) <= 0.f)
    return zero;
  const float NoL = saturate(dot(sn, wi));
  const float NoV = saturate(dot(sn, wo));
  if (NoL <= 0.f || NoV <= 0.f)
    return zero;
  D3 f = zero;
  { // diffuse
    const D w = (1.f - m.metallic) * (1.f - m.trans) * diffuse_scale_f(m, NoV);
    if (w.v > 0.f)
      f = m.base * (w * (INV_PI * NoL));
  }
  const D a = dmax(m.rough, 0.001f);
  if (!(m.rough.v < 0.001f)) { // GGX reflection (not the delta lobe)
    const V3 h = normalize(wi + wo);
    const float NoH = saturate(dot(sn, h));
    const float VoH = saturate(dot(wo, h));
    D3 F0, F90;
    spec_f0_f90_d(m, F0, F90);
    const D3 F = schlick_d(VoH, F0, F90);
    const D s = D_ggx_d(NoH, a) * G1_d(NoV, a) * G1_d(NoL, a) / (4.f * fmaxf(NoV, 1e-7f));
    f = f + F * s;
  }
  if (m.sheen.v > 0.f && m.metallic.v < 1.f) {
    const V3 h = normalize(wi + wo);
    const float HoL = fabsf(dot(h, wi));
    const D l = dlum(m.base);
    D3 tint = d3(V3{1.f, 1.f, 1.f});
    if (l.v > 0.f)
      tint = D3{m.base.x / l, m.base.y / l, m.base.z / l};
    const D half = dconst<NP>(0.5f);
    const D one = dconst<NP>(1.f);
    const D3 cs = D3{dlerp(one, tint.x, half), dlerp(one, tint.y, half), dlerp(one, tint.z, half)};
    const float c = 1.f - HoL;
    const float c2 = c * c;
    const float c5 = c2 * c2 * c;
    const D w = (1.f - m.metallic) * (1.f - m.trans);
    f = f + cs * (m.sheen * w * (c5 * NoL));
  }
  if (m.coat.v > 0.f) {
    const float ac = fmaxf(m.coat_rough, 0.001f);
    const V3 h = normalize(wi + wo);
    const float NoH = saturate(dot(sn, h));
    const float VoH = saturate(dot(wo, h));
    const float F0 = f0_of(1.5f);
    const float c = 1.f - saturate(VoH);
    const float c2 = c * c;
    const float F = F0 + (1.f - F0) * (c2 * c2 * c);
    const float s = F * D_ggx_f(NoH, ac) * G1_f(NoV, ac) * G1_f(NoL, ac) / (4.f * fmaxf(NoV, 1e-7f));
    const D w = m.coat * (0.25f * s);
    f = f + D3{w, w, w};
  }
  return f;
}

// Weight of a delta lobe (the path weight bsdf_sample returns) up to the
// constant factor 1 / (selection probability), as duals.
__device__ __forceinline__ D3 delta_weight_d(const MatD &m, int lobe, V3 wo, V3 n, V3 sn)
{
  const bool front = dot(wo, n) > 0.f;
  if (lobe == LOBE_SPEC_DELTA) {
    D3 F0, F90;
    spec_f0_f90_d(m, F0, F90);
    return schlick_d(saturate(dot(wo, sn)), F0, F90);
  }
  // dielectric boundary: t_energy / p_t, times the base colour when transmitted
  const D w = front ? dsat(m.trans) * (1.f - dsat(m.metallic)) : dconst<NP>(1.f);
  if (lobe == LOBE_TRANS)
    return D3{m.base.x * w, m.base.y * w, m.base.z * w};
  return D3{w, w, w};
}

// lobe_weights (disney_bsdf.h) with dual parameters.
__device__ __forceinline__ void lobe_weights_d(const MatD &m, float NoV, D &wd, D &ws, D &wt, D &wc)
{
  const D opaque = 1.f - dsat(m.trans);
  const D dielectric = 1.f - dsat(m.metallic);
  const D de = dielectric * opaque * diffuse_scale_f(m, NoV);
  wd = de.v > 0.f ? de * dmax(dlum(m.base), 0.05f) : dconst<NP>(0.f);
  if (m.sheen.v > 0.f && (dielectric * opaque).v > 0.f)
    wd = wd + m.sheen * 0.1f;
  D3 F0, F90;
  spec_f0_f90_d(m, F0, F90);
  const D spec = dlum(schlick_d(NoV, F0, F90));
  ws = spec.v > 0.f ? dmax(spec, 0.05f) : dconst<NP>(0.f);
  wt = dsat(m.trans) * dielectric;
  wc = dconst<NP>(0.f);
  if (m.coat.v > 0.f) {
    const float c = 1.f - saturate(NoV);
    const float c2 = c * c;
    wc = dmax(m.coat * (0.25f * (0.04f + 0.96f * c2 * c2 * c)), 0.02f);
  }
}

__device__ __forceinline__ D ggx_pdf_refl_d(float NoH, float VoH, const D &a)
{
  return D_ggx_d(NoH, a) * (NoH / (4.f * fmaxf(VoH, 1e-7f)));
}
__device__ __forceinline__ float ggx_pdf_refl_f(float NoH, float VoH, float a)
{
  return D_ggx_f(NoH, a) * NoH / (4.f * fmaxf(VoH, 1e-7f));
}

// The direction density of bsdf_sample's non-delta lobes, two ways:
//   pu  the mixture pdf the estimator divides by (bsdf_pdf, disney_bsdf.h);
//   pt  the density the sampler actually draws from.  Its diffuse lobe maps
//       the unit square through sample_concentric_disk (sampling.h:53-75),
//       whose radius |u| (resp. |v|) folds the disk onto the half x + y > 0
//       with twice the density, so the diffuse part is 2 cos / pi on that
//       half of the hemisphere (in the onb of the shading normal) and 0 on
//       the other.
// The renderer's expected image is the integral of pt * f / pu, so its
// derivative carries d log pt - d log pu besides d log f.
__device__ __noinline__ void pdf_pair_d(const MatD &m, V3 wo, V3 wi, V3 n, V3 sn, D &pu, D &pt)
{
  pu = dconst<NP>(0.f);
  pt = pu;
  if (dot(wo, n) <= 0.f || dot(wi, n) <= 0.f)
    return;
  const float NoL = saturate(dot(sn, wi));
  const float NoV = saturate(dot(sn, wo));
  if (NoL <= 0.f || NoV <= 0.f)
    return;
  D wd, ws, wt, wc;
  lobe_weights_d(m, NoV, wd, ws, wt, wc);
  const D sum = wd + ws + wt + wc;
  if (!(sum.v > 0.f))
    return;
  const D pd = wd / sum, ps = ws / sum, pc = wc / sum;
  if (pd.v > 0.f) {
    V3 t, b;
    onb(sn, t, b);
    pu = pu + pd * (NoL * INV_PI);
    if (dot(wi, t) + dot(wi, b) > 0.f)
      pt = pt + pd * (2.f * NoL * INV_PI);
  }
  if (ps.v > 0.f && !(m.rough.v < 0.001f)) {
    const V3 h = normalize(wi + wo);
    const D gs = ggx_pdf_refl_d(saturate(dot(sn, h)), saturate(dot(wo, h)), dmax(m.rough, 0.001f));
    pu = pu + ps * gs;
    pt = pt + ps * gs;
  }
  if (pc.v > 0.f) {
    const V3 h = normalize(wi + wo);
    const float gc = ggx_pdf_refl_f(saturate(dot(sn, h)), saturate(dot(wo, h)), fmaxf(m.coat_rough, 0.001f));
    pu = pu + pc * gc;
    pt = pt + pc * gc;
  }
}

// ----------------------------------------------------------------- grads
struct Grads {
  float *smat;      // shared: material_count * NP (or nullptr: global)
  float *gmat;      // global material grads
  float *svol;      // shared: volume_count * 4
  float4 *texels;   // global texel grads
  uint32_t nmat;
  // per-thread cache of one material's gradient, flushed when another
  // material comes (consecutive vertices, and NEE + sample of one vertex,
  // mostly share one): fewer contended shared-memory atomics
  uint32_t cur;
  float cache[NP];
};

__device__ __forceinline__ void flush_mat(Grads &g)
{
  if (g.cur == 0xffffffffu)
    return;
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    const float v = g.cache[k];
    g.cache[k] = 0.f;
    if (v == 0.f || !(v == v))
      continue;
    if (g.smat)
      atomicAdd(&g.smat[g.cur * NP + k], v);
    else
      atomicAdd(&g.gmat[g.cur * NP + k], v);
  }
}
__device__ __forceinline__ void add_mat(Grads &g, uint32_t m, const float *gp, uint32_t allowed)
{
  if (m != g.cur) {
    flush_mat(g);
    g.cur = m;
  }
#pragma unroll
  for (int k = 0; k < NP; ++k)
    if ((allowed >> k) & 1u)
      g.cache[k] += gp[k];
}

// Adds v to *p, the lanes of the warp that add to the same address at this
// call first combined (one atomic per distinct address instead of one per
// lane: neighbouring paths read the same texels).  Every lane converged here
// calls it; `on` says whether it has a value.
__device__ __forceinline__ void warp_add(float *p, float v, bool on, unsigned act)
{
  const unsigned long long key = on ? reinterpret_cast<unsigned long long>(p) : 0ull;
  const unsigned grp = __match_any_sync(act, key);
  float sum = 0.f;
  for (unsigned m = grp; m; m &= m - 1u)
    sum += __shfl_sync(grp, v, __ffs(int(m)) - 1);
  if (on && lane_id() == uint32_t(__ffs(int(grp)) - 1) && sum != 0.f && sum == sum)
    atomicAdd(p, sum);
}

// Texel gradients of one parameter source read from an image sampler at a
// hit: the sampler's taps (texels and bilinear / trilinear weights, as
// sampler_sample reads them) times the chain factor d param_c / d acc_j of
// resolve_material (the out transform, then max(., 0) for the base colour,
// the clamp to [0, 1] for roughness / metallic / specTrans) times the
// parameter gradients gpc[c] (three channels for the base colour, one for
// the scalars).  No-op for lanes without such a source (has = false); all
// lanes of `act` call it.
__device__ void scatter_source(float4 *texels, const DevScene &sc, bool has, int32_t id, int nch, const Query &q,
    const float *gpc, unsigned act)
{
  int n = 0;
  uint32_t idx[8];
  float w[8];
  float chain[3][4];
  for (int c = 0; c < 3; ++c)
    for (int j = 0; j < 4; ++j)
      chain[c][j] = 0.f;
  const DevSampler *sp = nullptr;
  if (has && id >= 0 && uint32_t(id) < sc.sampler_count && sc.samplers[uint32_t(id)].type != 3)
    sp = sc.samplers + uint32_t(id);
  if (sp) {
    const DevSampler &si = *sp;
    const float4 attr = fetch_attribute(sc, si.in_attribute, q);
    float4 c = mat4_mul(si.in_t, attr);
    c.x += si.in_o[0];
    c.y += si.in_o[1];
    c.z += si.in_o[2];
    const int dims = si.type == 0 ? 1 : (si.type == 1 ? 2 : 3);
    const float coord[3] = {c.x, c.y, c.z};
    int32_t i0[3] = {0, 0, 0}, i1[3] = {0, 0, 0};
    float fr[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < dims; ++d) {
      const int32_t nn = int32_t(si.size[d]);
      float x = coord[d];
      if (!(x > -1e6f && x < 1e6f))
        x = 0.f;
      if (si.linear) {
        const float f = x * float(nn) - 0.5f;
        const float fl = floorf(f);
        fr[d] = f - fl;
        i0[d] = wrap_index(int32_t(fl), nn, si.wrap[d]);
        i1[d] = wrap_index(int32_t(fl) + 1, nn, si.wrap[d]);
      } else {
        i0[d] = wrap_index(int32_t(floorf(x * float(nn))), nn, si.wrap[d]);
        i1[d] = i0[d];
      }
    }
    const uint32_t sx = si.size[0], sxy = si.size[0] * si.size[1];
    const int nz = dims > 2 ? 2 : 1, ny = dims > 1 ? 2 : 1;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int kz = 0; kz < nz; ++kz) {
      const float wz = dims > 2 ? (kz ? fr[2] : 1.f - fr[2]) : 1.f;
      const uint32_t z = uint32_t(kz ? i1[2] : i0[2]);
      for (int ky = 0; ky < ny; ++ky) {
        const float wy = dims > 1 ? (ky ? fr[1] : 1.f - fr[1]) : 1.f;
        const uint32_t y = uint32_t(ky ? i1[1] : i0[1]);
        for (int kx = 0; kx < 2; ++kx) {
          const uint32_t x = uint32_t(kx ? i1[0] : i0[0]);
          const float wt = (kx ? fr[0] : 1.f - fr[0]) * (wy * wz);
          const uint32_t ti = z * sxy + y * sx + x;
          idx[n] = si.grad_offset + ti;
          w[n] = wt;
          ++n;
          acc = add4(acc, mul4(sampler_texel(sc, si, ti), wt));
        }
      }
    }
    const float4 out = mat4_mul(si.out_t, acc);
    const float o[3] = {out.x + si.out_o[0], out.y + si.out_o[1], out.z + si.out_o[2]};
    for (int cc = 0; cc < nch; ++cc) {
      // base colour: max(o, 0); scalars: clamp01(o) (roughness: the
      // perceptual value, which the adjoint's gradient is taken against)
      const bool live = nch == 3 ? o[cc] > 0.f : (o[cc] > 0.f && o[cc] < 1.f);
      for (int j = 0; j < 4; ++j)
        chain[cc][j] = live ? si.out_t[4 * cc + j] * gpc[cc] : 0.f;
    }
  }
  // the warp's lanes walk the taps together; lanes with fewer (or none) add nothing
  __syncwarp(act);
  const int n_max = int(__reduce_max_sync(act, uint32_t(n)));
  for (int t = 0; t < n_max; ++t) {
    float *tp = reinterpret_cast<float *>(texels + (t < n ? idx[t] : 0u));
    for (int j = 0; j < 4; ++j) {
      const float v = t < n ? w[t] * (chain[0][j] + chain[1][j] + chain[2][j]) : 0.f;
      warp_add(tp + j, v, t < n && v != 0.f && v == v, act);
    }
  }
}

// gp += sum_c k_c * (d f_c / d theta) / f_c
__device__ __forceinline__ void add_dlog3(const D3 &f, V3 k, float *gp)
{
  const D *fc[3] = {&f.x, &f.y, &f.z};
  const float kc[3] = {k.x, k.y, k.z};
  for (int c = 0; c < 3; ++c) {
    const float fv = fc[c]->v;
    if (!(fv > 0.f) || kc[c] == 0.f)
      continue;
    const float s = kc[c] / fv;
#pragma unroll
    for (int p = 0; p < NP; ++p)
      gp[p] += s * fc[c]->d[p];
  }
}
// gp += K * d log x / d theta
__device__ __forceinline__ void add_dlog(const D &x, float K, float *gp)
{
  if (!(x.v > 0.f) || K == 0.f)
    return;
  const float s = K / x.v;
#pragma unroll
  for (int p = 0; p < NP; ++p)
    gp[p] += s * x.d[p];
}

// Scatters a vertex's parameter gradient gp into its material (the
// parameters it takes as constants) and, for parameters read from image
// samplers (base colour, roughness, metallic, specTrans), into their texels.
// All lanes converged here call it (the texel scatter is warp-cooperative).
__device__ void scatter_grads(Grads &g, const DevScene &sc, const DevMaterial &dm, uint32_t mat_id, const Query &q,
    const float *gp, bool on = true)
{
  const int src_of[NP] = {SRC_BASE, SRC_BASE, SRC_BASE, SRC_ROUGH, SRC_METAL, SRC_TRANS, -1, -1};
  if (on) {
    uint32_t allowed = 0;
#pragma unroll
    for (int p = 0; p < NP; ++p)
      if (src_of[p] < 0 || dm.src_kind[src_of[p]] == 0)
        allowed |= 1u << p;
    add_mat(g, mat_id, gp, allowed);
  }
  if (!g.texels)
    return;
  const unsigned act = __activemask();
  const bool any_src = on && (dm.src_kind[SRC_BASE] == 2 || dm.src_kind[SRC_ROUGH] == 2 ||
      dm.src_kind[SRC_METAL] == 2 || dm.src_kind[SRC_TRANS] == 2);
  if (!__any_sync(act, any_src))
    return;
  const float gb[3] = {gp[0], gp[1], gp[2]};
  scatter_source(g.texels, sc, on && dm.src_kind[SRC_BASE] == 2, dm.src_index[SRC_BASE], 3, q, gb, act);
  const int scalars[3] = {SRC_ROUGH, SRC_METAL, SRC_TRANS};
  for (int k = 0; k < 3; ++k) {
    const bool has = on && dm.src_kind[scalars[k]] == 2;
    if (!__any_sync(act, has))
      continue;
    const float gs[3] = {gp[3 + k], 0.f, 0.f};
    scatter_source(g.texels, sc, has, dm.src_index[scalars[k]], 1, q, gs, act);
  }
}

// ------------------------------------------------- volumes with d log weight
// VolumeSet::track (tf_volume.h:150-232) that also adds to dlog the
// derivative of the log tracking weight per unit of the volume's density
// scale.
__device__ float vol_track_d(const DevScene &sc, const DevVolume &v, V3 org, V3 dir, float t0, float t1, Rng &rng,
    bool scatter, V3 &albedo, float &tr, float &dlog)
{
  const float o[3] = {org.x, org.y, org.z}, d[3] = {dir.x, dir.y, dir.z};
  const float ds = v.density_scale;
  int cell[3], step[3];
  float t_next[3], t_delta[3];
  for (int a = 0; a < 3; ++a) {
    const int m = int(v.macro_dims[a]);
    const float extent = v.spacing[a] * float(v.dims[a] > 1 ? v.dims[a] - 1 : 1);
    const float cpu = float(m) / extent;
    const float g = (o[a] + d[a] * t0 - v.origin[a]) * cpu;
    int c = int(g);
    c = c < 0 ? 0 : (c > m - 1 ? m - 1 : c);
    cell[a] = c;
    const float speed = d[a] * cpu;
    if (speed > 0.f) {
      step[a] = 1;
      t_delta[a] = 1.f / speed;
      t_next[a] = t0 + (float(c + 1) - g) * t_delta[a];
    } else if (speed < 0.f) {
      step[a] = -1;
      t_delta[a] = -1.f / speed;
      t_next[a] = t0 + (g - float(c)) * t_delta[a];
    } else {
      step[a] = 0;
      t_delta[a] = 1e30f;
      t_next[a] = 1e30f;
    }
  }
  // Every majorant (macro cell) is proportional to the density scale ds, so
  // the real / null split and the ratio-tracking factors do not depend on it:
  // only the Poisson process of tentative collisions does.  Its log density
  // is  n log mu - tau  (n collisions, tau = majorant optical depth covered),
  // whose derivative per unit of ds is (n - tau) / ds.
  float t = t0;
  int lookups = 0;
  float n = 0.f, tau = 0.f;
  auto finish = [&]() {
    if (ds > 0.f)
      dlog += (n - tau) / ds;
  };
  for (int visited = 0; visited < 4096; ++visited) {
    const int axis = t_next[0] < t_next[1] ? (t_next[0] < t_next[2] ? 0 : 2) : (t_next[1] < t_next[2] ? 1 : 2);
    const float t_exit = t_next[axis] < t1 ? t_next[axis] : t1;
    const float bound = __ldg(sc.vol_majorants + v.macro_offset +
        (uint32_t(cell[2]) * v.macro_dims[1] + uint32_t(cell[1])) * v.macro_dims[0] + uint32_t(cell[0]));
    if (bound > 0.f) {
      const float inv_bound = 1.f / bound;
      const float cell_start = t;
      while (lookups < 8192) {
        t -= m_log(1.f - rng.next()) * inv_bound;
        if (t >= t_exit)
          break;
        ++lookups;
        n += 1.f;
        const float4 c = vol_classify(sc, v, org + dir * t);
        if (scatter) {
          if (rng.next() * bound < c.w) {
            albedo = V3{c.x, c.y, c.z};
            tau += bound * (t - cell_start);
            finish();
            return t;
          }
        } else {
          tr *= 1.f - c.w * inv_bound;
          if (tr < 0.05f) {
            if (!(tr > 0.f) || rng.next() * 0.05f >= tr) {
              tr = 0.f;
              tau += bound * (t - cell_start);
              finish();
              return -1.f;
            }
            tr = 0.05f;
          }
        }
      }
      tau += bound * (fminf(t, t_exit) - cell_start);
    }
    t = t_exit;
    if (t_exit >= t1 || lookups >= 8192)
      break;
    cell[axis] += step[axis];
    if (cell[axis] < 0 || cell[axis] >= int(v.macro_dims[axis]))
      break;
    t_next[axis] += t_delta[axis];
  }
  finish();
  return -1.f;
}

__device__ float vol_scatter_d(const DevScene &sc, V3 ro, V3 rd, float tmin, float tmax, Rng &rng, V3 &albedo,
    float *dlog, int &event_vol)
{
  float t_event = -1.f, t_limit = tmax, unused = 1.f;
  event_vol = -1;
  for (uint32_t vi = 0; vi < sc.volume_count; ++vi) {
    const DevVolume &v = sc.volumes[vi];
    if (v.majorant <= 0.f || v.tf_size == 0)
      continue;
    const V3 org = vol_point(v, ro), dir = vol_vector(v, rd);
    float t0 = tmin, t1 = t_limit;
    if (!vol_clip(v, org, dir, t0, t1))
      continue;
    V3 ea{0.f, 0.f, 0.f};
    float dl = 0.f;
    const float t = vol_track_d(sc, v, org, dir, t0, t1, rng, true, ea, unused, dl);
    if (vi < uint32_t(MAX_VOLUMES))
      dlog[vi] += dl;
    if (t >= 0.f) {
      t_event = t;
      t_limit = t;
      albedo = ea;
      event_vol = int(vi);
    }
  }
  return t_event;
}

__device__ float vol_transmittance_d(const DevScene &sc, V3 ro, V3 rd, float tmin, float tmax, Rng &rng, float *dlog)
{
  float tr = 1.f;
  V3 unused{0.f, 0.f, 0.f};
  for (uint32_t vi = 0; vi < sc.volume_count; ++vi) {
    const DevVolume &v = sc.volumes[vi];
    if (v.majorant <= 0.f || v.tf_size == 0)
      continue;
    const V3 org = vol_point(v, ro), dir = vol_vector(v, rd);
    float t0 = tmin, t1 = tmax;
    if (!vol_clip(v, org, dir, t0, t1))
      continue;
    float dl = 0.f;
    vol_track_d(sc, v, org, dir, t0, t1, rng, false, unused, tr, dl);
    if (vi < uint32_t(MAX_VOLUMES))
      dlog[vi] += dl;
    if (tr <= 0.f)
      return 0.f;
  }
  return tr;
}

__device__ __forceinline__ void add_vol(Grads &g, const float *dlog, uint32_t nvol, float k)
{
  for (uint32_t vi = 0; vi < nvol && vi < uint32_t(MAX_VOLUMES); ++vi)
    if (dlog[vi] != 0.f && k != 0.f)
      atomicAdd(&g.svol[4 * vi], k * dlog[vi]);
}

// ---------------------------------------------------------------- grads
// Per-block gradient accumulators: materials in shared memory (up to
// MAX_SMEM_MATERIALS, else straight to global), volumes in shared memory;
// flushed to global memory once per block.
__device__ __forceinline__ Grads begin_grads(float *smat, float *svol, const DevScene &sc, const AdjointArgs &a)
{
  const bool shared_mat = sc.material_count <= uint32_t(MAX_SMEM_MATERIALS);
  for (uint32_t i = threadIdx.x; i < MAX_SMEM_MATERIALS * NP; i += blockDim.x)
    smat[i] = 0.f;
  for (uint32_t i = threadIdx.x; i < MAX_VOLUMES * 4; i += blockDim.x)
    svol[i] = 0.f;
  __syncthreads();
  Grads g;
  g.smat = shared_mat ? smat : nullptr;
  g.gmat = a.mat_grads;
  g.svol = svol;
  g.texels = a.texel_grads;
  g.nmat = sc.material_count;
  g.cur = 0xffffffffu;
#pragma unroll
  for (int k = 0; k < NP; ++k)
    g.cache[k] = 0.f;
  return g;
}
__device__ __forceinline__ void end_grads(Grads &g, const DevScene &sc, const AdjointArgs &a)
{
  flush_mat(g);
  __syncthreads();
  if (g.smat)
    for (uint32_t i = threadIdx.x; i < sc.material_count * NP; i += blockDim.x)
      if (g.smat[i] != 0.f)
        atomicAdd(&a.mat_grads[i], g.smat[i]);
  for (uint32_t i = threadIdx.x; i < MAX_VOLUMES * 4 && i < sc.volume_count * 4; i += blockDim.x)
    if (g.svol[i] != 0.f)
      atomicAdd(&a.vol_grads[i], g.svol[i]);
}

__device__ __forceinline__ void put_vtx(const VtxSoA &v, uint32_t i, const Query &q, uint32_t mat)
{
  v.q[i] = make_uint4(q.prim, __float_as_uint(q.b1), __float_as_uint(q.b2), mat | ADJ_VTX_VALID);
  v.p[i] = f4(q.p, 0.f);
  v.sn[i] = f4(q.sn, 0.f);
}
// The material and hit query of a stored vertex; false: none stored.
__device__ bool get_vtx(const DevScene &sc, const VtxSoA &v, uint32_t i, uint32_t &mat, Query &q)
{
  const uint4 q4 = v.q[i];
  if (!(q4.w & ADJ_VTX_VALID))
    return false;
  mat = q4.w & ~ADJ_VTX_VALID;
  q.prim = q4.x;
  q.vidx = __ldg(sc.prim_vidx + q4.x);
  q.b1 = __uint_as_float(q4.y);
  q.b2 = __uint_as_float(q4.z);
  q.p = v3(v.p[i]);
  q.sn = v3(v.sn[i]);
  return true;
}

// d log w / d theta of the power-heuristic weight w that the previous
// surface sample's pdf pu entered (BSDF side): 2 (1 - w) d log pu, applied
// to the emission e that the weight multiplied, at the previous vertex.
__device__ void mis_prev(Grads &g, const DevScene &sc, const AdjPathSoA &in, uint32_t i, V3 delta, V3 e, float w)
{
  if (!(w < 1.f))
    return;
  const float K = dot(delta, e) * 2.f * (1.f - w);
  if (K == 0.f)
    return;
  uint32_t mat;
  Query q;
  if (!get_vtx(sc, in.v, i, mat, q))
    return;
  const float4 a = in.g0[i], b = in.g1[i];
  const float gp[NP] = {K * a.x, K * a.y, K * a.z, K * a.w, K * b.x, K * b.y, K * b.z, K * b.w};
  scatter_grads(g, sc, sc.materials[mat], mat, q, gp);
}

// What one replayed path hands on: its continuation and its shadow ray.
struct AdjNext {
  float4 o, d, tp;
  uint4 info;
  float pdist;
  float4 rem, g0, g1;
  bool has_vtx;
  Query vq;
  uint32_t vmat;
};
struct AdjShadow {
  float4 a, b, c, g0, g1;
  bool has_vtx;
};

// One bounce of one replayed path: shade_path (shade_kernels.cu) with the
// derivative bookkeeping of the path-replay adjoint.  Contributions known now
// (emission, environment) are collected here; the NEE contribution waits for
// its shadow ray (k_adj_resolve), so the BSDF sample's gradient is taken with
// the remainder before NEE and the shadow ray carries the correction.
__device__ __forceinline__ void adj_shade_path(const RenderConst &rc, const DevScene &sc, const AdjPathSoA &in,
    uint32_t i, float4 hit, int it, const AdjointArgs &a, Grads &g, bool &cont, AdjNext &nx, bool &has_sh,
    AdjShadow &sh)
{
  cont = false;
  has_sh = false;
  const float4 ro4 = in.p.ray_o[i], rd4 = in.p.ray_d[i], tp4 = in.p.tp[i];
  const uint4 info = in.p.info[i];
  const float pdist = in.p.pdist[i];
  const uint32_t slot = info.x, sample_index = info.y;
  const uint32_t pixel = slot % rc.npix;
  uint32_t kinds = info.z;
  const uint32_t depth = info.w & 0xffffu;
  bool primary = (info.w >> 16) & 1u;
  const bool prev_valid = (info.w & ADJ_PREV_VALID) != 0u;
  const bool emission_only = (kinds & EMISSION_ONLY) != 0u;
  const V3 ray_org = v3(ro4), ray_dir = v3(rd4);
  V3 tp = v3(tp4);
  const float prev_pdf = tp4.w;
  const uint32_t max_depth = rc.max_depth;
  const float eps = sc.eps;
  const uint32_t nvol = sc.volume_count;
  const uint32_t prim = __float_as_uint(hit.y);
  const bool is_hit = prim != 0xffffffffu;
  V3 rem = it == 0 ? v3(a.primal[slot]) : v3(in.rem[i]);
  const float4 dI = a.d_image[pixel];
  const V3 delta{dI.x * a.inv_spp, dI.y * a.inv_spp, dI.z * a.inv_spp};
  float4 col = a.collected[slot];
  auto collect = [&](V3 c) {
    rem = rem - c;
    col.x = col.x + c.x;
    col.y = col.y + c.y;
    col.z = col.z + c.z;
  };
  auto done = [&]() { a.collected[slot] = col; };
  Rng rng = path_rng(pixel, sample_index, 1u + uint32_t(it));

  if (nvol > 0) { // volume segment (pathtracer.cpp:789-858)
    V3 albedo{0.f, 0.f, 0.f};
    float dlog[MAX_VOLUMES] = {0.f, 0.f, 0.f, 0.f};
    int ev = -1;
    const float t_end = is_hit ? hit.x : rd4.w;
    const float t_sc = vol_scatter_d(sc, ray_org, ray_dir, ro4.w, t_end, rng, albedo, dlog, ev);
    add_vol(g, dlog, nvol, dot(delta, rem)); // the segment scales everything collected from here on
    if (t_sc >= 0.f && ev >= 0 && ev < MAX_VOLUMES) { // the scatter weight is the albedo
      if (albedo.x > 0.f)
        atomicAdd(&g.svol[4 * ev + 1], delta.x * rem.x / albedo.x);
      if (albedo.y > 0.f)
        atomicAdd(&g.svol[4 * ev + 2], delta.y * rem.y / albedo.y);
      if (albedo.z > 0.f)
        atomicAdd(&g.svol[4 * ev + 3], delta.z * rem.z / albedo.z);
    }
    if (t_sc >= 0.f) {
      const V3 p = ray_org + ray_dir * t_sc;
      primary = false;
      if (depth >= max_depth || emission_only) {
        done();
        return;
      }
      const V3 tpa = tp * albedo;
      const float phase = 0.25f * INV_PI;
      const DirectSample ds = sample_direct<true>(sc, p, rng);
      if (ds.valid) {
        const float w_mis = ds.mis ? power_heuristic(ds.pdf, phase) : 1.f;
        const V3 c = clamp_contrib(tpa * ds.radiance * (phase * w_mis / ds.pdf), int(depth), rc.clamp_direct,
            rc.clamp_indirect);
        const float stmax = ds.dist < 1e29f ? ds.dist * (1.f - 1e-4f) : 1e30f;
        has_sh = true;
        sh.a = f4(p, stmax);
        sh.b = f4(ds.wi, c.x);
        sh.c = make_float4(c.y, c.z, __uint_as_float(slot), __uint_as_float(sample_index));
        sh.g0 = make_float4(0.f, 0.f, 0.f, 0.f);
        sh.g1 = sh.g0;
        sh.has_vtx = false;
      }
      V3 tp_next = tpa;
      if (depth >= 2) {
        const float max_tp = fmaxf(tpa.x, fmaxf(tpa.y, tpa.z));
        const float survive = fminf(fmaxf(max_tp, 0.05f), 0.95f);
        if (rng.next() >= survive) {
          done();
          return;
        }
        tp_next = tpa * (1.f / survive);
      }
      if (count_bounce(kinds, 24u, rc.max_volume))
        kinds |= EMISSION_ONLY;
      const V3 nd = uniform_sphere(rng);
      cont = true;
      nx.o = f4(p, 0.f);
      nx.d = f4(nd, 1e30f);
      nx.tp = f4(tp_next, phase);
      nx.info = make_uint4(slot, sample_index, kinds, depth + 1u);
      nx.pdist = pdist;
      nx.rem = f4(rem, 0.f);
      nx.has_vtx = false;
      done();
      return;
    }
  }

  if (!is_hit) { // miss (pathtracer.cpp:860-899)
    V3 Lm{0.f, 0.f, 0.f};
    if (primary) {
      if (sc.has_env && sc.env_visible)
        Lm = env_eval(sc, ray_dir);
      else if (rc.bg_image) {
        const uint32_t x = pixel % rc.w, y = pixel / rc.w;
        const float4 bg = bg_image(rc, (float(x) + 0.5f) / float(rc.w), (float(y) + 0.5f) / float(rc.h));
        Lm = V3{bg.x, bg.y, bg.z} * bg.w;
      } else
        Lm = rc3(rc.bg) * rc.bg[3];
    } else {
      Lm = rc3(rc.ambient);
      if (sc.has_env) {
        float w_mis = 1.f;
        if (prev_pdf > 0.f)
          w_mis = power_heuristic(prev_pdf, env_pdf(sc, ray_dir) / float(sc.strategy_count));
        const V3 le = env_eval(sc, ray_dir);
        Lm = Lm + le * w_mis;
        if (prev_valid)
          mis_prev(g, sc, in, i, delta, tp * le * w_mis, w_mis);
      }
    }
    V3 c = tp * Lm;
    if (!primary || (sc.has_env && sc.env_visible))
      c = clamp_contrib(c, int(depth) - 1, rc.clamp_direct, rc.clamp_indirect);
    collect(c);
    done();
    return;
  }

  const RayHit rh{hit.x, prim, hit.z, hit.w};
  const HitAttr ha = hit_attributes(sc, ray_org, ray_dir, rh);
  const V3 p = ha.p;
  const V3 wo = -ray_dir;
  V3 hit_sn = ha.sn;
  if (!(dot(hit_sn, hit_sn) > 0.25f))
    hit_sn = ha.n;
  else if (dot(hit_sn, ha.n) < 0.f)
    hit_sn = hit_sn * -1.f;
  Query q;
  q.prim = prim;
  q.vidx = ha.vidx;
  q.b1 = rh.u;
  q.b2 = rh.v;
  q.p = p;
  q.sn = hit_sn;
  float alpha_val = 1.f;
  const DevMaterial &dm = sc.materials[ha.material_id];
  const Mat mat = resolve_material<true>(sc, dm, q, alpha_val);
  const bool hidden = (mat.flags & MF_HIDDEN) != 0 && primary;
  if (hidden || (alpha_val < 1.f && rng.next() >= alpha_val)) { // stochastic transparency
    float tmin = eps, tmax = 1e30f;
    const float nd = pdist + rh.t;
    if (primary) {
      float tn, tf;
      clip_range(rc, ray_dir, tn, tf);
      if (tf < 1e30f) {
        tmax = tf - nd;
        if (tmax < eps) {
          tmin = 1.f;
          tmax = 0.f;
        }
      }
    }
    cont = true;
    nx.o = f4(p, tmin);
    nx.d = f4(ray_dir, tmax);
    nx.tp = f4(tp, -1.f);
    nx.info = make_uint4(slot, sample_index, kinds, depth | (primary ? 1u << 16 : 0u));
    nx.pdist = nd;
    nx.rem = f4(rem, 0.f);
    nx.has_vtx = false;
    done();
    return;
  }
  V3 n = ha.n, sn = hit_sn;
  const bool front = dot(n, wo) >= 0.f;
  if (!(mat.transmission > 0.f) && !front) {
    n = n * -1.f;
    sn = sn * -1.f;
  }
  if (dm.src_kind[SRC_NORMAL] != 0)
    sn = apply_normal_map(sc, dm.src_kind[SRC_NORMAL], dm.src_index[SRC_NORMAL], q, sn);
  primary = false;
  if (may_emit(dm) && emits_on_side(mat.flags, front)) {
    float w_mis = 1.f;
    if (prev_pdf > 0.f && sc.emissive_count > 0) {
      const float pdf_area = __ldg(sc.prim_light_pdf + prim);
      const float cos_light = fabsf(dot(ha.n, wo));
      if (pdf_area > 0.f && cos_light > 0.f)
        w_mis = power_heuristic(prev_pdf, pdf_area * rh.t * rh.t / cos_light / float(sc.strategy_count));
    }
    const V3 e = clamp_contrib(tp * mat_emission(mat) * w_mis, int(depth) - 1, rc.clamp_direct, rc.clamp_indirect);
    collect(e);
    if (prev_valid)
      mis_prev(g, sc, in, i, delta, e, w_mis);
  }
  if ((mat.flags & MF_EMITTER_ONLY) != 0 || depth >= max_depth || emission_only) {
    done();
    return;
  }
  const MatD md = make_matd(mat);
  float gnee[NP];
#pragma unroll
  for (int k = 0; k < NP; ++k)
    gnee[k] = 0.f;
  V3 cnee{0.f, 0.f, 0.f};
  { // next event estimation: the shadow ray and its gradient per unit transmittance
    const DirectSample ds = sample_direct<true>(sc, p, rng);
    if (ds.valid) {
      const V3 f = bsdf_eval(mat, wo, ds.wi, n, sn);
      if (f.x > 0.f || f.y > 0.f || f.z > 0.f) {
        float w_mis = 1.f;
        if (ds.mis)
          w_mis = power_heuristic(ds.pdf, bsdf_pdf(mat, wo, ds.wi, n, sn));
        const V3 c = clamp_contrib(tp * f * ds.radiance * (w_mis / ds.pdf), int(depth), rc.clamp_direct,
            rc.clamp_indirect);
        const V3 so = p + n * eps;
        V3 sd;
        float stmax;
        if (ds.dist < 1e29f) {
          const V3 to_light = p + ds.wi * ds.dist - so;
          const float sdist = length(to_light);
          sd = sdist > 0.f ? to_light * (1.f / sdist) : ds.wi;
          stmax = sdist * (1.f - 1e-3f);
        } else {
          sd = ds.wi;
          stmax = 1e30f;
        }
        has_sh = true;
        sh.a = f4(so, stmax);
        sh.b = f4(sd, c.x);
        sh.c = make_float4(c.y, c.z, __uint_as_float(slot), __uint_as_float(sample_index));
        sh.has_vtx = true;
        cnee = c;
        add_dlog3(bsdf_eval_d(md, wo, ds.wi, n, sn), delta * c, gnee);
        if (ds.mis && w_mis < 1.f) { // d log w_nee = -2 (1 - w_nee) d log pu
          D pu, pt;
          pdf_pair_d(md, wo, ds.wi, n, sn, pu, pt);
          add_dlog(pu, -2.f * (1.f - w_mis) * dot(delta, c), gnee);
        }
      }
    }
  }
  const BSample bs = bsdf_sample(mat, wo, n, sn, rng);
  const bool sampled = !(bs.pdf <= 0.f || (bs.f.x <= 0.f && bs.f.y <= 0.f && bs.f.z <= 0.f));
  float grem[NP], gc[NP];
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    grem[k] = 0.f;
    gc[k] = 0.f;
  }
  bool prev_next = false;
  float gpu[NP];
  if (sampled) { // everything still to come passes through this sample's weight
    const V3 krem = delta * rem, kc = delta * cnee;
    const float Krem = krem.x + krem.y + krem.z, Kc = kc.x + kc.y + kc.z;
    if (bs.lobe == LOBE_DIFFUSE || bs.lobe == LOBE_GLOSSY || bs.lobe == LOBE_COAT) {
      D pu, pt; // weight f / pu of a direction drawn from pt
      pdf_pair_d(md, wo, bs.wi, n, sn, pu, pt);
      const D3 fd = bsdf_eval_d(md, wo, bs.wi, n, sn);
      add_dlog3(fd, krem, grem);
      add_dlog(pt, Krem, grem);
      add_dlog(pu, -Krem, grem);
      add_dlog3(fd, kc, gc);
      add_dlog(pt, Kc, gc);
      add_dlog(pu, -Kc, gc);
      if (pu.v > 0.f) {
        prev_next = true;
#pragma unroll
        for (int k = 0; k < NP; ++k)
          gpu[k] = pu.d[k] / pu.v;
      }
    } else {
      const D3 wd = delta_weight_d(md, bs.lobe, wo, n, sn);
      add_dlog3(wd, krem, grem);
      add_dlog3(wd, kc, gc);
      if (bs.noh > 0.f) { // the microfacet normal's density D(h) cos (ggx_half)
        const D dh = D_ggx_d(bs.noh, dmax(md.rough, 0.001f));
        add_dlog(dh, Krem, grem);
        add_dlog(dh, Kc, gc);
      }
    }
    scatter_grads(g, sc, dm, ha.material_id, q, grem);
  }
  if (has_sh) { // per unit transmittance: the NEE gradient minus the part the sample's term took
    sh.g0 = make_float4(gnee[0] - gc[0], gnee[1] - gc[1], gnee[2] - gc[2], gnee[3] - gc[3]);
    sh.g1 = make_float4(gnee[4] - gc[4], gnee[5] - gc[5], gnee[6] - gc[6], gnee[7] - gc[7]);
  }
  nx.vq = q;
  nx.vmat = ha.material_id;
  done();
  if (!sampled)
    return;
  V3 tpn = tp * (bs.f * (1.f / bs.pdf));
  if (depth >= 2) {
    const float max_tp = fmaxf(tpn.x, fmaxf(tpn.y, tpn.z));
    const float survive = fminf(fmaxf(max_tp, 0.05f), 0.95f);
    if (rng.next() >= survive)
      return;
    tpn = tpn * (1.f / survive);
  }
  if (rc.tp_clamp > 0.f) {
    const float mx = fmaxf(tpn.x, fmaxf(tpn.y, tpn.z));
    if (mx > rc.tp_clamp)
      tpn = tpn * (rc.tp_clamp / mx);
  }
  if (!finite3(tpn))
    return;
  const V3 wi = normalize(bs.wi);
  const float side = dot(wi, ha.n) < 0.f ? -1.f : 1.f;
  const bool through = (dot(wi, ha.n) < 0.f) != (dot(wo, ha.n) < 0.f);
  const bool exceeded = through ? count_bounce(kinds, 16u, rc.max_transmission)
                                : (bs.diff ? count_bounce(kinds, 0u, rc.max_diffuse)
                                           : count_bounce(kinds, 8u, rc.max_glossy));
  if (exceeded)
    kinds |= EMISSION_ONLY;
  cont = true;
  nx.o = f4(p + ha.n * (side * eps), 0.f);
  nx.d = f4(wi, 1e30f);
  nx.tp = f4(tpn, bs.spec ? -1.f : bs.pdf);
  nx.info = make_uint4(slot, sample_index, kinds, (depth + 1u) | (prev_next && !bs.spec ? ADJ_PREV_VALID : 0u));
  nx.pdist = pdist;
  nx.rem = f4(rem, 0.f);
  nx.has_vtx = prev_next && !bs.spec;
  if (nx.has_vtx) {
    nx.g0 = make_float4(gpu[0], gpu[1], gpu[2], gpu[3]);
    nx.g1 = make_float4(gpu[4], gpu[5], gpu[6], gpu[7]);
  }
}

// Minimum resident 128-thread blocks per SM for the replay shading kernel
// (caps its registers; see k_shade).
#ifndef PHC_ADJ_MIN_BLOCKS
#define PHC_ADJ_MIN_BLOCKS 10
#endif
// hq.hitq (optional): the closest-hit kernel's hit / miss queues, the hits
// sorted by material when there are at least hq.sort_threshold of them; the
// paths are then replayed hits first, in that order, then the misses, so
// that a warp's lanes mostly run one material's code.
__global__ void __launch_bounds__(128, PHC_ADJ_MIN_BLOCKS) k_adj_shade(const RenderConst *__restrict__ rcp, DevScene sc, AdjPathSoA in,
    AdjPathSoA out, const float4 *__restrict__ hits, AdjShadowSoA sh, WaveCounters wc, int it, AdjointArgs a,
    HitQueues hq)
{
  if (wave_failed(wc)) // a traversal warp stopped at its trip cap: its results are incomplete
    return;
  __shared__ float smat[MAX_SMEM_MATERIALS * NP];
  __shared__ float svol[MAX_VOLUMES * 4];
  Grads g = begin_grads(smat, svol, sc, a);
  const RenderConst &rc = *rcp;
  const uint32_t n = wc.count[it];
  uint32_t *fetch = wc.fetch + 4 * it + 1;
  for (;;) {
    const uint32_t base = warp_fetch(fetch);
    if (base >= n)
      break;
    const uint32_t j = base + lane_id();
    bool cont = false, has_sh = false;
    AdjNext nx;
    AdjShadow sr;
    if (j < n) {
      uint32_t i = j;
      if (hq.hitq) {
        const uint32_t hc = wc.hcount[it];
        const bool sorted = hq.sorted != nullptr && hq.sort_threshold != 0u && hc >= hq.sort_threshold;
        i = j < hc ? (sorted ? hq.sorted[j] : hq.hitq[j]) : hq.missq[j - hc];
      }
      adj_shade_path(rc, sc, in, i, hits[i], it, a, g, cont, nx, has_sh, sr);
    }
    const uint32_t o = warp_append(wc.count + it + 1, cont);
    if (cont) {
      out.p.ray_o[o] = nx.o;
      out.p.ray_d[o] = nx.d;
      out.p.tp[o] = nx.tp;
      out.p.info[o] = nx.info;
      out.p.pdist[o] = nx.pdist;
      out.rem[o] = nx.rem;
      if (nx.has_vtx) {
        out.g0[o] = nx.g0;
        out.g1[o] = nx.g1;
        put_vtx(out.v, o, nx.vq, nx.vmat);
      }
    }
    const uint32_t so = warp_append(wc.scount + it, has_sh);
    if (has_sh) {
      sh.s.a[so] = sr.a;
      sh.s.b[so] = sr.b;
      sh.s.c[so] = sr.c;
      sh.next[so] = cont ? o : ADJ_NO_NEXT;
      sh.g0[so] = sr.g0;
      sh.g1[so] = sr.g1;
      if (sr.has_vtx)
        put_vtx(sh.v, so, nx.vq, nx.vmat);
      else
        sh.v.q[so] = make_uint4(0u, 0u, 0u, 0u);
    }
  }
  end_grads(g, sc, a);
}

// The shadow rays of one bounce after k_shadow (deferred mode): for each
// unoccluded one the transmittance (with its derivative), the contribution
// collected, the continued path's remainder reduced, the vertex's gradient.
__global__ void __launch_bounds__(128) k_adj_resolve(const RenderConst *__restrict__ rcp, DevScene sc,
    AdjShadowSoA sh, AdjPathSoA next, WaveCounters wc, int it, AdjointArgs a)
{
  if (wave_failed(wc)) // a traversal warp stopped at its trip cap: its results are incomplete
    return;
  __shared__ float smat[MAX_SMEM_MATERIALS * NP];
  __shared__ float svol[MAX_VOLUMES * 4];
  Grads g = begin_grads(smat, svol, sc, a);
  const uint32_t n = wc.scount[it];
  const uint32_t npix = rcp->npix;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 s4 = sh.s.a[i];
    if (!(s4.w >= 0.f))
      continue;
    const float4 b4 = sh.s.b[i], c4 = sh.s.c[i];
    const uint32_t slot = __float_as_uint(c4.z), sample_index = __float_as_uint(c4.w);
    const uint32_t pixel = slot % npix;
    float T = 1.f;
    float dlt[MAX_VOLUMES] = {0.f, 0.f, 0.f, 0.f};
    if (sc.volume_count > 0) {
      Rng rs = path_rng(pixel, sample_index, 0x10000u + uint32_t(it));
      T = vol_transmittance_d(sc, v3(s4), v3(b4), 0.f, s4.w, rs, dlt);
    }
    const V3 c = V3{b4.w, c4.x, c4.y} * T;
    if (!finite3(c))
      continue;
    float4 col = a.collected[slot];
    col.x = col.x + c.x;
    col.y = col.y + c.y;
    col.z = col.z + c.z;
    a.collected[slot] = col;
    const uint32_t nx = sh.next[i];
    if (nx != ADJ_NO_NEXT) {
      float4 r = next.rem[nx];
      r.x = r.x - c.x;
      r.y = r.y - c.y;
      r.z = r.z - c.z;
      next.rem[nx] = r;
    }
    const float4 dI = a.d_image[pixel];
    const V3 delta{dI.x * a.inv_spp, dI.y * a.inv_spp, dI.z * a.inv_spp};
    add_vol(g, dlt, sc.volume_count, dot(delta, c));
    uint32_t mat;
    Query q;
    if (get_vtx(sc, sh.v, i, mat, q)) {
      const float4 u = sh.g0[i], w = sh.g1[i];
      const float gp[NP] = {T * u.x, T * u.y, T * u.z, T * u.w, T * w.x, T * w.y, T * w.z, T * w.w};
      scatter_grads(g, sc, sc.materials[mat], mat, q, gp);
    }
  }
  end_grads(g, sc, a);
}

// The replay collected what the forward pass did (same path), and the image
// of the pass's samples.
__global__ void __launch_bounds__(256) k_adj_finish(uint32_t slots, AdjointArgs a)
{
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < slots; i += gridDim.x * blockDim.x) {
    const float4 L = a.primal[i], C = a.collected[i];
    const float tol = 1e-4f * fmaxf(fabsf(L.x) + fabsf(L.y) + fabsf(L.z), 1e-2f);
    if (!(fabsf(C.x - L.x) + fabsf(C.y - L.y) + fabsf(C.z - L.z) <= tol))
      atomicAdd(a.mismatches, 1ull);
    if (a.radiance) {
      const uint32_t pixel = i % a.npix;
      atomicAdd(a.radiance + 3 * pixel, L.x);
      atomicAdd(a.radiance + 3 * pixel + 1, L.y);
      atomicAdd(a.radiance + 3 * pixel + 2, L.z);
    }
  }
}

} // namespace

void launch_adj_shade(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, AdjPathSoA in,
    AdjPathSoA out, const float4 *hits, AdjShadowSoA sh, WaveCounters wc, int it, AdjointArgs a, HitQueues hq)
{
  k_adj_shade<<<c.blocks_shade, 128, 0, s>>>(rc, sc, in, out, hits, sh, wc, it, a, hq);
}

void launch_adj_resolve(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, AdjShadowSoA sh,
    AdjPathSoA next, WaveCounters wc, int it, AdjointArgs a)
{
  k_adj_resolve<<<c.blocks_shade, 128, 0, s>>>(rc, sc, sh, next, wc, it, a);
}

void launch_adj_finish(cudaStream_t s, int blocks, uint32_t slots, AdjointArgs a)
{
  k_adj_finish<<<blocks, 256, 0, s>>>(slots, a);
}

int adj_shade_max_active_blocks(int threads)
{
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_adj_shade, threads, 0) != cudaSuccess)
    return 1;
  return n > 0 ? n : 1;
}

} // namespace phc
