// C entry points of the CPU restatement oracle (oracle/_build/libphoton_oracle.so).
// TEST INFRASTRUCTURE ONLY — see photon_oracle.cpp.
#pragma once
#include <stdint.h>

#include "photon_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

const char *orc_global_error(void);
void *orc_renderer_create(void);
void orc_renderer_destroy(void *h);
const char *orc_last_error(void *h);
int orc_set_scene(void *h, const phc_scene_desc *desc);
int orc_render(void *h, const phc_camera *cam, const phc_settings *settings, int reset);
uint32_t orc_accumulated_samples(void *h);
int orc_read_color(void *h, float *out);
int orc_read_depth(void *h, float *out);
int orc_read_normal(void *h, float *out);
int orc_read_albedo(void *h, float *out);
int orc_trace(const float *positions, uint64_t vertex_count, const uint32_t *indices, uint64_t triangle_count,
    const float *normals, const uint32_t *material_ids, const float *orgs, const float *dirs, const float *tmin,
    const float *tmax, uint32_t n, int any_hit, phc_hit_result *hits, uint32_t *occluded);
int orc_bsdf_probe(const phc_material *m, const float *n_geo, const float *n_shade, const float *wo, const float *wi,
    const uint32_t *seeds, uint32_t n, float *out, float *out2);
/* Radiance of every path of one sample, per pixel (rgb), for per-sample
   parity: renders sample index `sample_index` alone (spp 1, no adaptive). */
int orc_render_sample(void *h, const phc_camera *cam, const phc_settings *settings, uint32_t sample_index,
    float *rgb_out);
/* FP64 CPU adjoint of the image loss sum(d_color * I) (oracle/adjoint_fp64.inc). */
int orc_adjoint_fp64(void *h, const phc_camera *camera, const phc_settings *settings, uint32_t sample_offset,
    const float *d_color, uint32_t n_params, const int32_t *kind, const int32_t *index, const int32_t *comp,
    const float *const *directions, double h_step, double *grad);

#ifdef __cplusplus
}
#endif
