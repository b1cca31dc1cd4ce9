/*
 * ibl_oracle.h -- CPU oracle for the IBL precompute.  TEST INFRASTRUCTURE
 * ONLY: the tests, the smoke check and the CPU-baseline leg of the bench
 * call it to check the product's results.  Nothing in the product library
 * links or calls it.
 *
 * O1 (restatement of the reference estimator, parity oracle of the plain
 *     path): env mip chain (vkCmdBlitImage LINEAR), Vulkan trilinear REPEAT
 *     sampling, GenIrradianceMap.comp and PreFilterEnvMap.comp.
 * O2 (FP64 quadrature, ground truth for error statements).
 * O3 (split-sum BRDF LUT, Karis 2013; FP32 same-N and FP64 forms).
 *
 * All images are RGBA32F, row-major, row 0 = v = 0.  A "chain" is every level
 * of the env mip chain stored back to back (level 0 first).
 */
#ifndef ALTHEA_IBL_ORACLE_H
#define ALTHEA_IBL_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_GEN_REF_HASH = 0, ORACLE_GEN_HAMMERSLEY = 1 };
enum { ORACLE_LUT_ASSET = 0, ORACLE_LUT_CORRECTED = 1 };

int oracle_level_count(int w, int h);
void oracle_level_dims(int w, int h, int level, int* lw, int* lh);
size_t oracle_level_offset(int w, int h, int level); /* in texels */
size_t oracle_chain_texels(int w, int h);
void oracle_build_chain(const float* level0, int w, int h, float* chain);

/* Vulkan textureLod(sampler2D REPEAT/LINEAR/LINEAR, uv, lod).rgba */
void oracle_texture_lod(const float* chain, int w, int h, float u, float v,
                        float lod, float* rgba);

/* Prefilter (PreFilterEnvMap.comp:126-177): texels listed as (x, y) pairs.
 * out: 4 floats per listed texel.  nthreads <= 0 means all cores. */
void oracle_prefilter_texels(const float* chain, int w, int h, int ow, int oh,
                             float roughness, int samples, int generator,
                             const int* xy, int n, float* out, int nthreads);
/* Whole output image (ow*oh*4 floats). */
void oracle_prefilter_image(const float* chain, int w, int h, int ow, int oh,
                            float roughness, int samples, int generator,
                            float* out, int nthreads);

/* Irradiance (GenIrradianceMap.comp:106-155) generalised to any output size:
 * grid counts and LOD come from the env size, directions from the output. */
void oracle_irradiance_texels(const float* chain, int w, int h, int ow, int oh,
                              const int* xy, int n, float* out, int nthreads);
void oracle_irradiance_image(const float* chain, int w, int h, int ow, int oh,
                             float* out, int nthreads);

/* Split-sum BRDF LUT: n x n texels of (scale, bias), FP32 with N Hammersley
 * samples (out: n*n*2 floats). */
void oracle_brdf_lut_f32(int n, int samples, int orientation, float* out,
                         int nthreads);
/* The same integral in FP64 with libm (out: n*n*2 doubles). */
void oracle_brdf_lut_f64(int n, int samples, int orientation, double* out,
                         int nthreads);

/* O2: FP64 quadrature over level-0 texels for listed output texels.
 * prefilter: sum L*w / sum w with w = D_GGX(n.h)*max(0,n.w)*Omega.
 * irradiance: (1/pi) * sum L*max(0,n.w)*Omega.  out: 4 doubles per texel
 * (rgb + the weight sum). */
void oracle_quad_prefilter_texels(const float* level0, int w, int h, int ow,
                                  int oh, double roughness, const int* xy,
                                  int n, double* out, int nthreads);
void oracle_quad_irradiance_texels(const float* level0, int w, int h, int ow,
                                   int oh, const int* xy, int n, double* out,
                                   int nthreads);

/* First outputs of the ShaderToy hash (PreFilterEnvMap.comp:38-44). */
void oracle_rng_stream(uint32_t sx, uint32_t sy, int count, float* out);

int oracle_max_threads(void);

/* Portable GLSL built-in over an array: 0 sin, 1 cos, 2 atan, 3 atan2(a,b), 4 log2. */
void oracle_builtin_eval(int fn, const float* a, const float* b, float* out, int n);

/* Reflection-buffer glossy convolution (ssr_oracle.c; Shaders/SSRGlossyConvolve.comp
 * as dispatched by Src/ReflectionBuffer.cpp:163-275).  chain: RGBA16F levels
 * packed back to back (4 uint16 per texel, level 0 first); fills levels
 * 1..mips-1 from level 0.  IEEE binary16 conversions, round to nearest even. */
float oracle_half_to_float(uint16_t h);
uint16_t oracle_float_to_half(float f);
size_t oracle_ssr_level_offset(int w, int h, int level); /* in texels */
void oracle_ssr_convolve(uint16_t* chain, int w, int h, int mips);

#ifdef __cplusplus
}
#endif
#endif
