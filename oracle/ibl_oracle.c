/*
 * ibl_oracle.c -- CPU oracle for the IBL precompute (TEST INFRASTRUCTURE:
 * only tests/, the smoke check and the bench's CPU-baseline leg use it).
 *
 * A plain-C restatement of the reference algorithm, written from the
 * reference sources cited at each function.  Floating-point expressions keep
 * the operation order of the GLSL source (left-to-right, no contraction: build
 * with -ffp-contract=off), and the GLSL transcendental built-ins are bound to
 * the portable implementations in glsl_builtins.h, so this oracle is
 * bit-for-bit reproducible on any IEEE-754 host.
 */
#include "ibl_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../althea_gb300/csrc/glsl_builtins.h"

#define PI_F 3.14159265359f /* PreFilterEnvMap.comp:4 (a float literal in GLSL) */

typedef struct {
  float x, y, z;
} v3;

static v3 mk3(float x, float y, float z) {
  v3 r = {x, y, z};
  return r;
}

static int set_threads(int nthreads) {
#ifdef _OPENMP
  return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  (void)nthreads;
  return 1;
#endif
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ---------------------------------------------------------------------------
 * Mip chain.  Level count: Src/Utilities.cpp:97-100 (1 + floor(log2(max))).
 * Level sizes: Src/Image.cpp:157-166 (w >> l, minimum 1).
 * Content: Src/Image.cpp:184-213, vkCmdBlitImage with VK_FILTER_LINEAR from
 * level l-1 into level l; per the Vulkan blit rules the destination texel
 * centre (x+0.5) is scaled by src/dst extent and filtered bilinearly with
 * clamp-to-edge addressing.  For even sizes this is an exact 2x2 box.
 * ------------------------------------------------------------------------- */
int oracle_level_count(int w, int h) {
  int m = w > h ? w : h;
  return 1 + (int)floor(log2((double)m));
}

void oracle_level_dims(int w, int h, int level, int* lw, int* lh) {
  int a = w >> level, b = h >> level;
  *lw = a < 1 ? 1 : a;
  *lh = b < 1 ? 1 : b;
}

size_t oracle_level_offset(int w, int h, int level) {
  size_t off = 0;
  for (int l = 0; l < level; ++l) {
    int lw, lh;
    oracle_level_dims(w, h, l, &lw, &lh);
    off += (size_t)lw * (size_t)lh;
  }
  return off;
}

size_t oracle_chain_texels(int w, int h) {
  return oracle_level_offset(w, h, oracle_level_count(w, h));
}

/* Bilinear combination in the order used everywhere in this project:
 * ((w00*t00 + w10*t10) + w01*t01) + w11*t11, w00=(1-a)(1-b), w10=a(1-b),
 * w01=(1-a)b, w11=ab (Vulkan spec, "Linear filtering"). */
static void bilerp(const float* t00, const float* t10, const float* t01,
                   const float* t11, float a, float b, float* out) {
  float w00 = (1.0f - a) * (1.0f - b);
  float w10 = a * (1.0f - b);
  float w01 = (1.0f - a) * b;
  float w11 = a * b;
  for (int c = 0; c < 4; ++c)
    out[c] = ((w00 * t00[c] + w10 * t10[c]) + w01 * t01[c]) + w11 * t11[c];
}

static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

void oracle_build_chain(const float* level0, int w, int h, float* chain) {
  int levels = oracle_level_count(w, h);
  memcpy(chain, level0, (size_t)w * h * 4 * sizeof(float));
  for (int l = 1; l < levels; ++l) {
    int sw, sh, dw, dh;
    oracle_level_dims(w, h, l - 1, &sw, &sh);
    oracle_level_dims(w, h, l, &dw, &dh);
    const float* src = chain + 4 * oracle_level_offset(w, h, l - 1);
    float* dst = chain + 4 * oracle_level_offset(w, h, l);
    float sx = (float)sw / (float)dw, sy = (float)sh / (float)dh;
    for (int y = 0; y < dh; ++y) {
      float v = ((float)y + 0.5f) * sy - 0.5f;
      float fy = floorf(v);
      float b = v - fy;
      int j0 = clampi((int)fy, 0, sh - 1), j1 = clampi((int)fy + 1, 0, sh - 1);
      for (int x = 0; x < dw; ++x) {
        float u = ((float)x + 0.5f) * sx - 0.5f;
        float fx = floorf(u);
        float a = u - fx;
        int i0 = clampi((int)fx, 0, sw - 1), i1 = clampi((int)fx + 1, 0, sw - 1);
        bilerp(src + 4 * ((size_t)j0 * sw + i0), src + 4 * ((size_t)j0 * sw + i1),
               src + 4 * ((size_t)j1 * sw + i0), src + 4 * ((size_t)j1 * sw + i1),
               a, b, dst + 4 * ((size_t)y * dw + x));
      }
    }
  }
}

/* ---------------------------------------------------------------------------
 * textureLod with the precompute sampler: REPEAT in u and v, LINEAR min/mag,
 * LINEAR mipmap, minLod 0, maxLod mipCount-1 (Src/ImageBasedLighting.cpp:
 * 168-174, Src/Sampler.cpp:90-113).  Vulkan spec texel filtering: the LOD is
 * clamped to [0, q]; levels floor(lod) and min(floor(lod)+1, q) are blended
 * by frac(lod); each level samples at (u*w - 0.5, v*h - 0.5) with REPEAT
 * wrap of the integer texel coordinates.
 * ------------------------------------------------------------------------- */
static int wrap(int i, int n) {
  int r = i % n;
  return r < 0 ? r + n : r;
}

static void sample_level(const float* chain, int w, int h, int level, float u,
                         float v, float* out) {
  int lw, lh;
  oracle_level_dims(w, h, level, &lw, &lh);
  const float* img = chain + 4 * oracle_level_offset(w, h, level);
  float x = u * (float)lw - 0.5f;
  float y = v * (float)lh - 0.5f;
  float fx = floorf(x), fy = floorf(y);
  float a = x - fx, b = y - fy;
  int i0 = wrap((int)fx, lw), i1 = wrap((int)fx + 1, lw);
  int j0 = wrap((int)fy, lh), j1 = wrap((int)fy + 1, lh);
  bilerp(img + 4 * ((size_t)j0 * lw + i0), img + 4 * ((size_t)j0 * lw + i1),
         img + 4 * ((size_t)j1 * lw + i0), img + 4 * ((size_t)j1 * lw + i1), a,
         b, out);
}

void oracle_texture_lod(const float* chain, int w, int h, float u, float v,
                        float lod, float* rgba) {
  int q = oracle_level_count(w, h) - 1;
  float lam = lod;
  if (lam < 0.0f) lam = 0.0f;
  if (lam > (float)q) lam = (float)q;
  float fl = floorf(lam);
  int l0 = (int)fl;
  float d = lam - fl;
  sample_level(chain, w, h, l0, u, v, rgba);
  if (d > 0.0f) {
    float hi[4];
    int l1 = l0 + 1 > q ? q : l0 + 1;
    sample_level(chain, w, h, l1, u, v, hi);
    for (int c = 0; c < 4; ++c) rgba[c] = (1.0f - d) * rgba[c] + d * hi[c];
  }
}

/* ---------------------------------------------------------------------------
 * Shared shader helpers (identical in both .comp files).
 * ------------------------------------------------------------------------- */

/* coordinateSystem / LocalToWorld: PreFilterEnvMap.comp:22-34,
 * GenIrradianceMap.comp:19-31.  Columns (t, b, n). */
static void local_to_world(v3 n, v3* t, v3* b) {
  if (agb_abs(n.x) > agb_abs(n.y)) {
    float s = sqrtf(n.x * n.x + n.z * n.z);
    *t = mk3(-n.z / s, 0.0f / s, n.x / s);
  } else {
    float s = sqrtf(n.y * n.y + n.z * n.z);
    *t = mk3(0.0f / s, n.z / s, -n.y / s);
  }
  /* cross(n, t) */
  *b = mk3(n.y * t->z - n.z * t->y, n.z * t->x - n.x * t->z,
           n.x * t->y - n.y * t->x);
}

/* mat3(t, b, n) * v = t*v.x + b*v.y + n*v.z, component-wise left to right. */
static v3 mat_mul(v3 t, v3 b, v3 n, v3 v) {
  return mk3((t.x * v.x + b.x * v.y) + n.x * v.z,
             (t.y * v.x + b.y * v.y) + n.y * v.z,
             (t.z * v.x + b.z * v.y) + n.z * v.z);
}

/* Texel corner direction: texelUv = texelPos / size (no +0.5),
 * yaw = PI*(2u-1), pitch = PI*(v-0.5) (PreFilterEnvMap.comp:129-134). */
static v3 texel_dir(int x, int y, int ow, int oh) {
  float u = (float)x / (float)ow;
  float v = (float)y / (float)oh;
  float yaw = PI_F * (2.0f * u - 1.0f);
  float pitch = PI_F * (v - 0.5f);
  float cp = agb_cos(pitch);
  return mk3(cp * agb_cos(yaw), agb_sin(pitch), cp * agb_sin(yaw));
}

/* sampleEnvMap: PreFilterEnvMap.comp:98-122 (GenIrradianceMap.comp:78-102). */
static void sample_env(const float* chain, int w, int h, v3 dir, float mip,
                       float* rgba) {
  float pitch = 0.0f, yaw = 0.0f;
  float len_xz = sqrtf(dir.x * dir.x + dir.z * dir.z);
  if (len_xz > 0.001f) {
    yaw = agb_atan2(dir.z, dir.x);
    pitch = agb_atan(dir.y / len_xz);
  } else if (dir.y > 0.0f) {
    pitch = 0.5f * PI_F;
  } else {
    pitch = -0.5f * PI_F;
  }
  float u = yaw / (2.0f * PI_F) + 0.5f;
  float v = pitch / PI_F + 0.5f;
  oracle_texture_lod(chain, w, h, u, v, mip, rgba);
}

/* GLSL max(x, y) = x < y ? y : x (GLSL spec 8.3). */
static float glsl_max(float x, float y) { return x < y ? y : x; }

/* ---------------------------------------------------------------------------
 * Sample generators.
 * ref-hash: rng() of PreFilterEnvMap.comp:38-44, seeded with the texel
 * position (:127); two calls per sample (:85).
 * hammersley: xi = (i/N, bitreverse(i) * 2^-32) for sample i.
 * ------------------------------------------------------------------------- */
static float rng_next(uint32_t* sx, uint32_t* sy) {
  *sx += 1u;
  *sy += 1u;
  uint32_t qx = 1103515245u * ((*sx >> 1u) ^ *sy);
  uint32_t qy = 1103515245u * ((*sy >> 1u) ^ *sx);
  uint32_t n = 1103515245u * (qx ^ (qy >> 3u));
  return (float)n * (1.0f / 4294967296.0f);
}

void oracle_rng_stream(uint32_t sx, uint32_t sy, int count, float* out) {
  for (int i = 0; i < count; ++i) out[i] = rng_next(&sx, &sy);
}

static uint32_t bitrev32(uint32_t v) {
  v = ((v >> 1) & 0x55555555u) | ((v & 0x55555555u) << 1);
  v = ((v >> 2) & 0x33333333u) | ((v & 0x33333333u) << 2);
  v = ((v >> 4) & 0x0f0f0f0fu) | ((v & 0x0f0f0f0fu) << 4);
  v = ((v >> 8) & 0x00ff00ffu) | ((v & 0x00ff00ffu) << 8);
  return (v >> 16) | (v << 16);
}

static void hammersley(int i, int n, float* x, float* y) {
  *x = (float)i / (float)n;
  *y = (float)bitrev32((uint32_t)i) * (1.0f / 4294967296.0f);
}

/* distributionGGX: PreFilterEnvMap.comp:78-82. */
static float distribution_ggx(float ndoth, float a2) {
  float denom = (ndoth * ndoth * (a2 - 1.0f) + 1.0f);
  return a2 / (PI_F * denom * denom);
}

/* sampleGGX: PreFilterEnvMap.comp:84-92 (xi supplied by the generator). */
static v3 sample_ggx(float xi_x, float xi_y, float a2) {
  float phi = 2.0f * PI_F * xi_x;
  float cos_t = sqrtf((1.0f - xi_y) / (1.0f + (a2 - 1.0f) * xi_y));
  float sin_t = sqrtf(1.0f - cos_t * cos_t);
  return mk3(agb_cos(phi) * sin_t, agb_sin(phi) * sin_t, cos_t);
}

/* main of PreFilterEnvMap.comp:126-177 for one output texel. */
static void prefilter_texel(const float* chain, int w, int h, int ow, int oh,
                            float roughness, int samples, int generator, int x,
                            int y, float* out) {
  uint32_t sx = (uint32_t)x, sy = (uint32_t)y;
  v3 n = texel_dir(x, y, ow, oh);
  v3 r = n, v = r;
  float a = roughness;
  float a2 = a * a;
  v3 t, b;
  local_to_world(n, &t, &b);
  float acc[3] = {0.0f, 0.0f, 0.0f};
  float total = 0.0f;
  for (int i = 0; i < samples; ++i) {
    float xi_x, xi_y;
    if (generator == ORACLE_GEN_HAMMERSLEY) {
      hammersley(i, samples, &xi_x, &xi_y);
    } else {
      xi_x = rng_next(&sx, &sy);
      xi_y = rng_next(&sx, &sy);
    }
    v3 hv = mat_mul(t, b, n, sample_ggx(xi_x, xi_y, a2));
    float vdh = (v.x * hv.x + v.y * hv.y) + v.z * hv.z;
    float k = 2.0f * vdh;
    v3 l = mk3(k * hv.x - v.x, k * hv.y - v.y, k * hv.z - v.z);
    float len = sqrtf((l.x * l.x + l.y * l.y) + l.z * l.z);
    l = mk3(l.x / len, l.y / len, l.z / len);
    float ndotl = glsl_max((n.x * l.x + n.y * l.y) + n.z * l.z, 0.0f);
    float ndoth = glsl_max((n.x * hv.x + n.y * hv.y) + n.z * hv.z, 0.0f);
    float hdotv = glsl_max((hv.x * v.x + hv.y * v.y) + hv.z * v.z, 0.0f);
    float d = distribution_ggx(ndoth, a2);
    float pdf = d * ndoth / (4.0f * hdotv + 0.00001f);
    float sa_texel = 4.0f * PI_F / (6.0f * (float)w * (float)h);
    float sa_sample = 1.0f / ((float)samples * pdf + 0.0001f);
    float mip = roughness == 0.0f ? 0.0f : 0.5f * agb_log2(sa_sample / sa_texel);
    if (ndotl > 0.0f) {
      float c[4];
      sample_env(chain, w, h, l, mip, c);
      acc[0] += c[0] * ndotl;
      acc[1] += c[1] * ndotl;
      acc[2] += c[2] * ndotl;
      total += ndotl;
    }
  }
  out[0] = acc[0] / total;
  out[1] = acc[1] / total;
  out[2] = acc[2] / total;
  out[3] = 1.0f;
}

void oracle_prefilter_texels(const float* chain, int w, int h, int ow, int oh,
                             float roughness, int samples, int generator,
                             const int* xy, int n, float* out, int nthreads) {
  int nt = set_threads(nthreads);
  (void)nt;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
  for (int i = 0; i < n; ++i)
    prefilter_texel(chain, w, h, ow, oh, roughness, samples, generator,
                    xy[2 * i], xy[2 * i + 1], out + 4 * (size_t)i);
}

void oracle_prefilter_image(const float* chain, int w, int h, int ow, int oh,
                            float roughness, int samples, int generator,
                            float* out, int nthreads) {
  int nt = set_threads(nthreads);
  (void)nt;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
  for (long i = 0; i < (long)ow * oh; ++i)
    prefilter_texel(chain, w, h, ow, oh, roughness, samples, generator,
                    (int)(i % ow), (int)(i / ow), out + 4 * (size_t)i);
}

/* main of GenIrradianceMap.comp:106-155, output size decoupled from the env
 * size: the grid counts (:119-121) and LOD (:124) use the env size. */
static void irradiance_texel(const float* chain, int w, int h, int ow, int oh,
                             int x, int y, float* out) {
  v3 n = texel_dir(x, y, ow, oh);
  v3 t, b;
  local_to_world(n, &t, &b);
  float acc[3] = {0.0f, 0.0f, 0.0f};
  int theta_samples = 300;
  int phi_samples = (int)((float)h * (float)theta_samples / (float)w);
  float mip = agb_log2((float)w / (float)theta_samples);
  for (int i = 0; i < theta_samples; ++i) {
    float theta = (float)(i * 2) * PI_F / (float)theta_samples;
    float ct = agb_cos(theta), st = agb_sin(theta);
    for (int j = 0; j < phi_samples; ++j) {
      float phi = (float)j * 0.5f * PI_F / (float)phi_samples;
      float cp = agb_cos(phi), sp = agb_sin(phi);
      v3 d = mat_mul(t, b, n, mk3(ct * sp, st * sp, cp));
      float c[4];
      sample_env(chain, w, h, d, mip, c);
      acc[0] += c[0] * cp * sp;
      acc[1] += c[1] * cp * sp;
      acc[2] += c[2] * cp * sp;
    }
  }
  out[0] = PI_F * acc[0] / (float)theta_samples / (float)phi_samples;
  out[1] = PI_F * acc[1] / (float)theta_samples / (float)phi_samples;
  out[2] = PI_F * acc[2] / (float)theta_samples / (float)phi_samples;
  out[3] = 1.0f;
}

void oracle_irradiance_texels(const float* chain, int w, int h, int ow, int oh,
                              const int* xy, int n, float* out, int nthreads) {
  int nt = set_threads(nthreads);
  (void)nt;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
  for (int i = 0; i < n; ++i)
    irradiance_texel(chain, w, h, ow, oh, xy[2 * i], xy[2 * i + 1],
                     out + 4 * (size_t)i);
}

void oracle_irradiance_image(const float* chain, int w, int h, int ow, int oh,
                             float* out, int nthreads) {
  int nt = set_threads(nthreads);
  (void)nt;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
  for (long i = 0; i < (long)ow * oh; ++i)
    irradiance_texel(chain, w, h, ow, oh, (int)(i % ow), (int)(i / ow),
                     out + 4 * (size_t)i);
}

/* ---------------------------------------------------------------------------
 * O3: split-sum BRDF LUT (Karis, "Real Shading in Unreal Engine 4",
 * SIGGRAPH 2013 course notes, IntegrateBRDF).  The reference ships only the
 * baked asset Content/PrecomputedMaps/brdf_lut.png (loaded at
 * Src/ImageBasedLighting.cpp:570-603, read as (NdotV, roughness) at
 * Shaders/PBR/PBRMaterial.glsl:110-111).  GGX alpha = roughness^2,
 * Smith-Schlick k = alpha/2, Hammersley samples, Fc = (1 - VoH)^5.
 * Column i: NoV = (i + 0.5)/n.  Row j: roughness = 1 - (j + 0.5)/n in the
 * asset orientation (row 0 = roughness 1), (j + 0.5)/n when corrected.
 * ------------------------------------------------------------------------- */
static float lut_roughness(int j, int n, int orientation) {
  float t = ((float)j + 0.5f) / (float)n;
  return orientation == ORACLE_LUT_ASSET ? 1.0f - t : t;
}

static void lut_texel_f32(int i, int j, int n, int samples, int orientation,
                          float* out) {
  float nov = ((float)i + 0.5f) / (float)n;
  float rough = lut_roughness(j, n, orientation);
  float vx = sqrtf(1.0f - nov * nov), vz = nov;
  float alpha = rough * rough;
  float a2 = alpha * alpha;
  float k = alpha / 2.0f;
  /* G_vis = G1(L) G1(V) VoH / (NoH NoV) with G1(V) / NoV = 1 / (NoV (1 - k) + k)
   * taken once per texel and 1 / NoH once per sample */
  float gv = 1.0f / (nov * (1.0f - k) + k);
  float sum_a = 0.0f, sum_b = 0.0f;
  for (int s = 0; s < samples; ++s) {
    float xi_x, xi_y;
    hammersley(s, samples, &xi_x, &xi_y);
    float phi = 2.0f * PI_F * xi_x;
    float cos_t = sqrtf((1.0f - xi_y) / (1.0f + (a2 - 1.0f) * xi_y));
    float sin_t = sqrtf(1.0f - cos_t * cos_t);
    float hx = sin_t * agb_cos(phi), hz = cos_t;
    float noh = hz > 0.0f ? (hz < 1.0f ? hz : 1.0f) : 0.0f;
    /* V.y = 0; the sample's terms as the LUT kernels compute them */
    agb_lut_sample(vx, vz, hx, hz, 1.0f / noh, 1.0f - k, k, gv, &sum_a, &sum_b);
  }
  out[0] = sum_a / (float)samples;
  out[1] = sum_b / (float)samples;
}

void oracle_brdf_lut_f32(int n, int samples, int orientation, float* out,
                         int nthreads) {
  int nt = set_threads(nthreads);
  (void)nt;
#pragma omp parallel for schedule(dynamic, 8) num_threads(nt)
  for (long p = 0; p < (long)n * n; ++p)
    lut_texel_f32((int)(p % n), (int)(p / n), n, samples, orientation,
                  out + 2 * (size_t)p);
}

static void lut_texel_f64(int i, int j, int n, int samples, int orientation,
                          double* out) {
  double nov = ((double)i + 0.5) / (double)n;
  double t0 = ((double)j + 0.5) / (double)n;
  double rough = orientation == ORACLE_LUT_ASSET ? 1.0 - t0 : t0;
  double vx = sqrt(1.0 - nov * nov), vz = nov;
  double alpha = rough * rough, a2 = alpha * alpha, k = alpha / 2.0;
  double sum_a = 0.0, sum_b = 0.0;
  for (int s = 0; s < samples; ++s) {
    double xi_x = (double)s / (double)samples;
    double xi_y = (double)bitrev32((uint32_t)s) / 4294967296.0;
    double phi = 2.0 * M_PI * xi_x;
    double cos_t = sqrt((1.0 - xi_y) / (1.0 + (a2 - 1.0) * xi_y));
    double sin_t = sqrt(1.0 - cos_t * cos_t);
    double hx = sin_t * cos(phi), hz = cos_t;
    double vdh = vx * hx + vz * hz;
    double lz = 2.0 * vdh * hz - vz;
    double nol = lz > 0.0 ? (lz < 1.0 ? lz : 1.0) : 0.0;
    double noh = hz > 0.0 ? (hz < 1.0 ? hz : 1.0) : 0.0;
    double voh = vdh > 0.0 ? (vdh < 1.0 ? vdh : 1.0) : 0.0;
    if (nol > 0.0) {
      double g = nol / (nol * (1.0 - k) + k) * (nov / (nov * (1.0 - k) + k));
      double g_vis = g * voh / (noh * nov);
      double fc = pow(1.0 - voh, 5.0);
      sum_a += (1.0 - fc) * g_vis;
      sum_b += fc * g_vis;
    }
  }
  out[0] = sum_a / samples;
  out[1] = sum_b / samples;
}

void oracle_brdf_lut_f64(int n, int samples, int orientation, double* out,
                         int nthreads) {
  int nt = set_threads(nthreads);
  (void)nt;
#pragma omp parallel for schedule(dynamic, 8) num_threads(nt)
  for (long p = 0; p < (long)n * n; ++p)
    lut_texel_f64((int)(p % n), (int)(p / n), n, samples, orientation,
                  out + 2 * (size_t)p);
}

/* ---------------------------------------------------------------------------
 * O2: FP64 quadrature over level-0 texels.  Each source texel (x, y) is a
 * constant patch at its centre direction (yaw = pi*(2(x+.5)/W - 1),
 * pitch = pi*((y+.5)/H - .5)) with solid angle
 * Omega = (2 pi / W) * (sin(pitch_top) - sin(pitch_bottom)).
 * Output directions are the reference's texel corners.  For the GGX weight,
 * with v = n and h = normalize(n + w): n.h = sqrt((1 + n.w)/2), so the weight
 * depends on c = n.w only: D(n.h) * max(0, c) * Omega, the expectation of
 * the estimator of PreFilterEnvMap.comp:147-169 without LOD blur.
 * ------------------------------------------------------------------------- */
typedef struct {
  double* sin_p;
  double* cos_p;
  double* omega;
  double* sin_y;
  double* cos_y;
} quad_tables;

static void quad_tables_make(int w, int h, quad_tables* t) {
  t->sin_p = (double*)malloc(sizeof(double) * h);
  t->cos_p = (double*)malloc(sizeof(double) * h);
  t->omega = (double*)malloc(sizeof(double) * h);
  t->sin_y = (double*)malloc(sizeof(double) * w);
  t->cos_y = (double*)malloc(sizeof(double) * w);
  for (int y = 0; y < h; ++y) {
    double p = M_PI * (((double)y + 0.5) / h - 0.5);
    double p0 = M_PI * ((double)y / h - 0.5), p1 = M_PI * ((double)(y + 1) / h - 0.5);
    t->sin_p[y] = sin(p);
    t->cos_p[y] = cos(p);
    t->omega[y] = (2.0 * M_PI / w) * (sin(p1) - sin(p0));
  }
  for (int x = 0; x < w; ++x) {
    double yaw = M_PI * (2.0 * ((double)x + 0.5) / w - 1.0);
    t->sin_y[x] = sin(yaw);
    t->cos_y[x] = cos(yaw);
  }
}

static void quad_tables_free(quad_tables* t) {
  free(t->sin_p);
  free(t->cos_p);
  free(t->omega);
  free(t->sin_y);
  free(t->cos_y);
}

static void out_dir_f64(int x, int y, int ow, int oh, double* n) {
  double yaw = M_PI * (2.0 * (double)x / ow - 1.0);
  double pitch = M_PI * ((double)y / oh - 0.5);
  n[0] = cos(pitch) * cos(yaw);
  n[1] = sin(pitch);
  n[2] = cos(pitch) * sin(yaw);
}

static void quad_texel(const float* level0, int w, int h, const quad_tables* tb,
                       const double* n, double a2, int ggx, double* out) {
  double s0 = 0, s1 = 0, s2 = 0, sw = 0;
  for (int y = 0; y < h; ++y) {
    double cp = tb->cos_p[y], sp = tb->sin_p[y], om = tb->omega[y];
    double ny = n[1] * sp;
    const float* row = level0 + 4 * (size_t)y * w;
    for (int x = 0; x < w; ++x) {
      double c = (n[0] * tb->cos_y[x] + n[2] * tb->sin_y[x]) * cp + ny;
      if (c <= 0.0) continue;
      double wgt;
      if (ggx) {
        double nh2 = 0.5 * (1.0 + c);
        double den = nh2 * (a2 - 1.0) + 1.0;
        wgt = a2 / (M_PI * den * den) * c * om;
      } else {
        wgt = c * om;
      }
      s0 += wgt * row[4 * x];
      s1 += wgt * row[4 * x + 1];
      s2 += wgt * row[4 * x + 2];
      sw += wgt;
    }
  }
  if (ggx) {
    out[0] = s0 / sw;
    out[1] = s1 / sw;
    out[2] = s2 / sw;
  } else {
    out[0] = s0 / M_PI;
    out[1] = s1 / M_PI;
    out[2] = s2 / M_PI;
  }
  out[3] = sw;
}

void oracle_quad_prefilter_texels(const float* level0, int w, int h, int ow,
                                  int oh, double roughness, const int* xy,
                                  int n, double* out, int nthreads) {
  quad_tables tb;
  quad_tables_make(w, h, &tb);
  double a2 = roughness * roughness * roughness * roughness;
  /* a = roughness, a2 = a*a in the shader (:139-140): D uses a2 = r^2 where
   * the GGX alpha is r.  Keep the shader's convention: */
  a2 = roughness * roughness;
  int nt = set_threads(nthreads);
  (void)nt;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
  for (int i = 0; i < n; ++i) {
    double nd[3];
    out_dir_f64(xy[2 * i], xy[2 * i + 1], ow, oh, nd);
    quad_texel(level0, w, h, &tb, nd, a2, 1, out + 4 * (size_t)i);
  }
  quad_tables_free(&tb);
}

void oracle_quad_irradiance_texels(const float* level0, int w, int h, int ow,
                                   int oh, const int* xy, int n, double* out,
                                   int nthreads) {
  quad_tables tb;
  quad_tables_make(w, h, &tb);
  int nt = set_threads(nthreads);
  (void)nt;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
  for (int i = 0; i < n; ++i) {
    double nd[3];
    out_dir_f64(xy[2 * i], xy[2 * i + 1], ow, oh, nd);
    quad_texel(level0, w, h, &tb, nd, 0.0, 0, out + 4 * (size_t)i);
  }
  quad_tables_free(&tb);
}

/* Evaluates one portable GLSL built-in over an array (tests of their
 * accuracy): fn 0 sin, 1 cos, 2 atan, 3 atan2(a, b), 4 log2. */
void oracle_builtin_eval(int fn, const float* a, const float* b, float* out, int n) {
  for (int i = 0; i < n; ++i) {
    switch (fn) {
      case 0: out[i] = agb_sin(a[i]); break;
      case 1: out[i] = agb_cos(a[i]); break;
      case 2: out[i] = agb_atan(a[i]); break;
      case 3: out[i] = agb_atan2(a[i], b[i]); break;
      default: out[i] = agb_log2(a[i]); break;
    }
  }
}
