// ibl_texel.cuh -- per-texel bodies of the plain path, shared by the
// single-probe kernels (ibl_plain.cu) and the batched ones (ibl_batch.cu).
// Compiled only in -fmad=false units: bit parity with the CPU oracle.
#pragma once

#include "althea_ibl.h"
#include "ibl_device.cuh"

namespace ibl {

// One texel of vkCmdBlitImage(VK_FILTER_LINEAR) from an sw x sh level to a
// dw x dh level (Src/Image.cpp:184-213): destination centre scaled by the
// extent ratio, bilinear with clamp to edge.
__device__ __forceinline__ float4 blit_texel(const float4* __restrict__ src, int sw, int sh, int dw,
                                             int dh, int x, int y) {
  float kx = (float)sw / (float)dw, ky = (float)sh / (float)dh;
  float u = ((float)x + 0.5f) * kx - 0.5f;
  float v = ((float)y + 0.5f) * ky - 0.5f;
  float fx = floorf(u), fy = floorf(v);
  float a = u - fx, b = v - fy;
  int i0 = min(max((int)fx, 0), sw - 1), i1 = min(max((int)fx + 1, 0), sw - 1);
  int j0 = min(max((int)fy, 0), sh - 1), j1 = min(max((int)fy + 1, 0), sh - 1);
  const float4* r0 = src + (long long)j0 * sw;
  const float4* r1 = src + (long long)j1 * sw;
  float4 t00 = __ldg(r0 + i0), t10 = __ldg(r0 + i1), t01 = __ldg(r1 + i0), t11 = __ldg(r1 + i1);
  float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b);
  float w01 = (1.0f - a) * b, w11 = a * b;
  float4 o;
  o.x = ((w00 * t00.x + w10 * t10.x) + w01 * t01.x) + w11 * t11.x;
  o.y = ((w00 * t00.y + w10 * t10.y) + w01 * t01.y) + w11 * t11.y;
  o.z = ((w00 * t00.z + w10 * t10.z) + w01 * t01.z) + w11 * t11.z;
  o.w = ((w00 * t00.w + w10 * t10.w) + w01 * t01.w) + w11 * t11.w;
  return o;
}

// Hammersley xi does not depend on the texel, so neither does sampleGGX's
// local half-vector: blocks of a roughness > 0 mip tabulate it once in shared
// memory when it fits (same operations, same values).
constexpr int kMaxTabulatedSamples = 2048;

// Block-cooperative: h_local[3*i..3*i+2] = sampleGGX(Hammersley(i), r^2).
__device__ __forceinline__ void tabulate_hammersley(float* h_local, int samples, float roughness) {
  const float a2 = roughness * roughness;
  for (int i = threadIdx.x; i < samples; i += blockDim.x) {
    float xi_x, xi_y;
    hammersley(i, samples, xi_x, xi_y);
    Float3 hl = sample_ggx(xi_x, xi_y, a2);
    h_local[3 * i] = hl.x;
    h_local[3 * i + 1] = hl.y;
    h_local[3 * i + 2] = hl.z;
  }
}

__device__ __forceinline__ void prefilter_texel_degenerate(const float4* __restrict__ chain,
                                                           const ChainTable& tab, Float3 n,
                                                           Float3 t, Float3 b, uint32_t sx,
                                                           uint32_t sy, int samples, int gen,
                                                           float* acc, float& total) {
  // roughness == 0: a2 = 0 makes sampleGGX return (cos(phi)*0, sin(phi)*0, 1),
  // so every sample with xi.y < 1 yields the same H = n, the same L and the
  // same texel value; xi.y == 1 gives 0/0 and the sample fails NdotL > 0
  // (PreFilterEnvMap.comp:163).  Evaluate the first kept sample once, then
  // repeat the serial float accumulation for every kept sample, which is what
  // the loop of :147-167 computes.
  float c0 = 0.0f, c1 = 0.0f, c2 = 0.0f, ndotl = 0.0f;
  bool have = false;
#pragma unroll 4
  for (int i = 0; i < samples; ++i) {
    // Only xi.y decides whether a sample survives; xi.x is drawn for the
    // first kept sample alone.
    float xi_y;
    if (gen == ALTHEA_IBL_GEN_HAMMERSLEY) {
      xi_y = __uint2float_rn(__brev((uint32_t)i)) * (1.0f / 4294967296.0f);
    } else {
      xi_y = hash_float(hash_bits(sx + 2u * (uint32_t)i + 2u, sy + 2u * (uint32_t)i + 2u));
    }
    if (xi_y == 1.0f) continue;  // NaN sample, dropped by NdotL > 0
    if (!have) {
      float xi_x = gen == ALTHEA_IBL_GEN_HAMMERSLEY
                       ? (float)i / (float)samples
                       : hash_float(hash_bits(sx + 2u * (uint32_t)i + 1u,
                                              sy + 2u * (uint32_t)i + 1u));
      Float3 hv = to_world(t, b, n, sample_ggx(xi_x, xi_y, 0.0f));
      float vdh = (n.x * hv.x + n.y * hv.y) + n.z * hv.z;
      float k = 2.0f * vdh;
      Float3 l = normalize3(f3(k * hv.x - n.x, k * hv.y - n.y, k * hv.z - n.z));
      ndotl = glsl_max((n.x * l.x + n.y * l.y) + n.z * l.z, 0.0f);
      if (ndotl > 0.0f) {
        Float3 c = sample_env(chain, tab, l, 0.0f);
        c0 = c.x * ndotl;
        c1 = c.y * ndotl;
        c2 = c.z * ndotl;
      }
      have = true;
    }
    if (ndotl > 0.0f) {
      acc[0] += c0;
      acc[1] += c1;
      acc[2] += c2;
      total += ndotl;
    }
  }
}

// main of PreFilterEnvMap.comp:126-177 for output texel (x, y) of an ow x oh
// mip of an env map of size w x h.  h_local: tabulated Hammersley
// half-vectors or nullptr.
__device__ __forceinline__ float4 prefilter_texel(const float4* __restrict__ chain,
                                                  const ChainTable& tab, int w, int h, int x,
                                                  int y, int ow, int oh, float roughness,
                                                  int samples, int generator,
                                                  const float* h_local) {
  Float3 n = texel_dir(x, y, ow, oh);
  Float3 t, b;
  local_frame(n, t, b);
  const float a2 = roughness * roughness;
  float acc[3] = {0.0f, 0.0f, 0.0f};
  float total = 0.0f;

  if (roughness == 0.0f) {
    prefilter_texel_degenerate(chain, tab, n, t, b, (uint32_t)x, (uint32_t)y, samples,
                               generator, acc, total);
  } else {
    const float sa_texel = 4.0f * kPi / (6.0f * (float)w * (float)h);
    const float rcp_sa_texel = 1.0f / sa_texel;
    const float fsamples = (float)samples;
    uint32_t sx = (uint32_t)x, sy = (uint32_t)y;
#pragma unroll 1
    for (int i = 0; i < samples; ++i) {
      Float3 hl;
      if (h_local) {
        hl = f3(h_local[3 * i], h_local[3 * i + 1], h_local[3 * i + 2]);
      } else {
        float xi_x, xi_y;
        if (generator == ALTHEA_IBL_GEN_HAMMERSLEY) {
          hammersley(i, samples, xi_x, xi_y);
        } else {
          sx += 1u;
          sy += 1u;
          xi_x = hash_float(hash_bits(sx, sy));
          sx += 1u;
          sy += 1u;
          xi_y = hash_float(hash_bits(sx, sy));
        }
        hl = sample_ggx(xi_x, xi_y, a2);
      }
      Float3 hv = to_world(t, b, n, hl);
      // V = R = N (:136-137): V.H, N.H and H.V are one and the same sum.
      float vdh = (n.x * hv.x + n.y * hv.y) + n.z * hv.z;
      float k = 2.0f * vdh;
      Float3 l = normalize3(f3(k * hv.x - n.x, k * hv.y - n.y, k * hv.z - n.z));
      float ndotl = glsl_max((n.x * l.x + n.y * l.y) + n.z * l.z, 0.0f);
      if (ndotl > 0.0f) {
        float ndoth = glsl_max(vdh, 0.0f);
        float d = distribution_ggx(ndoth, a2);
        float pdf = d * ndoth / (4.0f * ndoth + 0.00001f);
        float sa_sample = 1.0f / (fsamples * pdf + 0.0001f);
        float mip = 0.5f * agb_log2(agb_div_rcp(sa_sample, sa_texel, rcp_sa_texel));
        Float3 c = sample_env(chain, tab, l, mip);
        acc[0] += c.x * ndotl;
        acc[1] += c.y * ndotl;
        acc[2] += c.z * ndotl;
        total += ndotl;
      }
    }
  }
  float4 o;
  o.x = acc[0] / total;
  o.y = acc[1] / total;
  o.z = acc[2] / total;
  o.w = 1.0f;
  return o;
}

// ---------------------------------------------------------------------------
// Irradiance (GenIrradianceMap.comp:106-155) building blocks.
// ---------------------------------------------------------------------------
constexpr int kIrrWarps = 8;
constexpr int kPatchT = 4, kPatchP = 8;
constexpr int kThetaSamples = 300;  // GenIrradianceMap.comp:119
constexpr int kMaxPhiSamples = 4096;

__host__ __device__ inline int irr_phi_samples(int w, int h) {
  // int(pushConstants.height * thetaSamples / pushConstants.width) (:120-121)
  return (int)((float)h * (float)kThetaSamples / (float)w);
}

// Block-cooperative sin/cos tables of the theta (:127) and phi (:132) steps.
__device__ __forceinline__ void irradiance_tables(float* cos_t, float* sin_t, float* cos_p,
                                                  float* sin_p, int phi_samples) {
  for (int i = threadIdx.x; i < kThetaSamples; i += blockDim.x) {
    // theta = i * 2 * PI / thetaSamples: int i*2, then float.
    float theta = (float)(i * 2) * kPi / (float)kThetaSamples;
    agb_sincos(theta, &sin_t[i], &cos_t[i]);
  }
  for (int j = threadIdx.x; j < phi_samples; j += blockDim.x) {
    float phi = (float)j * 0.5f * kPi / (float)phi_samples;
    agb_sincos(phi, &sin_p[j], &cos_p[j]);
  }
}

// The grid of one texel is cut into kBands fixed bands of theta rows.  Each
// band is summed by one warp (lanes on a 4 (theta) x 8 (phi) patch, then a
// fixed xor-shuffle tree), and the kBands band sums are combined by one fixed
// binary tree.  Blocks may own 32, 16 or 8 consecutive bands (1, 2 or 4 blocks
// per texel): they reduce their aligned subtree and the finish step applies
// the remaining top levels, so the result does not depend on the split.
constexpr int kBands = 32;

// Bands hold whole groups of kPatchT rows (75 groups over 32 bands: 2 or 3
// groups each) so no theta lane of the patch idles.
__host__ __device__ inline void band_rows(int band, int& row0, int& row1) {
  constexpr int groups = kThetaSamples / kPatchT;
  row0 = kPatchT * (band * groups / kBands);
  row1 = kPatchT * ((band + 1) * groups / kBands);
}

// In-place pairwise tree over n (a power of two) values; returns v[0].
__device__ __forceinline__ Float3 tree_sum3(float (*v)[3], int n) {
  for (int s = 1; s < n; s <<= 1)
    for (int i = 0; i + s < n; i += 2 * s) {
      v[i][0] += v[i + s][0];
      v[i][1] += v[i + s][1];
      v[i][2] += v[i + s][2];
    }
  return f3(v[0][0], v[0][1], v[0][2]);
}

// One warp's sum over theta rows [row0, row1) of one texel.
__device__ __forceinline__ Float3 irradiance_warp_sum(const float4* __restrict__ chain,
                                                      const ChainTable& tab, int w, Float3 n,
                                                      Float3 t, Float3 b, int row0, int row1,
                                                      int phi_samples, const float* cos_t,
                                                      const float* sin_t, const float* cos_p,
                                                      const float* sin_p) {
  const int lane = threadIdx.x & 31;
  const float mip = agb_log2((float)w / (float)kThetaSamples);  // :124
  const int lt = lane / kPatchP, lp = lane % kPatchP;
  float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
#pragma unroll 1
  for (int i = row0 + lt; i < row1; i += kPatchT) {
    const float ct = cos_t[i], st = sin_t[i];
#pragma unroll 1
    for (int j = lp; j < phi_samples; j += kPatchP) {
      const float cp = cos_p[j], sp = sin_p[j];
      Float3 d = to_world(t, b, n, f3(ct * sp, st * sp, cp));
      Float3 c = sample_env(chain, tab, d, mip);
      a0 += c.x * cp * sp;
      a1 += c.y * cp * sp;
      a2 += c.z * cp * sp;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a0 += __shfl_xor_sync(0xffffffffu, a0, o);
    a1 += __shfl_xor_sync(0xffffffffu, a1, o);
    a2 += __shfl_xor_sync(0xffffffffu, a2, o);
  }
  return f3(a0, a1, a2);
}

// Block part of one texel: bands [first, first + count) (count = 32/gb), each
// warp taking bands warp, warp+8, ...; returns (in thread 0) the aligned
// subtree sum.  band_smem: kBands x 3 floats of shared memory.
__device__ __forceinline__ Float3 irradiance_block_bands(
    const float4* __restrict__ chain, const ChainTable& tab, int w, int x, int y, int ow, int oh,
    int first, int count, int phi_samples, const float* cos_t, const float* sin_t,
    const float* cos_p, const float* sin_p, float (*band_smem)[3]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  Float3 n = texel_dir(x, y, ow, oh);
  Float3 t, b;
  local_frame(n, t, b);
  for (int k = warp; k < count; k += kIrrWarps) {
    int row0, row1;
    band_rows(first + k, row0, row1);
    Float3 s = irradiance_warp_sum(chain, tab, w, n, t, b, row0, row1, phi_samples, cos_t,
                                   sin_t, cos_p, sin_p);
    if (lane == 0) {
      band_smem[k][0] = s.x;
      band_smem[k][1] = s.y;
      band_smem[k][2] = s.z;
    }
  }
  __syncthreads();
  Float3 r = f3(0.0f, 0.0f, 0.0f);
  if (threadIdx.x == 0) r = tree_sum3(band_smem, count);
  return r;
}

// Top levels of the band tree over the gb (1, 2 or 4) block partials of one
// texel, stored consecutively.
__device__ __forceinline__ Float3 combine_partials(const float4* __restrict__ p, int gb) {
  float4 a = p[0];
  if (gb == 1) return f3(a.x, a.y, a.z);
  float4 b = p[1];
  Float3 l = f3(a.x + b.x, a.y + b.y, a.z + b.z);
  if (gb == 2) return l;
  float4 c = p[2], d = p[3];
  Float3 r = f3(c.x + d.x, c.y + d.y, c.z + d.z);
  return f3(l.x + r.x, l.y + r.y, l.z + r.z);
}

// Blocks per texel for a split target: 1, 2 or 4 (a power of two dividing the
// kBands bands into aligned groups of at least one band per warp).
__host__ __device__ inline int irradiance_split(long long texels, long long target_blocks) {
  long long want = (target_blocks + texels - 1) / texels;
  return want >= 4 ? 4 : (want >= 2 ? 2 : 1);
}

// vec4(PI * irradiance / float(thetaSamples) / float(phiSamples), 1.0) (:145)
__device__ __forceinline__ float4 irradiance_finish(float s0, float s1, float s2, int phi_samples) {
  float4 o;
  o.x = kPi * s0 / (float)kThetaSamples / (float)phi_samples;
  o.y = kPi * s1 / (float)kThetaSamples / (float)phi_samples;
  o.z = kPi * s2 / (float)kThetaSamples / (float)phi_samples;
  o.w = 1.0f;
  return o;
}

}  // namespace ibl
