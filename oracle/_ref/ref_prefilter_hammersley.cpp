// GENERATED by oracle/make_ref.py from PreFilterEnvMap.comp -- do not edit.
#include <omp.h>
#include "../glsl_compat.hpp"
namespace ref_prefilter_hammersley {
GLSLC_USING
static int glslc_max_samples = 0;
#define ALTHEA_XI() glslc::hammersley_next()
#define PI 3.14159265359f
#define MAX_SAMPLES (glslc_max_samples)
sampler2D environmentMap;
image2D prefilteredMip;
struct PushConstants {
  float envMapWidth;
  float envMapHeight;
  float width;
  float height;
  float roughness;
} pushConstants;
void coordinateSystem(vec3 v1, vec3& v2, vec3& v3) {
    if (abs(v1.x) > abs(v1.y))
            v2 = vec3(-v1.z, 0, v1.x) / sqrt(v1.x * v1.x + v1.z * v1.z);
        else
            v2 = vec3(0, v1.z, -v1.y) / sqrt(v1.y * v1.y + v1.z * v1.z);
        v3 = cross(v1, v2);
}
mat3 LocalToWorld(vec3 nor) {
    vec3 tan, bit;
    coordinateSystem(nor, tan, bit);
    return mat3(tan, bit, nor);
}
thread_local uvec2 seed;
float rng() {
    seed += uvec2(1);
    uvec2 q = 1103515245U * ( (seed >> 1U) ^ (seed.yx()) );
    uint  n = 1103515245U * ( (q.x) ^ (q.y >> 3U) );
    return float(n) * (1.0f / float(0xffffffffU));
}
vec3 squareToDiskConcentric(vec2 xi) {
  vec2 remappedRange = 2.0f * xi - 1.0f;
  if (remappedRange.x == 0.0f && remappedRange.y == 0.0f) {
    return vec3(0.0f);
  }
  float theta;
  float r;
  if (abs(remappedRange.x) > abs(remappedRange.y)) {
    r = remappedRange.x;
    theta = 0.25f * PI * remappedRange.y / remappedRange.x;
  } else {
    r = remappedRange.y;
    theta = 0.5f * PI - 0.25f * PI * remappedRange.x / remappedRange.y;
  }
  return r * vec3(cos(theta), sin(theta), 0.0f);
}
vec3 squareToHemisphereCosine(vec2 xi) {
    vec3 diskSample = squareToDiskConcentric(xi);
    return vec3(
        diskSample.x,
        diskSample.y,
        sqrt(clamp(1.0f - length(diskSample), 0.0f, 1.0f)));
}
vec3 sampleHemisphereCosine() {
  return squareToHemisphereCosine(ALTHEA_XI());
}
float distributionGGX(float NdotH, float a2)
{
    float denom  = (NdotH * NdotH * (a2 - 1.0f) + 1.0f);
    return a2 / (PI * denom * denom);
}
vec3 sampleGGX(float a2) {
  vec2 xi = ALTHEA_XI();
  float phi = 2.0f * PI * xi.x;
  float cosTheta = sqrt((1.0f - xi.y) / (1.0f + (a2 - 1.0f) * xi.y));
  float sinTheta = sqrt(1.0f - cosTheta * cosTheta);
  return vec3(cos(phi) * sinTheta, sin(phi) * sinTheta, cosTheta);
}
vec3 sampleEnvMap(vec3 dir, float mip) {
  float pitch = 0.0f;
  float yaw = 0.0f;
  float lenXz = length(dir.xz());
  if (lenXz > 0.001f) {
    yaw = atan(dir.z, dir.x);
    pitch = atan(dir.y / lenXz);
  } else if (dir.y > 0.0f) {
    pitch = 0.5f * PI;
  } else {
    pitch = -0.5f * PI;
  }
  vec2 uv = vec2(
      yaw / (2.0f * PI) + 0.5f,
      pitch / PI + 0.5f);
  vec3 color = textureLod(environmentMap, uv, mip).rgb();
  return color;
}
void shader_main() {
  seed = uvec2(gl_GlobalInvocationID.xy());
  ivec2 texelPos = ivec2(gl_GlobalInvocationID.xy());
  vec2 texelUv = vec2(texelPos) / vec2(pushConstants.width, pushConstants.height);
  float yaw = PI * (2.0f * texelUv.x - 1.0f);
  float pitch = PI * (texelUv.y - 0.5f);
  vec3 N = vec3(cos(pitch) * cos(yaw), sin(pitch), cos(pitch) * sin(yaw));
  vec3 R = N;
  vec3 V = R;
  float a = pushConstants.roughness;
  float a2 = a * a;
  mat3 localToWorld = LocalToWorld(N);
  vec3 prefilteredColor = vec3(0.0f);
  float totalWeight = 0.0f;
  int sampleCount = 0;
  for (int i = 0; i < MAX_SAMPLES; ++i) {
    vec3 H = localToWorld * sampleGGX(a2);
    vec3 L = normalize(2.0f * dot(V, H) * H - V);
    float NdotL = max(dot(N, L), 0.0f);
    float NdotH = max(dot(N, H), 0.0f);
    float HDotV = max(dot(H, V), 0.0f);
    float D = distributionGGX(NdotH, a2);
    float pdf = D * NdotH / (4.0f * HDotV + 0.00001f);
    float saTexel = 4.0f * PI / (6.0f * pushConstants.envMapWidth * pushConstants.envMapHeight);
    float saSample = 1.0f / (float(MAX_SAMPLES) * pdf + 0.0001f);
    float mipLevel =
        pushConstants.roughness == 0.0f ? 0.0f : 0.5f * log2(saSample / saTexel);
    if (NdotL > 0.0f) {
      prefilteredColor += sampleEnvMap(L, mipLevel) * NdotL;
      totalWeight += NdotL;
    }
  }
  vec4 color = vec4(prefilteredColor / totalWeight, 1.0f);
  imageStore(prefilteredMip, texelPos, color);
}

// ---- driver (generated) ----------------------------------------------------
extern "C" void ref_prefilter_hammersley(const float* chain, int w, int h, int levels, float* out,
                     int ow, int oh, float roughness, int samples, const int* xy, int n,
                     int nthreads) {
  glslc::g_res.chain = chain;
  glslc::g_res.w = w;
  glslc::g_res.h = h;
  glslc::g_res.levels = levels;
  glslc::g_res.out = out;
  glslc::g_res.ow = ow;
  glslc::g_res.oh = oh;
  pushConstants.envMapWidth = (float)w;
  pushConstants.envMapHeight = (float)h;
  pushConstants.width = (float)ow;
  pushConstants.height = (float)oh;
  pushConstants.roughness = roughness;
  glslc_max_samples = samples;
  glslc::g_sample_count = samples;
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(nt)
  for (int i = 0; i < n; ++i) {
    glslc::gl_GlobalInvocationID.x = (uint32_t)xy[2 * i];
    glslc::gl_GlobalInvocationID.y = (uint32_t)xy[2 * i + 1];
    glslc::gl_GlobalInvocationID.z = 0;
    glslc::g_sample_index = 0;
    shader_main();
  }
}
}
#undef ALTHEA_XI
#undef PI
#undef MAX_SAMPLES
