// GENERATED by oracle/make_ref.py from GenIrradianceMap.comp -- do not edit.
#include <omp.h>
#include "../glsl_compat.hpp"
namespace ref_irradiance {
GLSLC_USING
static int glslc_max_samples = 0;
#define ALTHEA_XI() vec2{rng(), rng()}
#define PI 3.14159265359f
sampler2D environmentMap;
image2D irradianceMap;
struct PushConstants {
  float width;
  float height;
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
  vec3 nor = vec3(cos(pitch) * cos(yaw), sin(pitch), cos(pitch) * sin(yaw));
  mat3 localToWorld = LocalToWorld(nor);
  vec3 irradiance = vec3(0.0f);
  int thetaSamples = 300;
  int phiSamples =
      int(pushConstants.height * thetaSamples / pushConstants.width);
  float mip = log2(pushConstants.width / float(thetaSamples));
  for (int i = 0; i < thetaSamples; ++i) {
    float theta = i * 2 * PI / thetaSamples;
    float cosTheta = cos(theta);
    float sinTheta = sin(theta);
    for (int j = 0; j < phiSamples; ++j) {
      float phi = j * 0.5f * PI / phiSamples;
      float cosPhi = cos(phi);
      float sinPhi = sin(phi);
      vec3 sampleDir =
          localToWorld * vec3(cosTheta * sinPhi, sinTheta * sinPhi, cosPhi);
      irradiance += sampleEnvMap(sampleDir, mip) * cosPhi * sinPhi;
    }
  }
  vec4 color = vec4(PI * irradiance / float(thetaSamples) / float(phiSamples), 1.0f);
  imageStore(irradianceMap, texelPos, color);
}

// ---- driver (generated) ----------------------------------------------------
extern "C" void ref_irradiance_raw(const float* chain, int w, int h, int levels, float* out,
                     int ow, int oh,  const int* xy, int n,
                     int nthreads) {
  glslc::g_res.chain = chain;
  glslc::g_res.w = w;
  glslc::g_res.h = h;
  glslc::g_res.levels = levels;
  glslc::g_res.out = out;
  glslc::g_res.ow = ow;
  glslc::g_res.oh = oh;
  pushConstants.width = (float)w;
  pushConstants.height = (float)h;
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
