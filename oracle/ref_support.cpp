// ref_support.cpp -- globals and the blit-equivalent mip chain for the
// reference-shader CPU library built by oracle/make_ref.py.
// TEST INFRASTRUCTURE ONLY.
#include <cmath>
#include <cstring>

#include "glsl_compat.hpp"

namespace glslc {
Resources g_res;
thread_local uvec3 gl_GlobalInvocationID;
thread_local int g_sample_index = 0;
int g_sample_count = 1;
HalfView g_heap_tex[4], g_heap_img[4];
}  // namespace glslc

namespace {
int dim_at(int d, int l) {
  int v = d >> l;
  return v < 1 ? 1 : v;
}
int clamp_edge(int i, int n) { return i < 0 ? 0 : (i >= n ? n - 1 : i); }
}  // namespace

extern "C" int ref_level_count(int w, int h) {
  return 1 + (int)std::floor(std::log2((double)(w > h ? w : h)));
}

// Src/Image.cpp:135-239: level l = vkCmdBlitImage(level l-1, LINEAR) with the
// Vulkan blit mapping (dst centre scaled by src/dst extent, clamp to edge).
extern "C" void ref_build_chain(const float* level0, int w, int h, float* chain) {
  int levels = ref_level_count(w, h);
  std::memcpy(chain, level0, sizeof(float) * 4 * (size_t)w * h);
  size_t src_off = 0, dst_off = (size_t)w * h;
  for (int l = 1; l < levels; ++l) {
    int sw = dim_at(w, l - 1), sh = dim_at(h, l - 1), dw = dim_at(w, l), dh = dim_at(h, l);
    const float* s = chain + 4 * src_off;
    float* d = chain + 4 * dst_off;
    float kx = (float)sw / (float)dw, ky = (float)sh / (float)dh;
    for (int y = 0; y < dh; ++y) {
      float v = ((float)y + 0.5f) * ky - 0.5f, fy = std::floor(v), b = v - fy;
      int j0 = clamp_edge((int)fy, sh), j1 = clamp_edge((int)fy + 1, sh);
      for (int x = 0; x < dw; ++x) {
        float u = ((float)x + 0.5f) * kx - 0.5f, fx = std::floor(u), a = u - fx;
        int i0 = clamp_edge((int)fx, sw), i1 = clamp_edge((int)fx + 1, sw);
        glslc::vec4 r = glslc::bilinear(glslc::fetch(s, sw, i0, j0), glslc::fetch(s, sw, i1, j0),
                                        glslc::fetch(s, sw, i0, j1), glslc::fetch(s, sw, i1, j1),
                                        a, b);
        float* o = d + 4 * ((size_t)y * dw + x);
        o[0] = r.x;
        o[1] = r.y;
        o[2] = r.z;
        o[3] = r.w;
      }
    }
    src_off = dst_off;
    dst_off += (size_t)dw * dh;
  }
}
