// ibl_suns.cu -- analytic sun lobes added to an equirect sky map on the device.
//
// A probe re-bake is usually caused by a change of the lights, not of the
// whole sky: the sun moves with the time of day.  The server keeps the sky map
// resident and each request names the suns to add before the bake, so a
// request moves no env map across the host link.  The lobe is the one the
// synthetic benchmark maps use: on R, G and B,
//   out = base + sum_s L_s exp(-theta_s^2 / (2 sigma_s^2)),
// theta_s = the angle between the texel centre's direction and sun s, with
// texel (x, y) of a W x H map at yaw = pi (2 (x + 0.5) / W - 1),
// pitch = pi ((y + 0.5) / H - 0.5), direction (cos p cos yaw, sin p,
// cos p sin yaw) -- the mapping of sampleEnvMap, PreFilterEnvMap.comp:98-122.
// theta = 2 asin(|d - s| / 2) keeps full FP32 accuracy near the sun's centre
// (acos of a dot product would lose it).  Alpha is copied.  The kernel is
// elementwise, so out may be base itself.
#include <cuda_runtime.h>

#include <cstring>

#include "althea_ibl.h"
#include "ibl_internal.h"

namespace ibl {
namespace {

struct SunArgs {
  float dx[ALTHEA_IBL_MAX_SUNS], dy[ALTHEA_IBL_MAX_SUNS], dz[ALTHEA_IBL_MAX_SUNS];
  float inv2s2[ALTHEA_IBL_MAX_SUNS];  // 1 / (2 sigma^2)
  float lum[ALTHEA_IBL_MAX_SUNS];
  int n;
};

__global__ void __launch_bounds__(256) apply_suns_kernel(const float4* __restrict__ base,
                                                         float4* __restrict__ out, int w, int h,
                                                         const SunArgs a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= w) return;
  const float kPi = 3.14159265358979f;
  float sp, cp, sy, cy;
  sincosf(kPi * (((float)y + 0.5f) / (float)h - 0.5f), &sp, &cp);
  sincosf(kPi * (2.0f * ((float)x + 0.5f) / (float)w - 1.0f), &sy, &cy);
  const float vx = cp * cy, vy = sp, vz = cp * sy;
  float add = 0.0f;
  for (int k = 0; k < a.n; ++k) {
    const float ex = vx - a.dx[k], ey = vy - a.dy[k], ez = vz - a.dz[k];
    const float chord = sqrtf(ex * ex + ey * ey + ez * ez);
    const float theta = 2.0f * asinf(fminf(0.5f * chord, 1.0f));
    add += a.lum[k] * expf(-theta * theta * a.inv2s2[k]);
  }
  const size_t i = (size_t)y * w + x;
  float4 v = base[i];
  v.x += add;
  v.y += add;
  v.z += add;
  out[i] = v;
}

}  // namespace

int launch_apply_suns(const float* base, float* out, int w, int h, const althea_ibl_sun* suns,
                      int n, cudaStream_t st) {
  int r = check_env(w, h);
  if (r) return r;
  if (!base || !out || ((uintptr_t)base) % 16 || ((uintptr_t)out) % 16)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "suns: base/out null or not 16-byte aligned");
  if (n < 0 || n > ALTHEA_IBL_MAX_SUNS || (n > 0 && !suns))
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "sun_count %d outside 0..%d", n,
                     ALTHEA_IBL_MAX_SUNS);
  SunArgs a;
  memset(&a, 0, sizeof(a));
  a.n = n;
  for (int k = 0; k < n; ++k) {
    const althea_ibl_sun& s = suns[k];
    const double len = sqrt((double)s.dir[0] * s.dir[0] + (double)s.dir[1] * s.dir[1] +
                            (double)s.dir[2] * s.dir[2]);
    if (!(len > 0.5 && len < 2.0) || !(s.sigma > 0.0f) || !(s.sigma < 4.0f) ||
        !(s.radiance >= 0.0f) || !(s.radiance < 3.0e38f))
      return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT,
                       "sun %d: direction not near unit length, sigma outside (0, 4) rad or "
                       "radiance outside [0, 3e38)",
                       k);
    a.dx[k] = (float)(s.dir[0] / len);
    a.dy[k] = (float)(s.dir[1] / len);
    a.dz[k] = (float)(s.dir[2] / len);
    a.inv2s2[k] = (float)(1.0 / (2.0 * (double)s.sigma * s.sigma));
    a.lum[k] = s.radiance;
  }
  const dim3 grid((unsigned)((w + 255) / 256), (unsigned)h);
  apply_suns_kernel<<<grid, 256, 0, st>>>(reinterpret_cast<const float4*>(base),
                                          reinterpret_cast<float4*>(out), w, h, a);
  return cuda_status(cudaGetLastError(), "apply suns launch");
}

}  // namespace ibl

extern "C" int althea_ibl_apply_suns(const float* base_dev, float* out_dev, int w, int h,
                                     const althea_ibl_sun* suns, int n, void* stream) {
  return ibl::launch_apply_suns(base_dev, out_dev, w, h, suns, n, (cudaStream_t)stream);
}
