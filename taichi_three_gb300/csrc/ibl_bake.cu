// ibl_bake.cu -- the bake of SkyboxLighting's prefiltered maps.
//
// CookTorrance.cook_for_ibl (tina/matr/material.py:279-316) and
// Lambert.cook_for_ibl (:407-438): every texel of the output map averages
// the environment about its own direction (Skybox.unmapcoor,
// tina/skybox.py:131-135) over `nsamples` directions
// tangentspace(dir) @ spherical(h, xi2) weighted by h, where
// h = sqrt((1 - xi1) / (1 - xi1 (1 - roughness^2))) for a CookTorrance level
// and h = xi1 for the Lambert map.  One warp per texel: the lanes split the
// samples and the sums are reduced across the warp.  The uniforms come from
// the counter-based stream of t3_ibl.cuh (seed, texel, sample), not from
// Taichi's generator, so the maps equal the reference's only in expectation.
#include "t3_shading.cuh"

namespace t3 {

// Skybox.unmapcoor: coor = (i, j) / (shape - 1) = (v, u); spherical(2u - 1, v)
// with y and z exchanged (tina/skybox.py:31-36)
__device__ __forceinline__ V3 texel_dir(int i, int j, int w, int h) {
  const float v = (float)i / (float)(w - 1), u = (float)j / (float)(h - 1);
  const float hh = u * 2.0f - 1.0f;
  const float r = sqrtf(fmaxf(0.0f, 1.0f - hh * hh));
  float s, c;
  sincospif(2.0f * v, &s, &c);
  return v3(r * c, hh, -(r * s));
}

__global__ void __launch_bounds__(256)
k_ibl_bake(Env env, float roughness, int nsamples, uint32_t seed, float* __restrict__ out, int w, int h) {
  const int lane = threadIdx.x & 31;
  const int64_t texel = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (texel >= (int64_t)w * h) return;  // whole warps leave together
  const int i = (int)(texel / h), j = (int)(texel - (int64_t)i * h);
  const V3 dir = texel_dir(i, j, w, h);
  const float a2 = fmaxf(0.0f, roughness * roughness);
  const uint32_t base = rng_base(seed, (uint32_t)texel);
  V3 res = v3(0.f, 0.f, 0.f);
  float dem = 0.0f;
  for (int s = lane; s < nsamples; s += 32) {
    const float x1 = rng_draw(base, (uint32_t)s, 0), x2 = rng_draw(base, (uint32_t)s, 1);
    const float hh = roughness >= 0.0f ? sqrtf((1.0f - x1) / (1.0f - x1 * (1.0f - a2))) : x1;
    const V3 odir = tangent_dir(dir, hh, x2);
    res = res + hh * env_sample(env, odir);
    dem += hh;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    res.x += __shfl_xor_sync(0xFFFFFFFFu, res.x, o);
    res.y += __shfl_xor_sync(0xFFFFFFFFu, res.y, o);
    res.z += __shfl_xor_sync(0xFFFFFFFFu, res.z, o);
    dem += __shfl_xor_sync(0xFFFFFFFFu, dem, o);
  }
  if (lane == 0) {
    float* p = out + texel * 3;
    p[0] = res.x / dem;
    p[1] = res.y / dem;
    p[2] = res.z / dem;
  }
}

} // namespace t3

using namespace t3;

extern "C" int t3_ibl_bake(const void* env, int env_w, int env_h, int env_half, float roughness, int nsamples,
                           uint32_t seed, float* out, int out_w, int out_h, void* stream) {
  if (!env || !out || env_w < 2 || env_h < 2 || out_w < 2 || out_h < 2 || nsamples < 1) return T3_EINVAL;
  if (!(roughness <= 1.0f)) return T3_EINVAL;  // above 1, or NaN
  const int64_t threads = (int64_t)out_w * out_h * 32;
  const int64_t grid = (threads + 255) / 256;
  if (grid > 0x7FFFFFFF) return T3_ETOOBIG;
  const Env e{env, env_w, env_h, env_half};
  k_ibl_bake<<<(unsigned)grid, 256, 0, (cudaStream_t)stream>>>(e, roughness, nsamples, seed, out, out_w, out_h);
  return cudaGetLastError() == cudaSuccess ? T3_OK : T3_ECUDA;
}
