// t3_ibl.cuh -- image-based lighting: environment lookup and the Monte Carlo
// IBL estimator built from the materials' own importance samplers.
//
// Environment (tina/skybox.py:23-28, 138-145; tina/common.py:140-149):
//   spheremap(dir): (x, y, z) -> (x, -z, y); u = y; p = atan2(-z, x) / tau mod 1;
//   coor = (p, u * 0.5 + 0.5); I = (shape - 1) * coor; bilerp(img, I).
//   The reference's bilerp reads I + 1 unclamped; here the +1 texel is clamped
//   to the map (it only matters on the last row / column).
//
// Estimator ("the method's own MC IBL"): the samplers of material.py --
// Lambert.sample :399-405 (cosine, weight 1), CookTorrance.sample :365-384
// (u = sqrt((1-xi)/(1-xi(1-a2))) about reflect(-V, n), weight F*G, zero and
// mirrored below the surface), Phong.sample :460-472, MixMaterial.sample
// :124-138 (lobe 2 with probability smoothlerp(avg(f), .12, .88), weight
// f / p) and ScaleMaterial.sample :180-184 -- with the radiance estimate of
// path/engine.py:243-266 for a ray that leaves to the sky: weight * env(dir).
// A pixel's colour is emission + (1/spp) * sum of those terms.  The flattened
// lobes carry the product of their Mix probabilities, so a lobe is drawn with
// one uniform against the cumulative probabilities (the same distribution
// as Tina's per-Mix draws).
//
// Random numbers: a counter-based hash (pcg_hash of Jarzynski & Olano,
// "Hash Functions for GPU Rendering", JCGT 2020) of (seed, pixel, sample,
// draw), so the oracle draws the identical stream.
#pragma once

#include <cuda_fp16.h>

// included by t3_shading.cuh after V3 / Frag / eval_value

namespace t3 {

__host__ __device__ __forceinline__ uint32_t pcg_hash(uint32_t v) {
  const uint32_t state = v * 747796405u + 2891336453u;
  const uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
  return (word >> 22u) ^ word;
}

// per-pixel stream base, then one hash per draw; uniform in [0, 1) with 24 bits
__host__ __device__ __forceinline__ uint32_t rng_base(uint32_t seed, uint32_t pixel) {
  return pcg_hash(seed ^ pcg_hash(pixel));
}
__host__ __device__ __forceinline__ float rng_draw(uint32_t base, uint32_t sample, uint32_t draw) {
  return (float)(pcg_hash(base ^ ((sample * 3u + draw) * 0x9E3779B9u)) >> 8) * 5.9604644775390625e-08f;
}

struct Env {
  const void* p;
  int w, h, half;
};

__device__ __forceinline__ V3 env_texel(const Env& e, int i, int j) {
  i = min(max(i, 0), e.w - 1);
  j = min(max(j, 0), e.h - 1);
  const int64_t o = ((int64_t)i * e.h + j) * 3;
  if (e.half) {
    const __half* t = reinterpret_cast<const __half*>(e.p) + o;
    return v3(__half2float(t[0]), __half2float(t[1]), __half2float(t[2]));
  }
  const float* t = reinterpret_cast<const float*>(e.p) + o;
  return v3(__ldg(t), __ldg(t + 1), __ldg(t + 2));
}

// Skybox.sample(dir)
__device__ __forceinline__ V3 env_sample(const Env& e, V3 dir) {
  const float u = dir.y;
  float p = atan2f(-dir.z, dir.x) * 0.15915494309189535f;  // / tau
  p = p - floorf(p);
  const float cx = p * (float)(e.w - 1), cy = (u * 0.5f + 0.5f) * (float)(e.h - 1);
  const float fx = floorf(cx), fy = floorf(cy);
  const int ix = (int)fx, iy = (int)fy;
  const float x1 = cx - fx, y1 = cy - fy, x0 = 1.0f - x1, y0 = 1.0f - y1;
  const V3 a = env_texel(e, ix + 1, iy + 1), b = env_texel(e, ix + 1, iy);
  const V3 c = env_texel(e, ix, iy), d = env_texel(e, ix, iy + 1);
  return ((x1 * y1) * a + (x1 * y0) * b) + ((x0 * y0) * c + (x0 * y1) * d);
}

// tangentspace(nrm) @ spherical(h, p)   (tina/advans.py:97-108)
__device__ __forceinline__ V3 tangent_dir(V3 n, float h, float p) {
  const V3 up = v3(233.0f, 666.0f, 512.0f);
  const V3 bitan = normalized(cross(n, up));
  const V3 tan = cross(bitan, n);
  float s, c;
  sincospif(2.0f * p, &s, &c);
  const float r = sqrtf(fmaxf(0.0f, 1.0f - h * h));
  return (r * c) * tan + (r * s) * bitan + h * n;
}

__device__ __forceinline__ V3 reflect3(V3 I, V3 n) { return I - (2.0f * dot(n, I)) * n; }

// smoothlerp(fac, .12, .88) (tina/common.py:215-231)
__device__ __forceinline__ float mix_prob(float fac) {
  if (fac != 0.0f && fac != 1.0f) {
    const float t = fminf(1.0f, fmaxf(0.0f, fac));
    const float s = t * t * (3.0f - 2.0f * t);
    return 0.12f * (1.0f - s) + 0.88f * s;
  }
  return fac;
}

// Per-lobe sampler state for the Monte Carlo estimator.
template <int NL>
struct IblLobes {
  int kind[NL];
  V3 w[NL];     // lobe weight / selection probability
  V3 f0[NL];    // COOK
  float r2[NL]; // COOK: roughness**2; PHONG: shineness
  float cdf[NL];
  int n;
};

template <int NL, bool TEX = true>
__device__ __forceinline__ void eval_ibl_lobes(const DevMaterial& mat, const Frag& fg,
                                               IblLobes<NL>& L, V3& emission) {
  L.n = mat.nlobes;
  emission = v3(0.f, 0.f, 0.f);
  float c = 0.0f;
#pragma unroll
  for (int k = 0; k < NL; k++) {
    L.kind[k] = -1;
    L.cdf[k] = c;
    if (k >= L.n) continue;
    const DevLobe& lb = mat.lobes[k];
    V3 w = v3(1.f, 1.f, 1.f);
    float prob = 1.0f;
    for (int j = 0; j < lb.nfac; j++) {
      const int fj = lb.fac[j];
      const V3 f = eval_value<TEX>(mat, fj & 0xFFFF, fg);
      const bool om = (fj & T3_FAC_ONE_MINUS) != 0;
      w = w * (om ? one_minus(f) : f);
      if (fj & T3_FAC_MIX) {
        const float q = mix_prob((f.x + f.y + f.z) * (1.0f / 3.0f));
        prob *= om ? 1.0f - q : q;
      }
    }
    if (lb.kind == T3_OP_EMISSION) {
      emission = emission + w;
      prob = 0.0f;  // Emission.sample returns weight 0
    }
    L.kind[k] = lb.kind;
    L.w[k] = prob > 0.0f ? (1.0f / prob) * w : v3(0.f, 0.f, 0.f);
    if (lb.kind == T3_OP_COOK) {
      const float r = eval_value<TEX>(mat, lb.p0, fg).x;
      L.r2[k] = r * r;
      L.f0[k] = eval_value<TEX>(mat, lb.p1, fg);
    } else if (lb.kind == T3_OP_PHONG) {
      L.r2[k] = eval_value<TEX>(mat, lb.p0, fg).x;
    }
    c += prob;
    L.cdf[k] = c;  // upper edge of lobe k's interval
  }
  // lobes are drawn with probability prob / c (Add nodes make c exceed 1, as
  // AddMaterial.sample picks each child with probability 1/2 and weight 2)
#pragma unroll
  for (int k = 0; k < NL; k++) L.w[k] = c * L.w[k];
}

// one sample of lobe k: direction and scalar-or-colour weight
template <int NL>
__device__ __forceinline__ V3 sample_lobe(const IblLobes<NL>& L, int k, V3 n, V3 vdir, float xu,
                                          float xv, V3& dir) {
  const int kind = L.kind[k];
  if (kind == T3_OP_LAMBERT) {
    dir = normalized(tangent_dir(n, sqrtf(xu), xv));
    return L.w[k];
  }
  if (kind == T3_OP_COOK) {
    const float a2s = fmaxf(0.0f, L.r2[k]);
    const float u = sqrtf((1.0f - xu) / (1.0f - xu * (1.0f - a2s)));
    const V3 rdir = reflect3(v3(-vdir.x, -vdir.y, -vdir.z), n);
    V3 o = tangent_dir(rdir, u, xv);
    // CookTorrance.sub_brdf(n, idir = V, odir = o)
    const float a2 = fmaxf(1e-6f, L.r2[k]);
    const V3 half = normalized(vdir + o);
    const float NoH = fmaxf(1e-10f, dot(half, n));
    const float NoL = fmaxf(1e-10f, dot(vdir, n));
    const float NoV = fmaxf(1e-10f, dot(o, n));
    const float VoH = fminf(1.0f, fmaxf(1e-10f, dot(half, o)));
    (void)NoH;
    const float kk = a2 * 0.5f;
    const float vdf = 1.0f / (((NoV * kk + 1.0f) - kk) * ((NoL * kk + 1.0f) - kk) *
                              (1.0f * (1.0f - a2) + 12.566370614359172f * a2));
    const float om = 1.0f - VoH;
    const float om2 = om * om;
    const float p5 = om * (om2 * om2);
    const V3 f0 = L.f0[k];
    V3 fdf = f0 + p5 * one_minus(f0);
    if (dot(o, n) < 0.0f) {
      o = v3(-o.x, -o.y, -o.z);
      fdf = v3(0.f, 0.f, 0.f);
    }
    dir = o;
    return vdf * (L.w[k] * fdf);
  }
  if (kind == T3_OP_PHONG) {
    const float m = L.r2[k];
    const float u = powf(xu, 1.0f / (m + 1.0f));
    const V3 rdir = reflect3(v3(-vdir.x, -vdir.y, -vdir.z), n);
    V3 o = tangent_dir(rdir, u, xv);
    float wt = 1.0f;
    if (dot(o, n) < 0.0f) {
      o = v3(-o.x, -o.y, -o.z);
      wt = 0.0f;
    }
    dir = o;
    return wt * L.w[k];
  }
  dir = n;
  return v3(0.f, 0.f, 0.f);
}

// emission + (1/spp) sum_s weight_s * env(dir_s)
template <int NL>
__device__ __forceinline__ V3 ibl_mc(const IblLobes<NL>& L, V3 n, V3 vdir, const Env& env, int spp,
                                     uint32_t seed, uint32_t pixel) {
  const uint32_t base = rng_base(seed, pixel);
  V3 acc = v3(0.f, 0.f, 0.f);
  const float total = L.cdf[NL - 1];
  if (!(total > 0.0f)) return acc;
  for (int s = 0; s < spp; s++) {
    const float xs = rng_draw(base, (uint32_t)s, 0u) * total;
    const float xu = rng_draw(base, (uint32_t)s, 1u);
    const float xv = rng_draw(base, (uint32_t)s, 2u);
    int k = 0;
#pragma unroll
    for (int j = 0; j < NL - 1; j++)
      if (xs >= L.cdf[j]) k = j + 1;
    V3 dir;
    const V3 w = sample_lobe<NL>(L, k, n, vdir, xu, xv, dir);
    if (w.x != 0.0f || w.y != 0.0f || w.z != 0.0f) acc = acc + w * env_sample(env, dir);
  }
  return (1.0f / (float)spp) * acc;
}

// ---- SkyboxLighting's prefiltered lookup (T3_LIGHT_IBL_PREFILTERED) ---------
__device__ __forceinline__ Env map_env(const t3_ibl_map& m) { return Env{m.data, m.w, m.h, m.half}; }

// bilerp(lut, (VoH, roughness)) (tina/common.py:141-150) at the point in
// texel units, as CookTorrance.sample_ibl reads it (material.py:275); the +1
// texels clamped to the table
__device__ __forceinline__ void lut_ab(const t3_ibl_tables& T, float px, float py, float& A, float& B) {
  const float Ix = floorf(px), Iy = floorf(py);
  const float x0 = px - Ix, x1 = py - Iy, y0 = 1.0f - x0, y1 = 1.0f - x1;
  const int ix = (int)Ix, iy = (int)Iy;
  auto at = [&](int i, int j) {
    i = min(max(i, 0), T.lut_w - 1);
    j = min(max(j, 0), T.lut_h - 1);
    return __ldg(reinterpret_cast<const float2*>(T.lut) + ((int64_t)i * T.lut_h + j));
  };
  const float2 a = at(ix + 1, iy + 1), b = at(ix + 1, iy), c = at(ix, iy), d = at(ix, iy + 1);
  A = ((a.x * x0) * x1 + (b.x * x0) * y1) + ((c.x * y0) * y1 + (d.x * y0) * x1);
  B = ((a.y * x0) * x1 + (b.y * x0) * y1) + ((c.y * y0) * y1 + (d.y * y0) * x1);
}

// CookTorrance.sample_ibl (tina/matr/material.py:256-277): the maps of the two
// roughness levels around `r` at the mirror direction, lerped, times
// f0 * A + B.  rough_levels (:251-253) pair each level with its step from the
// previous one; the ranges are tested in order and the last match wins.
__device__ __forceinline__ V3 cook_prefiltered(const t3_ibl_tables& T, float r, V3 f0, V3 n, V3 vdir) {
  constexpr double lv[7] = {0.0, 0.03, 0.08, 0.18, 0.35, 0.65, 1.0};
  const V3 rdir = reflect3(v3(-vdir.x, -vdir.y, -vdir.z), n);
  V3 wei = v3(1.f, 1.f, 1.f);
#pragma unroll
  for (int id = 0; id < 6; id++) {
    const float rough = (float)lv[id + 1], step = (float)(lv[id + 1] - lv[id]);
    const float lo = (float)(lv[id + 1] - (lv[id + 1] - lv[id]));
    if (lo <= r && r <= rough) {
      const V3 w1 = env_sample(map_env(T.spec[id]), rdir);
      const V3 w2 = env_sample(map_env(T.spec[id + 1]), rdir);
      const float fac2 = (rough - r) / step;
      wei = (1.0f - fac2) * w2 + fac2 * w1;  // lerp(fac2, wei2, wei1)
    }
  }
  const V3 half = normalized(vdir + rdir);
  const float VoH = fminf(1.0f, fmaxf(1e-10f, dot(half, rdir)));
  float A, B;
  lut_ab(T, VoH, r, A, B);
  return v3(wei.x * (f0.x * A + B), wei.y * (f0.y * A + B), wei.z * (f0.z * A + B));
}

// material.sample_ibl summed over the flattened lobes: each lobe's weight is
// the product of the Mix / Scale factors on its path (Mix: (1 - f) w1 + f w2,
// material.py:141-145; Scale: f w, :187-191); Lambert reads the diffuse map at
// the normal (:441-442).  Returns the emission separately.
template <int NL, bool TEX>
__device__ __forceinline__ V3 ibl_prefiltered(const DevMaterial& mat, const t3_ibl_tables& T, const Frag& fg,
                                              V3 vdir, V3& emission) {
  V3 acc = v3(0.f, 0.f, 0.f);
  emission = v3(0.f, 0.f, 0.f);
#pragma unroll
  for (int k = 0; k < NL; k++) {
    if (k >= mat.nlobes) continue;
    const DevLobe& lb = mat.lobes[k];
    V3 w = v3(1.f, 1.f, 1.f);
    for (int j = 0; j < lb.nfac; j++) {
      const V3 f = eval_value<TEX>(mat, lb.fac[j] & 0xFFFF, fg);
      w = w * ((lb.fac[j] & T3_FAC_ONE_MINUS) ? one_minus(f) : f);
    }
    if (lb.kind == T3_OP_EMISSION) {
      emission = emission + w;
    } else if (lb.kind == T3_OP_LAMBERT) {
      acc = acc + w * env_sample(map_env(T.diffuse), fg.normal);
    } else if (lb.kind == T3_OP_COOK) {
      const float r = eval_value<TEX>(mat, lb.p0, fg).x;
      acc = acc + w * cook_prefiltered(T, r, eval_value<TEX>(mat, lb.p1, fg), fg.normal, vdir);
    }
  }
  return acc;
}

} // namespace t3
