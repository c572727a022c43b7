// postfx.cu -- full-screen passes after shading: blooming, FXAA and the TAA
// accumulator (tina/postp/blooming.py, tina/postp/fxaa.py,
// tina/util/accumator.py), in Scene.render's order (raster.py:200-207):
// blooming on the HDR image, tonemap, FXAA, accumulate.
//
// Images use Tina's field indexing: pixel (x, y) at x*H + y, RGB float32.
// Where the reference reads a neighbour outside the image (FXAA's 3x3
// stencil and shifted bilerp, the bloom upsampling's +1 texel) the index is
// clamped to the image.  All passes are HBM / L2 bound and fully coalesced
// along y.
#include "t3_internal.cuh"

namespace t3 {

struct F3 { float x, y, z; };
__device__ __forceinline__ F3 ld_rgb(const float* img, int64_t i) {
  return F3{img[3 * i], img[3 * i + 1], img[3 * i + 2]};
}
__device__ __forceinline__ void st_rgb(float* img, int64_t i, F3 c) {
  img[3 * i] = c.x;
  img[3 * i + 1] = c.y;
  img[3 * i + 2] = c.z;
}
__device__ __forceinline__ F3 fma3(float s, F3 a, F3 acc) {
  return F3{acc.x + a.x * s, acc.y + a.y * s, acc.z + a.z * s};
}

// bilerp (common.py:141-150) of a [w, h, 3] image at (px, py), indices clamped
__device__ __forceinline__ F3 bilerp_img(const float* img, int w, int h, float px, float py) {
  const float fx = floorf(px), fy = floorf(py);
  const int ix = (int)fx, iy = (int)fy;
  const float x0 = px - fx, x1 = py - fy, y0 = 1.0f - x0, y1 = 1.0f - x1;
  auto at = [&](int i, int j) {
    i = min(max(i, 0), w - 1);
    j = min(max(j, 0), h - 1);
    return ld_rgb(img, (int64_t)i * h + j);
  };
  F3 r{0.f, 0.f, 0.f};
  r = fma3(x0 * x1, at(ix + 1, iy + 1), r);
  r = fma3(x0 * y1, at(ix + 1, iy), r);
  r = fma3(y0 * y1, at(ix, iy), r);
  r = fma3(y0 * x1, at(ix, iy + 1), r);
  return r;
}

// ---- blooming ----------------------------------------------------------------
struct BloomArgs {
  float thresh, factor, scale;
  int radius;
  float gwei[129];
};

__device__ __forceinline__ float bloom_filter(const BloomArgs& a, float x) {
  float t = fmaxf(0.0f, x - a.thresh);
  t = 1.0f - 1.0f / (1.0f + a.scale * t);
  return a.factor * t;
}

// half-resolution average of the filtered image (blooming.py:53-57)
__global__ void k_bloom_down(const float* __restrict__ img, int W, int H, float* __restrict__ half,
                             const __grid_constant__ BloomArgs a) {
  const int w = W / 2, h = H / 2;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)w * h) return;
  const int x = (int)(i / h), y = (int)(i - (int64_t)x * h);
  F3 r{0.f, 0.f, 0.f};
  for (int dx = 0; dx < 2; dx++)
    for (int dy = 0; dy < 2; dy++) {
      const F3 c = ld_rgb(img, (int64_t)(2 * x + dx) * H + (2 * y + dy));
      r = F3{r.x + bloom_filter(a, c.x), r.y + bloom_filter(a, c.y), r.z + bloom_filter(a, c.z)};
    }
  st_rgb(half, i, F3{r.x / 4.0f, r.y / 4.0f, r.z / 4.0f});
}

// separable Gaussian along x (axis 0) or y (axis 1), clamped (blooming.py:58-73)
__global__ void k_bloom_blur(const float* __restrict__ src, float* __restrict__ dst, int w, int h, int axis,
                             const __grid_constant__ BloomArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)w * h) return;
  const int x = (int)(i / h), y = (int)(i - (int64_t)x * h);
  F3 r = ld_rgb(src, i);
  r = F3{r.x * a.gwei[0], r.y * a.gwei[0], r.z * a.gwei[0]};
  for (int k = 1; k <= a.radius; k++) {
    F3 v0, v1;
    if (axis == 0) {
      v0 = ld_rgb(src, (int64_t)max(0, x - k) * h + y);
      v1 = ld_rgb(src, (int64_t)min(w - 1, x + k) * h + y);
    } else {
      v0 = ld_rgb(src, (int64_t)x * h + max(0, y - k));
      v1 = ld_rgb(src, (int64_t)x * h + min(h - 1, y + k));
    }
    r = fma3(a.gwei[k], F3{v0.x + v1.x, v0.y + v1.y, v0.z + v1.z}, r);
  }
  st_rgb(dst, i, r);
}

// image += bilerp(half, I / 2) (blooming.py:74-75)
__global__ void k_bloom_up(float* __restrict__ img, int W, int H, const float* __restrict__ half) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)W * H) return;
  const int x = (int)(i / H), y = (int)(i - (int64_t)x * H);
  const F3 b = bilerp_img(half, W / 2, H / 2, (float)x / 2.0f, (float)y / 2.0f);
  const F3 c = ld_rgb(img, i);
  st_rgb(img, i, F3{c.x + b.x, c.y + b.y, c.z + b.z});
}

// ---- FXAA ----------------------------------------------------------------------
__device__ __forceinline__ float clamp01(float x) { return fminf(1.0f, fmaxf(0.0f, x)); }

// luminance clamp(0.2989 r + 0.587 g + 0.114 b) and a copy of the image
// (fxaa.py:27-29).  The luminances and the edge decisions below are evaluated
// in source order without FMA contraction, so which pixels are filtered, and
// in which direction, does not depend on the compiler.
__global__ void k_fxaa_lumi(const float* __restrict__ img, int64_t n, float* __restrict__ lumi,
                            float* __restrict__ copy) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const F3 c = ld_rgb(img, i);
  lumi[i] = clamp01(xadd(xadd(xmul(0.2989f, c.x), xmul(0.587f, c.y)), xmul(0.114f, c.z)));
  st_rgb(copy, i, c);
}

__global__ void k_fxaa(float* __restrict__ img, int W, int H, const float* __restrict__ lumi,
                       const float* __restrict__ copy, float abs_thresh, float rel_thresh, float factor) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)W * H) return;
  const int x = (int)(i / H), y = (int)(i - (int64_t)x * H);
  auto L = [&](int dx, int dy) {
    const int xx = min(max(x + dx, 0), W - 1), yy = min(max(y + dy, 0), H - 1);
    return lumi[(int64_t)xx * H + yy];
  };
  const float m = L(0, 0), nn = L(0, 1), e = L(1, 0), s = L(0, -1), w = L(-1, 0);
  const float ne = L(1, 1), nw = L(-1, 1), se = L(1, -1), sw = L(-1, -1);
  const float hi = fmaxf(fmaxf(fmaxf(fmaxf(m, nn), e), s), w);
  const float lo = fminf(fminf(fminf(fminf(m, nn), e), s), w);
  const float c = xsub(hi, lo);
  if (c < abs_thresh || c < xmul(rel_thresh, hi)) return;
  float filt = xmul(2.0f, xadd(xadd(xadd(nn, e), s), w));
  filt = xadd(filt, xadd(xadd(xadd(ne, nw), se), sw));
  filt = fabsf(xsub(xdiv(filt, 12.0f), m));
  filt = clamp01(xdiv(filt, c));
  const float t = clamp01(filt);  // smoothstep(filt, 0, 1)
  const float sm = xmul(xmul(t, t), xsub(3.0f, xmul(2.0f, t)));
  float blend = xmul(xmul(sm, sm), factor);
  auto edge = [](float a, float b, float mid) { return fabsf(xsub(xadd(a, b), xmul(2.0f, mid))); };
  float hori = xmul(edge(nn, s, m), 2.0f);
  hori = xadd(hori, edge(ne, se, e));
  hori = xadd(hori, edge(nw, sw, w));
  float vert = xmul(edge(e, w, m), 2.0f);
  vert = xadd(vert, edge(ne, nw, nn));
  vert = xadd(vert, edge(se, sw, s));
  const bool is_hori = hori >= vert;
  const float plumi = is_hori ? nn : e, nlumi = is_hori ? s : w;
  if (fabsf(plumi - m) < fabsf(nlumi - m)) blend = -blend;
  const float px = xadd((float)x, is_hori ? 0.0f : blend), py = xadd((float)y, is_hori ? blend : 0.0f);
  st_rgb(img, i, bilerp_img(copy, W, H, px, py));
}

// ---- TAA accumulator -------------------------------------------------------------
// acc = acc * (1 - 1/count) + src * (1/count)  (accumator.py:17-23)
__global__ void k_accumulate(float* __restrict__ acc, const float* __restrict__ src, int64_t n, float inv) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float a = acc[i] * (1.0f - inv);
  acc[i] = a + src[i] * inv;
}

static unsigned blocks(int64_t n) { return (unsigned)((n + 255) / 256); }

} // namespace t3

using namespace t3;

extern "C" {

int64_t t3_bloom_workspace_floats(int width, int height) {
  return 2 * 3 * (int64_t)(width / 2) * (height / 2);
}

int t3_bloom(float* rgb, int width, int height, float thresh, float factor, float scale, float sigma,
             int radius, float* workspace, int64_t workspace_floats, void* stream) {
  if (!rgb || !workspace || width < 2 || height < 2 || radius < 1 || radius > 128) return T3_EINVAL;
  if (workspace_floats < t3_bloom_workspace_floats(width, height)) return T3_EINVAL;
  BloomArgs a;
  a.thresh = thresh;
  a.factor = factor;
  a.scale = scale;
  a.radius = radius;
  // init_gwei (blooming.py:30-40) in float32
  float sum = -1.0f;
  for (int i = 0; i <= radius; i++) {
    const float x = sigma * (float)i / (float)radius;
    a.gwei[i] = expf(-(x * x));
    sum += a.gwei[i] * 2.0f;
  }
  for (int i = 0; i <= radius; i++) a.gwei[i] /= sum;
  const int w = width / 2, h = height / 2;
  const int64_t hn = (int64_t)w * h;
  float* half = workspace;
  float* tmp = workspace + 3 * hn;
  cudaStream_t st = (cudaStream_t)stream;
  k_bloom_down<<<blocks(hn), 256, 0, st>>>(rgb, width, height, half, a);
  k_bloom_blur<<<blocks(hn), 256, 0, st>>>(half, tmp, w, h, 0, a);
  k_bloom_blur<<<blocks(hn), 256, 0, st>>>(tmp, half, w, h, 1, a);
  k_bloom_up<<<blocks((int64_t)width * height), 256, 0, st>>>(rgb, width, height, half);
  return cudaGetLastError() == cudaSuccess ? T3_OK : T3_ECUDA;
}

int64_t t3_fxaa_workspace_floats(int width, int height) { return 4 * (int64_t)width * height; }

int t3_fxaa(float* rgb, int width, int height, float abs_thresh, float rel_thresh, float factor,
            float* workspace, int64_t workspace_floats, void* stream) {
  if (!rgb || !workspace || width < 1 || height < 1) return T3_EINVAL;
  if (workspace_floats < t3_fxaa_workspace_floats(width, height)) return T3_EINVAL;
  const int64_t n = (int64_t)width * height;
  float* lumi = workspace;
  float* copy = workspace + n;
  cudaStream_t st = (cudaStream_t)stream;
  k_fxaa_lumi<<<blocks(n), 256, 0, st>>>(rgb, n, lumi, copy);
  k_fxaa<<<blocks(n), 256, 0, st>>>(rgb, width, height, lumi, copy, abs_thresh, rel_thresh, factor);
  return cudaGetLastError() == cudaSuccess ? T3_OK : T3_ECUDA;
}

int t3_accumulate(float* acc, const float* src, int64_t n, int count, void* stream) {
  if (!acc || !src || n < 0 || count < 1) return T3_EINVAL;
  if (n == 0) return T3_OK;
  k_accumulate<<<blocks(n), 256, 0, (cudaStream_t)stream>>>(acc, src, n, 1.0f / (float)count);
  return cudaGetLastError() == cudaSuccess ? T3_OK : T3_ECUDA;
}

} // extern "C"
