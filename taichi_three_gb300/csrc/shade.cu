// shade.cu -- the deferred interpolate-and-shade pass of the direct path.
//
// TriangleRaster.render_color (tina/core/triangle.py:134-153) with the shader it
// calls inlined (t3_shading.cuh).  One thread per pixel: it decodes the winning
// face from the packed key, recomputes that face's setup and barycentric weights
// exactly as the rasteriser did (so depth_f is bit-exact), interpolates
// position / normal / texcoord, evaluates the material once per pixel, then
// sums the lamps and applies ACES.
#include "t3_shading.cuh"

namespace t3 {

// Copies the scene descriptor (a kernel parameter) into the workspace and zeroes
// the per-frame counters: one launch makes the scene readable by every later
// kernel of the frame, including inside a captured CUDA graph.
__global__ void k_upload_scene(const DevScene sc, DevScene* __restrict__ dst,
                               uint32_t* __restrict__ counters, int ncounters,
                               int32_t* __restrict__ status) {
  if (blockIdx.x == 0) {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&sc);
    uint32_t* d = reinterpret_cast<uint32_t*>(dst);
    constexpr int nwords = (int)(sizeof(DevScene) / 4);
    for (int i = threadIdx.x; i < nwords; i += blockDim.x) d[i] = src[i];
    if (threadIdx.x == 0 && status) *status = 0;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ncounters; i += gridDim.x * blockDim.x)
    counters[i] = 0u;
}

cudaError_t launch_upload_scene(const DevScene& sc, DevScene* dst, uint32_t* counters,
                                int ncounters, int32_t* status, cudaStream_t st) {
  int grid = (ncounters + 255) / 256;
  grid = grid < 1 ? 1 : grid > 64 ? 64 : grid;
  k_upload_scene<<<grid, 256, 0, st>>>(sc, dst, counters, ncounters, status);
  return cudaGetLastError();
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
k_shade(const DevScene* __restrict__ sc, const unsigned long long* __restrict__ keys,
        t3_outputs out, int64_t npix, int H) {
  const int64_t i = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  if (i >= npix) return;
  const int x = (int)(i / H), y = (int)(i - (int64_t)x * H);
  shade_pixel_from_key(sc, nullptr, keys[i], x, y, out);
}

cudaError_t launch_shade(const DevScene* sc_dev, const t3_frame& fr, const unsigned long long* keys,
                         const t3_outputs& out, cudaStream_t st) {
  constexpr int BLOCK = 256;
  const int64_t npix = (int64_t)fr.width * fr.height;
  const int64_t grid = (npix + BLOCK - 1) / BLOCK;
  k_shade<BLOCK><<<(unsigned)grid, BLOCK, 0, st>>>(sc_dev, keys, out, npix, fr.height);
  return cudaGetLastError();
}

} // namespace t3
