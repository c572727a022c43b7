// raster.cu -- depth-buffer clear and the direct rasteriser.
//
// TriangleRaster.render_occup (tina/core/triangle.py:89-131) as a GB300 kernel:
// one thread per face runs the vertex transform, back-face cull, trivial clip,
// viewport map, bbox and edge setup, then walks the bbox and folds every covered
// pixel into a packed 64-bit key (depth ^ sign bit) << 32 | face id with
// atomicMin.  The unsigned minimum of that key is the serial reference's winner:
// lowest int32 depth, ties to the lowest face id (the strict `>` at
// triangle.py:123), so the result does not depend on thread order and the
// reference's racy `occup[P] = f` store disappears.
//
// Face-soup vertex positions (9 floats per face) are staged into shared memory
// with 16-byte vector loads so a warp reads its 1152 contiguous bytes once.
// Faces whose clamped bbox exceeds `big_threshold` pixels are pushed to a queue
// and rasterised by k_raster_big, one CTA per face.
#include "t3_internal.cuh"

namespace t3 {

__global__ void k_clear(unsigned long long* __restrict__ keys, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if ((reinterpret_cast<uintptr_t>(keys) & 15) == 0) {
    ulonglong2* k2 = reinterpret_cast<ulonglong2*>(keys);
    const int64_t n2 = n >> 1;
    for (int64_t j = i; j < n2; j += stride) k2[j] = make_ulonglong2(T3_EMPTY_KEY, T3_EMPTY_KEY);
    if (i == 0 && (n & 1)) keys[n - 1] = T3_EMPTY_KEY;
  } else {
    for (int64_t j = i; j < n; j += stride) keys[j] = T3_EMPTY_KEY;
  }
}

// Folds one face's covered pixels in [x0, x1] x [y0, y1] into the key buffer.
__device__ __forceinline__ void raster_rect(const t3_frame& fr, const Setup& s, uint32_t id,
                                            int32_t x0, int32_t x1, int32_t y0, int32_t y1,
                                            unsigned long long* __restrict__ keys) {
  const int64_t H = fr.height;
  const float maxd = (float)fr.maxdepth;
  for (int32_t x = x0; x <= x1; x++) {
    const float px = xadd((float)x, fr.bias[0]);
    for (int32_t y = y0; y <= y1; y++) {
      const float py = xadd((float)y, fr.bias[1]);
      float wx, wy, wz, sum;
      face_raw_weights(s, px, py, wx, wy, wz, sum);
      f3 wei;
      if (!face_inside(wx, wy, wz, sum, wei)) continue;
      const int32_t d = trunc_i32(xmul(face_depth(s, wei), maxd));
      if (d >= fr.maxdepth) continue;  // can never pass `old > depth`
      const unsigned long long key = pack_key(d, id);
      unsigned long long* p = keys + (int64_t)x * H + y;
      // keys only decrease: a stale read can only send us to the atomic
      if (key < *reinterpret_cast<volatile unsigned long long*>(p)) atomicMin(p, key);
    }
  }
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
k_raster_direct(const t3_frame fr, const t3_mesh mesh, int64_t nfaces, uint32_t face_base,
                unsigned long long* __restrict__ keys, BigQueue big, int32_t big_threshold) {
  __shared__ __align__(16) float sv[BLOCK * 9];
  const int64_t f0 = (int64_t)blockIdx.x * BLOCK;
  const bool staged = mesh.kind == T3_MESH_SOUP && !(mesh.flags & T3_MESH_NOCULL);
  if (staged) {
    const int64_t rem = nfaces - f0;
    const int nf = rem < BLOCK ? (int)rem : BLOCK;
    const float* src = mesh.verts + f0 * 9;
    const int nflt = nf * 9;
    if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
      const int n4 = nflt >> 2;
      const float4* s4 = reinterpret_cast<const float4*>(src);
      float4* d4 = reinterpret_cast<float4*>(sv);
      for (int i = threadIdx.x; i < n4; i += BLOCK) d4[i] = __ldg(s4 + i);
      for (int i = (n4 << 2) + threadIdx.x; i < nflt; i += BLOCK) sv[i] = __ldg(src + i);
    } else {
      for (int i = threadIdx.x; i < nflt; i += BLOCK) sv[i] = __ldg(src + i);
    }
    __syncthreads();
  }
  const int64_t n = f0 + threadIdx.x;
  if (n >= nfaces) return;
  f3 v[3];
  if (staged) {
    const float* p = sv + threadIdx.x * 9;
    f3 t[3] = {f3{p[0], p[1], p[2]}, f3{p[3], p[4], p[5]}, f3{p[6], p[7], p[8]}};
    if (mesh.flags & T3_MESH_TRANSFORM) {
#pragma unroll
      for (int k = 0; k < 3; k++) t[k] = mapply_pos_x(mesh.trans, t[k]);
    }
    const bool flip = (mesh.flags & T3_MESH_FLIP_ORDER) != 0;
    v[0] = flip ? t[2] : t[0];
    v[1] = t[1];
    v[2] = flip ? t[0] : t[2];
  } else {
    face_verts(mesh, face_ref(mesh, n), v);
  }
  Setup s;
  if (!face_setup(fr, v, s)) return;
  if (s.botx > s.topx || s.boty > s.topy) return;
  const int64_t area = (int64_t)(s.topx - s.botx + 1) * (int64_t)(s.topy - s.boty + 1);
  if (area > big_threshold) {
    const uint32_t slot = atomicAdd(big.count, 1u);
    if (slot < big.capacity) {
      big.items[slot] = (uint32_t)n;
    } else {
      atomicOr(big.status, T3_STATUS_BIG_OVERFLOW);
    }
    return;
  }
  raster_rect(fr, s, face_base + (uint32_t)n, s.botx, s.topx, s.boty, s.topy, keys);
}

// One CTA per queued large face: threads stride over the face's bbox pixels.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
k_raster_big(const t3_frame fr, const t3_mesh mesh, uint32_t face_base,
             unsigned long long* __restrict__ keys, BigQueue big) {
  const uint32_t count = min(*big.count, big.capacity);
  const int64_t H = fr.height;
  const float maxd = (float)fr.maxdepth;
  for (uint32_t e = blockIdx.x; e < count; e += gridDim.x) {
    const uint32_t n = big.items[e];
    f3 v[3];
    face_verts(mesh, face_ref(mesh, n), v);
    Setup s;
    if (!face_setup(fr, v, s)) continue;
    const int32_t w = s.topx - s.botx + 1, h = s.topy - s.boty + 1;
    const int64_t area = (int64_t)w * h;
    const uint32_t id = face_base + n;
    for (int64_t k = threadIdx.x; k < area; k += BLOCK) {
      const int32_t x = s.botx + (int32_t)(k / h);
      const int32_t y = s.boty + (int32_t)(k - (k / h) * h);
      const float px = xadd((float)x, fr.bias[0]);
      const float py = xadd((float)y, fr.bias[1]);
      float wx, wy, wz, sum;
      face_raw_weights(s, px, py, wx, wy, wz, sum);
      f3 wei;
      if (!face_inside(wx, wy, wz, sum, wei)) continue;
      const int32_t d = trunc_i32(xmul(face_depth(s, wei), maxd));
      if (d >= fr.maxdepth) continue;
      const unsigned long long key = pack_key(d, id);
      unsigned long long* p = keys + (int64_t)x * H + y;
      if (key < *reinterpret_cast<volatile unsigned long long*>(p)) atomicMin(p, key);
    }
  }
}

cudaError_t launch_clear(unsigned long long* keys, int64_t n, cudaStream_t st) {
  const int block = 256;
  int64_t want = ((n >> 1) + block - 1) / block;
  const int grid = (int)(want < 4 * 152 * 8 ? (want > 0 ? want : 1) : 4 * 152 * 8);
  k_clear<<<grid, block, 0, st>>>(keys, n);
  return cudaGetLastError();
}

cudaError_t launch_raster_direct(const t3_frame& fr, const t3_object& ob, unsigned long long* keys,
                                 const BigQueue& big, int32_t big_threshold, cudaStream_t st) {
  if (ob.nfaces <= 0) return cudaSuccess;
  constexpr int BLOCK = 256;
  const int64_t grid = (ob.nfaces + BLOCK - 1) / BLOCK;
  // big.count was zeroed by the scene upload at the start of the frame
  k_raster_direct<BLOCK><<<(unsigned)grid, BLOCK, 0, st>>>(fr, ob.mesh, ob.nfaces,
                                                          (uint32_t)ob.face_base, keys, big,
                                                          big_threshold);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_raster_big<BLOCK><<<2 * 152, BLOCK, 0, st>>>(fr, ob.mesh, (uint32_t)ob.face_base, keys, big);
  return cudaGetLastError();
}

} // namespace t3
