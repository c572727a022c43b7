// vertex.cu -- per-vertex stages that run before the rasteriser.
//
// MeshGrid.pre_compute (tina/mesh/grid.py:27-36): smooth grid normals by
// central differences with clamped neighbours,
//   dy = pos[i, j+1] - pos[i, j-1],  dx = pos[i+1, j] - pos[i-1, j],
//   nrm[i, j] = normalize(cross(dx, dy)),
// evaluated with the exact-order helpers so the normals are bit-identical to a
// serial FP32 evaluation of that source.
#include "t3_internal.cuh"

namespace t3 {

__global__ void k_grid_normals(const float* __restrict__ pos, float* __restrict__ nrm, int nx,
                               int ny) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)nx * ny) return;
  const int i = (int)(idx / ny), j = (int)(idx - (int64_t)i * ny);
  const int i2 = i - 1 > 0 ? i - 1 : 0, j2 = j - 1 > 0 ? j - 1 : 0;
  const int i1 = i + 1 < nx - 1 ? i + 1 : nx - 1, j1 = j + 1 < ny - 1 ? j + 1 : ny - 1;
  const f3 dy = sub_x(ld3(pos + ((int64_t)i * ny + j1) * 3), ld3(pos + ((int64_t)i * ny + j2) * 3));
  const f3 dx = sub_x(ld3(pos + ((int64_t)i1 * ny + j) * 3), ld3(pos + ((int64_t)i2 * ny + j) * 3));
  const f3 n = normalized_x(cross_x(dx, dy));
  nrm[idx * 3] = n.x;
  nrm[idx * 3 + 1] = n.y;
  nrm[idx * 3 + 2] = n.z;
}

} // namespace t3

extern "C" int t3_grid_normals(const float* pos, float* nrm, int nx, int ny, void* stream) {
  if (!pos || !nrm || nx < 1 || ny < 1) return T3_EINVAL;
  const int64_t n = (int64_t)nx * ny;
  const int block = 256;
  t3::k_grid_normals<<<(unsigned)((n + block - 1) / block), block, 0, (cudaStream_t)stream>>>(
      pos, nrm, nx, ny);
  return cudaGetLastError() == cudaSuccess ? T3_OK : T3_ECUDA;
}

namespace t3 {
__global__ void k_tonemap(float* __restrict__ rgb, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float c = rgb[i];
  // source order, no contraction: the same bits as the serial evaluation
  const float num = xmul(c, xadd(xmul(2.51f, c), 0.03f));
  const float den = xadd(xmul(c, xadd(xmul(2.43f, c), 0.59f)), 0.14f);
  rgb[i] = xdiv(num, den);
}
} // namespace t3

// ToneMapping.apply (tina/postp/tonemap.py:10-12): in-place ACES on n floats.
extern "C" int t3_tonemap(float* rgb, int64_t n, void* stream) {
  if (!rgb || n < 0) return T3_EINVAL;
  if (n == 0) return T3_OK;
  const int block = 256;
  t3::k_tonemap<<<(unsigned)((n + block - 1) / block), block, 0, (cudaStream_t)stream>>>(rgb, n);
  return cudaGetLastError() == cudaSuccess ? T3_OK : T3_ECUDA;
}

namespace t3 {
// z = amp * sin(fx * x + wx * t) * cos(fy * y + wy * t) at every grid vertex
// (x, y read from the vertex itself)
__global__ void k_grid_wave(float* __restrict__ pos, int64_t n, float amp, float fx, float fy, float wx,
                            float wy, float t) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float x = pos[i * 3], y = pos[i * 3 + 1];
  pos[i * 3 + 2] = amp * sinf(fx * x + wx * t) * cosf(fy * y + wy * t);
}
} // namespace t3

// Height-field animation of a grid: pos[i, j].z = amp sin(fx x + wx t) cos(fy y + wy t).
extern "C" int t3_grid_wave(float* pos, int nx, int ny, float amp, float fx, float fy, float wx, float wy,
                            float t, void* stream) {
  if (!pos || nx < 1 || ny < 1) return T3_EINVAL;
  const int64_t n = (int64_t)nx * ny;
  const int block = 256;
  t3::k_grid_wave<<<(unsigned)((n + block - 1) / block), block, 0, (cudaStream_t)stream>>>(
      pos, n, amp, fx, fy, wx, wy, t);
  return cudaGetLastError() == cudaSuccess ? T3_OK : T3_ECUDA;
}

namespace t3 {
// The vertex stage of indexed meshes and grids: each vertex's NDC position and
// clip w once (after MeshTransform), instead of once per face corner in the
// rasteriser's setup (the same operations on the same inputs, so the same bits).
__global__ void k_vertex_ndc(const t3_frame fr, const t3_mesh mesh, int64_t nverts, float4* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nverts) return;
  f3 v = ld3(mesh.verts + i * 3);
  if (mesh.flags & T3_MESH_TRANSFORM) v = mapply_pos_x(mesh.trans, v);
  out[i] = vertex_ndc(fr, v);
}

cudaError_t launch_vertex_ndc(const t3_frame& fr, const t3_mesh& mesh, int64_t nverts, float4* out,
                              cudaStream_t st) {
  if (nverts <= 0) return cudaSuccess;
  k_vertex_ndc<<<(unsigned)((nverts + 255) / 256), 256, 0, st>>>(fr, mesh, nverts, out);
  return cudaGetLastError();
}
} // namespace t3
