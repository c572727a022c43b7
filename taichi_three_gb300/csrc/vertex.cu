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

// ---- MeshSmoothNormal (tina/mesh/norm.py:17-55) --------------------------------
// The reference accumulates each face's unit normal onto its three vertices in
// face order, then normalises.  Here the (vertex, face) pairs of all corners are
// sorted by vertex with a stable radix sort, which keeps every vertex's faces in
// face order, and one thread per vertex sums its faces' normals in that order:
// the same additions in the same order as the serial loop, so the result is
// bit-identical and independent of scheduling.
#include <cub/device/device_radix_sort.cuh>

namespace t3 {

__global__ void k_sn_pairs(const t3_mesh mesh, int64_t nfaces, int32_t* __restrict__ keys,
                           int32_t* __restrict__ vals) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nfaces * 3) return;
  const int64_t n = e / 3;
  const int k = (int)(e - n * 3);
  keys[e] = __ldg(mesh.faces + n * mesh.face_stride + k * mesh.corner_stride + mesh.slot_vert);
  vals[e] = (int32_t)n;
}

// [start, end) of every vertex's run of sorted pairs (runs of vertices outside
// [0, nverts) are dropped)
__global__ void k_sn_runs(const int32_t* __restrict__ keys, int64_t m, int64_t nverts,
                          int32_t* __restrict__ start, int32_t* __restrict__ end) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= m) return;
  const int32_t v = keys[p];
  if (v < 0 || v >= nverts) return;
  if (p == 0 || keys[p - 1] != v) start[v] = (int32_t)p;
  if (p == m - 1 || keys[p + 1] != v) end[v] = (int32_t)(p + 1);
}

__global__ void k_sn_normals(const t3_mesh mesh, int64_t nverts, const int32_t* __restrict__ faces,
                             const int32_t* __restrict__ start, const int32_t* __restrict__ end,
                             float* __restrict__ out) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nverts) return;
  f3 acc = f3{0.0f, 0.0f, 0.0f};
  for (int32_t p = start[v]; p < end[v]; p++) {
    const int64_t n = faces[p];
    const f3 a = ld3(base_ptr(mesh, n, 0, 0)), b = ld3(base_ptr(mesh, n, 1, 0));
    const f3 c = ld3(base_ptr(mesh, n, 2, 0));
    const f3 nrm = normalized_x(cross_x(sub_x(b, a), sub_x(c, a)));
    acc = f3{xadd(acc.x, nrm.x), xadd(acc.y, nrm.y), xadd(acc.z, nrm.z)};
  }
  const f3 r = normalized_x(acc);
  out[v * 3] = r.x;
  out[v * 3 + 1] = r.y;
  out[v * 3 + 2] = r.z;
}

struct SmoothLayout {
  size_t temp, temp_bytes, keys_in, vals_in, keys_out, vals_out, start, end, total;
};

static size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

static int smooth_layout(int64_t nfaces, int64_t nverts, SmoothLayout& L) {
  if (nfaces < 0 || nverts < 0) return T3_EINVAL;
  if (nfaces * 3 > (int64_t)0x7FFFFFFF || nverts > (int64_t)0x7FFFFFFF) return T3_ETOOBIG;
  const int m = (int)(nfaces * 3);
  size_t temp = 0;
  if (m > 0 &&
      cub::DeviceRadixSort::SortPairs(nullptr, temp, (const int32_t*)nullptr, (int32_t*)nullptr,
                                      (const int32_t*)nullptr, (int32_t*)nullptr, m) != cudaSuccess)
    return T3_ECUDA;
  const size_t pairs = al256(sizeof(int32_t) * (size_t)(m > 0 ? m : 1));
  const size_t runs = al256(sizeof(int32_t) * (size_t)(nverts > 0 ? nverts : 1));
  L.temp = 0;
  L.temp_bytes = temp;
  L.keys_in = al256(temp);
  L.vals_in = L.keys_in + pairs;
  L.keys_out = L.vals_in + pairs;
  L.vals_out = L.keys_out + pairs;
  L.start = L.vals_out + pairs;
  L.end = L.start + runs;
  L.total = L.end + runs;
  return T3_OK;
}

} // namespace t3

extern "C" int t3_smooth_normals_workspace_size(int64_t nfaces, int64_t nverts, size_t* bytes) {
  if (!bytes) return T3_EINVAL;
  t3::SmoothLayout L;
  const int r = t3::smooth_layout(nfaces, nverts, L);
  if (r) return r;
  *bytes = L.total;
  return T3_OK;
}

extern "C" int t3_smooth_normals(const t3_mesh* mesh, int64_t nverts, float* norms_out, void* workspace,
                                 size_t workspace_bytes, void* stream) {
  if (!mesh || !norms_out || !workspace || nverts < 0) return T3_EINVAL;
  if (mesh->kind != T3_MESH_INDEXED || mesh->flags != 0) return T3_EINVAL;
  if (mesh->nfaces > 0 && (!mesh->verts || !mesh->faces || mesh->face_stride <= 0 || mesh->corner_stride <= 0))
    return T3_EINVAL;
  if ((reinterpret_cast<uintptr_t>(workspace) & 15) != 0) return T3_EINVAL;
  t3::SmoothLayout L;
  int r = t3::smooth_layout(mesh->nfaces, nverts, L);
  if (r) return r;
  if (workspace_bytes < L.total) return T3_EINVAL;
  if (nverts == 0) return T3_OK;
  cudaStream_t st = (cudaStream_t)stream;
  uint8_t* ws = reinterpret_cast<uint8_t*>(workspace);
  int32_t* keys_in = reinterpret_cast<int32_t*>(ws + L.keys_in);
  int32_t* vals_in = reinterpret_cast<int32_t*>(ws + L.vals_in);
  int32_t* keys_out = reinterpret_cast<int32_t*>(ws + L.keys_out);
  int32_t* vals_out = reinterpret_cast<int32_t*>(ws + L.vals_out);
  int32_t* start = reinterpret_cast<int32_t*>(ws + L.start);
  int32_t* end = reinterpret_cast<int32_t*>(ws + L.end);
  const int64_t m = mesh->nfaces * 3;
  const int block = 256;
  cudaError_t e = cudaMemsetAsync(start, 0, sizeof(int32_t) * (size_t)nverts, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(end, 0, sizeof(int32_t) * (size_t)nverts, st);
  if (e == cudaSuccess && m > 0) {
    t3::k_sn_pairs<<<(unsigned)((m + block - 1) / block), block, 0, st>>>(*mesh, mesh->nfaces, keys_in,
                                                                          vals_in);
    e = cudaGetLastError();
    size_t temp = L.temp_bytes;
    if (e == cudaSuccess)
      e = cub::DeviceRadixSort::SortPairs(ws + L.temp, temp, keys_in, keys_out, vals_in, vals_out, (int)m,
                                          0, 32, st);
    if (e == cudaSuccess) {
      t3::k_sn_runs<<<(unsigned)((m + block - 1) / block), block, 0, st>>>(keys_out, m, nverts, start, end);
      e = cudaGetLastError();
    }
  }
  if (e == cudaSuccess) {
    t3::k_sn_normals<<<(unsigned)((nverts + block - 1) / block), block, 0, st>>>(*mesh, nverts, vals_out,
                                                                                 start, end, norms_out);
    e = cudaGetLastError();
  }
  return e == cudaSuccess ? T3_OK : T3_ECUDA;
}
