// t3_device.cuh -- device-side building blocks shared by the raster and shade
// kernels: exact-order FP32 arithmetic, the mesh protocol, per-face setup and
// barycentric weights.
//
// Bit-exactness contract: face setup, weights and depth are evaluated with the
// round-to-nearest intrinsics (__fadd_rn, __fmul_rn, __fdiv_rn ...), which the
// compiler never contracts into FMA, in the operation order of Tina's Taichi
// source (tina/core/triangle.py:93-122, tina/common.py:170-184).  The triangle
// id and depth buffers are therefore bit-identical to a serial FP32 evaluation
// of that source.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/tina3.h"

namespace t3 {

#define T3_MAX_LOBES 4
#define T3_MAX_FACTORS 4
#define T3_EMPTY_KEY 0xFFFFFFFFFFFFFFFFull

// ---- exact-order arithmetic -------------------------------------------------
__device__ __forceinline__ float xadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float xsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float xmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xdiv(float a, float b) { return __fdiv_rn(a, b); }
// 1 / b, correctly rounded: the same bits as xdiv(1.0f, b)
__device__ __forceinline__ float xrcp(float b) { return __frcp_rn(b); }

struct f2 { float x, y; };
struct f3 { float x, y, z; };

__device__ __forceinline__ f3 mk3(float a, float b, float c) { return f3{a, b, c}; }

// float -> int32 truncation; out-of-range saturates, NaN -> INT32_MIN
__device__ __forceinline__ int32_t trunc_i32(float x) {
  if (!(x >= -2147483648.0f)) return INT32_MIN;
  if (x >= 2147483648.0f) return INT32_MAX;
  return (int32_t)x;
}

// mapply (tina/common.py:170-177), exact order
__device__ __forceinline__ void mapply_x(const float* m, f3 p, float wei, f3& r, float& w) {
  float r0 = xmul(m[3], wei), r1 = xmul(m[7], wei), r2 = xmul(m[11], wei);
  r0 = xadd(r0, xmul(m[0], p.x)); r0 = xadd(r0, xmul(m[1], p.y)); r0 = xadd(r0, xmul(m[2], p.z));
  r1 = xadd(r1, xmul(m[4], p.x)); r1 = xadd(r1, xmul(m[5], p.y)); r1 = xadd(r1, xmul(m[6], p.z));
  r2 = xadd(r2, xmul(m[8], p.x)); r2 = xadd(r2, xmul(m[9], p.y)); r2 = xadd(r2, xmul(m[10], p.z));
  float ww = xmul(m[15], wei);
  ww = xadd(ww, xmul(m[12], p.x)); ww = xadd(ww, xmul(m[13], p.y)); ww = xadd(ww, xmul(m[14], p.z));
  r = f3{r0, r1, r2};
  w = ww;
}
__device__ __forceinline__ f3 mapply_pos_x(const float* m, f3 p) {
  f3 r; float w;
  mapply_x(m, p, 1.0f, r, w);
  return f3{xdiv(r.x, w), xdiv(r.y, w), xdiv(r.z, w)};
}
// 3x3 @ v (Taichi Matrix.__matmul__ order)
__device__ __forceinline__ f3 matvec3_x(const float* m, f3 v) {
  float a0 = xmul(m[0], v.x); a0 = xadd(a0, xmul(m[1], v.y)); a0 = xadd(a0, xmul(m[2], v.z));
  float a1 = xmul(m[3], v.x); a1 = xadd(a1, xmul(m[4], v.y)); a1 = xadd(a1, xmul(m[5], v.z));
  float a2 = xmul(m[6], v.x); a2 = xadd(a2, xmul(m[7], v.y)); a2 = xadd(a2, xmul(m[8], v.z));
  return f3{a0, a1, a2};
}
__device__ __forceinline__ f3 sub_x(f3 a, f3 b) { return f3{xsub(a.x, b.x), xsub(a.y, b.y), xsub(a.z, b.z)}; }
__device__ __forceinline__ f3 cross_x(f3 a, f3 b) {
  return f3{xsub(xmul(a.y, b.z), xmul(a.z, b.y)), xsub(xmul(a.z, b.x), xmul(a.x, b.z)),
            xsub(xmul(a.x, b.y), xmul(a.y, b.x))};
}
__device__ __forceinline__ float dot_x(f3 a, f3 b) {
  return xadd(xadd(xmul(a.x, b.x), xmul(a.y, b.y)), xmul(a.z, b.z));
}
__device__ __forceinline__ f3 normalized_x(f3 a) {
  float inv = xrcp(__fsqrt_rn(dot_x(a, a)));
  return f3{xmul(inv, a.x), xmul(inv, a.y), xmul(inv, a.z)};
}
__device__ __forceinline__ float cross2_x(float ax, float ay, float bx, float by) {
  return xsub(xmul(ax, by), xmul(ay, bx));
}

__device__ __forceinline__ f3 ld3(const float* p) { return f3{__ldg(p), __ldg(p + 1), __ldg(p + 2)}; }

// ---- mesh protocol -----------------------------------------------------------
// Mesh-edit flags apply in the fixed nesting
//   MeshNoCulling(MeshFlipNormal(MeshFlipCulling(MeshFlatNormal(MeshTransform(base)))))

// pointer to attribute `attr` (0 vert, 1 norm, 2 coor) of corner k of base face f
__device__ __forceinline__ const float* base_ptr(const t3_mesh& d, int64_t f, int k, int attr) {
  const float* arr = attr == 0 ? d.verts : attr == 1 ? d.norms : d.coors;
  const int width = attr == 2 ? 2 : 3;
  if (d.kind == T3_MESH_SOUP) {
    return arr + (f * 3 + k) * width;
  } else if (d.kind == T3_MESH_GRID) {
    // MeshGrid._get_face_props (tina/mesh/grid.py:46-58); the cell stride is
    // the second axis's cell count (the reference's res.x - 1 equals it on
    // square grids and reads outside a rectangular one)
    const uint32_t stride = (uint32_t)d.grid_ny - 1u;
    const uint32_t m = (uint32_t)(f >> 1);
    const uint32_t i = m / stride, j = m - i * stride;
    // corners a=(i,j) b=(i+1,j) c=(i+1,j+1) d=(i,j+1); odd faces take (a, c, d)
    int c = k;
    if (f & 1) c = k == 0 ? 0 : k + 1;
    const uint32_t ii = i + (c == 1 || c == 2 ? 1u : 0u);
    const uint32_t jj = j + (c >= 2 ? 1u : 0u);
    return arr + ((int64_t)ii * d.grid_ny + jj) * width;
  } else {
    const int slot = attr == 0 ? d.slot_vert : attr == 1 ? d.slot_norm : d.slot_coor;
    const int32_t idx = __ldg(d.faces + f * d.face_stride + k * d.corner_stride + slot);
    return arr + (int64_t)idx * width;
  }
}

struct FaceRef {
  int64_t f;   // base face
  bool flip;   // corner order reversed
  bool negate; // normals negated
};

__device__ __forceinline__ FaceRef face_ref(const t3_mesh& d, int64_t n) {
  FaceRef r{n, (d.flags & T3_MESH_FLIP_ORDER) != 0, (d.flags & T3_MESH_FLIP_NORMAL) != 0};
  if (d.flags & T3_MESH_NOCULL) {
    r.f = n >> 1;
    if (n & 1) { r.flip = !r.flip; r.negate = !r.negate; }
  }
  return r;
}

// the three corners of face n of a face soup's position or normal array
__device__ __forceinline__ void soup_corners(const float* arr, int64_t n, f3 v[3]) {
  const float* p = arr + n * 9;
#pragma unroll
  for (int k = 0; k < 3; k++) v[k] = ld3(p + 3 * k);
}

__device__ __forceinline__ void base_verts(const t3_mesh& d, int64_t f, f3 v[3]) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    v[k] = ld3(base_ptr(d, f, k, 0));
    if (d.flags & T3_MESH_TRANSFORM) v[k] = mapply_pos_x(d.trans, v[k]);
  }
}

__device__ __forceinline__ void face_verts(const t3_mesh& d, const FaceRef& r, f3 v[3]) {
  f3 t[3];
  base_verts(d, r.f, t);
  v[0] = r.flip ? t[2] : t[0];
  v[1] = t[1];
  v[2] = r.flip ? t[0] : t[2];
}

__device__ __forceinline__ void face_norms(const t3_mesh& d, const FaceRef& r, f3 v[3]) {
  f3 t[3];
  if (d.flags & T3_MESH_FLAT_NORMAL) {
    f3 p[3];
    base_verts(d, r.f, p);
    f3 nn = normalized_x(cross_x(sub_x(p[1], p[0]), sub_x(p[2], p[0])));
    t[0] = t[1] = t[2] = nn;
  } else {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      t[k] = ld3(base_ptr(d, r.f, k, 1));
      if (d.flags & T3_MESH_TRANSFORM) t[k] = matvec3_x(d.trans_normal, t[k]);
    }
  }
  v[0] = r.flip ? t[2] : t[0];
  v[1] = t[1];
  v[2] = r.flip ? t[0] : t[2];
  if (r.negate) {
#pragma unroll
    for (int k = 0; k < 3; k++) v[k] = f3{-v[k].x, -v[k].y, -v[k].z};
  }
}

__device__ __forceinline__ void face_coors(const t3_mesh& d, const FaceRef& r, f2 v[3]) {
  f2 t[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float* p = base_ptr(d, r.f, k, 2);
    t[k] = f2{__ldg(p), __ldg(p + 1)};
  }
  v[0] = r.flip ? t[2] : t[0];
  v[1] = t[1];
  v[2] = r.flip ? t[0] : t[2];
}

// ---- per-face setup (triangle.py:93-113) -------------------------------------
struct Setup {
  float Az, Bz, Cz;       // NDC depth of the corners
  float bx, by, cx, cy;   // viewport corners b, c
  float bcnx, bcny, canx, cany;
  float wsa, wsb, wsc;    // 1 / clip w
  int32_t botx, boty, topx, topy;
};

__device__ __forceinline__ bool inside_clip(f3 p) {
  return (-1.0f <= p.x && p.x <= 1.0f) && (-1.0f <= p.y && p.y <= 1.0f) &&
         (-1.0f <= p.z && p.z <= 1.0f);
}

// The reference walks every pixel of [floor(min), ceil(max)] (triangle.py:108-114),
// but a pixel whose centre lies well outside [min, max] cannot pass the inside
// test, so only centres in [min - eps, max + eps] are tested (about half the
// pixel tests of small faces).  The bound, in terms of the setup's FP32
// values: with positive clip-w reciprocals a pixel passes only if its three
// computed weights are >= 0.  Each is the exact barycentric coordinate lambda_i
// plus evaluation and coefficient rounding of at most 8u (T + 1) + 4u T, where
// u = 2^-24 and T = (ext_x + ext_y + 4) (|bcn| + |can|)_1 bounds every product
// in the weights over the walked range; the rounding of the face's doubled
// area n adds at most 8u T to the third.  A centre with lambda_i >= -E lies
// within E * extent of the corners' [min, max] (it is their affine
// combination), so eps = 2^-18 (T + 1) (extent + 1), about three times the
// bound, plus 2^-16 (2 + |coord| + extent) for the viewport coordinates'
// own rounding.  T is large exactly where cancellation makes the weights
// inaccurate: thin wedges with a far corner (a centre 0.4 px outside the
// corners' range can pass there) keep nearly the reference's whole range.
// Faces whose clip-w reciprocals are not all positive and finite accept
// centres outside the corners' range and are not tightened.
__device__ __forceinline__ void tighten_to_centres(float lo, float hi, float T, int32_t& bot, int32_t& top) {
  const float mag = fmaxf(fabsf(lo), fabsf(hi));
  if (!(mag < 16777216.0f)) return;  // also NaN / inf: keep the reference's range
  const float ext = hi - lo;
  const float eps = (2.0f + mag + ext) * 1.52587890625e-05f +        // 2^-16
                    (T + 1.0f) * (ext + 1.0f) * 3.814697265625e-06f;  // 2^-18
  if (!(eps < 4.0f)) return;  // no centre of the range is excluded (also inf / NaN)
  const int32_t b = (int32_t)ceilf(lo - 0.5f - eps);
  const int32_t t = (int32_t)floorf(hi - 0.5f + eps);
  bot = b > bot ? b : bot;
  top = t < top ? t : top;
}

// the vertex transform of the setup: NDC position and clip w of one corner
// (mapply_pos, common.py:170-184)
__device__ __forceinline__ float4 vertex_ndc(const t3_frame& fr, f3 v) {
  f3 r;
  float w;
  mapply_x(fr.W2V, v, 1.0f, r, w);
  return make_float4(xdiv(r.x, w), xdiv(r.y, w), xdiv(r.z, w), w);
}

// setup from the corners' NDC positions and clip w (the rest of
// render_occup's per-face part); returns false when the face is culled or clipped
__device__ __forceinline__ bool face_setup_ndc(const t3_frame& fr, float4 A4, float4 B4, float4 C4,
                                               Setup& s) {
  const f3 Av = f3{A4.x, A4.y, A4.z}, Bv = f3{B4.x, B4.y, B4.z}, Cv = f3{C4.x, C4.y, C4.z};
  const float wa = A4.w, wb = B4.w, wc = C4.w;
  const float facing = cross2_x(xsub(Bv.x, Av.x), xsub(Bv.y, Av.y), xsub(Cv.x, Av.x), xsub(Cv.y, Av.y));
  if (facing <= 0.0f && (fr.flags & T3_CULLING)) return false;
  if (fr.flags & T3_CLIPPING) {
    if (!inside_clip(Av) && !inside_clip(Bv) && !inside_clip(Cv)) return false;
  }
  const float W = (float)fr.width, H = (float)fr.height;
  const float ax = xmul(xadd(xmul(Av.x, 0.5f), 0.5f), W), ay = xmul(xadd(xmul(Av.y, 0.5f), 0.5f), H);
  const float bx = xmul(xadd(xmul(Bv.x, 0.5f), 0.5f), W), by = xmul(xadd(xmul(Bv.y, 0.5f), 0.5f), H);
  const float cx = xmul(xadd(xmul(Cv.x, 0.5f), 0.5f), W), cy = xmul(xadd(xmul(Cv.y, 0.5f), 0.5f), H);
  const int32_t lox = trunc_i32(floorf(fminf(fminf(ax, bx), cx)));
  const int32_t loy = trunc_i32(floorf(fminf(fminf(ay, by), cy)));
  const int32_t hix = trunc_i32(ceilf(fmaxf(fmaxf(ax, bx), cx)));
  const int32_t hiy = trunc_i32(ceilf(fmaxf(fmaxf(ay, by), cy)));
  s.botx = lox > 0 ? lox : 0;
  s.boty = loy > 0 ? loy : 0;
  s.topx = hix < fr.width - 1 ? hix : fr.width - 1;
  s.topy = hiy < fr.height - 1 ? hiy : fr.height - 1;
  const float n = cross2_x(xsub(bx, ax), xsub(by, ay), xsub(cx, ax), xsub(cy, ay));
  s.bcnx = xdiv(xsub(bx, cx), n);
  s.bcny = xdiv(xsub(by, cy), n);
  s.canx = xdiv(xsub(cx, ax), n);
  s.cany = xdiv(xsub(cy, ay), n);
  s.bx = bx; s.by = by; s.cx = cx; s.cy = cy;
  s.wsa = xrcp(wa);
  s.wsb = xrcp(wb);
  s.wsc = xrcp(wc);
  if (s.wsa > 0.0f && s.wsb > 0.0f && s.wsc > 0.0f && s.wsa < INFINITY && s.wsb < INFINITY &&
      s.wsc < INFINITY) {
    const float lox_f = fminf(fminf(ax, bx), cx), hix_f = fmaxf(fmaxf(ax, bx), cx);
    const float loy_f = fminf(fminf(ay, by), cy), hiy_f = fmaxf(fmaxf(ay, by), cy);
    const float S = fabsf(s.bcnx) + fabsf(s.bcny) + fabsf(s.canx) + fabsf(s.cany);
    const float T = ((hix_f - lox_f) + (hiy_f - loy_f) + 4.0f) * S;  // inf / NaN: no tightening
    tighten_to_centres(lox_f, hix_f, T, s.botx, s.topx);
    tighten_to_centres(loy_f, hiy_f, T, s.boty, s.topy);
  }
  s.Az = Av.z; s.Bz = Bv.z; s.Cz = Cv.z;
  return true;
}

// returns false when the face is culled or clipped
__device__ __forceinline__ bool face_setup(const t3_frame& fr, const f3 v[3], Setup& s) {
  return face_setup_ndc(fr, vertex_ndc(fr, v[0]), vertex_ndc(fr, v[1]), vertex_ndc(fr, v[2]), s);
}

// vertex row of corner k of base face f (GRID and INDEXED meshes; base_ptr's indexing)
__device__ __forceinline__ int64_t corner_vertex(const t3_mesh& d, int64_t f, int k) {
  if (d.kind == T3_MESH_GRID) {
    const uint32_t stride = (uint32_t)d.grid_ny - 1u;
    const uint32_t m = (uint32_t)(f >> 1);
    const uint32_t i = m / stride, j = m - i * stride;
    int c = k;
    if (f & 1) c = k == 0 ? 0 : k + 1;
    const uint32_t ii = i + (c == 1 || c == 2 ? 1u : 0u);
    const uint32_t jj = j + (c >= 2 ? 1u : 0u);
    return (int64_t)ii * d.grid_ny + jj;
  }
  return __ldg(d.faces + f * d.face_stride + k * d.corner_stride + d.slot_vert);
}

// Unnormalised weights at pixel centre (px, py) and their sum (triangle.py:115-119).
__device__ __forceinline__ void face_raw_weights(const Setup& s, float px, float py, float& wx,
                                                 float& wy, float& wz, float& sum) {
  const float w_bc = cross2_x(xsub(px, s.bx), xsub(py, s.by), s.bcnx, s.bcny);
  const float w_ca = cross2_x(xsub(px, s.cx), xsub(py, s.cy), s.canx, s.cany);
  wx = xmul(w_bc, s.wsa);
  wy = xmul(w_ca, s.wsb);
  wz = xmul(xsub(xsub(1.0f, w_bc), w_ca), s.wsc);
  sum = xadd(xadd(wx, wy), wz);
}

// Exact `all(wei / sum >= 0)`.  For 0 < sum < 1 a negative finite weight stays
// negative after the division (|w| / sum > |w| >= 2^-149 never rounds to -0), so
// those pixels are rejected without dividing; every other case divides.
__device__ __forceinline__ bool face_inside(float wx, float wy, float wz, float sum, f3& wei) {
  if (sum > 0.0f && sum < 1.0f && (wx < 0.0f || wy < 0.0f || wz < 0.0f)) return false;
  wei = f3{xdiv(wx, sum), xdiv(wy, sum), xdiv(wz, sum)};
  return wei.x >= 0.0f && wei.y >= 0.0f && wei.z >= 0.0f;
}

__device__ __forceinline__ f3 face_weights(const Setup& s, float px, float py) {
  float wx, wy, wz, sum;
  face_raw_weights(s, px, py, wx, wy, wz, sum);
  return f3{xdiv(wx, sum), xdiv(wy, sum), xdiv(wz, sum)};
}

__device__ __forceinline__ float face_depth(const Setup& s, f3 wei) {
  return xadd(xadd(xmul(wei.x, s.Az), xmul(wei.y, s.Bz)), xmul(wei.z, s.Cz));
}

__device__ __forceinline__ uint64_t pack_key(int32_t depth, uint32_t id) {
  return ((uint64_t)((uint32_t)depth ^ 0x80000000u) << 32) | (uint64_t)id;
}

// ---- particles (tina/core/particle.py) -----------------------------------------

// mapply_dir (common.py:186-189): mapply with w = 0, in source order
__device__ __forceinline__ f3 mapply_dir_x(const float* m, f3 d) {
  f3 r;
  float w;
  mapply_x(m, d, 0.0f, r, w);
  return r;
}

// from_viewport (engine.py:63-65): p / res * 2 - 1
__device__ __forceinline__ float from_viewport_x(float p, float res) {
  return xsub(xmul(xdiv(p, res), 2.0f), 1.0f);
}

struct ParSetup {
  float ax, ay, az, r2;  // world centre, radius**2
  float vz;              // NDC depth of the centre (the depth of every pixel)
  int32_t depth;         // int(vz * maxdepth)
  int32_t botx, boty, topx, topy;
};

// ParticleRaster.render_occup's per-particle part (particle.py:77-101); false
// when clipped away or the bbox is empty
__device__ __forceinline__ bool particle_setup(const t3_frame& fr, f3 A, float R, ParSetup& p) {
  const f3 Av = mapply_pos_x(fr.W2V, A);
  if ((fr.flags & T3_CLIPPING) && !(-1.0f <= Av.z && Av.z <= 1.0f)) return false;
  const f3 DX = normalized_x(mapply_dir_x(fr.V2W, f3{1.0f, 0.0f, 0.0f}));
  const f3 DY = normalized_x(mapply_dir_x(fr.V2W, f3{0.0f, 1.0f, 0.0f}));
  const f3 AX = f3{xadd(A.x, xmul(DX.x, R)), xadd(A.y, xmul(DX.y, R)), xadd(A.z, xmul(DX.z, R))};
  const f3 AY = f3{xadd(A.x, xmul(DY.x, R)), xadd(A.y, xmul(DY.y, R)), xadd(A.z, xmul(DY.z, R))};
  const float rvx = xsub(mapply_pos_x(fr.W2V, AX).x, Av.x);
  const float rvy = xsub(mapply_pos_x(fr.W2V, AY).y, Av.y);
  const float W = (float)fr.width, H = (float)fr.height;
  auto vp = [](float c, float res) { return xmul(xadd(xmul(c, 0.5f), 0.5f), res); };
  // b = viewport of (Av - (rx,0)), (Av + (rx,0)), (Av - (0,ry)), (Av + (0,ry))
  const float b0x = vp(xsub(Av.x, rvx), W), b0y = vp(xsub(Av.y, 0.0f), H);
  const float b1x = vp(xadd(Av.x, rvx), W), b1y = vp(xadd(Av.y, 0.0f), H);
  const float b2x = vp(xsub(Av.x, 0.0f), W), b2y = vp(xsub(Av.y, rvy), H);
  const float b3x = vp(xadd(Av.x, 0.0f), W), b3y = vp(xadd(Av.y, rvy), H);
  const int32_t lox = trunc_i32(floorf(fminf(b0x, b2x))), loy = trunc_i32(floorf(fminf(b0y, b2y)));
  const int32_t hix = trunc_i32(ceilf(fmaxf(b1x, b3x))), hiy = trunc_i32(ceilf(fmaxf(b1y, b3y)));
  p.botx = lox > 0 ? lox : 0;
  p.boty = loy > 0 ? loy : 0;
  p.topx = hix < fr.width - 1 ? hix : fr.width - 1;
  p.topy = hiy < fr.height - 1 ? hiy : fr.height - 1;
  p.ax = A.x; p.ay = A.y; p.az = A.z;
  p.r2 = xmul(R, R);
  p.vz = Av.z;
  p.depth = trunc_i32(xmul(Av.z, (float)fr.maxdepth));
  return p.botx <= p.topx && p.boty <= p.topy;
}

// the world point of pixel centre (px, py) at the particle's depth
// (particle.py:103-105): mapply_pos(V2W, (from_viewport(p), Av.z))
__device__ __forceinline__ f3 particle_pixel_world(const t3_frame& fr, float px, float py, float vz) {
  const f3 Pv = f3{from_viewport_x(px, (float)fr.width), from_viewport_x(py, (float)fr.height), vz};
  return mapply_pos_x(fr.V2W, Pv);
}

// (Pl - Al).norm_sqr() <= Rl**2
__device__ __forceinline__ bool particle_covers(const ParSetup& p, f3 Pl) {
  const float dx = xsub(Pl.x, p.ax), dy = xsub(Pl.y, p.ay), dz = xsub(Pl.z, p.az);
  return !(xadd(xadd(xmul(dx, dx), xmul(dy, dy)), xmul(dz, dz)) > p.r2);
}

// ---- wireframe (WireframeRaster, tina/core/wireframe.py) ----------------------
__host__ __device__ __forceinline__ bool is_wire(const t3_mesh& d) {
  return d.kind == T3_MESH_LINES || (d.flags & T3_MESH_WIREFRAME) != 0;
}

// world endpoints of line n of a wire object: SimpleMesh(npolygon=2) lines, or
// MeshToWire's corners (n % p, (n + 1) % p) of face n / p (wire.py:20-27)
__device__ __forceinline__ void wire_endpoints(const t3_mesh& d, int64_t n, f3& A, f3& B) {
  if (d.kind == T3_MESH_LINES) {
    int64_t l = n;
    bool swap = false;
    if (d.flags & T3_MESH_WIREFRAME) { l = n >> 1; swap = (n & 1) != 0; }
    f3 p0 = ld3(d.verts + l * 6), p1 = ld3(d.verts + l * 6 + 3);
    if (d.flags & T3_MESH_TRANSFORM) { p0 = mapply_pos_x(d.trans, p0); p1 = mapply_pos_x(d.trans, p1); }
    A = swap ? p1 : p0;
    B = swap ? p0 : p1;
    return;
  }
  if (d.flags & T3_MESH_QUADS) {
    // MeshGrid(as_quad=True) (grid.py:46-58): quad f = cell f's corners
    // a=(i,j) b=(i+1,j) c=(i+1,j+1) d=(i,j+1); line n joins corners n % 4 and (n + 1) % 4
    const int64_t f = n >> 2;
    const int e = (int)(n & 3);
    const int64_t stride = (int64_t)d.grid_ny - 1;
    const int64_t i = f / stride, j = f - i * stride;
    auto corner = [&](int c) {
      const int64_t ii = i + (c == 1 || c == 2 ? 1 : 0), jj = j + (c >= 2 ? 1 : 0);
      f3 p = ld3(d.verts + (ii * d.grid_ny + jj) * 3);
      if (d.flags & T3_MESH_TRANSFORM) p = mapply_pos_x(d.trans, p);
      return p;
    };
    A = corner(e);
    B = corner((e + 1) & 3);
    return;
  }
  const int64_t f = n / 3;
  const int e = (int)(n - f * 3);
  f3 v[3];
  face_verts(d, face_ref(d, f), v);
  A = e == 0 ? v[0] : e == 1 ? v[1] : v[2];
  B = e == 0 ? v[1] : e == 1 ? v[2] : v[0];
}

struct WireSetup {
  float ax, ay;    // viewport start a
  float kx, ky;    // per-step increment k (draw_line)
  float az, bz;    // NDC depth of the endpoints
  float wsa, wsb;  // 1 / clip w of the endpoints
  int32_t siz;     // the line's last step (steps 0..siz)
  int32_t lo, hi;  // the steps whose pixel lies inside the frame
};

// the pixel coordinate of step i along one axis (pos = src + k * i + bias)
__device__ __forceinline__ float wire_coord(float a, float k, float bias, int32_t i) {
  return xadd(xadd(a, xmul(k, (float)i)), bias);
}

// first i in [lo, hi + 1) where pred, for a predicate false..false true..true
template <class Pred>
__device__ __forceinline__ int32_t wire_first(int32_t lo, int32_t hi, Pred pred) {
  int64_t a = lo, b = (int64_t)hi + 1;
  while (a < b) {
    const int64_t m = a + ((b - a) >> 1);
    if (pred((int32_t)m)) b = m; else a = m + 1;
  }
  return (int32_t)a;
}

// the steps of [0, siz] whose coordinate lies in [0, res): every operation of
// wire_coord is monotone in i (k * float(i) for a fixed k, then two roundings
// of a sum), so the in-range steps form one interval, found by bisection
__device__ __forceinline__ void wire_axis_range(float a, float k, float bias, int32_t res, int32_t siz,
                                                int32_t& lo, int32_t& hi) {
  const float r = (float)res;
  if (k >= 0.0f) {
    lo = wire_first(0, siz, [&](int32_t i) { return wire_coord(a, k, bias, i) >= 0.0f; });
    hi = wire_first(0, siz, [&](int32_t i) { return !(wire_coord(a, k, bias, i) < r); }) - 1;
  } else {
    lo = wire_first(0, siz, [&](int32_t i) { return wire_coord(a, k, bias, i) < r; });
    hi = wire_first(0, siz, [&](int32_t i) { return !(wire_coord(a, k, bias, i) >= 0.0f); }) - 1;
  }
}

// WireframeRaster.render_color's per-line part (wireframe.py:72-83, draw_line
// :49-64); false when clipped or no step lands in the frame
__device__ __forceinline__ bool wire_setup(const t3_frame& fr, f3 A, f3 B, WireSetup& s) {
  f3 ra, rb;
  float wa, wb;
  mapply_x(fr.W2V, A, 1.0f, ra, wa);
  mapply_x(fr.W2V, B, 1.0f, rb, wb);
  const f3 Av = f3{xdiv(ra.x, wa), xdiv(ra.y, wa), xdiv(ra.z, wa)};
  const f3 Bv = f3{xdiv(rb.x, wb), xdiv(rb.y, wb), xdiv(rb.z, wb)};
  if ((fr.flags & T3_WIRE_CLIPPING) && !inside_clip(Av) && !inside_clip(Bv)) return false;
  auto vp = [](float c, float res) { return xmul(xadd(xmul(c, 0.5f), 0.5f), res); };
  s.ax = vp(Av.x, (float)fr.width);
  s.ay = vp(Av.y, (float)fr.height);
  const float bx = vp(Bv.x, (float)fr.width), by = vp(Bv.y, (float)fr.height);
  s.az = Av.z;
  s.bz = Bv.z;
  s.wsa = xdiv(1.0f, wa);
  s.wsb = xdiv(1.0f, wb);
  const float dx = xsub(bx, s.ax), dy = xsub(by, s.ay);
  const float adx = fabsf(dx), ady = fabsf(dy);
  if (adx >= ady) {
    s.kx = dx >= 0.0f ? 1.0f : -1.0f;
    s.ky = xdiv(xmul(s.kx, dy), dx);
    s.siz = trunc_i32(adx);
  } else {
    s.ky = dy >= 0.0f ? 1.0f : -1.0f;
    s.kx = xdiv(xmul(s.ky, dx), dy);
    s.siz = trunc_i32(ady);
  }
  // range(siz + 1) in int32: empty for siz < 0 and for siz = INT32_MAX (overflow)
  if (s.siz < 0 || s.siz == INT32_MAX) return false;
  int32_t lx, hx, ly, hy;
  wire_axis_range(s.ax, s.kx, fr.bias[0], fr.width, s.siz, lx, hx);
  wire_axis_range(s.ay, s.ky, fr.bias[1], fr.height, s.siz, ly, hy);
  s.lo = lx > ly ? lx : ly;
  s.hi = hx < hy ? hx : hy;
  return s.lo <= s.hi;
}

// step i of the line (wireframe.py:84-92): its pixel and int depth; false when
// the pixel is outside the frame or the depth cannot pass the depth test
__device__ __forceinline__ bool wire_step(const t3_frame& fr, const WireSetup& s, int32_t i, int& x, int& y,
                                          int32_t& depth) {
  const float fi = (float)i;
  x = trunc_i32(floorf(xadd(xadd(s.ax, xmul(s.kx, fi)), fr.bias[0])));
  y = trunc_i32(floorf(xadd(xadd(s.ay, xmul(s.ky, fi)), fr.bias[1])));
  if (!(0 <= x && x < fr.width && 0 <= y && y < fr.height)) return false;
  const float cor = xdiv(fi, (float)s.siz);
  float w0 = xmul(xsub(1.0f, cor), s.wsa), w1 = xmul(cor, s.wsb);
  const float sum = xadd(w0, w1);
  w0 = xdiv(w0, sum);
  w1 = xdiv(w1, sum);
  const float df = xadd(xmul(w0, s.az), xmul(w1, s.bz));
  depth = trunc_i32(xmul(df, (float)fr.maxdepth));
  return depth < fr.maxdepth;
}

} // namespace t3
