// tina_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement of Tina's triangle rasteriser and deferred shading pass
// (taichi-dev/taichi_three, "Tina" v0.1.1), used by tests/ and by bench.py's
// CPU-baseline leg as the checker.  It is never part of the product path.
//
// Parity status: the reference is Python on the Taichi JIT, Taichi is not
// installable here, and the reference ships no golden vectors or tests with
// assertions.  This restatement is pinned against the reference's own Python
// source executed by tests/golden/make_golden.py (a pure-Python stand-in for the
// subset of the Taichi DSL the path uses); where that pin does not reach, the
// restatement is "parity unpinned".
//
// Semantics restated (file:line are within the reference project):
//   * Engine              tina/core/engine.py:6-76   (W2V/V2W, bias, maxdepth 2**30)
//   * mapply / mapply_pos tina/common.py:170-184     (op order below)
//   * TriangleRaster      tina/core/triangle.py:89-153
//   * interpolate         tina/core/triangle.py:32-49
//   * calc_view_ray       tina/core/shader.py:82-93
//   * Lighting            tina/core/lighting.py:84-98
//   * materials           tina/matr/material.py:69-472, 659-706
//   * nodes               tina/matr/nodes.py:42-96
//   * ACES tonemap        tina/advans.py:32-34, tina/postp/tonemap.py:10-12
//   * mesh getters        tina/mesh/simple.py:34-48, grid.py:27-70, trans.py:29-40,
//                         cull.py:5-66, norm.py:5-14, model.py:50-73, conn.py:117-140
//
// Floating point: every expression is evaluated in the Real type (float for the
// bit-exact oracle, double for the FP64 twin) left to right as the Taichi source
// is written, with IEEE division and square root, and the file is compiled with
// -ffp-contract=off so no multiply-add is fused.  Vector helpers follow Taichi's
// Matrix methods: dot = ((x0*y0 + x1*y1) + x2*y2), norm = sqrt(dot(v, v)),
// normalized = v * (1 / norm), 2-D cross = a.x*b.y - a.y*b.x, integer powers by
// repeated squaring (x**2 = x*x, x**5 = x * ((x*x)*(x*x))).
//
// The serial mode walks faces in index order, which makes the reference's
// `atomic_min(depth) > depth` (triangle.py:123) deterministic: the lowest depth
// wins and ties keep the lowest face id.  The parallel mode (OpenMP) reaches the
// same result through a 64-bit packed (depth, face id) compare-and-swap minimum;
// it is the timed CPU baseline.

#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/tina3.h"

namespace {

template <class R> struct v2 { R x, y; };
template <class R> struct v3 { R x, y, z; };

template <class R> inline v3<R> mk3(R a, R b, R c) { return v3<R>{a, b, c}; }
template <class R> inline v3<R> add(v3<R> a, v3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> inline v3<R> sub(v3<R> a, v3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> inline v3<R> mul(v3<R> a, v3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> inline v3<R> muls(R s, v3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> inline v3<R> mulv(v3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> inline v3<R> divs(v3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> inline v3<R> neg(v3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> inline R dot(v3<R> a, v3<R> b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <class R> inline R norm(v3<R> a) { return std::sqrt(dot(a, a)); }
template <class R> inline v3<R> normalized(v3<R> a) {
  R inv = R(1) / norm(a);
  return muls(inv, a);
}
template <class R> inline v3<R> cross(v3<R> a, v3<R> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> inline R cross2(v2<R> a, v2<R> b) { return a.x * b.y - a.y * b.x; }
// reflect(I, N) = I - 2 * N.dot(I) * N   (tina/common.py:197-199)
template <class R> inline v3<R> reflect(v3<R> I, v3<R> N) {
  R d = R(2) * dot(N, I);
  return sub(I, muls(d, N));
}
// A Taichi-source literal: an f32 constant in the FP32 oracle, the exact decimal in FP64.
template <class R> inline R cst(double x) { return sizeof(R) == 4 ? (R)(float)x : (R)x; }
template <class R> inline R pow2(R x) { return x * x; }
template <class R> inline R ipow(R x, int n) {
  R result = R(1), base = x;
  bool first = true;
  while (n > 0) {
    if (n & 1) { result = first ? base : result * base; first = false; }
    n >>= 1;
    if (n) base = base * base;
  }
  return first ? R(1) : result;
}
template <class R> inline R pow5(R x) {
  R x2 = x * x;
  R x4 = x2 * x2;
  return x * x4;
}
// Taichi `min`/`max` on floats keep the non-NaN operand (LLVM minnum/maxnum).
template <class R> inline R fmin_(R a, R b) { return std::fmin(a, b); }
template <class R> inline R fmax_(R a, R b) { return std::fmax(a, b); }

// float -> int32 with truncation; out-of-range values saturate (the Taichi source
// leaves them undefined) and NaN maps to INT32_MIN.
template <class R> inline int32_t trunc_i32(R x) {
  if (!(x >= R(-2147483648.0))) return INT32_MIN;
  if (x >= R(2147483648.0)) return INT32_MAX;
  return (int32_t)x;
}

// mapply(mat, pos, wei) (tina/common.py:170-177):
//   res_i = M[i][3]*wei; res_i += M[i][0]*p0; res_i += M[i][1]*p1; res_i += M[i][2]*p2
//   rew   = M[3][3]*wei; rew  += M[3][0]*p0; rew  += M[3][1]*p1; rew  += M[3][2]*p2
template <class R> struct mat4 { R m[16]; };
template <class R> inline void mapply(const mat4<R>& M, v3<R> p, R wei, v3<R>& res, R& rew) {
  const R* m = M.m;
  R r0 = m[3] * wei, r1 = m[7] * wei, r2 = m[11] * wei;
  r0 = r0 + m[0] * p.x; r0 = r0 + m[1] * p.y; r0 = r0 + m[2] * p.z;
  r1 = r1 + m[4] * p.x; r1 = r1 + m[5] * p.y; r1 = r1 + m[6] * p.z;
  r2 = r2 + m[8] * p.x; r2 = r2 + m[9] * p.y; r2 = r2 + m[10] * p.z;
  R w = m[15] * wei;
  w = w + m[12] * p.x; w = w + m[13] * p.y; w = w + m[14] * p.z;
  res = {r0, r1, r2};
  rew = w;
}
template <class R> inline v3<R> mapply_pos(const mat4<R>& M, v3<R> p) {
  v3<R> r; R w;
  mapply(M, p, R(1), r, w);
  return divs(r, w);
}
// 3x3 @ vec (Taichi Matrix.__matmul__: acc = M[i][0]*v0; acc += M[i][1]*v1; ...)
template <class R> inline v3<R> matvec3(const R* m, v3<R> v) {
  R a0 = m[0] * v.x; a0 = a0 + m[1] * v.y; a0 = a0 + m[2] * v.z;
  R a1 = m[3] * v.x; a1 = a1 + m[4] * v.y; a1 = a1 + m[5] * v.z;
  R a2 = m[6] * v.x; a2 = a2 + m[7] * v.y; a2 = a2 + m[8] * v.z;
  return {a0, a1, a2};
}

template <class R> inline v3<R> ld3(const float* p) { return {(R)p[0], (R)p[1], (R)p[2]}; }
template <class R> inline v3<R> ld2(const float* p) { return {(R)p[0], (R)p[1], R(0)}; }

// ---------------------------------------------------------------------------
// Mesh protocol (get_face_verts / get_face_norms / get_face_coors).
// Mesh-edit flags are applied in one fixed nesting:
//   MeshNoCulling(MeshFlipNormal(MeshFlipCulling(MeshFlatNormal(MeshTransform(base)))))
// ---------------------------------------------------------------------------
template <class R> struct Mesh {
  const t3_mesh* d;
  mat4<R> trans;
  R tn[9];
  explicit Mesh(const t3_mesh* desc) : d(desc) {
    for (int i = 0; i < 16; i++) trans.m[i] = (R)desc->trans[i];
    for (int i = 0; i < 9; i++) tn[i] = (R)desc->trans_normal[i];
  }
  // corner k, attribute 0 = vert, 1 = norm, 2 = coor, of a base-mesh face
  const float* base_ptr(int64_t f, int k, int attr) const {
    const float* arr = attr == 0 ? d->verts : attr == 1 ? d->norms : d->coors;
    int width = attr == 2 ? 2 : 3;
    if (d->kind == T3_MESH_SOUP) {
      return arr + (f * 3 + k) * width;
    } else if (d->kind == T3_MESH_GRID) {
      // MeshGrid._get_face_props (tina/mesh/grid.py:46-58); cell stride =
      // the second axis's cell count (res.x - 1 there: equal on square grids,
      // out of bounds on rectangular ones)
      int64_t stride = d->grid_ny - 1;
      int64_t m = f / 2;
      int64_t i = m / stride, j = m % stride;
      int64_t ii[4] = {i, i + 1, i + 1, i};
      int64_t jj[4] = {j, j, j + 1, j + 1};
      int sel[3] = {0, 1, 2};
      if (f % 2 != 0) { sel[0] = 0; sel[1] = 2; sel[2] = 3; }
      int c = sel[k];
      return arr + (ii[c] * d->grid_ny + jj[c]) * width;
    } else {
      int slot = attr == 0 ? d->slot_vert : attr == 1 ? d->slot_norm : d->slot_coor;
      int64_t idx = d->faces[f * d->face_stride + k * d->corner_stride + slot];
      return arr + idx * width;
    }
  }
  void verts(int64_t n, v3<R> v[3]) const {
    int64_t f = n;
    bool flip = (d->flags & T3_MESH_FLIP_ORDER) != 0;
    if (d->flags & T3_MESH_NOCULL) { f = n / 2; if (n % 2 != 0) flip = !flip; }
    v3<R> t[3];
    for (int k = 0; k < 3; k++) {
      t[k] = ld3<R>(base_ptr(f, k, 0));
      if (d->flags & T3_MESH_TRANSFORM) t[k] = mapply_pos(trans, t[k]);
    }
    for (int k = 0; k < 3; k++) v[k] = flip ? t[2 - k] : t[k];
  }
  void norms(int64_t n, v3<R> v[3]) const {
    int64_t f = n;
    bool flip = (d->flags & T3_MESH_FLIP_ORDER) != 0;
    bool negate = (d->flags & T3_MESH_FLIP_NORMAL) != 0;
    if (d->flags & T3_MESH_NOCULL) {
      f = n / 2;
      if (n % 2 != 0) { flip = !flip; negate = !negate; }
    }
    v3<R> t[3];
    if (d->flags & T3_MESH_FLAT_NORMAL) {
      // MeshFlatNormal._calc_norm (tina/mesh/norm.py:7-9) on the transformed verts
      v3<R> p[3];
      for (int k = 0; k < 3; k++) {
        p[k] = ld3<R>(base_ptr(f, k, 0));
        if (d->flags & T3_MESH_TRANSFORM) p[k] = mapply_pos(trans, p[k]);
      }
      v3<R> nn = normalized(cross(sub(p[1], p[0]), sub(p[2], p[0])));
      t[0] = t[1] = t[2] = nn;
    } else {
      for (int k = 0; k < 3; k++) {
        t[k] = ld3<R>(base_ptr(f, k, 1));
        if (d->flags & T3_MESH_TRANSFORM) t[k] = matvec3(tn, t[k]);
      }
    }
    for (int k = 0; k < 3; k++) {
      v[k] = flip ? t[2 - k] : t[k];
      if (negate) v[k] = neg(v[k]);
    }
  }
  void coors(int64_t n, v3<R> v[3]) const {
    int64_t f = n;
    bool flip = (d->flags & T3_MESH_FLIP_ORDER) != 0;
    if (d->flags & T3_MESH_NOCULL) { f = n / 2; if (n % 2 != 0) flip = !flip; }
    v3<R> t[3];
    for (int k = 0; k < 3; k++) t[k] = ld2<R>(base_ptr(f, k, 2));
    for (int k = 0; k < 3; k++) v[k] = flip ? t[2 - k] : t[k];
  }
  int64_t base_face(int64_t n) const { return (d->flags & T3_MESH_NOCULL) ? n / 2 : n; }
};

// ---------------------------------------------------------------------------
// Per-face setup, shared by render_occup and render_color (triangle.py:93-113)
// ---------------------------------------------------------------------------
template <class R> struct Setup {
  v3<R> Av, Bv, Cv;
  v2<R> a, b, c;
  v2<R> bcn, can;
  v3<R> wscale;
  int32_t botx, boty, topx, topy;
  bool culled;
};

template <class R>
inline v2<R> to_viewport(v3<R> p, int W, int H) {
  // (p.xy * 0.5 + 0.5) * res   (tina/core/engine.py:59-61)
  return {(p.x * R(0.5) + R(0.5)) * (R)W, (p.y * R(0.5) + R(0.5)) * (R)H};
}

template <class R> inline bool inside_clip(v3<R> p) {
  return (R(-1) <= p.x && p.x <= R(1)) && (R(-1) <= p.y && p.y <= R(1)) &&
         (R(-1) <= p.z && p.z <= R(1));
}

template <class R>
void face_setup(const mat4<R>& W2V, const t3_frame& fr, const v3<R> v[3], Setup<R>& s) {
  s.culled = false;
  s.Av = mapply_pos(W2V, v[0]);
  s.Bv = mapply_pos(W2V, v[1]);
  s.Cv = mapply_pos(W2V, v[2]);
  v2<R> e1 = {s.Bv.x - s.Av.x, s.Bv.y - s.Av.y};
  v2<R> e2 = {s.Cv.x - s.Av.x, s.Cv.y - s.Av.y};
  R facing = cross2(e1, e2);
  if (facing <= R(0) && (fr.flags & T3_CULLING)) { s.culled = true; return; }
  if (fr.flags & T3_CLIPPING) {
    if (!inside_clip(s.Av) && !inside_clip(s.Bv) && !inside_clip(s.Cv)) { s.culled = true; return; }
  }
  s.a = to_viewport(s.Av, fr.width, fr.height);
  s.b = to_viewport(s.Bv, fr.width, fr.height);
  s.c = to_viewport(s.Cv, fr.width, fr.height);
  R minx = fmin_(fmin_(s.a.x, s.b.x), s.c.x), miny = fmin_(fmin_(s.a.y, s.b.y), s.c.y);
  R maxx = fmax_(fmax_(s.a.x, s.b.x), s.c.x), maxy = fmax_(fmax_(s.a.y, s.b.y), s.c.y);
  int32_t bx = trunc_i32(std::floor(minx)), by = trunc_i32(std::floor(miny));
  int32_t tx = trunc_i32(std::ceil(maxx)), ty = trunc_i32(std::ceil(maxy));
  s.botx = bx > 0 ? bx : 0;
  s.boty = by > 0 ? by : 0;
  s.topx = tx < fr.width - 1 ? tx : fr.width - 1;
  s.topy = ty < fr.height - 1 ? ty : fr.height - 1;
  v2<R> ba = {s.b.x - s.a.x, s.b.y - s.a.y};
  v2<R> ca = {s.c.x - s.a.x, s.c.y - s.a.y};
  R n = cross2(ba, ca);
  s.bcn = {(s.b.x - s.c.x) / n, (s.b.y - s.c.y) / n};
  s.can = {(s.c.x - s.a.x) / n, (s.c.y - s.a.y) / n};
  v3<R> r; R wa, wb, wc;
  mapply(W2V, v[0], R(1), r, wa);
  mapply(W2V, v[1], R(1), r, wb);
  mapply(W2V, v[2], R(1), r, wc);
  s.wscale = {R(1) / wa, R(1) / wb, R(1) / wc};
}

// barycentric weights at pixel (x, y) (triangle.py:115-119 and :147-151)
template <class R>
inline v3<R> face_weights(const Setup<R>& s, const t3_frame& fr, int32_t x, int32_t y) {
  v2<R> pos = {(R)x + (R)fr.bias[0], (R)y + (R)fr.bias[1]};
  R w_bc = cross2(v2<R>{pos.x - s.b.x, pos.y - s.b.y}, s.bcn);
  R w_ca = cross2(v2<R>{pos.x - s.c.x, pos.y - s.c.y}, s.can);
  v3<R> wei = {w_bc * s.wscale.x, w_ca * s.wscale.y, ((R(1) - w_bc) - w_ca) * s.wscale.z};
  R sum = (wei.x + wei.y) + wei.z;
  return divs(wei, sum);
}

template <class R> inline R face_depth(const Setup<R>& s, v3<R> wei) {
  return (wei.x * s.Av.z + wei.y * s.Bv.z) + wei.z * s.Cv.z;
}

// ---------------------------------------------------------------------------
// Materials (tina/matr/material.py, nodes.py).  Values are carried as 3-vectors
// with a width tag; width-1 values broadcast like Taichi scalar * vector.
// ---------------------------------------------------------------------------
template <class R> struct Val { v3<R> v; int w; };
template <class R> inline Val<R> sval(R s) { return {{s, s, s}, 1}; }
template <class R> inline Val<R> vmul(Val<R> a, Val<R> b) { return {mul(a.v, b.v), a.w > b.w ? a.w : b.w}; }
template <class R> inline Val<R> vadd(Val<R> a, Val<R> b) { return {add(a.v, b.v), a.w > b.w ? a.w : b.w}; }
template <class R> inline Val<R> one_minus(Val<R> a) { return {{R(1) - a.v.x, R(1) - a.v.y, R(1) - a.v.z}, a.w}; }

template <class R> struct Frag {
  v3<R> pos, normal, texcoord;
  const float* attr; // per-face attributes of this fragment's face
  v3<R> color = {R(1), R(1), R(1)};  // Input('color'): white on triangles, the particle's colour
};

template <class R> struct MaterialEval {
  const t3_material* m;
  const Frag<R>* fr;

  Val<R> value(int i) const {
    const t3_node& n = m->nodes[i];
    switch (n.op) {
    case T3_OP_CONST:
      return {{(R)n.v[0], (R)n.v[1], (R)n.v[2]}, n.b == 3 ? 3 : 1};
    case T3_OP_ATTR: {
      if (n.b == 1) return sval<R>((R)fr->attr[n.a]);
      return {{(R)fr->attr[n.a], (R)fr->attr[n.a + 1], (R)fr->attr[n.a + 2]}, 3};
    }
    case T3_OP_INPUT:
      if (n.a == 0) return {fr->pos, 3};
      if (n.a == 1) return {fr->color, 3};  // V(1,1,1) on triangles (triangle.py:48), particle colour
      if (n.a == 2) return {fr->normal, 3};
      return {fr->texcoord, 2};
    case T3_OP_TEXTURE: {
      // Texture.__call__ nodes.py:105-111: bilerp(tex, texcoord * (shape - 1)),
      // bilerp of common.py:141-150 (the +1 texel clamped to the image)
      const t3_texture& t = m->textures[n.b];
      const Val<R> uv = value(n.a);
      const R px = uv.v.x * (R)(t.w - 1), py = uv.v.y * (R)(t.h - 1);
      const R Ix = std::floor(px), Iy = std::floor(py);
      const R x0 = px - Ix, x1 = py - Iy, y0 = R(1) - x0, y1 = R(1) - x1;
      auto texel = [&](int64_t i, int64_t j) {
        i = i < 0 ? 0 : i >= t.w ? t.w - 1 : i;
        j = j < 0 ? 0 : j >= t.h ? t.h - 1 : j;
        const float* p = t.data + (i * t.h + j) * t.channels;
        return t.channels == 1 ? v3<R>{(R)p[0], (R)p[0], (R)p[0]} : v3<R>{(R)p[0], (R)p[1], (R)p[2]};
      };
      const int64_t ix = (int64_t)Ix, iy = (int64_t)Iy;
      v3<R> r = muls(x0 * x1, texel(ix + 1, iy + 1));
      r = add(r, muls(x0 * y1, texel(ix + 1, iy)));
      r = add(r, muls(y0 * y1, texel(ix, iy)));
      r = add(r, muls(y0 * x1, texel(ix, iy + 1)));
      return {r, t.channels == 1 ? 1 : 3};
    }
    case T3_OP_CHECKER: {
      // ChessboardTexture nodes.py:114-126: lerp((texcoord // size).sum() % 2, c0, c1)
      const Val<R> uv = value(n.a);
      const R size = value(n.b).v.x;
      const R s = std::floor(uv.v.x / size) + std::floor(uv.v.y / size);
      const R t = s - R(2) * std::floor(s / R(2));
      const Val<R> c0 = value(n.c), c1 = value((int)n.v[0]);
      return vadd(vmul(c0, sval<R>(R(1) - t)), vmul(c1, sval<R>(t)));
    }
    case T3_OP_FRESNEL: {
      // f0 = metallic * albedo + (1 - metallic) * 0.16 * specular**2  material.py:69-71
      Val<R> met = value(n.a), alb = value(n.b), spc = value(n.c);
      Val<R> t1 = vmul(met, alb);
      Val<R> om = one_minus(met);
      Val<R> t2 = vmul(vmul(om, sval<R>(cst<R>(0.16))), vmul(spc, spc));
      return vadd(t1, t2);
    }
    default:
      return sval<R>(R(0));
    }
  }

  // brdf(nrm, idir=L, odir=V)
  Val<R> brdf(int i, v3<R> nrm, v3<R> idir, v3<R> odir) const {
    const t3_node& n = m->nodes[i];
    switch (n.op) {
    case T3_OP_LAMBERT:
      return sval<R>(inv_pi());
    case T3_OP_PHONG: {
      Val<R> mm = value(n.a);
      R m_ = mm.v.x;
      v3<R> rdir = reflect(neg(idir), nrm);
      R VoR = fmax_(R(0), dot(odir, rdir));
      // VoR**m: a Python-int shineness (node flag c == 1) is an integer power by
      // repeated squaring, a float one is pow().
      const t3_node& mn = m->nodes[n.a];
      R p = (mn.op == T3_OP_CONST && mn.c == 1) ? ipow(VoR, (int)mn.v[0]) : std::pow(VoR, m_);
      return sval<R>((p * (m_ + R(2))) / R(2));
    }
    case T3_OP_COOK:
      return cook_brdf(n, nrm, idir, odir);
    case T3_OP_EMISSION:
      return sval<R>(R(0));
    case T3_OP_MIX: {
      Val<R> fac = value(n.c);
      Val<R> w1 = brdf(n.a, nrm, idir, odir), w2 = brdf(n.b, nrm, idir, odir);
      return vadd(vmul(one_minus(fac), w1), vmul(fac, w2));
    }
    case T3_OP_SCALE: {
      Val<R> fac = value(n.b);
      return vmul(fac, brdf(n.a, nrm, idir, odir));
    }
    case T3_OP_ADD:
      return vadd(brdf(n.a, nrm, idir, odir), brdf(n.b, nrm, idir, odir));
    default:
      return sval<R>(R(0));
    }
  }

  static R inv_pi() { return cst<R>(1.0 / M_PI); }        // 1 / ti.pi
  static R c_eps_big() { return cst<R>(1.0 - 1e-10); }    // 1 - EPS
  static R c_eps() { return cst<R>(1e-10); }              // EPS
  static R c_eps6() { return cst<R>(1e-6); }              // advans.eps
  static R c_4pi() { return cst<R>(4.0 * M_PI); }         // 4 * ti.pi

  // CookTorrance.sub_brdf / brdf (material.py:322-362)
  Val<R> cook_brdf(const t3_node& n, v3<R> nrm, v3<R> idir, v3<R> odir) const {
    R roughness = value(n.a).v.x;
    Val<R> f0 = value(n.b);
    const R EPS = c_eps();
    v3<R> half = normalized(add(idir, odir));
    R NoH = fmax_(EPS, dot(half, nrm));
    R NoL = fmax_(EPS, dot(idir, nrm));
    R NoV = fmax_(EPS, dot(odir, nrm));
    R VoH = fmin_(c_eps_big(), fmax_(EPS, dot(half, odir)));
    R alpha2 = fmax_(c_eps6(), pow2(roughness));
    R denom = R(1) - pow2(NoH) * (R(1) - alpha2);
    R ndf = alpha2 / pow2(denom);
    R k = alpha2 / R(2);
    R vdf = R(1) / ((NoV * k + R(1)) - k);
    vdf = vdf * (R(1) / ((NoL * k + R(1)) - k));
    vdf = vdf / (R(1) * (R(1) - alpha2) + c_4pi() * alpha2);
    R p5 = pow5(R(1) - VoH);
    Val<R> fdf = {{f0.v.x + (R(1) - f0.v.x) * p5, f0.v.y + (R(1) - f0.v.y) * p5,
                   f0.v.z + (R(1) - f0.v.z) * p5}, f0.w};
    // fdf * vdf * ndf
    return {{(fdf.v.x * vdf) * ndf, (fdf.v.y * vdf) * ndf, (fdf.v.z * vdf) * ndf}, fdf.w};
  }

  Val<R> ambient(int i) const {
    const t3_node& n = m->nodes[i];
    switch (n.op) {
    case T3_OP_LAMBERT: case T3_OP_PHONG: case T3_OP_COOK:
      return sval<R>(R(1));
    case T3_OP_EMISSION:
      return sval<R>(R(0));
    case T3_OP_MIX: {
      Val<R> fac = value(n.c);
      return vadd(vmul(one_minus(fac), ambient(n.a)), vmul(fac, ambient(n.b)));
    }
    case T3_OP_SCALE:
      return vmul(value(n.b), ambient(n.a));
    case T3_OP_ADD:
      return vadd(ambient(n.a), ambient(n.b));
    default:
      return sval<R>(R(0));
    }
  }

  Val<R> emission(int i) const {
    const t3_node& n = m->nodes[i];
    switch (n.op) {
    case T3_OP_EMISSION:
      return sval<R>(R(1));
    case T3_OP_MIX: {
      Val<R> fac = value(n.c);
      return vadd(vmul(one_minus(fac), emission(n.a)), vmul(fac, emission(n.b)));
    }
    case T3_OP_SCALE:
      return vmul(value(n.b), emission(n.a));
    case T3_OP_ADD:
      return vadd(emission(n.a), emission(n.b));
    default:
      return sval<R>(R(0));
    }
  }
};

// ACES (tina/advans.py:32-34)
template <class R> inline R aces1(R c) {
  return (c * (cst<R>(2.51) * c + cst<R>(0.03))) / (c * (cst<R>(2.43) * c + cst<R>(0.59)) + cst<R>(0.14));
}

// ---------------------------------------------------------------------------
// Image-based lighting (SkyboxLighting, tina/core/lighting.py:5-21) by the
// materials' own importance samplers (material.py sample(): Lambert :399-405,
// CookTorrance :365-384, Phong :460-472, Mix :124-138, Scale :180-184), with
// the sky-ray estimate of path/engine.py:243-266: emission + mean of
// weight * env(dir).  The material tree is flattened into weighted lobes
// (the product of Mix / Scale factors along the path); a lobe is drawn with
// probability equal to the product of its Mix choices (smoothlerp(avg f, .12,
// .88) or its complement), normalised over the lobes, and weighted by
// lobe weight / probability.  Random numbers: pcg_hash (Jarzynski & Olano,
// JCGT 2020) of (seed, pixel, sample, draw).
// ---------------------------------------------------------------------------
inline uint32_t pcg_hash(uint32_t v) {
  const uint32_t state = v * 747796405u + 2891336453u;
  const uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
  return (word >> 22u) ^ word;
}
inline uint32_t rng_base(uint32_t seed, uint32_t pixel) { return pcg_hash(seed ^ pcg_hash(pixel)); }
inline float rng_draw(uint32_t base, uint32_t sample, uint32_t draw) {
  return (float)(pcg_hash(base ^ ((sample * 3u + draw) * 0x9E3779B9u)) >> 8) * 5.9604644775390625e-08f;
}

// IEEE binary16 -> float
inline float half_to_float(uint16_t h) {
  const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  uint32_t exp = (h >> 10) & 0x1Fu, man = h & 0x3FFu, bits;
  if (exp == 0) {
    if (man == 0) {
      bits = sign;
    } else {  // subnormal: renormalise
      int e = -1;
      do { e++; man <<= 1; } while (!(man & 0x400u));
      bits = sign | ((uint32_t)(127 - 15 - e) << 23) | ((man & 0x3FFu) << 13);
    }
  } else if (exp == 31) {
    bits = sign | 0x7F800000u | (man << 13);
  } else {
    bits = sign | ((exp + 127 - 15) << 23) | (man << 13);
  }
  float f;
  std::memcpy(&f, &bits, 4);
  return f;
}

template <class R> struct EnvMap {
  const t3_lighting* lt;
  v3<R> texel(int64_t i, int64_t j) const {
    i = i < 0 ? 0 : i >= lt->env_w ? lt->env_w - 1 : i;
    j = j < 0 ? 0 : j >= lt->env_h ? lt->env_h - 1 : j;
    const int64_t o = (i * lt->env_h + j) * 3;
    if (lt->env_half) {
      const uint16_t* t = reinterpret_cast<const uint16_t*>(lt->env) + o;
      return {(R)half_to_float(t[0]), (R)half_to_float(t[1]), (R)half_to_float(t[2])};
    }
    const float* t = reinterpret_cast<const float*>(lt->env) + o;
    return {(R)t[0], (R)t[1], (R)t[2]};
  }
  // Skybox.sample: spheremap (tina/skybox.py:23-28) + bilerp (tina/common.py:140-149),
  // the +1 texel clamped to the map
  v3<R> sample(v3<R> dir) const {
    const R u = dir.y;
    R p = std::atan2(-dir.z, dir.x) / R(2.0 * M_PI);
    p = p - std::floor(p);
    const R cx = p * (R)(lt->env_w - 1), cy = (u * R(0.5) + R(0.5)) * (R)(lt->env_h - 1);
    const R fx = std::floor(cx), fy = std::floor(cy);
    const int64_t ix = (int64_t)fx, iy = (int64_t)fy;
    const R x1 = cx - fx, y1 = cy - fy, x0 = R(1) - x1, y0 = R(1) - y1;
    v3<R> r = add(add(muls(x1 * y1, texel(ix + 1, iy + 1)), muls(x1 * y0, texel(ix + 1, iy))),
                  add(muls(x0 * y0, texel(ix, iy)), muls(x0 * y1, texel(ix, iy + 1))));
    return r;
  }
};

// tangentspace(nrm) @ spherical(h, p)  (tina/advans.py:97-108)
template <class R> inline v3<R> tangent_dir(v3<R> n, R h, R p) {
  const v3<R> bitan = normalized(cross(n, v3<R>{R(233), R(666), R(512)}));
  const v3<R> tan = cross(bitan, n);
  const R r = std::sqrt(std::max(R(0), R(1) - h * h));
  const R a = R(2.0 * M_PI) * p;
  return add(add(muls(r * std::cos(a), tan), muls(r * std::sin(a), bitan)), muls(h, n));
}

template <class R> inline R mix_prob(R fac) {
  if (fac != R(0) && fac != R(1)) {
    const R t = std::min(R(1), std::max(R(0), fac));
    const R s = t * t * (R(3) - R(2) * t);
    return R(0.12) * (R(1) - s) + R(0.88) * s;
  }
  return fac;
}

struct FlatLobe {
  int leaf;
  int nfac;
  int fac[8];     // node index
  bool onem[8];
  bool mix[8];
};

inline void flatten(const t3_material& m, int node, FlatLobe cur, std::vector<FlatLobe>& out) {
  const t3_node& nd = m.nodes[node];
  if (nd.op == T3_OP_LAMBERT || nd.op == T3_OP_PHONG || nd.op == T3_OP_COOK || nd.op == T3_OP_EMISSION) {
    cur.leaf = node;
    out.push_back(cur);
    return;
  }
  if (nd.op == T3_OP_MIX) {
    FlatLobe a = cur, b = cur;
    a.fac[a.nfac] = nd.c; a.onem[a.nfac] = true; a.mix[a.nfac] = true; a.nfac++;
    b.fac[b.nfac] = nd.c; b.onem[b.nfac] = false; b.mix[b.nfac] = true; b.nfac++;
    flatten(m, nd.a, a, out);
    flatten(m, nd.b, b, out);
  } else if (nd.op == T3_OP_SCALE) {
    cur.fac[cur.nfac] = nd.b; cur.onem[cur.nfac] = false; cur.mix[cur.nfac] = false; cur.nfac++;
    flatten(m, nd.a, cur, out);
  } else if (nd.op == T3_OP_ADD) {
    flatten(m, nd.a, cur, out);
    flatten(m, nd.b, cur, out);
  }
}

// One draw of a leaf material's sampler (tina/matr/material.py sample()) from
// the uniforms (xu, xv): the direction and the weight the estimator applies.
//   Lambert (:399-405): u = sqrt(xu) about the normal, weight 1.
//   CookTorrance (:365-384): u = sqrt((1 - xu) / (1 - xu (1 - a2))) about
//     reflect(-V, n), weight F * G of sub_brdf(n, V, dir); mirrored with F = 0
//     below the surface.  r2 = roughness**2.
//   Phong (:459-472): u = xu^(1 / (m + 1)) about reflect(-V, n), weight 1 (0
//     mirrored below the surface).  r2 = shineness.
template <class R>
v3<R> sample_leaf(int op, R r2, v3<R> f0, v3<R> viewdir, v3<R> normal, R xu, R xv, v3<R>& dir) {
  if (op == T3_OP_LAMBERT) {
    dir = normalized(tangent_dir(normal, std::sqrt(xu), xv));
    return {R(1), R(1), R(1)};
  }
  if (op == T3_OP_COOK) {
    const R a2s = std::max(R(0), r2);
    const R u = std::sqrt((R(1) - xu) / (R(1) - xu * (R(1) - a2s)));
    const v3<R> rdir = reflect(neg(viewdir), normal);
    v3<R> o = tangent_dir(rdir, u, xv);
    const R a2 = std::max(MaterialEval<R>::c_eps6(), r2);
    const v3<R> half = normalized(add(viewdir, o));
    const R NoL = std::max(MaterialEval<R>::c_eps(), dot(viewdir, normal));
    const R NoV = std::max(MaterialEval<R>::c_eps(), dot(o, normal));
    const R VoH = std::min(MaterialEval<R>::c_eps_big(), std::max(MaterialEval<R>::c_eps(), dot(half, o)));
    const R kk = a2 / R(2);
    R vdf = R(1) / ((NoV * kk + R(1)) - kk);
    vdf = vdf * (R(1) / ((NoL * kk + R(1)) - kk));
    vdf = vdf / (R(1) * (R(1) - a2) + MaterialEval<R>::c_4pi() * a2);
    const R p5 = pow5(R(1) - VoH);
    v3<R> fdf = {f0.x + (R(1) - f0.x) * p5, f0.y + (R(1) - f0.y) * p5, f0.z + (R(1) - f0.z) * p5};
    if (dot(o, normal) < R(0)) { o = neg(o); fdf = {R(0), R(0), R(0)}; }
    dir = o;
    return muls(vdf, fdf);
  }
  if (op == T3_OP_PHONG) {
    const R m = r2;
    const R u = std::pow(xu, R(1) / (m + R(2) - R(1)));
    const v3<R> rdir = reflect(neg(viewdir), normal);
    v3<R> o = tangent_dir(rdir, u, xv);
    R wt = 1;
    if (dot(o, normal) < R(0)) { o = neg(o); wt = 0; }
    dir = o;
    return {wt, wt, wt};
  }
  dir = normal;
  return {R(0), R(0), R(0)};
}

template <class R>
v3<R> shade_ibl_mc(const t3_lighting& L, const MaterialEval<R>& me, v3<R> normal, v3<R> viewdir,
                   uint32_t pixel, int spp, uint32_t seed) {
  std::vector<FlatLobe> lobes;
  FlatLobe root{};
  flatten(*me.m, me.m->root, root, lobes);
  const int nl = (int)lobes.size();
  std::vector<v3<R>> W(nl), f0(nl);
  std::vector<R> prob(nl), cdf(nl), r2(nl);
  v3<R> emission = {R(0), R(0), R(0)};
  R c = 0;
  for (int k = 0; k < nl; k++) {
    v3<R> w = {R(1), R(1), R(1)};
    R pr = 1;
    for (int j = 0; j < lobes[k].nfac; j++) {
      v3<R> f = me.value(lobes[k].fac[j]).v;
      if (lobes[k].onem[j]) f = {R(1) - f.x, R(1) - f.y, R(1) - f.z};
      w = mul(w, f);
      if (lobes[k].mix[j]) {
        v3<R> g = me.value(lobes[k].fac[j]).v;
        const R q = mix_prob((g.x + g.y + g.z) * (R(1) / R(3)));
        pr *= lobes[k].onem[j] ? R(1) - q : q;
      }
    }
    const t3_node& leaf = me.m->nodes[lobes[k].leaf];
    if (leaf.op == T3_OP_EMISSION) { emission = add(emission, w); pr = 0; }
    W[k] = pr > 0 ? muls(R(1) / pr, w) : v3<R>{R(0), R(0), R(0)};
    if (leaf.op == T3_OP_COOK) {
      const R r = me.value(leaf.a).v.x;
      r2[k] = r * r;
      f0[k] = me.value(leaf.b).v;
    } else if (leaf.op == T3_OP_PHONG) {
      r2[k] = me.value(leaf.a).v.x;
    }
    c += pr;
    cdf[k] = c;
  }
  for (int k = 0; k < nl; k++) W[k] = muls(c, W[k]);
  v3<R> acc = {R(0), R(0), R(0)};
  if (c > 0) {
    EnvMap<R> env{&L};
    const uint32_t base = rng_base(seed, pixel);
    for (int s = 0; s < spp; s++) {
      const R xs = (R)rng_draw(base, (uint32_t)s, 0u) * c;
      const R xu = (R)rng_draw(base, (uint32_t)s, 1u), xv = (R)rng_draw(base, (uint32_t)s, 2u);
      int k = 0;
      for (int j = 0; j < nl - 1; j++)
        if (xs >= cdf[j]) k = j + 1;
      const t3_node& leaf = me.m->nodes[lobes[k].leaf];
      if (leaf.op != T3_OP_LAMBERT && leaf.op != T3_OP_COOK && leaf.op != T3_OP_PHONG) continue;
      v3<R> dir;
      const v3<R> lw = sample_leaf<R>(leaf.op, r2[k], f0[k], viewdir, normal, xu, xv, dir);
      const v3<R> w = mul(W[k], lw);
      if (w.x != R(0) || w.y != R(0) || w.z != R(0)) acc = add(acc, mul(w, env.sample(dir)));
    }
    acc = muls(R(1) / (R)spp, acc);
  }
  return add(emission, acc);
}

// ---------------------------------------------------------------------------
// SkyboxLighting's own lookup of prefiltered maps (tina/core/lighting.py:20-21):
// material.sample_ibl(tab, viewdir, normal) + material.emission().
// ---------------------------------------------------------------------------

// An equirect map of the prefiltered tables, sampled like Skybox.sample.
template <class R> struct MapView {
  const void* data;
  int w, h, half;
  v3<R> texel(int64_t i, int64_t j) const {
    i = i < 0 ? 0 : i >= w ? w - 1 : i;
    j = j < 0 ? 0 : j >= h ? h - 1 : j;
    const int64_t o = (i * h + j) * 3;
    if (half) {
      const uint16_t* t = reinterpret_cast<const uint16_t*>(data) + o;
      return {(R)half_to_float(t[0]), (R)half_to_float(t[1]), (R)half_to_float(t[2])};
    }
    const float* t = reinterpret_cast<const float*>(data) + o;
    return {(R)t[0], (R)t[1], (R)t[2]};
  }
  v3<R> sample(v3<R> dir) const {
    const R u = dir.y;
    R p = std::atan2(-dir.z, dir.x) / R(2.0 * M_PI);
    p = p - std::floor(p);
    const R cx = p * (R)(w - 1), cy = (u * R(0.5) + R(0.5)) * (R)(h - 1);
    const R fx = std::floor(cx), fy = std::floor(cy);
    const int64_t ix = (int64_t)fx, iy = (int64_t)fy;
    const R x1 = cx - fx, y1 = cy - fy, x0 = R(1) - x1, y0 = R(1) - y1;
    return add(add(muls(x1 * y1, texel(ix + 1, iy + 1)), muls(x1 * y0, texel(ix + 1, iy))),
               add(muls(x0 * y0, texel(ix, iy)), muls(x0 * y1, texel(ix, iy + 1))));
  }
};
template <class R> inline MapView<R> map_view(const t3_ibl_map& m) { return {m.data, m.w, m.h, m.half}; }

// bilerp(lut, (VoH, roughness)) of tina/common.py:141-150 at the point in
// texel units (the reference does not scale it to the table); A, B = the
// table's first two channels, +1 texels clamped to the table
template <class R> inline void lut_ab(const t3_ibl_tables& T, R px, R py, R& A, R& B) {
  const R Ix = std::floor(px), Iy = std::floor(py);
  const R x0 = px - Ix, x1 = py - Iy, y0 = R(1) - x0, y1 = R(1) - x1;
  auto at = [&](int64_t i, int64_t j, int c) {
    i = i < 0 ? 0 : i >= T.lut_w ? T.lut_w - 1 : i;
    j = j < 0 ? 0 : j >= T.lut_h ? T.lut_h - 1 : j;
    return (R)T.lut[(i * T.lut_h + j) * 2 + c];
  };
  const int64_t ix = (int64_t)Ix, iy = (int64_t)Iy;
  for (int c = 0; c < 2; c++) {
    R r = (at(ix + 1, iy + 1, c) * x0) * x1;
    r = r + (at(ix + 1, iy, c) * x0) * y1;
    r = r + (at(ix, iy, c) * y0) * y1;
    r = r + (at(ix, iy + 1, c) * y0) * x1;
    (c ? B : A) = r;
  }
}

// CookTorrance.rough_levels (tina/matr/material.py:251-253): pairs (a, a - b)
// of consecutive levels, evaluated in double (Python) and used as float
// constants in the kernel
inline void rough_level(int id, double& rough, double& step) {
  static const double lv[6] = {0.03, 0.08, 0.18, 0.35, 0.65, 1.0};
  rough = lv[id];
  step = lv[id] - (id ? lv[id - 1] : 0.0);
}

// CookTorrance.sample_ibl (tina/matr/material.py:256-277)
template <class R>
v3<R> cook_sample_ibl(const t3_ibl_tables& T, R roughness, v3<R> f0, v3<R> idir, v3<R> nrm) {
  const v3<R> rdir = reflect(neg(idir), nrm);
  v3<R> wei = {R(1), R(1), R(1)};
  for (int id = 0; id < 6; id++) {
    double rough_d, step_d;
    rough_level(id, rough_d, step_d);
    const R lo = cst<R>(rough_d - step_d), rough = cst<R>(rough_d), step = cst<R>(step_d);
    if (lo <= roughness && roughness <= rough) {
      const v3<R> w1 = map_view<R>(T.spec[id]).sample(rdir);
      const v3<R> w2 = map_view<R>(T.spec[id + 1]).sample(rdir);
      const R fac2 = (rough - roughness) / step;
      wei = add(muls(R(1) - fac2, w2), muls(fac2, w1));  // lerp(fac2, wei2, wei1)
    }
  }
  const v3<R> half = normalized(add(idir, rdir));
  const R VoH = fmin_(MaterialEval<R>::c_eps_big(), fmax_(MaterialEval<R>::c_eps(), dot(half, rdir)));
  R A, B;
  lut_ab<R>(T, VoH, roughness, A, B);
  return {wei.x * (f0.x * A + B), wei.y * (f0.y * A + B), wei.z * (f0.z * A + B)};
}

// material.sample_ibl over the material tree: Lambert (:441-442), CookTorrance,
// Mix (:141-145), Scale (:187-191); Add sums its children and Emission gives 0
// (the reference has neither; Phong has no lookup there and is refused)
template <class R>
v3<R> sample_ibl(const MaterialEval<R>& me, const t3_ibl_tables& T, int i, v3<R> idir, v3<R> nrm) {
  const t3_node& n = me.m->nodes[i];
  switch (n.op) {
  case T3_OP_LAMBERT:
    return map_view<R>(T.diffuse).sample(nrm);
  case T3_OP_COOK:
    return cook_sample_ibl<R>(T, me.value(n.a).v.x, me.value(n.b).v, idir, nrm);
  case T3_OP_MIX: {
    const v3<R> fac = me.value(n.c).v;
    const v3<R> w1 = sample_ibl(me, T, n.a, idir, nrm), w2 = sample_ibl(me, T, n.b, idir, nrm);
    return add(mul(v3<R>{R(1) - fac.x, R(1) - fac.y, R(1) - fac.z}, w1), mul(fac, w2));
  }
  case T3_OP_SCALE:
    return mul(me.value(n.b).v, sample_ibl(me, T, n.a, idir, nrm));
  case T3_OP_ADD:
    return add(sample_ibl(me, T, n.a, idir, nrm), sample_ibl(me, T, n.b, idir, nrm));
  default:
    return {R(0), R(0), R(0)};
  }
}

// Lighting.shade_color (tina/core/lighting.py:84-98)
template <class R>
v3<R> shade_lamps(const t3_lighting& L, const MaterialEval<R>& me, v3<R> pos, v3<R> normal,
                  v3<R> viewdir) {
  v3<R> res = {R(0), R(0), R(0)};
  int root = me.m->root;
  res = add(res, me.emission(root).v);
  v3<R> amb = {(R)L.ambient[0], (R)L.ambient[1], (R)L.ambient[2]};
  res = add(res, mul(amb, me.ambient(root).v));
  for (int l = 0; l < L.nlights; l++) {
    const t3_light& lt = L.lights[l];
    v3<R> lxyz = {(R)lt.dir[0], (R)lt.dir[1], (R)lt.dir[2]};
    R lw = (R)lt.dir[3];
    v3<R> lcolor = {(R)lt.color[0], (R)lt.color[1], (R)lt.color[2]};
    v3<R> light_dir = sub(lxyz, mulv(pos, lw));
    R dist = norm(light_dir);
    light_dir = divs(light_dir, dist);
    R cos_i = dot(normal, light_dir);
    if (cos_i > R(0)) {
      lcolor = divs(lcolor, pow2(dist));
      v3<R> mcolor = me.brdf(root, normal, light_dir, viewdir).v;
      res = add(res, mul(muls(cos_i, lcolor), mcolor));
    }
  }
  return res;
}

template <class R> struct Ctx {
  const t3_scene* sc;
  mat4<R> W2V, V2W;
  int spp = 0;        // > 0: IBL sample count / seed override (ground-truth runs)
  uint32_t seed = 0;
};

// render_color for one pixel of one object (triangle.py:134-153 -> shader.py:119-131)
// ---------------------------------------------------------------------------
// Particles (tina/core/particle.py, SimpleParticles tina/pars/simple.py):
// verts = positions, coors = radii, norms = colours (nullable).
// ---------------------------------------------------------------------------
template <class R> inline v3<R> mapply_dir(const mat4<R>& M, v3<R> d) {
  v3<R> r;
  R w;
  mapply(M, d, R(0), r, w);
  return r;
}

template <class R> struct ParS {
  v3<R> A;
  R Rl, r2, vz;
  int32_t depth;
  int32_t botx, boty, topx, topy;
};

// render_occup's per-particle part (particle.py:77-101); false when clipped or empty
template <class R> bool particle_setup(const Ctx<R>& cx, const t3_mesh& m, int64_t n, ParS<R>& p) {
  const t3_frame& fr = cx.sc->frame;
  p.A = ld3<R>(m.verts + n * 3);
  p.Rl = (R)m.coors[n];
  const v3<R> Av = mapply_pos(cx.W2V, p.A);
  if ((fr.flags & T3_CLIPPING) && !(R(-1) <= Av.z && Av.z <= R(1))) return false;
  const v3<R> DX = normalized(mapply_dir(cx.V2W, v3<R>{R(1), R(0), R(0)}));
  const v3<R> DY = normalized(mapply_dir(cx.V2W, v3<R>{R(0), R(1), R(0)}));
  const R rx = mapply_pos(cx.W2V, add(p.A, mulv(DX, p.Rl))).x - Av.x;
  const R ry = mapply_pos(cx.W2V, add(p.A, mulv(DY, p.Rl))).y - Av.y;
  const v2<R> b0 = to_viewport(v3<R>{Av.x - rx, Av.y - R(0), Av.z}, fr.width, fr.height);
  const v2<R> b1 = to_viewport(v3<R>{Av.x + rx, Av.y + R(0), Av.z}, fr.width, fr.height);
  const v2<R> b2 = to_viewport(v3<R>{Av.x - R(0), Av.y - ry, Av.z}, fr.width, fr.height);
  const v2<R> b3 = to_viewport(v3<R>{Av.x + R(0), Av.y + ry, Av.z}, fr.width, fr.height);
  const int32_t lox = trunc_i32(std::floor(fmin_(b0.x, b2.x))), loy = trunc_i32(std::floor(fmin_(b0.y, b2.y)));
  const int32_t hix = trunc_i32(std::ceil(fmax_(b1.x, b3.x))), hiy = trunc_i32(std::ceil(fmax_(b1.y, b3.y)));
  p.botx = lox > 0 ? lox : 0;
  p.boty = loy > 0 ? loy : 0;
  p.topx = hix < fr.width - 1 ? hix : fr.width - 1;
  p.topy = hiy < fr.height - 1 ? hiy : fr.height - 1;
  p.r2 = p.Rl * p.Rl;
  p.vz = Av.z;
  p.depth = trunc_i32(Av.z * (R)fr.maxdepth);
  return p.botx <= p.topx && p.boty <= p.topy;
}

// Pl = mapply_pos(V2W, (from_viewport(P + bias), Av.z)) (particle.py:103-105)
template <class R> v3<R> particle_pixel_world(const Ctx<R>& cx, const ParS<R>& p, int32_t x, int32_t y) {
  const t3_frame& fr = cx.sc->frame;
  const R px = (R)x + (R)fr.bias[0], py = (R)y + (R)fr.bias[1];
  const v3<R> Pv = {(px / (R)fr.width) * R(2) - R(1), (py / (R)fr.height) * R(2) - R(1), p.vz};
  return mapply_pos(cx.V2W, Pv);
}

template <class R> bool particle_covers(const ParS<R>& p, v3<R> Pl) {
  const v3<R> d = sub(Pl, p.A);
  return !(((d.x * d.x + d.y * d.y) + d.z * d.z) > p.r2);
}

// render_color's particle geometry (particle.py:118-146): normal and position
template <class R> void particle_frag(const Ctx<R>& cx, const t3_mesh& m, int64_t n, int32_t x, int32_t y,
                                      v3<R>& pos, v3<R>& normal, v3<R>& color, R& depth_f) {
  ParS<R> p;
  p.A = ld3<R>(m.verts + n * 3);
  p.Rl = (R)m.coors[n];
  p.vz = mapply_pos(cx.W2V, p.A).z;
  depth_f = p.vz;
  const v3<R> Pl = particle_pixel_world(cx, p, x, y);
  v3<R> D = divs(sub(Pl, p.A), p.Rl);
  const v3<R> Z = normalized(mapply_dir(cx.V2W, v3<R>{R(0), R(0), R(1)}));
  D = sub(D, mulv(Z, std::sqrt(R(1) - dot(D, D))));
  D = normalized(D);
  normal = D;
  pos = add(p.A, mulv(D, p.Rl));
  color = m.norms ? ld3<R>(m.norms + n * 3) : v3<R>{R(1), R(1), R(1)};
}

// ---------------------------------------------------------------------------
// Wireframe (tina/core/wireframe.py; lines of SimpleMesh(npolygon=2),
// tina/mesh/simple.py, or MeshToWire, tina/mesh/wire.py).
// ---------------------------------------------------------------------------
inline bool is_wire(const t3_mesh& m) { return m.kind == T3_MESH_LINES || (m.flags & T3_MESH_WIREFRAME) != 0; }
inline bool is_point_or_line(const t3_mesh& m) { return m.kind == T3_MESH_PARTICLES || is_wire(m); }

// world endpoints of line n: MeshToWire._get_face_props (wire.py:20-27) takes
// corners n % p and (n + 1) % p of face n // p
template <class R> void wire_endpoints(const t3_mesh& m, int64_t n, v3<R>& A, v3<R>& B) {
  if (m.kind == T3_MESH_LINES) {
    const int p = (m.flags & T3_MESH_WIREFRAME) ? 2 : 1;
    const int64_t l = n / p;
    const int e = (int)(n % p);
    v3<R> c[2] = {ld3<R>(m.verts + l * 6), ld3<R>(m.verts + l * 6 + 3)};
    if (m.flags & T3_MESH_TRANSFORM) {
      mat4<R> T;
      for (int i = 0; i < 16; i++) T.m[i] = (R)m.trans[i];
      c[0] = mapply_pos(T, c[0]);
      c[1] = mapply_pos(T, c[1]);
    }
    A = c[e];
    B = c[(e + 1) % 2];
    return;
  }
  if (m.flags & T3_MESH_QUADS) {
    // MeshGrid(as_quad=True) (grid.py:46-58): _get_face_props returns the
    // cell's (a, b, c, d) = ((i,j), (i+1,j), (i+1,j+1), (i,j+1))
    const int64_t f = n / 4, stride = m.grid_ny - 1;
    const int64_t i = f / stride, j = f % stride;
    const int64_t ii[4] = {i, i + 1, i + 1, i}, jj[4] = {j, j, j + 1, j + 1};
    v3<R> c[4];
    for (int k = 0; k < 4; k++) {
      c[k] = ld3<R>(m.verts + (ii[k] * m.grid_ny + jj[k]) * 3);
      if (m.flags & T3_MESH_TRANSFORM) {
        mat4<R> T;
        for (int q = 0; q < 16; q++) T.m[q] = (R)m.trans[q];
        c[k] = mapply_pos(T, c[k]);
      }
    }
    A = c[n % 4];
    B = c[(n + 1) % 4];
    return;
  }
  Mesh<R> mesh(&m);
  v3<R> v[3];
  mesh.verts(n / 3, v);
  A = v[n % 3];
  B = v[(n % 3 + 1) % 3];
}

template <class R> struct WireS {
  v2<R> a, k;     // viewport start, step (draw_line, wireframe.py:49-64)
  R az, bz;       // NDC depths of the endpoints
  R wsa, wsb;     // wscale = 1 / clip w
  int32_t siz;
};

// render_color's per-line part (wireframe.py:72-83); false when clipped or
// when range(siz + 1) is empty in int32 (siz < 0, or siz + 1 overflowing)
template <class R> bool wire_setup(const Ctx<R>& cx, v3<R> A, v3<R> B, WireS<R>& s) {
  const t3_frame& fr = cx.sc->frame;
  v3<R> ra, rb;
  R wa, wb;
  mapply(cx.W2V, A, R(1), ra, wa);
  mapply(cx.W2V, B, R(1), rb, wb);
  const v3<R> Av = divs(ra, wa), Bv = divs(rb, wb);
  if ((fr.flags & T3_WIRE_CLIPPING) && !inside_clip(Av) && !inside_clip(Bv)) return false;
  s.a = to_viewport(Av, fr.width, fr.height);
  const v2<R> b = to_viewport(Bv, fr.width, fr.height);
  s.az = Av.z;
  s.bz = Bv.z;
  s.wsa = R(1) / wa;
  s.wsb = R(1) / wb;
  const v2<R> d = {b.x - s.a.x, b.y - s.a.y};
  if (std::fabs(d.x) >= std::fabs(d.y)) {
    s.k.x = d.x >= R(0) ? R(1) : R(-1);
    s.k.y = s.k.x * d.y / d.x;
    s.siz = trunc_i32(std::fabs(d.x));
  } else {
    s.k.y = d.y >= R(0) ? R(1) : R(-1);
    s.k.x = s.k.y * d.x / d.y;
    s.siz = trunc_i32(std::fabs(d.y));
  }
  return s.siz >= 0 && s.siz != INT32_MAX;
}

// step i (wireframe.py:84-92): pixel and int depth; false outside the frame
template <class R> bool wire_step(const t3_frame& fr, const WireS<R>& s, int32_t i, int32_t& x, int32_t& y,
                                  int32_t& depth) {
  const R fi = (R)i;
  x = trunc_i32(std::floor((s.a.x + s.k.x * fi) + (R)fr.bias[0]));
  y = trunc_i32(std::floor((s.a.y + s.k.y * fi) + (R)fr.bias[1]));
  if (!(0 <= x && x < fr.width && 0 <= y && y < fr.height)) return false;
  const R cor = fi / (R)s.siz;
  R w0 = (R(1) - cor) * s.wsa, w1 = cor * s.wsb;
  const R sum = w0 + w1;
  w0 = w0 / sum;
  w1 = w1 / sum;
  depth = trunc_i32((w0 * s.az + w1 * s.bz) * (R)fr.maxdepth);
  return true;
}

template <class R>
v3<R> shade_pixel(const Ctx<R>& cx, const t3_object& ob, const Mesh<R>& mesh, int64_t f,
                  int32_t x, int32_t y, R* depth_f_out) {
  const t3_frame& fr = cx.sc->frame;
  // Shader.blend_color(..., factor=1, linecolor) (wireframe.py:93-97, shader.py:133-135)
  if (is_wire(ob.mesh)) return {(R)fr.linecolor[0], (R)fr.linecolor[1], (R)fr.linecolor[2]};
  v3<R> pos, normal, tex = {R(0), R(0), R(0)}, color = {R(1), R(1), R(1)};
  if (ob.mesh.kind == T3_MESH_PARTICLES) {
    R df;
    particle_frag(cx, ob.mesh, f, x, y, pos, normal, color, df);
    if (depth_f_out) *depth_f_out = df;
  } else {
  v3<R> v[3];
  mesh.verts(f, v);
  Setup<R> s;
  face_setup(cx.W2V, fr, v, s);
  v3<R> wei = face_weights(s, fr, x, y);
  if (depth_f_out) *depth_f_out = face_depth(s, wei);
  // interpolate (triangle.py:32-49)
  pos = add(add(muls(wei.x, v[0]), muls(wei.y, v[1])), muls(wei.z, v[2]));
  if (fr.flags & T3_SMOOTHING) {
    v3<R> n[3];
    mesh.norms(f, n);
    normal = add(add(muls(wei.x, n[0]), muls(wei.y, n[1])), muls(wei.z, n[2]));
  } else {
    normal = cross(sub(v[1], v[0]), sub(v[2], v[0]));
  }
  normal = normalized(normal);
  if (fr.flags & T3_TEXTURING) {
    v3<R> t[3];
    mesh.coors(f, t);
    tex = add(add(muls(wei.x, t[0]), muls(wei.y, t[1])), muls(wei.z, t[2]));
    tex.z = R(0);
  }
  }
  // calc_viewdir (shader.py:82-93)
  R px = (R)x + (R)fr.bias[0], py = (R)y + (R)fr.bias[1];
  R ux = (px / (R)fr.width) * R(2) - R(1);
  R uy = (py / (R)fr.height) * R(2) - R(1);
  v3<R> ro = mapply_pos(cx.V2W, v3<R>{ux, uy, R(-1)});
  v3<R> ro1 = mapply_pos(cx.V2W, v3<R>{ux, uy, R(1)});
  v3<R> rd = normalized(sub(ro1, ro));
  v3<R> viewdir = neg(rd);

  Frag<R> fg;
  fg.pos = pos; fg.normal = normal; fg.texcoord = tex; fg.color = color;
  int64_t bf = ob.mesh.kind == T3_MESH_PARTICLES ? f : mesh.base_face(f);
  fg.attr = ob.mesh.face_attr ? ob.mesh.face_attr + bf * ob.mesh.attr_stride : nullptr;
  MaterialEval<R> me{&ob.material, &fg};
  const t3_lighting& L = cx.sc->lighting;
  // T3_LIGHT_IBL_MLP: the Monte Carlo estimator the network stands in for
  if (L.mode == T3_LIGHT_IBL_MC || L.mode == T3_LIGHT_IBL_MLP) {
    const uint32_t pixel = (uint32_t)((int64_t)x * fr.height + y);
    const int spp = cx.spp > 0 ? cx.spp : L.spp;
    const uint32_t seed = cx.spp > 0 ? cx.seed : L.seed;
    v3<R> c = shade_ibl_mc(L, me, normal, viewdir, pixel, spp, seed);
    if (L.nlights > 0) {
      t3_lighting lamps = L;
      lamps.ambient[0] = lamps.ambient[1] = lamps.ambient[2] = 0.0f;
      v3<R> l = shade_lamps(lamps, me, pos, normal, viewdir);
      c = add(c, sub(l, me.emission(me.m->root).v));  // lamps without a second emission
    }
    return c;
  }
  if (L.mode == T3_LIGHT_IBL_PREFILTERED && L.tables) {
    // SkyboxLighting.shade_color: sample_ibl(tab, viewdir, normal) + emission
    v3<R> c = add(sample_ibl(me, *L.tables, me.m->root, viewdir, normal), me.emission(me.m->root).v);
    if (L.nlights > 0) {
      t3_lighting lamps = L;
      lamps.ambient[0] = lamps.ambient[1] = lamps.ambient[2] = 0.0f;
      v3<R> l = shade_lamps(lamps, me, pos, normal, viewdir);
      c = add(c, sub(l, me.emission(me.m->root).v));
    }
    return c;
  }
  return shade_lamps(L, me, pos, normal, viewdir);
}

// Engine.render_background (tina/core/engine.py:42-49): the sky along the view ray
template <class R> v3<R> background_pixel(const Ctx<R>& cx, int32_t x, int32_t y) {
  const t3_frame& fr = cx.sc->frame;
  R px = (R)x + (R)fr.bias[0], py = (R)y + (R)fr.bias[1];
  R ux = (px / (R)fr.width) * R(2) - R(1);
  R uy = (py / (R)fr.height) * R(2) - R(1);
  v3<R> ro = mapply_pos(cx.V2W, v3<R>{ux, uy, R(-1)});
  v3<R> ro1 = mapply_pos(cx.V2W, v3<R>{ux, uy, R(1)});
  v3<R> rd = normalized(sub(ro1, ro));
  return EnvMap<R>{&cx.sc->lighting}.sample(rd);
}

inline uint64_t pack_key(int32_t depth, uint32_t id) {
  return ((uint64_t)((uint32_t)depth ^ 0x80000000u) << 32) | (uint64_t)id;
}

template <class R>
inline void raster_face(const Ctx<R>& cx, const Setup<R>& s, uint64_t id,
                        std::atomic<uint64_t>* keys) {
  const t3_frame& fr = cx.sc->frame;
  const int H = fr.height;
  for (int32_t x = s.botx; x <= s.topx; x++) {
    for (int32_t y = s.boty; y <= s.topy; y++) {
      v3<R> wei = face_weights(s, fr, x, y);
      if (wei.x >= R(0) && wei.y >= R(0) && wei.z >= R(0)) {
        R depth_f = face_depth(s, wei);
        int32_t d = trunc_i32(depth_f * (R)fr.maxdepth);
        if (d >= fr.maxdepth) continue; // can never pass `old > depth`
        uint64_t key = pack_key(d, (uint32_t)id);
        int64_t P_ = (int64_t)x * H + y;
        uint64_t cur = keys[P_].load(std::memory_order_relaxed);
        while (key < cur && !keys[P_].compare_exchange_weak(cur, key)) {
        }
      }
    }
  }
}

// one object into the packed (depth, global id) minimum, in parallel
template <class R>
void raster_object_keys(const Ctx<R>& cx, const t3_object& ob, std::atomic<uint64_t>* keys) {
  const t3_frame& fr = cx.sc->frame;
  const int H = fr.height;
  if (ob.mesh.kind == T3_MESH_PARTICLES) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t f = 0; f < ob.nfaces; f++) {
      ParS<R> p;
      if (!particle_setup(cx, ob.mesh, f, p) || p.depth >= fr.maxdepth) continue;
      const uint64_t key = pack_key(p.depth, (uint32_t)(ob.face_base + f));
      for (int32_t x = p.botx; x <= p.topx; x++)
        for (int32_t y = p.boty; y <= p.topy; y++) {
          if (!particle_covers(p, particle_pixel_world(cx, p, x, y))) continue;
          const int64_t P_ = (int64_t)x * H + y;
          uint64_t cur = keys[P_].load(std::memory_order_relaxed);
          while (key < cur && !keys[P_].compare_exchange_weak(cur, key)) {
          }
        }
    }
    return;
  }
  if (is_wire(ob.mesh)) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t f = 0; f < ob.nfaces; f++) {
      v3<R> A, B;
      wire_endpoints<R>(ob.mesh, f, A, B);
      WireS<R> s;
      if (!wire_setup(cx, A, B, s)) continue;
      for (int32_t i = 0; i <= s.siz; i++) {
        int32_t x, y, d;
        if (!wire_step(fr, s, i, x, y, d) || d >= fr.maxdepth) continue;
        const uint64_t key = pack_key(d, (uint32_t)(ob.face_base + f));
        const int64_t P_ = (int64_t)x * H + y;
        uint64_t cur = keys[P_].load(std::memory_order_relaxed);
        while (key < cur && !keys[P_].compare_exchange_weak(cur, key)) {
        }
      }
    }
    return;
  }
  Mesh<R> mesh(&ob.mesh);
#pragma omp parallel for schedule(dynamic, 2048)
  for (int64_t f = 0; f < ob.nfaces; f++) {
    v3<R> v[3];
    mesh.verts(f, v);
    Setup<R> s;
    face_setup(cx.W2V, fr, v, s);
    if (s.culled) continue;
    raster_face(cx, s, (uint64_t)(ob.face_base + f), keys);
  }
}

template <class R>
int render(const t3_scene* sc, int mode, float* rgb, float* rgb_pre, double* rgb64,
           int32_t* id_out, int32_t* depth_out, float* depth_f_out, int nthreads) {
  const t3_frame& fr = sc->frame;
  const int W = fr.width, H = fr.height;
  const int64_t P = (int64_t)W * H;
  Ctx<R> cx;
  cx.sc = sc;
  for (int i = 0; i < 16; i++) { cx.W2V.m[i] = (R)fr.W2V[i]; cx.V2W.m[i] = (R)fr.V2W[i]; }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  std::vector<int32_t> depth(P, fr.maxdepth);   // Engine.depth
  std::vector<int64_t> gid(P, -1);               // global winner id
  std::vector<v3<R>> img(P);                     // Scene.image
  for (int64_t i = 0; i < P; i++) img[i] = {(R)fr.bgcolor[0], (R)fr.bgcolor[1], (R)fr.bgcolor[2]};

  if (mode == 0) {
    // Scene.render's per-object loop (tina/scene/raster.py:183-187), serial faces
    std::vector<int64_t> occup(P);
    for (int o = 0; o < sc->nobjects; o++) {
      const t3_object& ob = sc->objects[o];
      Mesh<R> mesh(&ob.mesh);
      // render_occup (triangle.py:89-131; particle.py:74-114 for particles)
      std::fill(occup.begin(), occup.end(), -1);
      if (ob.mesh.kind == T3_MESH_PARTICLES) {
        for (int64_t f = 0; f < ob.nfaces; f++) {
          ParS<R> p;
          if (!particle_setup(cx, ob.mesh, f, p)) continue;
          for (int32_t x = p.botx; x <= p.topx; x++) {
            for (int32_t y = p.boty; y <= p.topy; y++) {
              if (!particle_covers(p, particle_pixel_world(cx, p, x, y))) continue;
              const int32_t d = p.depth;
              int64_t P_ = (int64_t)x * H + y;
              int32_t old = depth[P_];
              if (d < old) depth[P_] = d;
              if (old > d) {
                if (depth[P_] >= d) { occup[P_] = f; gid[P_] = ob.face_base + f; }
              }
            }
          }
        }
      }
      if (is_wire(ob.mesh)) {
        // WireframeRaster.render_color (wireframe.py:69-97): lines in order,
        // steps in order, each through the depth test
        for (int64_t f = 0; f < ob.nfaces; f++) {
          v3<R> A, B;
          wire_endpoints<R>(ob.mesh, f, A, B);
          WireS<R> s;
          if (!wire_setup(cx, A, B, s)) continue;
          for (int32_t i = 0; i <= s.siz; i++) {
            int32_t x, y, d;
            if (!wire_step(fr, s, i, x, y, d)) continue;
            int64_t P_ = (int64_t)x * H + y;
            int32_t old = depth[P_];
            if (d < old) depth[P_] = d;
            if (old > d) {
              if (depth[P_] >= d) { occup[P_] = f; gid[P_] = ob.face_base + f; }
            }
          }
        }
      }
      for (int64_t f = 0; f < ob.nfaces && !is_point_or_line(ob.mesh); f++) {
        v3<R> v[3];
        mesh.verts(f, v);
        Setup<R> s;
        face_setup(cx.W2V, fr, v, s);
        if (s.culled) continue;
        for (int32_t x = s.botx; x <= s.topx; x++) {
          for (int32_t y = s.boty; y <= s.topy; y++) {
            v3<R> wei = face_weights(s, fr, x, y);
            if (wei.x >= R(0) && wei.y >= R(0) && wei.z >= R(0)) {
              R depth_f = face_depth(s, wei);
              int32_t d = trunc_i32(depth_f * (R)fr.maxdepth);
              int64_t P_ = (int64_t)x * H + y;
              int32_t old = depth[P_];          // ti.atomic_min returns the old value
              if (d < old) depth[P_] = d;
              if (old > d) {
                if (depth[P_] >= d) { occup[P_] = f; gid[P_] = ob.face_base + f; }
              }
            }
          }
        }
      }
      // render_color (triangle.py:134-153)
      for (int64_t i = 0; i < P; i++) {
        if (occup[i] == -1) continue;
        img[i] = shade_pixel(cx, ob, mesh, occup[i], (int32_t)(i / H), (int32_t)(i % H), (R*)nullptr);
      }
    }
  } else {
    // all objects into one packed (depth, global id) minimum, then one shading
    // pass with each pixel's winner: the same image as the per-object loop.
    std::vector<std::atomic<uint64_t>> keys(P);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < P; i++) keys[i].store(~0ull, std::memory_order_relaxed);
    for (int o = 0; o < sc->nobjects; o++) {
      const t3_object& ob = sc->objects[o];
      Mesh<R> mesh(&ob.mesh);
      raster_object_keys(cx, ob, keys.data());
    }
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < P; i++) {
      uint64_t k = keys[i].load(std::memory_order_relaxed);
      if (k == ~0ull) continue;
      depth[i] = (int32_t)((uint32_t)(k >> 32) ^ 0x80000000u);
      gid[i] = (int64_t)(uint32_t)k;
      for (int o = 0; o < sc->nobjects; o++) {
        const t3_object& ob = sc->objects[o];
        if (gid[i] >= ob.face_base && gid[i] < ob.face_base + ob.nfaces) {
          Mesh<R> mesh(&ob.mesh);
          img[i] = shade_pixel(cx, ob, mesh, gid[i] - ob.face_base, (int32_t)(i / H),
                               (int32_t)(i % H), (R*)nullptr);
        }
      }
    }
  }

  if (sc->lighting.mode == T3_LIGHT_IBL_MC || sc->lighting.mode == T3_LIGHT_IBL_MLP ||
      sc->lighting.mode == T3_LIGHT_IBL_PREFILTERED) {
#pragma omp parallel for schedule(static) if (mode == 1)
    for (int64_t i = 0; i < P; i++)
      if (gid[i] < 0) img[i] = background_pixel(cx, (int32_t)(i / H), (int32_t)(i % H));
  }

  // ToneMapping.apply (postp/tonemap.py:10-12) and the outputs
#pragma omp parallel for schedule(static) if (mode == 1)
  for (int64_t i = 0; i < P; i++) {
    v3<R> c = img[i];
    if (rgb_pre) { rgb_pre[3 * i] = (float)c.x; rgb_pre[3 * i + 1] = (float)c.y; rgb_pre[3 * i + 2] = (float)c.z; }
    if (fr.flags & T3_TONEMAP) c = {aces1(c.x), aces1(c.y), aces1(c.z)};
    if (rgb) { rgb[3 * i] = (float)c.x; rgb[3 * i + 1] = (float)c.y; rgb[3 * i + 2] = (float)c.z; }
    if (rgb64) { rgb64[3 * i] = (double)c.x; rgb64[3 * i + 1] = (double)c.y; rgb64[3 * i + 2] = (double)c.z; }
    if (id_out) id_out[i] = (int32_t)gid[i];
    if (depth_out) depth_out[i] = depth[i];
    if (depth_f_out) {
      float df = std::numeric_limits<float>::infinity();
      for (int o = 0; o < sc->nobjects && gid[i] >= 0; o++) {
        const t3_object& ob = sc->objects[o];
        if (gid[i] >= ob.face_base && gid[i] < ob.face_base + ob.nfaces) {
          // the winning fragment's float depth, recomputed as render_color does
          if (ob.mesh.kind == T3_MESH_PARTICLES) {
            df = (float)mapply_pos(cx.W2V, ld3<R>(ob.mesh.verts + (gid[i] - ob.face_base) * 3)).z;
            continue;
          }
          if (is_wire(ob.mesh)) {  // a line pixel: its int depth over maxdepth
            df = (float)((R)depth[i] / (R)fr.maxdepth);
            continue;
          }
          Mesh<R> mesh(&ob.mesh);
          v3<R> v[3];
          mesh.verts(gid[i] - ob.face_base, v);
          Setup<R> s;
          face_setup(cx.W2V, fr, v, s);
          df = (float)face_depth(s, face_weights(s, fr, (int32_t)(i / H), (int32_t)(i % H)));
        }
      }
      depth_f_out[i] = df;
    }
  }
  return 0;
}

// FP32 raster of every object (packed-key minimum, OpenMP): the winning
// global face id per pixel, -1 where empty.
inline std::vector<int64_t> raster_gids_f32(const t3_scene* sc) {
  const t3_frame& fr = sc->frame;
  const int64_t P = (int64_t)fr.width * fr.height;
  Ctx<float> cx;
  cx.sc = sc;
  for (int i = 0; i < 16; i++) { cx.W2V.m[i] = fr.W2V[i]; cx.V2W.m[i] = fr.V2W[i]; }
  std::vector<std::atomic<uint64_t>> keys(P);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < P; i++) keys[i].store(~0ull, std::memory_order_relaxed);
  for (int o = 0; o < sc->nobjects; o++) {
    raster_object_keys(cx, sc->objects[o], keys.data());
  }
  std::vector<int64_t> gid(P);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < P; i++) {
    const uint64_t k = keys[i].load(std::memory_order_relaxed);
    gid[i] = k == ~0ull ? -1 : (int64_t)(uint32_t)k;
  }
  return gid;
}

} // namespace

// Shading of selected pixels (indices x*H + y) over the FP32 raster's
// winners, in precision R: rgb_pre / rgb_post [n, 3] before / after ACES,
// face_id [n] (nullable) the winning global face id (-1 empty).  spp > 0
// overrides the IBL sample count and seed (ground-truth runs); spp = 0 keeps
// the scene's own, the stream the CUDA path draws.
template <class R>
int shade_pixels(const t3_scene* sc, const int64_t* pixels, int64_t n, int spp, uint32_t seed,
                        int nthreads, R* rgb_pre, R* rgb_post, int32_t* face_id) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  const t3_frame& fr = sc->frame;
  const int H = fr.height;
  const int64_t P = (int64_t)fr.width * fr.height;
  for (int64_t q = 0; q < n; q++)
    if (pixels[q] < 0 || pixels[q] >= P) return -1;
  std::vector<int64_t> gid = raster_gids_f32(sc);
  Ctx<R> cx;
  cx.sc = sc;
  cx.spp = spp;
  cx.seed = seed;
  for (int i = 0; i < 16; i++) { cx.W2V.m[i] = fr.W2V[i]; cx.V2W.m[i] = fr.V2W[i]; }
  const bool ibl = sc->lighting.mode == T3_LIGHT_IBL_MC || sc->lighting.mode == T3_LIGHT_IBL_MLP ||
                   sc->lighting.mode == T3_LIGHT_IBL_PREFILTERED;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t q = 0; q < n; q++) {
    const int64_t i = pixels[q];
    const int32_t x = (int32_t)(i / H), y = (int32_t)(i % H);
    v3<R> c = {(R)fr.bgcolor[0], (R)fr.bgcolor[1], (R)fr.bgcolor[2]};
    if (gid[i] >= 0) {
      for (int o = 0; o < sc->nobjects; o++) {
        const t3_object& ob = sc->objects[o];
        if (gid[i] >= ob.face_base && gid[i] < ob.face_base + ob.nfaces) {
          Mesh<R> mesh(&ob.mesh);
          c = shade_pixel(cx, ob, mesh, gid[i] - ob.face_base, x, y, (R*)nullptr);
        }
      }
    } else if (ibl) {
      c = background_pixel(cx, x, y);
    }
    if (rgb_pre) { rgb_pre[3 * q] = c.x; rgb_pre[3 * q + 1] = c.y; rgb_pre[3 * q + 2] = c.z; }
    if (fr.flags & T3_TONEMAP) c = {aces1(c.x), aces1(c.y), aces1(c.z)};
    if (rgb_post) { rgb_post[3 * q] = c.x; rgb_post[3 * q + 1] = c.y; rgb_post[3 * q + 2] = c.z; }
    if (face_id) face_id[q] = (int32_t)gid[i];
  }
  return 0;
}

extern "C" {

// SkyboxLighting's lookup for n (view direction, normal) pairs of a material
// whose parameters are constants: out[n, 3] = material.sample_ibl(tab, idir,
// nrm) with the tables T (the pin against the reference's own sample_ibl).
int oracle_sample_ibl_f32(const t3_material* mat, const t3_ibl_tables* T, const float* idir, const float* nrm,
                          int64_t n, float* out) {
  for (int64_t q = 0; q < n; q++) {
    Frag<float> fr{};
    fr.normal = {nrm[3 * q], nrm[3 * q + 1], nrm[3 * q + 2]};
    fr.attr = nullptr;
    MaterialEval<float> me{mat, &fr};
    const v3<float> r = sample_ibl(me, *T, mat->root, v3<float>{idir[3 * q], idir[3 * q + 1], idir[3 * q + 2]},
                                   fr.normal);
    out[3 * q] = r.x; out[3 * q + 1] = r.y; out[3 * q + 2] = r.z;
  }
  return 0;
}

// One draw of a leaf sampler for n inputs: op (T3_OP_LAMBERT / COOK / PHONG),
// param = roughness (its square is taken) or shineness, f0 [n, 3], uniforms
// xi [n, 2]; out_dir / out_w [n, 3].
int oracle_sample_leaf_f32(int op, const float* param, const float* f0, const float* idir, const float* nrm,
                           const float* xi, int64_t n, float* out_dir, float* out_w) {
  for (int64_t q = 0; q < n; q++) {
    const float r2 = op == T3_OP_COOK ? param[q] * param[q] : param[q];
    v3<float> dir;
    const v3<float> w = sample_leaf<float>(op, r2, v3<float>{f0[3 * q], f0[3 * q + 1], f0[3 * q + 2]},
                                           v3<float>{idir[3 * q], idir[3 * q + 1], idir[3 * q + 2]},
                                           v3<float>{nrm[3 * q], nrm[3 * q + 1], nrm[3 * q + 2]}, xi[2 * q],
                                           xi[2 * q + 1], dir);
    out_dir[3 * q] = dir.x; out_dir[3 * q + 1] = dir.y; out_dir[3 * q + 2] = dir.z;
    out_w[3 * q] = w.x; out_w[3 * q + 1] = w.y; out_w[3 * q + 2] = w.z;
  }
  return 0;
}

// MixMaterial.sample's choice (tina/matr/material.py:124-138) for n draws:
// the second child when xi < smoothlerp(avg(fac), .12, .88), with weight
// fac / p, else the first with (1 - fac) / (1 - p); out_w [n, 3], pick [n].
int oracle_mix_choice_f32(const float* fac, const float* xi, int64_t n, float* out_w, int32_t* pick) {
  for (int64_t q = 0; q < n; q++) {
    const v3<float> f = {fac[3 * q], fac[3 * q + 1], fac[3 * q + 2]};
    const float p = mix_prob((f.x + f.y + f.z) / 3.0f);
    if (xi[q] < p) {
      pick[q] = 1;
      out_w[3 * q] = f.x / p; out_w[3 * q + 1] = f.y / p; out_w[3 * q + 2] = f.z / p;
    } else {
      pick[q] = 0;
      out_w[3 * q] = (1.0f - f.x) / (1.0f - p);
      out_w[3 * q + 1] = (1.0f - f.y) / (1.0f - p);
      out_w[3 * q + 2] = (1.0f - f.z) / (1.0f - p);
    }
  }
  return 0;
}

// FP64 shading of selected pixels with the IBL sample count / seed overridden
// (spp > 0): the converged reference image for error statements.
int oracle_pixels_f64(const t3_scene* sc, const int64_t* pixels, int64_t n, int spp, uint32_t seed,
                      int nthreads, double* rgb_pre, double* rgb_post) {
  return shade_pixels<double>(sc, pixels, n, spp, seed, nthreads, rgb_pre, rgb_post, nullptr);
}

// FP32 shading of selected pixels with the scene's own IBL stream: the parity
// oracle for frames too large to shade whole on the CPU.
int oracle_pixels_f32(const t3_scene* sc, const int64_t* pixels, int64_t n, int nthreads, float* rgb_post,
                      int32_t* face_id) {
  return shade_pixels<float>(sc, pixels, n, 0, 0, nthreads, (float*)nullptr, rgb_post, face_id);
}


// FP32 restatement (bit-exact target).  mode 0 = serial face order (the oracle),
// mode 1 = OpenMP with packed-key minimum (the timed CPU baseline).
int oracle_render_f32(const t3_scene* sc, int mode, int nthreads, float* rgb, float* rgb_pre,
                      int32_t* face_id, int32_t* depth, float* depth_f) {
  return render<float>(sc, mode, rgb, rgb_pre, nullptr, face_id, depth, depth_f, nthreads);
}

// FP64 twin: the same algorithm in double precision, for error statements.
int oracle_render_f64(const t3_scene* sc, int mode, int nthreads, double* rgb, float* rgb_pre,
                      int32_t* face_id, int32_t* depth) {
  return render<double>(sc, mode, nullptr, rgb_pre, rgb, face_id, depth, nullptr, nthreads);
}

// MeshGrid.pre_compute (tina/mesh/grid.py:27-36)
int oracle_grid_normals(const float* pos, float* nrm, int nx, int ny) {
  for (int i = 0; i < nx; i++) {
    for (int j = 0; j < ny; j++) {
      int i2 = i - 1 > 0 ? i - 1 : 0, j2 = j - 1 > 0 ? j - 1 : 0;
      int i1 = i + 1 < nx - 1 ? i + 1 : nx - 1, j1 = j + 1 < ny - 1 ? j + 1 : ny - 1;
      auto at = [&](int a, int b) { return ld3<float>(pos + ((int64_t)a * ny + b) * 3); };
      v3<float> dy = sub(at(i, j1), at(i, j2));
      v3<float> dx = sub(at(i1, j), at(i2, j));
      v3<float> n = normalized(cross(dx, dy));
      float* o = nrm + ((int64_t)i * ny + j) * 3;
      o[0] = n.x; o[1] = n.y; o[2] = n.z;
    }
  }
  return 0;
}

// MeshSmoothNormal._update_normal (tina/mesh/norm.py:34-46): every face's unit
// normal added onto its three vertices in face order, then normalised.
int oracle_smooth_normals(const t3_mesh* m, int64_t nverts, float* out) {
  std::vector<v3<float>> acc((size_t)nverts, v3<float>{0.0f, 0.0f, 0.0f});
  for (int64_t n = 0; n < m->nfaces; n++) {
    int64_t idx[3];
    v3<float> p[3];
    for (int k = 0; k < 3; k++) {
      idx[k] = m->faces[n * m->face_stride + k * m->corner_stride + m->slot_vert];
      p[k] = ld3<float>(m->verts + idx[k] * 3);
    }
    const v3<float> nrm = normalized(cross(sub(p[1], p[0]), sub(p[2], p[0])));
    for (int k = 0; k < 3; k++)
      if (idx[k] >= 0 && idx[k] < nverts) acc[(size_t)idx[k]] = add(acc[(size_t)idx[k]], nrm);
  }
  for (int64_t v = 0; v < nverts; v++) {
    const v3<float> r = normalized(acc[(size_t)v]);
    out[3 * v] = r.x;
    out[3 * v + 1] = r.y;
    out[3 * v + 2] = r.z;
  }
  return 0;
}

int oracle_aces_f32(const float* in, float* out, int64_t n) {
  for (int64_t i = 0; i < n; i++) out[i] = aces1<float>(in[i]);
  return 0;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

} // extern "C"
