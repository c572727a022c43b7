// t3_shading.cuh -- per-pixel deferred shading shared by the direct shade kernel
// and the binned tile kernel.
//
// Shader.shade_color (tina/core/shader.py:119-131) with calc_view_ray
// (shader.py:82-93), Lighting.shade_color (tina/core/lighting.py:84-98), the
// material BRDFs (tina/matr/material.py) and the ACES epilogue
// (tina/advans.py:32-34).  Materials arrive flattened into weighted lobes; node
// values are evaluated on the fly from the read-only node table (FRESNEL over
// leaf nodes, everything else a leaf), so no per-thread node array is kept.
#pragma once

#include "t3_internal.cuh"

namespace t3 {

struct V3 { float x, y, z; };
__device__ __forceinline__ V3 v3(float a, float b, float c) { return V3{a, b, c}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
// The products and sums of dot and lerp3 are written as explicit FMAs, so every
// kernel instance that interpolates a fragment gets the same bits (left to the
// compiler, the contraction of a sum of products can differ between instances
// with different surrounding code, and the network's Fourier features of the
// normal can then round to different BF16 values).
__device__ __forceinline__ float dot(V3 a, V3 b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }
// wa A + wb B + wc C, summed in that order
__device__ __forceinline__ V3 lerp3(float wa, float wb, float wc, V3 A, V3 B, V3 C) {
  return v3(fmaf(wc, C.x, fmaf(wb, B.x, wa * A.x)), fmaf(wc, C.y, fmaf(wb, B.y, wa * A.y)),
            fmaf(wc, C.z, fmaf(wb, B.z, wa * A.z)));
}
__device__ __forceinline__ V3 normalized(V3 a) { return rsqrtf(dot(a, a)) * a; }
// Approximate reciprocal, reciprocal square root and quotient for the
// shading-only arithmetic (lamp terms, BRDF lobes, view ray, ACES), whose
// inputs are normal numbers: the hardware approximations in their
// flush-to-zero form, without the denormal handling of rsqrtf / __fdividef.
__device__ __forceinline__ float rsqrt_fast(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rcp_fast(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float div_fast(float a, float b) { return a * rcp_fast(b); }
__device__ __forceinline__ V3 normalized_fast(V3 a) { return rsqrt_fast(dot(a, a)) * a; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return v3(fmaf(a.y, b.z, -(a.z * b.y)), fmaf(a.z, b.x, -(a.x * b.z)), fmaf(a.x, b.y, -(a.y * b.x)));
}
__device__ __forceinline__ V3 one_minus(V3 a) { return v3(1.0f - a.x, 1.0f - a.y, 1.0f - a.z); }
__device__ __forceinline__ V3 tov(f3 a) { return v3(a.x, a.y, a.z); }

__device__ __forceinline__ float aces(float c) {
  return div_fast(c * (2.51f * c + 0.03f), c * (2.43f * c + 0.59f) + 0.14f);
}

__device__ __forceinline__ float ipowf(float x, int n) {
  float result = 1.0f, base = x;
  bool first = true;
  while (n > 0) {
    if (n & 1) { result = first ? base : result * base; first = false; }
    n >>= 1;
    if (n) base = base * base;
  }
  return result;
}

struct Frag {
  V3 pos, normal;
  f2 tex;
  const float* attr;
  V3 color;  // Input('color'): white on triangles (triangle.py:48), the particle's colour
};

// CONST / ATTR / INPUT node value (scalars broadcast to all three lanes)
__device__ __forceinline__ V3 eval_basic(const t3_node& nd, const Frag& fg) {
  switch (nd.op) {
  case T3_OP_CONST:
    return nd.b == 3 ? v3(nd.v[0], nd.v[1], nd.v[2]) : v3(nd.v[0], nd.v[0], nd.v[0]);
  case T3_OP_ATTR:
    if (nd.b == 1) {
      const float a = __ldg(fg.attr + nd.a);
      return v3(a, a, a);
    }
    return v3(__ldg(fg.attr + nd.a), __ldg(fg.attr + nd.a + 1), __ldg(fg.attr + nd.a + 2));
  case T3_OP_INPUT:
    return nd.a == 0 ? fg.pos : nd.a == 1 ? fg.color : nd.a == 2 ? fg.normal
                                                                        : v3(fg.tex.x, fg.tex.y, 0.f);
  default:
    return v3(0.f, 0.f, 0.f);
  }
}

// Texture.__call__ (nodes.py:105-111): bilerp(texture, texcoord * (shape - 1))
// (common.py:141-150), indices clamped to the image
__device__ __forceinline__ V3 tex_texel(const t3_texture& t, int i, int j) {
  i = min(max(i, 0), t.w - 1);
  j = min(max(j, 0), t.h - 1);
  const float* p = t.data + ((int64_t)i * t.h + j) * t.channels;
  if (t.channels == 1) {
    const float s = __ldg(p);
    return v3(s, s, s);
  }
  return v3(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}

__device__ __forceinline__ V3 tex_sample(const t3_texture& t, V3 uv) {
  const float cx = uv.x * (float)(t.w - 1), cy = uv.y * (float)(t.h - 1);
  const float fx = floorf(cx), fy = floorf(cy);
  const int ix = (int)fx, iy = (int)fy;
  const float x0 = cx - fx, x1 = cy - fy, y0 = 1.0f - x0, y1 = 1.0f - x1;
  return ((x0 * x1) * tex_texel(t, ix + 1, iy + 1) + (x0 * y1) * tex_texel(t, ix + 1, iy)) +
         ((y0 * y1) * tex_texel(t, ix, iy) + (y0 * x1) * tex_texel(t, ix, iy + 1));
}

// Texture and ChessboardTexture (nodes.py:114-126:
// lerp((texcoord // size).sum() % 2, color0, color1)), one out-of-line copy.
static __device__ __noinline__ V3 eval_texture_node(const DevMaterial& m, int i, Frag fg) {
  const t3_node& nd = m.nodes[i];
  if (nd.op == T3_OP_TEXTURE) return tex_sample(m.textures[nd.b], eval_basic(m.nodes[nd.a], fg));
  const V3 uv = eval_basic(m.nodes[nd.a], fg);
  const float size = eval_basic(m.nodes[nd.b], fg).x;
  const float s = floorf(uv.x / size) + floorf(uv.y / size);
  const float t = s - 2.0f * floorf(s * 0.5f);
  const V3 c0 = eval_basic(m.nodes[nd.c], fg), c1 = eval_basic(m.nodes[(int)nd.v[0]], fg);
  return (1.0f - t) * c0 + t * c1;
}

// basic values and (TEX) the texture nodes.  TEX = false compiles the texture
// nodes out: the host picks that instance for untextured scenes, which keeps
// the call and its registers out of the lamp loop.
template <bool TEX>
__device__ __forceinline__ V3 eval_leaf(const DevMaterial& m, int i, const Frag& fg) {
  const t3_node& nd = m.nodes[i];
  if constexpr (TEX) {
    if (nd.op == T3_OP_TEXTURE || nd.op == T3_OP_CHECKER) return eval_texture_node(m, i, fg);
  }
  return eval_basic(nd, fg);
}

// value of node i; FRESNEL f0 = metallic * albedo + (1 - metallic) * 0.16 * specular**2
template <bool TEX = true>
__device__ __forceinline__ V3 eval_value(const DevMaterial& m, int i, const Frag& fg) {
  const t3_node nd = m.nodes[i];
  if (nd.op == T3_OP_FRESNEL) {
    const V3 met = eval_leaf<TEX>(m, nd.a, fg), alb = eval_leaf<TEX>(m, nd.b, fg);
    const V3 spc = eval_leaf<TEX>(m, nd.c, fg);
    return met * alb + (one_minus(met) * v3(0.16f, 0.16f, 0.16f)) * (spc * spc);
  }
  return eval_leaf<TEX>(m, i, fg);
}

// NL = lobe slots compiled in (the kernels are instantiated for 1, 2 and 4)
template <int NL>
struct LobeState {
  int kind[NL];
  V3 w[NL];   // lobe weight
  V3 f0[NL];  // COOK fresnel
  float a2[NL], oma2[NL], k[NL], gnorm[NL];
  float m[NL];
  int ipow[NL];
  int n;
};

// Lobe signatures: the kinds of a material's flattened lobes, one byte per
// slot (0 = none).  A kernel instantiated for a signature has the lobe kinds as
// constants (no per-lamp dispatch); SIG 0 reads them from the material.
constexpr int T3_SIG_DIFFUSE = T3_OP_LAMBERT;                      // Diffuse, Lambert * c
constexpr int T3_SIG_PBR = T3_OP_LAMBERT | (T3_OP_COOK << 8);      // PBR
constexpr int T3_SIG_CLASSIC = T3_OP_LAMBERT | (T3_OP_PHONG << 8); // Classic
template <int SIG>
__device__ __forceinline__ constexpr int sig_kind(int k) { return (SIG >> (8 * k)) & 0xFF; }
// instances whose every object has the FastMat shape of its signature
constexpr int T3_SIG_FAST = 1 << 24;

template <int NL, bool TEX = true, int SIG = 0>
__device__ __forceinline__ void eval_material(const DevMaterial& mat, const Frag& fg, V3 viewdir,
                                              LobeState<NL>& L, V3& ambient, V3& emission) {
  L.n = mat.nlobes;
  ambient = v3(0.f, 0.f, 0.f);
  emission = v3(0.f, 0.f, 0.f);
  const float NoV = fmaxf(1e-10f, dot(viewdir, fg.normal));
#pragma unroll
  for (int k = 0; k < NL; k++) {
    L.kind[k] = -1;
    if (k >= L.n) continue;
    const DevLobe& lb = mat.lobes[k];
    V3 w = v3(1.f, 1.f, 1.f);
    for (int j = 0; j < lb.nfac; j++) {
      const V3 f = eval_value<TEX>(mat, lb.fac[j] & 0xFFFF, fg);
      w = w * ((lb.fac[j] & T3_FAC_ONE_MINUS) ? one_minus(f) : f);
    }
    const int kind = SIG ? sig_kind<SIG & ~T3_SIG_FAST>(k) : lb.kind;
    L.kind[k] = kind;
    if (kind == T3_OP_EMISSION) emission = emission + w;
    else ambient = ambient + w;
    if (kind == T3_OP_COOK) {
      // per-pixel parts of CookTorrance.sub_brdf (material.py:323-357)
      const float r = eval_value<TEX>(mat, lb.p0, fg).x;
      const float a2 = fmaxf(1e-6f, r * r);
      const float kk = a2 * 0.5f;
      L.a2[k] = a2;
      L.k[k] = kk;
      L.gnorm[k] = div_fast(1.0f, ((NoV * kk + 1.0f) - kk) * (1.0f * (1.0f - a2) + 12.566370614359172f * a2));
      L.oma2[k] = 1.0f - a2;
      L.f0[k] = eval_value<TEX>(mat, lb.p1, fg);
    } else if (kind == T3_OP_PHONG) {
      L.m[k] = eval_value<TEX>(mat, lb.p0, fg).x;
      L.ipow[k] = lb.int_pow;
    }
    L.w[k] = w;
  }
}

// eval_material for an object whose material has its signature's FastMat
// shape: each parameter evaluated once; the same values as eval_material
template <int NL, int SIG>
__device__ __forceinline__ void eval_material_fast(const DevObject& ob, const Frag& fg, V3 viewdir,
                                                   LobeState<NL>& L, V3& ambient, V3& emission) {
  constexpr int S = SIG & ~T3_SIG_FAST;
  const DevMaterial& mat = ob.mat;
  const V3 c = eval_basic(mat.nodes[ob.fast.node[0]], fg);
  emission = v3(0.f, 0.f, 0.f);
  L.n = S == T3_SIG_DIFFUSE ? 1 : 2;
#pragma unroll
  for (int k = 0; k < NL; k++) L.kind[k] = sig_kind<S>(k);
  if constexpr (S == T3_SIG_DIFFUSE) {
    L.w[0] = c;
    ambient = c;
  } else {
    // Mix(Lambert * C, second, F): weights (1 - F) C and F
    const V3 f = S == T3_SIG_PBR ? eval_value<false>(mat, ob.fast.node[1], fg)
                                 : eval_basic(mat.nodes[ob.fast.node[1]], fg);
    L.w[0] = one_minus(f) * c;
    L.w[1] = f;
    ambient = L.w[0] + L.w[1];
    const float p = eval_basic(mat.nodes[ob.fast.node[2]], fg).x;
    if constexpr (S == T3_SIG_PBR) {
      const float NoV = fmaxf(1e-10f, dot(viewdir, fg.normal));
      const float a2 = fmaxf(1e-6f, p * p);
      const float kk = a2 * 0.5f;
      L.a2[1] = a2;
      L.k[1] = kk;
      L.gnorm[1] = div_fast(1.0f, ((NoV * kk + 1.0f) - kk) * (1.0f * (1.0f - a2) + 12.566370614359172f * a2));
      L.oma2[1] = 1.0f - a2;
      L.f0[1] = f;
    } else {
      L.m[1] = p;
      L.ipow[1] = ob.fast.int_pow;
    }
  }
}

// sum_k W_k * brdf_k(n, L, V)
template <int NL, int SIG = 0>
__device__ __forceinline__ V3 eval_brdf(const LobeState<NL>& L, V3 n, V3 ldir, V3 vdir) {
  V3 acc = v3(0.f, 0.f, 0.f);
#pragma unroll
  for (int k = 0; k < NL; k++) {
    const int kind = SIG ? sig_kind<SIG & ~T3_SIG_FAST>(k) : L.kind[k];
    if (kind == T3_OP_LAMBERT) {
      acc = acc + 0.31830988618379067f * L.w[k];
    } else if (kind == T3_OP_COOK) {
      const V3 half = normalized_fast(ldir + vdir);
      const float NoH = fmaxf(1e-10f, dot(half, n));
      const float NoL = fmaxf(1e-10f, dot(ldir, n));
      const float VoH = fminf(1.0f, fmaxf(1e-10f, dot(half, vdir)));
      const float a2 = L.a2[k];
      const float denom = 1.0f - (NoH * NoH) * L.oma2[k];
      const float ndf = div_fast(a2, denom * denom);
      const float vdf = div_fast(L.gnorm[k], (NoL * L.k[k] + 1.0f) - L.k[k]);
      const float om = 1.0f - VoH;
      const float om2 = om * om;
      const float p5 = om * (om2 * om2);
      const V3 f0 = L.f0[k];
      const V3 fdf = f0 + p5 * one_minus(f0);
      acc = acc + (vdf * ndf) * (L.w[k] * fdf);
    } else if (kind == T3_OP_PHONG) {
      // reflect(-L, n) = -L - 2 (n . -L) n
      const V3 I = v3(-ldir.x, -ldir.y, -ldir.z);
      const V3 rdir = I - (2.0f * dot(n, I)) * n;
      const float VoR = fmaxf(0.0f, dot(vdir, rdir));
      const float m = L.m[k];
      const float p = L.ipow[k] > 0 ? ipowf(VoR, L.ipow[k]) : powf(VoR, m);
      acc = acc + ((p * (m + 2.0f)) * 0.5f) * L.w[k];
    }
  }
  return acc;
}

__device__ __forceinline__ V3 background(const t3_frame& fr) {
  V3 c = v3(fr.bgcolor[0], fr.bgcolor[1], fr.bgcolor[2]);
  if (fr.flags & T3_TONEMAP) c = v3(aces(c.x), aces(c.y), aces(c.z));
  return c;
}

// Writes an empty pixel: background colour, id -1, maxdepth, +inf.
__device__ __forceinline__ void write_empty(const t3_frame& fr, const t3_outputs& out, int64_t i,
                                            V3 bg) {
  if (out.rgb) {
    out.rgb[3 * i] = bg.x;
    out.rgb[3 * i + 1] = bg.y;
    out.rgb[3 * i + 2] = bg.z;
  }
  if (out.face_id) out.face_id[i] = -1;
  if (out.depth) out.depth[i] = fr.maxdepth;
  if (out.depth_f) out.depth_f[i] = __int_as_float(0x7f800000);
}

} // namespace t3

#include "t3_ibl.cuh"

namespace t3 {

// calc_view_ray (shader.py:82-87): the ray through pixel centre (px, py),
// normalize(mapply_pos(V2W, (u, +1)) - mapply_pos(V2W, (u, -1)))
__device__ __forceinline__ V3 view_ray(const t3_frame& fr, float px, float py) {
  const float ux = div_fast(px, (float)fr.width) * 2.0f - 1.0f;
  const float uy = div_fast(py, (float)fr.height) * 2.0f - 1.0f;
  const float* M = fr.V2W;
  const float bx = M[3] + M[0] * ux + M[1] * uy, by = M[7] + M[4] * ux + M[5] * uy;
  const float bz = M[11] + M[8] * ux + M[9] * uy, bw = M[15] + M[12] * ux + M[13] * uy;
  const float w0 = rcp_fast(bw - M[14]), w1 = rcp_fast(bw + M[14]);
  const V3 ro = v3((bx - M[2]) * w0, (by - M[6]) * w0, (bz - M[10]) * w0);
  const V3 ro1 = v3((bx + M[2]) * w1, (by + M[6]) * w1, (bz + M[10]) * w1);
  return normalized_fast(ro1 - ro);
}

// the object owning the key's face id (-1: empty pixel, or an id no object owns)
__device__ __forceinline__ int key_owner(const DevScene* __restrict__ sc, unsigned long long key) {
  int o = -1;
  if (key != T3_EMPTY_KEY) {
    const int64_t gid = (int64_t)(uint32_t)key;
    const int nobj = sc->nobjects;
    for (int j = 0; j < nobj; j++) {
      if (gid >= sc->obj[j].face_base && gid < sc->obj[j].face_base + sc->obj[j].nfaces) o = j;
    }
  }
  return o;
}

// Everything shading needs about one covered pixel.
struct PixelGeom {
  int64_t i;          // pixel index x*H + y
  bool flat;          // a line pixel: fg.color is its final colour, nothing to shade
  const DevObject* ob;
  Frag fg;
  V3 vdir;            // calc_viewdir
};

// Decodes pixel (x, y)'s key, writes its raster outputs (face id, int depth,
// float depth) and, when covered, fills `g` (interpolation of
// triangle.py:32-49 and calc_viewdir of shader.py:82-93).  Returns false for
// an empty pixel.  `rec` (nullable) holds the rasteriser's setup records
// (64 bytes per face id); without it the face setup is recomputed,
// bit-identically.  COHERENT_REC: the records were written by the same kernel
// launch (read through L2, not the read-only path).  PLAIN: every object of
// the frame is a face soup without mesh edits (plain_soups), so the line,
// particle, transform and corner-order paths are compiled out (fewer
// registers and instructions; the raster outputs are the same bits, the
// shading arithmetic may round differently in its last bit where the
// compiler contracts it differently, well inside the RGB tolerance).
template <bool COHERENT_REC = false, bool PLAIN = false>
__device__ __forceinline__ bool pixel_geometry(const DevScene* __restrict__ sc,
                                               const float4* __restrict__ rec,
                                               unsigned long long key, int x, int y,
                                               const t3_outputs& out, PixelGeom& g) {
  const t3_frame& fr = sc->frame;
  const int H = fr.height;
  const int64_t i = (int64_t)x * H + y;
  g.i = i;
  g.flat = false;
  const int o = key_owner(sc, key);
  if (o < 0) {
    if (out.face_id) out.face_id[i] = -1;
    if (out.depth) out.depth[i] = fr.maxdepth;
    if (out.depth_f) out.depth_f[i] = __int_as_float(0x7f800000);
    return false;
  }
  const uint32_t gid = (uint32_t)key;
  const DevObject& ob = sc->obj[o];
  g.ob = &ob;
  const t3_mesh& mesh = ob.mesh;
  const int64_t n = (int64_t)gid - ob.face_base;
  if (!PLAIN && is_wire(mesh)) {
    // WireframeRaster: the raster's line colour, blended with factor 1 by
    // Shader.blend_color (wireframe.py:93-97, shader.py:133-135)
    const int32_t d = (int32_t)((uint32_t)(key >> 32) ^ 0x80000000u);
    if (out.face_id) out.face_id[i] = (int32_t)gid;
    if (out.depth) out.depth[i] = d;
    if (out.depth_f) out.depth_f[i] = xdiv((float)d, (float)fr.maxdepth);
    g.flat = true;
    g.fg.color = v3(fr.linecolor[0], fr.linecolor[1], fr.linecolor[2]);
    return true;
  }
  if (!PLAIN && mesh.kind == T3_MESH_PARTICLES) {
    // ParticleRaster.render_color (particle.py:116-146)
    const f3 A = ld3(mesh.verts + n * 3);
    const float Rl = __ldg(mesh.coors + n);
    const float vz = mapply_pos_x(fr.W2V, A).z;
    if (out.face_id) out.face_id[i] = (int32_t)gid;
    if (out.depth) out.depth[i] = (int32_t)((uint32_t)(key >> 32) ^ 0x80000000u);
    if (out.depth_f) out.depth_f[i] = vz;
    const float px = xadd((float)x, fr.bias[0]), py = xadd((float)y, fr.bias[1]);
    const f3 Pl = particle_pixel_world(fr, px, py, vz);
    f3 D = f3{xdiv(xsub(Pl.x, A.x), Rl), xdiv(xsub(Pl.y, A.y), Rl), xdiv(xsub(Pl.z, A.z), Rl)};
    const f3 Z = normalized_x(mapply_dir_x(fr.V2W, f3{0.0f, 0.0f, 1.0f}));
    const float h = __fsqrt_rn(xsub(1.0f, dot_x(D, D)));
    D = normalized_x(f3{xsub(D.x, xmul(Z.x, h)), xsub(D.y, xmul(Z.y, h)), xsub(D.z, xmul(Z.z, h))});
    Frag& fp = g.fg;
    fp.normal = tov(D);
    fp.pos = v3(xadd(A.x, xmul(D.x, Rl)), xadd(A.y, xmul(D.y, Rl)), xadd(A.z, xmul(D.z, Rl)));
    fp.tex = f2{0.f, 0.f};
    fp.attr = mesh.face_attr ? mesh.face_attr + n * mesh.attr_stride : nullptr;
    fp.color = mesh.norms ? tov(ld3(mesh.norms + n * 3)) : v3(1.f, 1.f, 1.f);
    const V3 rd = view_ray(fr, px, py);
    g.vdir = v3(-rd.x, -rd.y, -rd.z);
    return true;
  }
  const FaceRef ref = PLAIN ? FaceRef{n, false, false} : face_ref(mesh, n);
  // start every gather of this face now: normals and material attributes are
  // needed only after the weights, but their DRAM latency overlaps from here
  if ((fr.flags & T3_SMOOTHING) && mesh.norms && !(mesh.flags & T3_MESH_FLAT_NORMAL)) {
#pragma unroll
    for (int k = 0; k < 3; k++)
      asm volatile("prefetch.global.L1 [%0];" :: "l"(base_ptr(mesh, ref.f, k, 1)));
  }
  if (mesh.face_attr)
    asm volatile("prefetch.global.L1 [%0];" :: "l"(mesh.face_attr + ref.f * mesh.attr_stride));
  f3 v[3];
  if constexpr (PLAIN) soup_corners(mesh.verts, n, v);
  else face_verts(mesh, ref, v);
  Setup s;
  if (rec) {
    const float4* r = rec + (size_t)gid * 4;
    float4 a, b, c, d;
    if (COHERENT_REC) {
      a = __ldcg(r); b = __ldcg(r + 1); c = __ldcg(r + 2); d = __ldcg(r + 3);
    } else {
      a = __ldg(r); b = __ldg(r + 1); c = __ldg(r + 2); d = __ldg(r + 3);
    }
    s.bx = a.x; s.by = a.y; s.cx = a.z; s.cy = a.w;
    s.bcnx = b.x; s.bcny = b.y; s.canx = b.z; s.cany = b.w;
    s.wsa = c.x; s.wsb = c.y; s.wsc = c.z; s.Az = c.w;
    s.Bz = d.x; s.Cz = d.y;
  } else {
    face_setup(fr, v, s);
  }
  const float px = xadd((float)x, fr.bias[0]), py = xadd((float)y, fr.bias[1]);
  const f3 wei = face_weights(s, px, py);
  // the raster outputs are final: store them now (shorter live ranges)
  if (out.face_id) out.face_id[i] = (int32_t)gid;
  if (out.depth) out.depth[i] = (int32_t)((uint32_t)(key >> 32) ^ 0x80000000u);
  if (out.depth_f) out.depth_f[i] = face_depth(s, wei);

  // interpolate (triangle.py:32-49)
  Frag& fg = g.fg;
  const V3 A = tov(v[0]), B = tov(v[1]), C = tov(v[2]);
  fg.pos = lerp3(wei.x, wei.y, wei.z, A, B, C);
  V3 nrm;
  if (fr.flags & T3_SMOOTHING) {
    f3 nn[3];
    if constexpr (PLAIN) soup_corners(mesh.norms, n, nn);
    else face_norms(mesh, ref, nn);
    nrm = lerp3(wei.x, wei.y, wei.z, tov(nn[0]), tov(nn[1]), tov(nn[2]));
  } else {
    nrm = cross(B - A, C - A);
  }
  fg.normal = normalized(nrm);
  fg.tex = f2{0.f, 0.f};
  if (fr.flags & T3_TEXTURING) {
    f2 t[3];
    face_coors(mesh, ref, t);
    fg.tex = f2{fmaf(wei.z, t[2].x, fmaf(wei.y, t[1].x, wei.x * t[0].x)),
                fmaf(wei.z, t[2].y, fmaf(wei.y, t[1].y, wei.x * t[0].y))};
  }
  fg.attr = mesh.face_attr ? mesh.face_attr + ref.f * mesh.attr_stride : nullptr;
  fg.color = v3(1.f, 1.f, 1.f);
  const V3 rd = view_ray(fr, px, py);
  g.vdir = v3(-rd.x, -rd.y, -rd.z);
  return true;
}

// Lighting.shade_color's lamp loop (lighting.py:88-97) for the lobes in L
template <int NL, int SIG = 0>
__device__ __forceinline__ V3 lamps_term(const t3_lighting& lt, const LobeState<NL>& L,
                                         const Frag& fg, V3 vdir) {
  V3 color = v3(0.f, 0.f, 0.f);
  const int nl = lt.nlights;
  for (int l = 0; l < nl; l++) {
    const float4 ld = *reinterpret_cast<const float4*>(lt.lights[l].dir);
    V3 ldir = v3(ld.x - fg.pos.x * ld.w, ld.y - fg.pos.y * ld.w, ld.z - fg.pos.z * ld.w);
    const float d2 = dot(ldir, ldir);
    const float inv_d = rsqrt_fast(d2);
    ldir = inv_d * ldir;
    const float cos_i = dot(fg.normal, ldir);
    if (cos_i > 0.0f) {
      const float4 lc = *reinterpret_cast<const float4*>(lt.lights[l].color);
      const float s = cos_i * (inv_d * inv_d);
      const V3 mcol = eval_brdf<NL, SIG>(L, fg.normal, ldir, vdir);
      color = color + v3(s * lc.x, s * lc.y, s * lc.z) * mcol;
    }
  }
  return color;
}

__device__ __forceinline__ void store_rgb(const t3_frame& fr, const t3_outputs& out, int64_t i,
                                          V3 color) {
  if (fr.flags & T3_TONEMAP) color = v3(aces(color.x), aces(color.y), aces(color.z));
  if (out.rgb) {
    out.rgb[3 * i] = color.x;
    out.rgb[3 * i + 1] = color.y;
    out.rgb[3 * i + 2] = color.z;
  }
}

template <int NL, int MODE, bool TEX, int SIG = 0>
__device__ __forceinline__ void shade_lit(const DevScene* __restrict__ sc, const PixelGeom& g,
                                          const t3_outputs& out);

// Shades pixel (x, y) from its packed (depth, id) key and writes every output.
// MODE is the lighting (T3_LIGHT_LAMPS or T3_LIGHT_IBL_MC).
template <int NL, int MODE, bool COHERENT_REC = false, bool TEX = true, int SIG = 0, bool PLAIN = false>
__device__ __forceinline__ void shade_pixel_from_key(const DevScene* __restrict__ sc,
                                                     const float4* __restrict__ rec,
                                                     unsigned long long key, int x, int y,
                                                     const t3_outputs& out) {
  const t3_frame& fr = sc->frame;
  PixelGeom g;
  const t3_lighting& lt = sc->lighting;
  if (const int sel = fr.flags & (T3_SHADE_OWNED | T3_SHADE_EMPTY)) {
    // protocol frames: only the selected pixels are written
    const bool empty = key == T3_EMPTY_KEY;
    if (empty ? !(sel & T3_SHADE_EMPTY) : (!(sel & T3_SHADE_OWNED) || key_owner(sc, key) < 0)) return;
  }
  if (!pixel_geometry<COHERENT_REC, PLAIN>(sc, rec, key, x, y, out, g)) {
    V3 bg = v3(fr.bgcolor[0], fr.bgcolor[1], fr.bgcolor[2]);
    if (MODE != T3_LIGHT_LAMPS) {
      // Engine.render_background (engine.py:42-49): the sky along the view ray
      const Env env{lt.env, lt.env_w, lt.env_h, lt.env_half};
      bg = env_sample(env, view_ray(fr, xadd((float)x, fr.bias[0]), xadd((float)y, fr.bias[1])));
    }
    store_rgb(fr, out, (int64_t)x * fr.height + y, bg);
    return;
  }
  if (g.flat) {
    store_rgb(fr, out, g.i, g.fg.color);
    return;
  }
  shade_lit<NL, MODE, TEX, SIG>(sc, g, out);
}

// the lighting of one covered pixel from its geometry (Shader.shade_color)
template <int NL, int MODE, bool TEX, int SIG>
__device__ __forceinline__ void shade_lit(const DevScene* __restrict__ sc, const PixelGeom& g,
                                          const t3_outputs& out) {
  const t3_frame& fr = sc->frame;
  const t3_lighting& lt = sc->lighting;
  V3 color;
  if (MODE == T3_LIGHT_LAMPS) {
    LobeState<NL> L;
    V3 amb, emi;
    if constexpr ((SIG & T3_SIG_FAST) != 0) eval_material_fast<NL, SIG>(*g.ob, g.fg, g.vdir, L, amb, emi);
    else eval_material<NL, TEX, SIG>(g.ob->mat, g.fg, g.vdir, L, amb, emi);
    color = emi + v3(lt.ambient[0], lt.ambient[1], lt.ambient[2]) * amb;
    color = color + lamps_term<NL, SIG>(lt, L, g.fg, g.vdir);
  } else if (MODE == T3_LIGHT_IBL_PREFILTERED) {
    // SkyboxLighting.shade_color (lighting.py:20-21) with its prefiltered tables
    V3 emi;
    color = ibl_prefiltered<NL, TEX>(g.ob->mat, sc->tables, g.fg, g.vdir, emi);
    color = emi + color;
    if (lt.nlights > 0) {
      LobeState<NL> Ll;
      V3 amb, e2;
      eval_material<NL, TEX, SIG>(g.ob->mat, g.fg, g.vdir, Ll, amb, e2);
      color = color + lamps_term<NL, SIG>(lt, Ll, g.fg, g.vdir);
    }
  } else {
    // SkyboxLighting.shade_color (lighting.py:20-21): IBL + emission
    IblLobes<NL> L;
    V3 emi;
    eval_ibl_lobes<NL, TEX>(g.ob->mat, g.fg, L, emi);
    const Env env{lt.env, lt.env_w, lt.env_h, lt.env_half};
    color = emi + ibl_mc<NL>(L, g.fg.normal, g.vdir, env, lt.spp, lt.seed, (uint32_t)g.i);
    if (lt.nlights > 0) {
      LobeState<NL> Ll;
      V3 amb, e2;
      eval_material<NL, TEX, SIG>(g.ob->mat, g.fg, g.vdir, Ll, amb, e2);
      color = color + lamps_term<NL, SIG>(lt, Ll, g.fg, g.vdir);
    }
  }
  store_rgb(fr, out, g.i, color);
}

// Lamp-lit frames: this thread's four consecutive pixels [base + local0, +4).
// Their keys are read as two 16-byte loads; four empty pixels are written as
// background with 16-byte stores (three for the RGB triples, one each for id,
// depth and float depth) when the output buffers allow it; the covered pixels
// are appended to the block's list in pixel order (one shared atomic per warp).
template <bool COHERENT>
__device__ __forceinline__ void list_quad(const t3_frame& fr, const unsigned long long* __restrict__ keys,
                                          const t3_outputs& out, int64_t npix, int64_t base, int local0,
                                          V3 bg, int* s_list, int* s_count, unsigned long long* s_key,
                                          unsigned long long* reset_keys) {
  const int lane = threadIdx.x & 31;
  const int64_t i0 = base + local0;
  unsigned long long kk[4];
  unsigned valid = 0u;  // pixels inside the frame
  if (i0 + 3 < npix && (reinterpret_cast<uintptr_t>(keys + i0) & 15) == 0) {
    const ulonglong2* k2 = reinterpret_cast<const ulonglong2*>(keys + i0);
    const ulonglong2 a = COHERENT ? __ldcg(k2) : k2[0];
    const ulonglong2 b = COHERENT ? __ldcg(k2 + 1) : k2[1];
    kk[0] = a.x; kk[1] = a.y; kk[2] = b.x; kk[3] = b.y;
    valid = 15u;
  } else {
#pragma unroll
    for (int j = 0; j < 4; j++) {
      kk[j] = T3_EMPTY_KEY;
      if (i0 + j < npix) {
        kk[j] = COHERENT ? __ldcg(keys + i0 + j) : keys[i0 + j];
        valid |= 1u << j;
      }
    }
  }
  unsigned covered = 0u;
#pragma unroll
  for (int j = 0; j < 4; j++)
    if (kk[j] != T3_EMPTY_KEY) covered |= 1u << j;
  // protocol frames that select pixels write empty ones only with T3_SHADE_EMPTY
  if (!(fr.flags & T3_SHADE_OWNED) || (fr.flags & T3_SHADE_EMPTY)) {
    const uintptr_t align = reinterpret_cast<uintptr_t>(out.rgb) | reinterpret_cast<uintptr_t>(out.face_id) |
                            reinterpret_cast<uintptr_t>(out.depth) | reinterpret_cast<uintptr_t>(out.depth_f);
    if (covered == 0u && valid == 15u && (align & 15) == 0) {
      if (out.rgb) {
        float4* r4 = reinterpret_cast<float4*>(out.rgb + 3 * i0);
        r4[0] = make_float4(bg.x, bg.y, bg.z, bg.x);
        r4[1] = make_float4(bg.y, bg.z, bg.x, bg.y);
        r4[2] = make_float4(bg.z, bg.x, bg.y, bg.z);
      }
      if (out.face_id) *reinterpret_cast<int4*>(out.face_id + i0) = make_int4(-1, -1, -1, -1);
      if (out.depth) {
        const int32_t d = fr.maxdepth;
        *reinterpret_cast<int4*>(out.depth + i0) = make_int4(d, d, d, d);
      }
      if (out.depth_f) {
        const float inf = __int_as_float(0x7f800000);
        *reinterpret_cast<float4*>(out.depth_f + i0) = make_float4(inf, inf, inf, inf);
      }
    } else {
#pragma unroll
      for (int j = 0; j < 4; j++)
        if ((valid >> j & 1u) && !(covered >> j & 1u)) write_empty(fr, out, i0 + j, bg);
    }
  }
  if (reset_keys && covered) {
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (covered >> j & 1u) reset_keys[i0 + j] = T3_EMPTY_KEY;
  }
  // the warp's covered pixels, in pixel order, after one shared atomic
  const int cnt = __popc(covered);
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= o) incl += t;
  }
  const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
  if (total == 0) return;
  int slot = 0;
  if (lane == 31) slot = atomicAdd(s_count, total);
  slot = __shfl_sync(0xFFFFFFFFu, slot, 31);
  int at = slot + incl - cnt;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    if (covered >> j & 1u) {
      s_list[at] = local0 + j;
      s_key[at] = kk[j];
      at++;
    }
  }
}

// One block's share of the shading pass: pixels [base, base + BLOCK * PPT) of
// the frame.  Empty pixels are written as background at once; covered ones are
// compacted into a shared list (warp ballot + one shared atomic per warp), with
// their keys, so that full warps run the shading.  s_list and s_key hold
// BLOCK * PPT entries; s_count must be zero on entry and is left non-zero
// (callers reset it after a barrier).  reset_keys (nullable): the frame's key
// buffer, whose keys this block returns to empty as it reads them.
template <int BLOCK, int PPT, int NL, int MODE, bool COHERENT = false, bool TEX = true, int SIG = 0,
          bool PLAIN = false>
__device__ __forceinline__ void shade_block(const DevScene* __restrict__ sc,
                                            const unsigned long long* __restrict__ keys,
                                            const float4* __restrict__ rec, const t3_outputs& out,
                                            int64_t npix, int64_t base, int* s_list, int* s_count,
                                            unsigned long long* s_key,
                                            unsigned long long* reset_keys = nullptr) {
  const t3_frame& fr = sc->frame;
  const int H = fr.height;
  const V3 bg = background(fr);
  const int lane = threadIdx.x & 31;
  if constexpr (MODE == T3_LIGHT_LAMPS && PPT % 4 == 0) {
#pragma unroll
    for (int k = 0; k < PPT / 4; k++)
      list_quad<COHERENT>(fr, keys, out, npix, base, 4 * (k * BLOCK + threadIdx.x), bg, s_list, s_count,
                          s_key, reset_keys);
  } else {
#pragma unroll
    for (int k = 0; k < PPT; k++) {
      const int local = k * BLOCK + threadIdx.x;
      const int64_t i = base + local;
      bool covered = false;
      unsigned long long key = T3_EMPTY_KEY;
      if (i < npix) {
        // with IBL, empty pixels show the sky and go through the shading list too
        key = COHERENT ? __ldcg(keys + i) : keys[i];
        if (MODE == T3_LIGHT_LAMPS && key == T3_EMPTY_KEY) {
          // protocol frames that select pixels write empty ones only with T3_SHADE_EMPTY
          if (!(fr.flags & T3_SHADE_OWNED) || (fr.flags & T3_SHADE_EMPTY)) write_empty(fr, out, i, bg);
        } else {
          covered = true;
        }
        if (key != T3_EMPTY_KEY && reset_keys) reset_keys[i] = T3_EMPTY_KEY;
      }
      const unsigned m = __ballot_sync(0xFFFFFFFFu, covered);
      if (m) {
        int slot = 0;
        if (lane == 0) slot = atomicAdd(s_count, __popc(m));
        slot = __shfl_sync(0xFFFFFFFFu, slot, 0);
        if (covered) {
          const int at = slot + __popc(m & ((1u << lane) - 1u));
          s_list[at] = local;
          s_key[at] = key;
        }
      }
    }
  }
  __syncthreads();
  const int n = *s_count;
  for (int j = threadIdx.x; j < n; j += BLOCK) {
    const int64_t i = base + s_list[j];
    const int x = (int)(i / H), y = (int)(i - (int64_t)x * H);
    shade_pixel_from_key<NL, MODE, COHERENT, TEX, SIG, PLAIN>(sc, rec, s_key[j], x, y, out);
  }
}

} // namespace t3
