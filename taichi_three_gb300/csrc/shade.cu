// shade.cu -- deferred interpolate-and-shade pass.
//
// TriangleRaster.render_color (tina/core/triangle.py:134-153) with the shader it
// calls inlined: Shader.shade_color (tina/core/shader.py:119-131),
// calc_view_ray (shader.py:82-93), Lighting.shade_color
// (tina/core/lighting.py:84-98), the material BRDFs (tina/matr/material.py) and
// the ACES tonemap (tina/advans.py:32-34) fused as the epilogue.  One thread per
// pixel: it decodes the winning face from the packed key, recomputes that face's
// setup and barycentric weights exactly as the rasteriser did (so depth_f is
// bit-exact), interpolates position / normal / texcoord, evaluates the material
// expression once per pixel, then sums the lamps.
#include "t3_internal.cuh"

namespace t3 {

// Copies the scene descriptor (a kernel parameter) into the workspace and zeroes
// the per-frame counters: one launch makes the scene readable by every later
// kernel of the frame, including inside a captured CUDA graph.
__global__ void k_upload_scene(const DevScene sc, DevScene* __restrict__ dst,
                               uint32_t* __restrict__ counters, int ncounters) {
  const uint32_t* src = reinterpret_cast<const uint32_t*>(&sc);
  uint32_t* d = reinterpret_cast<uint32_t*>(dst);
  constexpr int nwords = (int)(sizeof(DevScene) / 4);
  for (int i = threadIdx.x; i < nwords; i += blockDim.x) d[i] = src[i];
  for (int i = threadIdx.x; i < ncounters; i += blockDim.x) counters[i] = 0u;
}

cudaError_t launch_upload_scene(const DevScene& sc, DevScene* dst, uint32_t* counters,
                                int ncounters, cudaStream_t st) {
  k_upload_scene<<<1, 256, 0, st>>>(sc, dst, counters, ncounters);
  return cudaGetLastError();
}

struct V3 { float x, y, z; };
__device__ __forceinline__ V3 v3(float a, float b, float c) { return V3{a, b, c}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ V3 normalized(V3 a) { return (1.0f / sqrtf(dot(a, a))) * a; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ V3 one_minus(V3 a) { return v3(1.0f - a.x, 1.0f - a.y, 1.0f - a.z); }
__device__ __forceinline__ V3 tov(f3 a) { return v3(a.x, a.y, a.z); }

__device__ __forceinline__ float aces(float c) {
  return (c * (2.51f * c + 0.03f)) / (c * (2.43f * c + 0.59f) + 0.14f);
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

// Per-pixel material state: the flattened lobes with their per-pixel parameters.
struct LobeState {
  int kind[T3_MAX_LOBES];
  V3 w[T3_MAX_LOBES];   // lobe weight
  V3 f0[T3_MAX_LOBES];  // COOK fresnel
  float a2[T3_MAX_LOBES], k[T3_MAX_LOBES], gnorm[T3_MAX_LOBES], gv[T3_MAX_LOBES];
  float m[T3_MAX_LOBES]; int ipow[T3_MAX_LOBES];
  int n;
};

__device__ __forceinline__ void eval_material(const DevMaterial& mat, V3 pos, V3 normal, f2 tex,
                                              const float* attr, V3 viewdir, LobeState& L,
                                              V3& ambient, V3& emission) {
  V3 val[T3_MAX_NODES];
  const int nn = mat.nnodes;
  for (int i = 0; i < nn; i++) {
    const t3_node nd = mat.nodes[i];
    V3 r = v3(0.f, 0.f, 0.f);
    switch (nd.op) {
    case T3_OP_CONST:
      r = nd.b == 3 ? v3(nd.v[0], nd.v[1], nd.v[2]) : v3(nd.v[0], nd.v[0], nd.v[0]);
      break;
    case T3_OP_ATTR:
      if (nd.b == 1) { float a = __ldg(attr + nd.a); r = v3(a, a, a); }
      else r = v3(__ldg(attr + nd.a), __ldg(attr + nd.a + 1), __ldg(attr + nd.a + 2));
      break;
    case T3_OP_INPUT:
      r = nd.a == 0 ? pos : nd.a == 1 ? v3(1.f, 1.f, 1.f) : nd.a == 2 ? normal : v3(tex.x, tex.y, 0.f);
      break;
    case T3_OP_FRESNEL: {
      V3 met = val[nd.a], alb = val[nd.b], spc = val[nd.c];
      r = met * alb + (one_minus(met) * v3(0.16f, 0.16f, 0.16f)) * (spc * spc);
      break;
    }
    default:
      break;
    }
    val[i] = r;
  }
  L.n = mat.nlobes;
  ambient = v3(0.f, 0.f, 0.f);
  emission = v3(0.f, 0.f, 0.f);
#pragma unroll
  for (int k = 0; k < T3_MAX_LOBES; k++) {
    if (k >= L.n) break;
    const DevLobe lb = mat.lobes[k];
    V3 w = v3(1.f, 1.f, 1.f);
    for (int j = 0; j < lb.nfac; j++) {
      V3 f = val[lb.fac[j] & 0xFFFF];
      w = w * ((lb.fac[j] & T3_FAC_ONE_MINUS) ? one_minus(f) : f);
    }
    L.kind[k] = lb.kind;
    L.w[k] = w;
    if (lb.kind == T3_OP_EMISSION) emission = emission + w;
    else ambient = ambient + w;
    if (lb.kind == T3_OP_COOK) {
      const float r = val[lb.p0].x;
      const float a2 = fmaxf(1e-6f, r * r);
      const float kk = a2 / 2.0f;
      L.a2[k] = a2;
      L.k[k] = kk;
      L.gnorm[k] = 1.0f / (1.0f * (1.0f - a2) + 12.566370614359172f * a2);
      const float NoV = fmaxf(1e-10f, dot(viewdir, normal));
      L.gv[k] = 1.0f / ((NoV * kk + 1.0f) - kk);
      L.f0[k] = val[lb.p1];
    } else if (lb.kind == T3_OP_PHONG) {
      L.m[k] = val[lb.p0].x;
      L.ipow[k] = lb.int_pow;
    }
  }
}

// sum_k W_k * brdf_k(n, L, V)
__device__ __forceinline__ V3 eval_brdf(const LobeState& L, V3 n, V3 ldir, V3 vdir) {
  V3 acc = v3(0.f, 0.f, 0.f);
#pragma unroll
  for (int k = 0; k < T3_MAX_LOBES; k++) {
    if (k >= L.n) break;
    if (L.kind[k] == T3_OP_LAMBERT) {
      acc = acc + 0.31830988618379067f * L.w[k];
    } else if (L.kind[k] == T3_OP_COOK) {
      const V3 half = normalized(ldir + vdir);
      const float NoH = fmaxf(1e-10f, dot(half, n));
      const float NoL = fmaxf(1e-10f, dot(ldir, n));
      const float VoH = fminf(1.0f, fmaxf(1e-10f, dot(half, vdir)));
      const float a2 = L.a2[k];
      const float denom = 1.0f - (NoH * NoH) * (1.0f - a2);
      const float ndf = a2 / (denom * denom);
      const float vdf = (L.gv[k] * (1.0f / ((NoL * L.k[k] + 1.0f) - L.k[k]))) * L.gnorm[k];
      const float om = 1.0f - VoH;
      const float om2 = om * om;
      const float p5 = om * (om2 * om2);
      const V3 f0 = L.f0[k];
      const V3 fdf = f0 + p5 * one_minus(f0);
      acc = acc + (vdf * ndf) * (L.w[k] * fdf);
    } else if (L.kind[k] == T3_OP_PHONG) {
      // reflect(-L, n) = -L - 2 (n . -L) n
      const V3 I = v3(-ldir.x, -ldir.y, -ldir.z);
      const V3 rdir = I - (2.0f * dot(n, I)) * n;
      const float VoR = fmaxf(0.0f, dot(vdir, rdir));
      const float m = L.m[k];
      const float p = L.ipow[k] > 0 ? ipowf(VoR, L.ipow[k]) : powf(VoR, m);
      acc = acc + ((p * (m + 2.0f)) / 2.0f) * L.w[k];
    }
  }
  return acc;
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
k_shade(const DevScene* __restrict__ sc, const unsigned long long* __restrict__ keys,
        t3_outputs out, int64_t npix) {
  const int64_t i = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  if (i >= npix) return;
  const t3_frame& fr = sc->frame;
  const int H = fr.height;
  const unsigned long long key = keys[i];
  V3 color;
  int32_t fid = -1, depth = fr.maxdepth;
  float depth_f = __int_as_float(0x7f800000);
  // the object owning this face id (-1: empty pixel, or an id no object owns)
  int o = -1;
  if (key != T3_EMPTY_KEY) {
    const int64_t gid = (int64_t)(uint32_t)key;
    const int nobj = sc->nobjects;
    for (int j = 0; j < nobj; j++) {
      const DevObject& ob = sc->obj[j];
      if (gid >= ob.face_base && gid < ob.face_base + ob.nfaces) o = j;
    }
  }
  if (o < 0) {
    color = v3(fr.bgcolor[0], fr.bgcolor[1], fr.bgcolor[2]);
  } else {
    const uint32_t gid = (uint32_t)key;
    fid = (int32_t)gid;
    depth = (int32_t)((uint32_t)(key >> 32) ^ 0x80000000u);
    const DevObject& ob = sc->obj[o];
    const t3_mesh& mesh = ob.mesh;
    const int64_t n = (int64_t)gid - ob.face_base;
    const FaceRef ref = face_ref(mesh, n);
    f3 v[3];
    face_verts(mesh, ref, v);
    Setup s;
    face_setup(fr, v, s);
    const int32_t x = (int32_t)(i / H), y = (int32_t)(i - (int64_t)x * H);
    const float px = xadd((float)x, fr.bias[0]), py = xadd((float)y, fr.bias[1]);
    const f3 wei = face_weights(s, px, py);
    depth_f = face_depth(s, wei);

    // interpolate (triangle.py:32-49)
    const V3 A = tov(v[0]), B = tov(v[1]), C = tov(v[2]);
    const V3 pos = (wei.x * A + wei.y * B) + wei.z * C;
    V3 nrm;
    if (fr.flags & T3_SMOOTHING) {
      f3 nn[3];
      face_norms(mesh, ref, nn);
      nrm = (wei.x * tov(nn[0]) + wei.y * tov(nn[1])) + wei.z * tov(nn[2]);
    } else {
      nrm = cross(B - A, C - A);
    }
    nrm = normalized(nrm);
    f2 tex = f2{0.f, 0.f};
    if (fr.flags & T3_TEXTURING) {
      f2 t[3];
      face_coors(mesh, ref, t);
      tex = f2{(wei.x * t[0].x + wei.y * t[1].x) + wei.z * t[2].x,
               (wei.x * t[0].y + wei.y * t[1].y) + wei.z * t[2].y};
    }
    // calc_viewdir (shader.py:82-93)
    const float ux = (px / (float)fr.width) * 2.0f - 1.0f;
    const float uy = (py / (float)H) * 2.0f - 1.0f;
    const f3 ro = mapply_pos_x(fr.V2W, f3{ux, uy, -1.0f});
    const f3 ro1 = mapply_pos_x(fr.V2W, f3{ux, uy, 1.0f});
    const V3 rd = normalized(v3(ro1.x - ro.x, ro1.y - ro.y, ro1.z - ro.z));
    const V3 vdir = v3(-rd.x, -rd.y, -rd.z);

    const float* attr = mesh.face_attr ? mesh.face_attr + ref.f * mesh.attr_stride : nullptr;
    LobeState L;
    V3 amb, emi;
    eval_material(ob.mat, pos, nrm, tex, attr, vdir, L, amb, emi);

    // Lighting.shade_color (lighting.py:84-98)
    const t3_lighting& lt = sc->lighting;
    color = emi;
    color = color + v3(lt.ambient[0], lt.ambient[1], lt.ambient[2]) * amb;
    const int nl = lt.nlights;
    for (int l = 0; l < nl; l++) {
      const float4 ld = *reinterpret_cast<const float4*>(lt.lights[l].dir);
      const float4 lc = *reinterpret_cast<const float4*>(lt.lights[l].color);
      V3 ldir = v3(ld.x - pos.x * ld.w, ld.y - pos.y * ld.w, ld.z - pos.z * ld.w);
      const float dist = sqrtf(dot(ldir, ldir));
      ldir = v3(ldir.x / dist, ldir.y / dist, ldir.z / dist);
      const float cos_i = dot(nrm, ldir);
      if (cos_i > 0.0f) {
        const float d2 = dist * dist;
        const V3 lcol = v3(lc.x / d2, lc.y / d2, lc.z / d2);
        const V3 mcol = eval_brdf(L, nrm, ldir, vdir);
        color = color + (cos_i * lcol) * mcol;
      }
    }
  }
  if (fr.flags & T3_TONEMAP) color = v3(aces(color.x), aces(color.y), aces(color.z));
  if (out.rgb) {
    out.rgb[3 * i] = color.x;
    out.rgb[3 * i + 1] = color.y;
    out.rgb[3 * i + 2] = color.z;
  }
  if (out.face_id) out.face_id[i] = fid;
  if (out.depth) out.depth[i] = depth;
  if (out.depth_f) out.depth_f[i] = depth_f;
}

cudaError_t launch_shade(const DevScene* sc_dev, const t3_frame& fr, const unsigned long long* keys,
                         const t3_outputs& out, cudaStream_t st) {
  constexpr int BLOCK = 256;
  const int64_t npix = (int64_t)fr.width * fr.height;
  const int64_t grid = (npix + BLOCK - 1) / BLOCK;
  k_shade<BLOCK><<<(unsigned)grid, BLOCK, 0, st>>>(sc_dev, keys, out, npix);
  return cudaGetLastError();
}

} // namespace t3
