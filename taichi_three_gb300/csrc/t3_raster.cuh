// t3_raster.cuh -- warp-cooperative, load-balanced rasterisation of 32 faces.
//
// Face sizes in a soup are lognormal, so "one thread walks its face's bbox"
// leaves a warp waiting on its largest face.  Here each lane contributes one
// face (its clipped bbox), the warp prefix-sums the bbox areas, and the lanes
// then walk the concatenated pixel list 32 pixels at a time: lane l takes
// pixel base + l, finds its face by binary search over the prefix sums and runs
// the exact inside / depth test of triangle.py:115-125 on it.  Setups live in
// shared memory (structure of arrays, one slot per lane).
#pragma once

#include "t3_internal.cuh"

namespace t3 {

// Setup records: 4 x float4 per global face id, written by the rasteriser for
// every visible face and read back by shading (no per-pixel setup recompute).
__device__ __forceinline__ void store_record(float4* __restrict__ rec, uint32_t gid, const Setup& s) {
  float4* r = rec + (size_t)gid * 4;
  r[0] = make_float4(s.bx, s.by, s.cx, s.cy);
  r[1] = make_float4(s.bcnx, s.bcny, s.canx, s.cany);
  r[2] = make_float4(s.wsa, s.wsb, s.wsc, s.Az);
  r[3] = make_float4(s.Bz, s.Cz, __int_as_float(s.botx | (s.boty << 16)),
                     __int_as_float(s.topx | (s.topy << 16)));
}

__device__ __forceinline__ void load_record(const float4* __restrict__ rec, uint32_t gid, Setup& s) {
  const float4* r = rec + (size_t)gid * 4;
  const float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2), d = __ldg(r + 3);
  s.bx = a.x; s.by = a.y; s.cx = a.z; s.cy = a.w;
  s.bcnx = b.x; s.bcny = b.y; s.canx = b.z; s.cany = b.w;
  s.wsa = c.x; s.wsb = c.y; s.wsc = c.z; s.Az = c.w;
  s.Bz = d.x; s.Cz = d.y;
  const int p0 = __float_as_int(d.z), p1 = __float_as_int(d.w);
  s.botx = p0 & 0xFFFF; s.boty = p0 >> 16; s.topx = p1 & 0xFFFF; s.topy = p1 >> 16;
}

// A warp's face setups in rank order (faces with a non-empty bbox), one 64-byte
// record per face (four 16-byte loads per tested pixel; lanes testing pixels
// of the same face read it as a broadcast), plus the bbox heights and the
// first index of each face's pixels in the warp's concatenated pixel list.
struct WarpFaces {
  float4 rec[32][4];  // (bx, by, cx, cy) (bcn, can) (wsa, wsb, wsc, Az) (Bz, Cz, x0 | y0 << 16, id)
  int h[32], start[32];
};

// One pixel's exact inside / depth test (triangle.py:115-125) against setup t.
template <class Sink>
__device__ __forceinline__ void test_pixel(const Setup& t, int x, int y, uint32_t id, float biasx,
                                           float biasy, float maxd, int32_t maxdepth, Sink& sink) {
  const float px = xadd((float)x, biasx), py = xadd((float)y, biasy);
  float wx, wy, wz, sum;
  face_raw_weights(t, px, py, wx, wy, wz, sum);
  f3 wei;
  if (face_inside(wx, wy, wz, sum, wei)) {
    const int32_t d = trunc_i32(xmul(face_depth(t, wei), maxd));
    if (d < maxdepth) sink(x, y, pack_key(d, id));
  }
}

// Every lane of the warp must call this.  `active` lanes contribute the face
// `s` clipped to [cx0, cx1] x [cy0, cy1]; sink(x, y, key) receives every
// covered pixel with its packed (depth, id) key.  Every face, however small,
// goes through the cooperative prefix-sum walk (measured faster than letting
// faces of a few pixels walk their own bbox per lane).  Finding a pixel's face:
// per round of 32 list positions, each face whose first pixel falls in the
// round sets that position's bit (one warp OR-reduction); a lane's face rank is
// the faces started before the round plus the set bits up to its position.
template <class Sink>
__device__ __forceinline__ void warp_raster(WarpFaces& wf, const Setup& s, bool active, uint32_t id,
                                            int cx0, int cx1, int cy0, int cy1,
                                            const t3_frame& fr, Sink sink) {
  const unsigned FULL = 0xFFFFFFFFu;
  const int lane = threadIdx.x & 31;
  const int x0 = max(s.botx, cx0), x1 = min(s.topx, cx1);
  const int y0 = max(s.boty, cy0), y1 = min(s.topy, cy1);
  const int area = (active && x0 <= x1 && y0 <= y1) ? (x1 - x0 + 1) * (y1 - y0 + 1) : 0;
  const float maxd = (float)fr.maxdepth;
  const float biasx = fr.bias[0], biasy = fr.bias[1];
  const unsigned live = __ballot_sync(FULL, area > 0);
  if (!live) return;
  int incl = area;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += t;
  }
  const int first = incl - area;  // this face's first position in the pixel list
  if (area > 0) {
    const int r = __popc(live & ((1u << lane) - 1u));
    wf.rec[r][0] = make_float4(s.bx, s.by, s.cx, s.cy);
    wf.rec[r][1] = make_float4(s.bcnx, s.bcny, s.canx, s.cany);
    wf.rec[r][2] = make_float4(s.wsa, s.wsb, s.wsc, s.Az);
    wf.rec[r][3] = make_float4(s.Bz, s.Cz, __int_as_float(x0 | (y0 << 16)), __uint_as_float(id));
    wf.h[r] = y1 - y0 + 1;
    wf.start[r] = first;
  }
  const int total = __shfl_sync(FULL, incl, 31);
  const unsigned upto = lane == 31 ? 0xFFFFFFFFu : ((2u << lane) - 1u);
  __syncwarp();
  int before = 0;  // faces whose first pixel precedes this round
  for (int base = 0; base < total; base += 32) {
    const unsigned bit = (area > 0 && first >= base && first < base + 32) ? 1u << (first - base) : 0u;
    const unsigned starts = __reduce_or_sync(FULL, bit);
    const int idx = base + lane;
    if (idx < total) {
      const int j = before + __popc(starts & upto) - 1;
      const int off = idx - wf.start[j];
      const int h = wf.h[j];
      int q = __float2int_rz(__fdividef((float)off + 0.5f, (float)h));
      int r = off - q * h;
      if (r < 0) { q--; r += h; } else if (r >= h) { q++; r -= h; }
      const float4 r0 = wf.rec[j][0], r1 = wf.rec[j][1], r2 = wf.rec[j][2], r3 = wf.rec[j][3];
      Setup t;
      t.bx = r0.x; t.by = r0.y; t.cx = r0.z; t.cy = r0.w;
      t.bcnx = r1.x; t.bcny = r1.y; t.canx = r1.z; t.cany = r1.w;
      t.wsa = r2.x; t.wsb = r2.y; t.wsc = r2.z; t.Az = r2.w;
      t.Bz = r3.x; t.Cz = r3.y;
      const int xy = __float_as_int(r3.z);
      test_pixel(t, (xy & 0xFFFF) + q, (xy >> 16) + r, __float_as_uint(r3.w), biasx, biasy, maxd,
                 fr.maxdepth, sink);
    }
    before += __popc(starts);
  }
  __syncwarp();
}

// Loads (and transforms) the corners of face n; soup positions come from the
// block's shared-memory staging area when `staged`.
__device__ __forceinline__ void load_face(const t3_mesh& mesh, int64_t n, bool staged,
                                          const float* sv, f3 v[3]) {
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
}

// Cooperative 16-byte loads of the block's face-soup positions into shared memory.
template <int BLOCK>
__device__ __forceinline__ bool stage_soup(const t3_mesh& mesh, int64_t nfaces, int64_t f0, float* sv) {
  const bool staged = mesh.kind == T3_MESH_SOUP && !(mesh.flags & T3_MESH_NOCULL);
  if (staged) {
    const int64_t rem = nfaces - f0;
    const int nf = rem < BLOCK ? (int)(rem > 0 ? rem : 0) : BLOCK;
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
  }
  __syncthreads();
  return staged;
}

} // namespace t3
