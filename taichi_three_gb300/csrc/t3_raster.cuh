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

// ---- column-span walk ---------------------------------------------------------
// The bbox walk above tests every pixel centre of a face's bbox; for the small
// faces of a soup about 30 % of those tests pass.  Here the warp first computes,
// for each column of each face's bbox, the rows whose centres can pass: each
// edge function is linear along a column, so "w >= 0" bounds the row from one
// side, and the bound is widened by a margin far above the rounding error of
// the exact evaluation (below).  Only those candidates get the exact test, so
// coverage is unchanged.
//
// Margin: the exact test computes w = (px - bx) * bcn.y - (py - by) * bcn.x in
// FP32 (each operation rounded, |error| <= 3u (|px - bx| |bcn.y| + |py - by|
// |bcn.x|), u = 2^-24) and the third weight as (1 - w_bc) - w_ca; a pixel passes
// only if every weight is >= 0 (with positive clip-w reciprocals the division
// by their sum keeps the signs, and the weights sum to 1, so not all can be
// negative).  A row bound B = -A / k from the FP32 coefficients is off by at
// most 4u |B| plus A's own rounding.  With N = 2 (dbx + dcx + hb + hc + |by| +
// |cy| + 2) (|bcn| + |can|)_1 + 4 bounding every |w| term that enters, the
// error in rows is below 3u N / |k| + 4u |B|; the margin taken is
// 2^-18 (N / |k| + |B|) + 2^-20, over 20 times that.  Faces whose clip-w
// reciprocals are not all positive and finite, or whose edge coefficients are
// not finite, keep their whole columns.
constexpr int kMaxWarpCols = 160;  // columns per warp walk (more: the bbox walk)

struct WarpCols {
  int2 col[kMaxWarpCols];  // non-empty columns: (x | face rank << 16, first row | first position << 15)
};

// rows [lo, hi] (within [y0, y1]) of column x whose centres can pass t's test
__device__ __forceinline__ void column_rows(const Setup& t, int x, int y0, int y1, float biasx, float biasy,
                                            int& lo, int& hi) {
  lo = y0;
  hi = y1;
  const bool ok = t.wsa > 0.0f && t.wsb > 0.0f && t.wsc > 0.0f && t.wsa < INFINITY && t.wsb < INFINITY &&
                  t.wsc < INFINITY;
  const float S = fabsf(t.bcnx) + fabsf(t.bcny) + fabsf(t.canx) + fabsf(t.cany);
  if (!ok || !(S < INFINITY)) return;  // also NaN
  const float px = xadd((float)x, biasx);
  const float ya = (float)y0 + biasy, yb = (float)y1 + biasy;
  const float dbx = fabsf(px - t.bx), dcx = fabsf(px - t.cx);
  const float hb = fmaxf(fabsf(ya - t.by), fabsf(yb - t.by)), hc = fmaxf(fabsf(ya - t.cy), fabsf(yb - t.cy));
  const float N = 2.0f * (dbx + dcx + hb + hc + fabsf(t.by) + fabsf(t.cy) + 2.0f) * S + 4.0f;
  // w(py) = A + k py for the edges bc, ca and ab
  const float A1 = (px - t.bx) * t.bcny + t.by * t.bcnx, k1 = -t.bcnx;
  const float A2 = (px - t.cx) * t.cany + t.cy * t.canx, k2 = -t.canx;
  const float A3 = 1.0f - A1 - A2, k3 = t.bcnx + t.canx;
  const float As[3] = {A1, A2, A3}, ks[3] = {k1, k2, k3};
  const float flo = (float)y0 - 1.0f, fhi = (float)y1 + 1.0f;
#pragma unroll
  for (int e = 0; e < 3; e++) {
    const float k = ks[e], ak = fabsf(k);
    if (!(ak * 1048576.0f > S)) continue;  // nearly constant along the column: no bound
    const float B = __fdividef(-As[e], k);
    const float m = 3.814697265625e-06f * (__fdividef(N, ak) + fabsf(B)) + 9.5367431640625e-07f;
    if (!(fabsf(B) < 1e30f) || !(m < 1e30f)) continue;
    if (k > 0.0f) {
      const float b = fminf(fmaxf(B - m - biasy, flo), fhi);
      const int r = (int)ceilf(b);
      lo = r > lo ? r : lo;
    } else {
      const float b = fminf(fmaxf(B + m - biasy, flo), fhi);
      const int r = (int)floorf(b);
      hi = r < hi ? r : hi;
    }
  }
}

// column_rows split in two: the per-face part (column_consts, once by the
// face's own lane) and the per-column part (column_rows_c), with the same
// bounds up to the order of N's sum and the approximate reciprocal of the
// edge slopes, both far inside the margin's 2^-18 factor.
struct ColConsts {
  float4 a;  // S (NaN: the face's columns get no bounds), H = hb + hc + |by| + |cy| + 2,
             // by * bcnx, cy * canx
  float4 b;  // 1 / k of the edges bc, ca, ab (0: the edge gives no bound), unused
};

__device__ __forceinline__ ColConsts column_consts(const Setup& t, int y0, int y1, float biasy) {
  const bool ok = t.wsa > 0.0f && t.wsb > 0.0f && t.wsc > 0.0f && t.wsa < INFINITY && t.wsb < INFINITY &&
                  t.wsc < INFINITY;
  float S = fabsf(t.bcnx) + fabsf(t.bcny) + fabsf(t.canx) + fabsf(t.cany);
  if (!ok || !(S < INFINITY)) S = __int_as_float(0x7fffffff);
  const float ya = (float)y0 + biasy, yb = (float)y1 + biasy;
  const float hb = fmaxf(fabsf(ya - t.by), fabsf(yb - t.by)), hc = fmaxf(fabsf(ya - t.cy), fabsf(yb - t.cy));
  const float ks[3] = {-t.bcnx, -t.canx, t.bcnx + t.canx};
  float ik[3];
#pragma unroll
  for (int e = 0; e < 3; e++)  // a slope nearly constant along the column gives no bound
    ik[e] = fabsf(ks[e]) * 1048576.0f > S ? __fdividef(1.0f, ks[e]) : 0.0f;
  ColConsts c;
  c.a = make_float4(S, hb + hc + fabsf(t.by) + fabsf(t.cy) + 2.0f, t.by * t.bcnx, t.cy * t.canx);
  c.b = make_float4(ik[0], ik[1], ik[2], 0.0f);
  return c;
}

// column_rows from the face's corners b, c, its coefficients bcn.y and can.y
// and its column_consts
__device__ __forceinline__ void column_rows_c(float bx, float cx, float bcny, float cany, const ColConsts& c,
                                              int x, int y0, int y1, float biasx, float biasy, int& lo,
                                              int& hi) {
  lo = y0;
  hi = y1;
  const float S = c.a.x;
  if (!(S < INFINITY)) return;  // also NaN
  const float px = xadd((float)x, biasx);
  const float dbx = fabsf(px - bx), dcx = fabsf(px - cx);
  const float N = 2.0f * ((dbx + dcx) + c.a.y) * S + 4.0f;
  const float A1 = (px - bx) * bcny + c.a.z;
  const float A2 = (px - cx) * cany + c.a.w;
  const float A3 = 1.0f - A1 - A2;
  const float As[3] = {A1, A2, A3}, iks[3] = {c.b.x, c.b.y, c.b.z};
  const float flo = (float)y0 - 1.0f, fhi = (float)y1 + 1.0f;
#pragma unroll
  for (int e = 0; e < 3; e++) {
    const float ik = iks[e];
    if (ik == 0.0f) continue;
    const float B = -As[e] * ik;
    const float m = 3.814697265625e-06f * (N * fabsf(ik) + fabsf(B)) + 9.5367431640625e-07f;
    if (!(fabsf(B) < 1e30f) || !(m < 1e30f)) continue;
    if (ik > 0.0f) {
      const float b = fminf(fmaxf(B - m - biasy, flo), fhi);
      const int r = (int)ceilf(b);
      lo = r > lo ? r : lo;
    } else {
      const float b = fminf(fmaxf(B + m - biasy, flo), fhi);
      const int r = (int)floorf(b);
      hi = r < hi ? r : hi;
    }
  }
}

// warp_raster over column spans: same interface and result; warps whose faces
// have more than kMaxWarpCols columns in total take the bbox walk.
// cc (nullable, 32 entries, the warp's own): the faces' column_consts are
// stored there once and the columns read them instead of recomputing them.
template <class Sink>
__device__ __forceinline__ void warp_raster_spans(WarpFaces& wf, WarpCols& wc, const Setup& s, bool active,
                                                  uint32_t id, int cx0, int cx1, int cy0, int cy1,
                                                  const t3_frame& fr, Sink sink, ColConsts* cc = nullptr) {
  const unsigned FULL = 0xFFFFFFFFu;
  const int lane = threadIdx.x & 31;
  const int x0 = max(s.botx, cx0), x1 = min(s.topx, cx1);
  const int y0 = max(s.boty, cy0), y1 = min(s.topy, cy1);
  const int ncols = (active && x0 <= x1 && y0 <= y1) ? x1 - x0 + 1 : 0;
  const unsigned live = __ballot_sync(FULL, ncols > 0);
  if (!live) return;
  int incl = ncols;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += t;
  }
  const int total = __shfl_sync(FULL, incl, 31);
  // candidate positions are packed in 17 bits: bboxes of up to 2^17 pixels per
  // warp; columns averaging under three rows (faces of a pixel or two) gain
  // nothing from the spans and take the bbox walk too
  const unsigned area = ncols > 0 ? min((unsigned)ncols * (unsigned)(y1 - y0 + 1), 1u << 20) : 0u;
  const unsigned warp_area = __reduce_add_sync(FULL, area);
  if (total > kMaxWarpCols || warp_area >= (1u << 17) || warp_area < 3u * (unsigned)total) {
    warp_raster(wf, s, active, id, cx0, cx1, cy0, cy1, fr, sink);
    return;
  }
  const int first = incl - ncols;  // this face's first column
  if (ncols > 0) {
    const int r = __popc(live & ((1u << lane) - 1u));
    wf.rec[r][0] = make_float4(s.bx, s.by, s.cx, s.cy);
    wf.rec[r][1] = make_float4(s.bcnx, s.bcny, s.canx, s.cany);
    wf.rec[r][2] = make_float4(s.wsa, s.wsb, s.wsc, s.Az);
    wf.rec[r][3] = make_float4(s.Bz, s.Cz, __int_as_float(x0 | (y0 << 16)), __uint_as_float(id));
    wf.h[r] = y1 - y0 + 1;
    wf.start[r] = first;
    if (cc) cc[r] = column_consts(s, y0, y1, fr.bias[1]);
  }
  const unsigned upto = lane == 31 ? 0xFFFFFFFFu : ((2u << lane) - 1u);
  const unsigned below = (1u << lane) - 1u;
  const float biasx = fr.bias[0], biasy = fr.bias[1];
  __syncwarp();
  // 1. the candidate rows of every column; non-empty columns are listed in
  // order with the position of their first candidate
  int ncand = 0, npix = 0, before = 0;
  for (int base = 0; base < total; base += 32) {
    const unsigned bit = (ncols > 0 && first >= base && first < base + 32) ? 1u << (first - base) : 0u;
    const unsigned starts = __reduce_or_sync(FULL, bit);
    const int ci = base + lane;
    int cnt = 0, rlo = 0, x = 0, j = 0;
    if (ci < total) {
      j = before + __popc(starts & upto) - 1;
      const int xy = __float_as_int(wf.rec[j][3].z);
      x = (xy & 0xFFFF) + (ci - wf.start[j]);
      const int fy0 = xy >> 16;
      int rhi;
      if (cc) {
        const float4 r0 = wf.rec[j][0], r1 = wf.rec[j][1];
        column_rows_c(r0.x, r0.z, r1.y, r1.w, cc[j], x, fy0, fy0 + wf.h[j] - 1, biasx, biasy, rlo, rhi);
      } else {
        const float4 r0 = wf.rec[j][0], r1 = wf.rec[j][1], r2 = wf.rec[j][2];
        Setup t;
        t.bx = r0.x; t.by = r0.y; t.cx = r0.z; t.cy = r0.w;
        t.bcnx = r1.x; t.bcny = r1.y; t.canx = r1.z; t.cany = r1.w;
        t.wsa = r2.x; t.wsb = r2.y; t.wsc = r2.z;
        column_rows(t, x, fy0, fy0 + wf.h[j] - 1, biasx, biasy, rlo, rhi);
      }
      cnt = rhi >= rlo ? rhi - rlo + 1 : 0;
    }
    const unsigned m = __ballot_sync(FULL, cnt > 0);
    int pre = cnt;  // positions: inclusive scan of the counts
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(FULL, pre, o);
      if (lane >= o) pre += t;
    }
    if (cnt > 0) {
      const int k = ncand + __popc(m & below);
      wc.col[k] = make_int2(x | (j << 16), rlo | ((npix + pre - cnt) << 15));
    }
    ncand += __popc(m);
    npix += __shfl_sync(FULL, pre, 31);
    before += __popc(starts);
  }
  __syncwarp();
  // 2. the candidates, 32 at a time: a candidate's column is the last one
  // starting at or before it (found as in warp_raster, with the column starts
  // held in registers, five per lane)
  int cst[kMaxWarpCols / 32];
#pragma unroll
  for (int q = 0; q < kMaxWarpCols / 32; q++) {
    const int k = lane + 32 * q;
    cst[q] = k < ncand ? (int)((uint32_t)wc.col[k].y >> 15) : -1;
  }
  const float maxd = (float)fr.maxdepth;
  int cbefore = 0;
  for (int base = 0; base < npix; base += 32) {
    unsigned bits = 0u;
#pragma unroll
    for (int q = 0; q < kMaxWarpCols / 32; q++) {
      if (32 * q >= ncand) break;  // warp-uniform: no column starts in the registers from here on
      const unsigned d = (unsigned)(cst[q] - base);
      if (d < 32u) bits |= 1u << d;
    }
    const unsigned starts = __reduce_or_sync(FULL, bits);
    const int idx = base + lane;
    if (idx < npix) {
      const int k = cbefore + __popc(starts & upto) - 1;
      const int2 cd = wc.col[k];
      const int j = (cd.x >> 16) & 31;
      const int y = (cd.y & 0x7FFF) + (idx - (int)((uint32_t)cd.y >> 15));
      const float4 r0 = wf.rec[j][0], r1 = wf.rec[j][1], r2 = wf.rec[j][2], r3 = wf.rec[j][3];
      Setup t;
      t.bx = r0.x; t.by = r0.y; t.cx = r0.z; t.cy = r0.w;
      t.bcnx = r1.x; t.bcny = r1.y; t.canx = r1.z; t.cany = r1.w;
      t.wsa = r2.x; t.wsb = r2.y; t.wsc = r2.z; t.Az = r2.w;
      t.Bz = r3.x; t.Cz = r3.y;
      test_pixel(t, cd.x & 0xFFFF, y, __float_as_uint(r3.w), biasx, biasy, maxd, fr.maxdepth, sink);
    }
    cbefore += __popc(starts);
  }
  __syncwarp();
}

// Loads (and transforms) the corners of face n; soup positions come from the
// block's shared-memory staging area when `staged`.
__device__ __forceinline__ void load_face(const t3_mesh& mesh, int64_t n, bool staged,
                                          const float* sv, f3 v[3], int slot = -1) {
  if (staged) {
    const float* p = sv + (slot < 0 ? (int)threadIdx.x : slot) * 9;
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
__device__ __forceinline__ bool stage_soup(const t3_mesh& mesh, int64_t nfaces, int64_t f0, float* sv,
                                           int nmax = BLOCK) {
  const bool staged = mesh.kind == T3_MESH_SOUP && !(mesh.flags & T3_MESH_NOCULL);
  if (staged) {
    const int64_t rem = nfaces - f0;
    const int nf = rem < nmax ? (int)(rem > 0 ? rem : 0) : nmax;
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
