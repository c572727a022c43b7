// raster.cu -- depth-key clear and the direct rasteriser.
//
// TriangleRaster.render_occup (tina/core/triangle.py:89-131) as a GB300 kernel:
// one thread per face runs the vertex transform, back-face cull, trivial clip,
// viewport map, bbox and edge setup; the warp then rasterises its 32 faces
// cooperatively (t3_raster.cuh) and folds every covered pixel into a packed
// 64-bit key (depth ^ sign bit) << 32 | face id with atomicMin.  The unsigned
// minimum of that key is the serial reference's winner: lowest int32 depth,
// ties to the lowest face id (the strict `>` at triangle.py:123), so the result
// does not depend on thread order and the reference's racy `occup[P] = f`
// store disappears.
//
// Face-soup vertex positions (9 floats per face) are staged into shared memory
// with 16-byte vector loads so a warp reads its 1152 contiguous bytes once.
// Faces whose clamped bbox exceeds `big_threshold` pixels are queued and
// rasterised by k_raster_big, where every CTA takes a slice of each queued
// face's bbox.
#include "t3_raster.cuh"

namespace t3 {

// key buffer <- empty; also zeroes `ncounters` frame counters and the status
// word (one launch where the frame needs no device copy of the scene).  With a
// key state (t3_render's direct frames) the keys are left alone when the tag
// says the previous frame's shading emptied them; the last block to finish
// then marks them as not known to be empty.
__global__ void k_clear(unsigned long long* __restrict__ keys, int64_t n, uint32_t* __restrict__ counters,
                        int ncounters, int32_t* __restrict__ status, KeyState ks) {
  __shared__ int s_skip;
  if (threadIdx.x == 0)
    s_skip = ks.tag_word && ks.tag != 0ull && *(volatile unsigned long long*)ks.tag_word == ks.tag;
  __syncthreads();
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ncounters) counters[i] = 0u;
  if (i == 0 && status) *status = 0;
  if (!s_skip) {
    if ((reinterpret_cast<uintptr_t>(keys) & 15) == 0) {
      ulonglong2* k2 = reinterpret_cast<ulonglong2*>(keys);
      const int64_t n2 = n >> 1;
      for (int64_t j = i; j < n2; j += stride) k2[j] = make_ulonglong2(T3_EMPTY_KEY, T3_EMPTY_KEY);
      if (i == 0 && (n & 1)) keys[n - 1] = T3_EMPTY_KEY;
    } else {
      for (int64_t j = i; j < n; j += stride) keys[j] = T3_EMPTY_KEY;
    }
  }
  if (ks.tag_word && threadIdx.x == 0) {
    // this block has read the tag: order that read before the ticket
    __threadfence();
    if (atomicAdd(ks.ticket, 1u) == gridDim.x - 1) {
      *ks.tag_word = 0ull;
      *ks.ticket = 0u;
    }
  }
}

template <bool COUNT>
struct GlobalKeySink {
  unsigned long long* keys;
  int64_t H;
  unsigned long long* fragments;  // COUNT (statistics runs only): every reduction is counted
  __device__ __forceinline__ void operator()(int x, int y, unsigned long long key) const {
    if constexpr (COUNT) atomicAdd(fragments, 1ull);
    // fire-and-forget reduction (no return value, so no load latency on the
    // fragment path)
    atomicMin(keys + (int64_t)x * H + y, key);
  }
};

// `fpw` faces per warp (a power of two up to 32): lanes below fpw take one
// face each.  Small meshes use fewer than 32 so that more warps share the
// walk of their pixels (a mesh of a few thousand faces fills only a few SMs
// at 32 faces per warp, and each warp's walk is a long serial chain).
template <int BLOCK, bool COUNT>
__global__ void __launch_bounds__(BLOCK, 1536 / BLOCK)
k_raster_direct(const t3_frame fr, const t3_mesh mesh, int64_t nfaces, uint32_t face_base,
                unsigned long long* __restrict__ keys, BigQueue big, int32_t big_threshold, int fpw) {
  __shared__ __align__(16) float sv[BLOCK * 9];
  __shared__ WarpFaces wfs[BLOCK / 32];
  __shared__ WarpCols wcs[BLOCK / 32];
  const int per_block = (BLOCK / 32) * fpw;
  const int64_t f0 = (int64_t)blockIdx.x * per_block;
  const bool staged = stage_soup<BLOCK>(mesh, nfaces, f0, sv, per_block);
  const int lane = threadIdx.x & 31;
  const int slot = (threadIdx.x >> 5) * fpw + lane;  // this lane's face within the block
  const int64_t n = f0 + slot;
  Setup s{};
  bool vis = false;
  if (lane < fpw && n < nfaces) {
    if (big.vndc) {
      // transformed corners from the vertex stage
      const FaceRef ref = face_ref(mesh, n);
      float4 c[3];
#pragma unroll
      for (int k = 0; k < 3; k++) c[k] = __ldg(big.vndc + corner_vertex(mesh, ref.f, k));
      vis = face_setup_ndc(fr, ref.flip ? c[2] : c[0], c[1], ref.flip ? c[0] : c[2], s);
    } else {
      f3 v[3];
      load_face(mesh, n, staged, sv, v, slot);
      vis = face_setup(fr, v, s);
    }
    vis = vis && s.botx <= s.topx && s.boty <= s.topy;
  }
  if (vis) {
    if (big.rec) store_record(big.rec, face_base + (uint32_t)n, s);
    const int64_t area = (int64_t)(s.topx - s.botx + 1) * (int64_t)(s.topy - s.boty + 1);
    if (area > big_threshold) {
      const uint32_t slot = atomicAdd(big.count, 1u);
      if (slot < big.capacity) big.items[slot] = (uint32_t)n;
      else atomicOr(big.status, T3_STATUS_BIG_OVERFLOW);
      vis = false;
    }
  }
  // the staged positions are read: each warp's 1,152 bytes of them hold its
  // faces' column constants from here on
  static_assert(sizeof(ColConsts) * 32 <= 32 * 9 * sizeof(float), "column constants outgrow the staging area");
  __syncthreads();
  ColConsts* cc = reinterpret_cast<ColConsts*>(sv + (threadIdx.x >> 5) * 32 * 9);
  GlobalKeySink<COUNT> sink{keys, fr.height, big.fragments};
  warp_raster_spans(wfs[threadIdx.x >> 5], wcs[threadIdx.x >> 5], s, vis, face_base + (uint32_t)n, 0,
                    fr.width - 1, 0, fr.height - 1, fr, sink, cc);
}

// Large faces: every CTA walks a slice of every queued face's bbox.  The
// queued faces' setups are read 32 at a time into shared memory (one round
// of loads for the chunk instead of a dependent load chain per face).
template <int BLOCK, bool COUNT>
__global__ void __launch_bounds__(BLOCK)
k_raster_big(const t3_frame fr, const t3_mesh mesh, uint32_t face_base,
             unsigned long long* __restrict__ keys, BigQueue big) {
  constexpr int kChunk = 32;
  __shared__ Setup s_face[kChunk];
  __shared__ uint32_t s_id[kChunk];
  const uint32_t count = min(*big.count, big.capacity);
  const float maxd = (float)fr.maxdepth;
  GlobalKeySink<COUNT> sink{keys, fr.height, big.fragments};
  const int64_t stride = (int64_t)gridDim.x * BLOCK;
  for (uint32_t e0 = 0; e0 < count; e0 += kChunk) {
    const uint32_t m = min((uint32_t)kChunk, count - e0);
    __syncthreads();  // the previous chunk's faces are walked
    if (threadIdx.x < m) {
      const uint32_t n = big.items[e0 + threadIdx.x];
      Setup s;
      if (big.rec) {
        // the setup record k_raster_direct stored for the face
        load_record(big.rec, face_base + n, s);
      } else {
        f3 v[3];
        face_verts(mesh, face_ref(mesh, n), v);
        if (!face_setup(fr, v, s)) s.topx = s.botx - 1;  // nothing to walk
      }
      s_face[threadIdx.x] = s;
      s_id[threadIdx.x] = face_base + n;
    }
    __syncthreads();
    for (uint32_t e = 0; e < m; e++) {
      const Setup& s = s_face[e];
      if (s.topx < s.botx || s.topy < s.boty) continue;
      const int32_t h = s.topy - s.boty + 1;
      const int64_t area = (int64_t)(s.topx - s.botx + 1) * h;
      const uint32_t id = s_id[e];
      for (int64_t k = (int64_t)blockIdx.x * BLOCK + threadIdx.x; k < area; k += stride) {
        // bboxes are clamped to the frame (at most 65535 rows), so the
        // column / row split fits 32-bit arithmetic when the area does
        int32_t q, r;
        if (area <= INT32_MAX) {
          q = (int32_t)k / h;
          r = (int32_t)k - q * h;
        } else {
          q = (int32_t)(k / h);
          r = (int32_t)(k - (int64_t)q * h);
        }
        const int32_t x = s.botx + q, y = s.boty + r;
        const float px = xadd((float)x, fr.bias[0]);
        const float py = xadd((float)y, fr.bias[1]);
        float wx, wy, wz, sum;
        face_raw_weights(s, px, py, wx, wy, wz, sum);
        f3 wei;
        if (!face_inside(wx, wy, wz, sum, wei)) continue;
        const int32_t d = trunc_i32(xmul(face_depth(s, wei), maxd));
        if (d >= fr.maxdepth) continue;
        sink(x, y, pack_key(d, id));
      }
    }
  }
}

cudaError_t launch_clear(unsigned long long* keys, int64_t n, cudaStream_t st, uint32_t* counters,
                         int ncounters, int32_t* status, KeyState ks) {
  const int block = 256;
  int64_t want = ((n >> 1) + block - 1) / block;
  // with a key state, a grid that exits quickly when the keys are already
  // empty (four CTAs per SM stride over the buffer when they are not); one
  // block when the host expects them to be empty
  const int64_t cap = ks.tag_word ? (ks.likely_empty ? 1 : 4 * 152) : 4 * 152 * 8;
  int64_t grid = want < cap ? want : cap;
  if (grid * block < ncounters) grid = (ncounters + block - 1) / block;
  if (grid < 1) grid = 1;
  k_clear<<<(unsigned)grid, block, 0, st>>>(keys, n, counters, ncounters, status, ks);
  return cudaGetLastError();
}

cudaError_t launch_raster_direct(const t3_frame& fr, const t3_object& ob, unsigned long long* keys,
                                 const BigQueue& big, int32_t big_threshold, cudaStream_t st) {
  if (ob.nfaces <= 0) return cudaSuccess;
  // four warps per CTA: a CTA's slot is held until its slowest warp's walk
  // ends, and smaller CTAs leave less of it idle (measured 0.7 us per 1080p
  // soup frame against eight warps)
  constexpr int BLOCK = 128;
  // faces per warp: 32 once the mesh fills every SM's warps (152 SMs x 48),
  // fewer below that, down to one face per warp
  int fpw = 32;
  while (fpw > 1 && ob.nfaces < (int64_t)152 * 48 * fpw) fpw >>= 1;
  const int64_t per_block = (BLOCK / 32) * fpw;
  const int64_t grid = (ob.nfaces + per_block - 1) / per_block;
  // big.count was zeroed at the start of the frame
  if (big.fragments) {
    k_raster_direct<BLOCK, true><<<(unsigned)grid, BLOCK, 0, st>>>(fr, ob.mesh, ob.nfaces,
                                                                  (uint32_t)ob.face_base, keys, big,
                                                                  big_threshold, fpw);
    k_raster_big<256, true><<<152, 256, 0, st>>>(fr, ob.mesh, (uint32_t)ob.face_base, keys, big);
    return cudaGetLastError();
  }
  k_raster_direct<BLOCK, false><<<(unsigned)grid, BLOCK, 0, st>>>(fr, ob.mesh, ob.nfaces,
                                                                 (uint32_t)ob.face_base, keys, big,
                                                                 big_threshold, fpw);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_raster_big<256, false><<<152, 256, 0, st>>>(fr, ob.mesh, (uint32_t)ob.face_base, keys, big);
  return cudaGetLastError();
}

// ---- particles (ParticleRaster.render_occup, tina/core/particle.py:74-114) ----
// One thread per particle computes its screen bbox; the warp then walks the
// 32 particles' bbox pixels cooperatively (as warp_raster does for faces) and
// keeps the pixels whose world point at the particle's depth lies within the
// radius; every pixel of a particle has the particle's depth.
struct WarpPars {
  float4 rec[32][2];  // (ax, ay, az, r2) (vz, depth, x0 | y0 << 16, id)
  int h[32];
  long long start[32];
};

template <int BLOCK, bool COUNT>
__global__ void __launch_bounds__(BLOCK)
k_raster_particles(const t3_frame fr, const t3_mesh mesh, int64_t npars, uint32_t face_base,
                   unsigned long long* __restrict__ keys, unsigned long long* fragments) {
  __shared__ WarpPars wps[BLOCK / 32];
  const unsigned FULL = 0xFFFFFFFFu;
  const int lane = threadIdx.x & 31;
  WarpPars& wp = wps[threadIdx.x >> 5];
  GlobalKeySink<COUNT> sink{keys, fr.height, fragments};
  const int64_t n = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  ParSetup p{};
  bool live = false;
  if (n < npars) {
    live = particle_setup(fr, ld3(mesh.verts + n * 3), __ldg(mesh.coors + n), p) && p.depth < fr.maxdepth;
  }
  const long long area = live ? (long long)(p.topx - p.botx + 1) * (p.topy - p.boty + 1) : 0;
  const unsigned lm = __ballot_sync(FULL, area > 0);
  if (!lm) return;
  long long incl = area;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long t = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += t;
  }
  const long long first = incl - area;
  if (area > 0) {
    const int r = __popc(lm & ((1u << lane) - 1u));
    wp.rec[r][0] = make_float4(p.ax, p.ay, p.az, p.r2);
    wp.rec[r][1] = make_float4(p.vz, __int_as_float(p.depth), __int_as_float(p.botx | (p.boty << 16)),
                               __uint_as_float(face_base + (uint32_t)n));
    wp.h[r] = p.topy - p.boty + 1;
    wp.start[r] = first;
  }
  const long long total = __shfl_sync(FULL, incl, 31);
  const unsigned upto = lane == 31 ? 0xFFFFFFFFu : ((2u << lane) - 1u);
  __syncwarp();
  int before = 0;
  for (long long base = 0; base < total; base += 32) {
    const unsigned bit = (area > 0 && first >= base && first < base + 32) ? 1u << (int)(first - base) : 0u;
    const unsigned starts = __reduce_or_sync(FULL, bit);
    const long long idx = base + lane;
    if (idx < total) {
      const int j = before + __popc(starts & upto) - 1;
      const long long off = idx - wp.start[j];
      const int h = wp.h[j];
      const int q = (int)(off / h), r = (int)(off - (long long)q * h);
      const float4 a = wp.rec[j][0], b = wp.rec[j][1];
      ParSetup t;
      t.ax = a.x; t.ay = a.y; t.az = a.z; t.r2 = a.w;
      const int xy = __float_as_int(b.z);
      const int x = (xy & 0xFFFF) + q, y = (xy >> 16) + r;
      const f3 Pl = particle_pixel_world(fr, xadd((float)x, fr.bias[0]), xadd((float)y, fr.bias[1]), b.x);
      if (particle_covers(t, Pl)) sink(x, y, pack_key(__float_as_int(b.y), __float_as_uint(b.w)));
    }
    before += __popc(starts);
  }
}

cudaError_t launch_raster_particles(const t3_frame& fr, const t3_object& ob, unsigned long long* keys,
                                    unsigned long long* fragments, cudaStream_t st) {
  if (ob.nfaces <= 0) return cudaSuccess;
  constexpr int BLOCK = 128;
  const unsigned grid = (unsigned)((ob.nfaces + BLOCK - 1) / BLOCK);
  if (fragments)
    k_raster_particles<BLOCK, true><<<grid, BLOCK, 0, st>>>(fr, ob.mesh, ob.nfaces, (uint32_t)ob.face_base,
                                                            keys, fragments);
  else
    k_raster_particles<BLOCK, false><<<grid, BLOCK, 0, st>>>(fr, ob.mesh, ob.nfaces, (uint32_t)ob.face_base,
                                                             keys, nullptr);
  return cudaGetLastError();
}

// ---- wireframe (WireframeRaster.render_color, tina/core/wireframe.py:69-97) ----
// One thread per line runs the setup and finds, by bisection, the steps whose
// pixel lies inside the frame; the warp then walks the 32 lines' steps
// cooperatively.  Every step is the reference's DDA step with its own depth
// interpolation, folded into the packed key like a triangle fragment (the
// shading pass writes the raster's line colour where a line wins).
struct WarpWires {
  float4 rec[32][2];  // (ax, ay, kx, ky) (az, bz, wsa, wsb)
  int4 meta[32];      // (siz, lo, id, -)
  long long start[32];
};

template <int BLOCK, bool COUNT>
__global__ void __launch_bounds__(BLOCK)
k_raster_wires(const t3_frame fr, const t3_mesh mesh, int64_t nwires, uint32_t face_base,
               unsigned long long* __restrict__ keys, unsigned long long* fragments) {
  __shared__ WarpWires wws[BLOCK / 32];
  const unsigned FULL = 0xFFFFFFFFu;
  const int lane = threadIdx.x & 31;
  WarpWires& ww = wws[threadIdx.x >> 5];
  GlobalKeySink<COUNT> sink{keys, fr.height, fragments};
  const int64_t n = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
  WireSetup s{};
  bool live = false;
  if (n < nwires) {
    f3 A, B;
    wire_endpoints(mesh, n, A, B);
    live = wire_setup(fr, A, B, s);
  }
  const long long cnt = live ? (long long)s.hi - s.lo + 1 : 0;
  const unsigned lm = __ballot_sync(FULL, cnt > 0);
  if (!lm) return;
  long long incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long t = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += t;
  }
  const long long first = incl - cnt;
  if (cnt > 0) {
    const int r = __popc(lm & ((1u << lane) - 1u));
    ww.rec[r][0] = make_float4(s.ax, s.ay, s.kx, s.ky);
    ww.rec[r][1] = make_float4(s.az, s.bz, s.wsa, s.wsb);
    ww.meta[r] = make_int4(s.siz, s.lo, (int)(face_base + (uint32_t)n), 0);
    ww.start[r] = first;
  }
  const long long total = __shfl_sync(FULL, incl, 31);
  const unsigned upto = lane == 31 ? 0xFFFFFFFFu : ((2u << lane) - 1u);
  __syncwarp();
  int before = 0;
  for (long long base = 0; base < total; base += 32) {
    const unsigned bit = (cnt > 0 && first >= base && first < base + 32) ? 1u << (int)(first - base) : 0u;
    const unsigned starts = __reduce_or_sync(FULL, bit);
    const long long idx = base + lane;
    if (idx < total) {
      const int j = before + __popc(starts & upto) - 1;
      const float4 a = ww.rec[j][0], b = ww.rec[j][1];
      const int4 m = ww.meta[j];
      WireSetup t;
      t.ax = a.x; t.ay = a.y; t.kx = a.z; t.ky = a.w;
      t.az = b.x; t.bz = b.y; t.wsa = b.z; t.wsb = b.w;
      t.siz = m.x;
      const int32_t i = m.y + (int32_t)(idx - ww.start[j]);
      int x, y;
      int32_t depth;
      if (wire_step(fr, t, i, x, y, depth)) sink(x, y, pack_key(depth, (uint32_t)m.z));
    }
    before += __popc(starts);
  }
}

cudaError_t launch_raster_wires(const t3_frame& fr, const t3_object& ob, unsigned long long* keys,
                                unsigned long long* fragments, cudaStream_t st) {
  if (ob.nfaces <= 0) return cudaSuccess;
  constexpr int BLOCK = 128;
  const unsigned grid = (unsigned)((ob.nfaces + BLOCK - 1) / BLOCK);
  if (fragments)
    k_raster_wires<BLOCK, true><<<grid, BLOCK, 0, st>>>(fr, ob.mesh, ob.nfaces, (uint32_t)ob.face_base,
                                                        keys, fragments);
  else
    k_raster_wires<BLOCK, false><<<grid, BLOCK, 0, st>>>(fr, ob.mesh, ob.nfaces, (uint32_t)ob.face_base,
                                                         keys, nullptr);
  return cudaGetLastError();
}

// u64 atomicMin throughput: n distinct addresses (L2 resident for n * 8 below
// the L2 size), `rounds` reductions each, with decreasing values so every
// reduction changes memory like a winning fragment does
__global__ void k_red_min_rate(unsigned long long* __restrict__ buf, int64_t n, int rounds) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int r = 0; r < rounds; r++)
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
      atomicMin(buf + i, (unsigned long long)(rounds - r) << 32 | (unsigned long long)i);
}

cudaError_t launch_red_min_rate(unsigned long long* buf, int64_t n, int rounds, cudaStream_t st) {
  k_red_min_rate<<<152 * 8, 256, 0, st>>>(buf, n, rounds);
  return cudaGetLastError();
}

} // namespace t3
