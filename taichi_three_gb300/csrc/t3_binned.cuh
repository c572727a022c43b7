// t3_binned.cuh -- the binned tile rasteriser with fused deferred shading:
// the per-block and per-tile bodies shared by the single-view kernels
// (binned.cu) and the batched ones (batch_binned.cu).
//
// Same results as the direct path (TriangleRaster.render_occup + render_color,
// tina/core/triangle.py:89-153): bit-exact face id / depth, identical shading.
// Two kernels per frame (after the scene upload):
//
//  k_bin   one thread per face: vertex transform, cull, clip and edge setup;
//          a visible face stores its 64-byte setup record at its global id and
//          appends that id to the fixed-capacity bin of every screen tile its
//          bbox touches.  Appends are warp-aggregated: __match_any_sync groups
//          the lanes that hit the same tile, the group leader reserves the
//          slots with one atomicAdd and every lane takes base + popc(lanes
//          below it in the group) -- a warp-ballot prefix sum.  Faces touching
//          more than `big_tiles` tiles go to a ballot-compacted big-face list.
//  k_tile  one CTA per tile: TMA (cp.async.bulk) stages the tile's bin into
//          shared memory under an mbarrier, in chunks of at most kQueueMax
//          entries (a chunk is rasterised before the next is copied, so a bin
//          of any capacity fits); the warps rasterise the binned
//          faces (and the big faces overlapping the tile) cooperatively
//          (t3_raster.cuh) into a tile of 64-bit packed (depth, id) keys in
//          shared memory with atomicMin; then the CTA shades the tile's pixels
//          from those keys, reusing the setup records, and writes rgb / id /
//          depth / depth_f once.  No global key buffer and no clear pass.
//
// The mbarrier wait is bounded: when it runs out the kernel records
// T3_STATUS_TIMEOUT, waits once more (bounded) for its own copy, and writes
// the tile as background.  A bin that overflows its capacity sets
// T3_STATUS_BIN_OVERFLOW (the host retries with a larger capacity).
#pragma once

#include "t3_raster.cuh"
#include "t3_shading.cuh"

namespace t3 {

// One block's share of k_bin: faces [f0, f0 + BLOCK) of one object.  Every
// thread of the block calls it (the soup staging has a block barrier).
template <int BLOCK>
__device__ __forceinline__ void bin_faces(const t3_frame& fr, const t3_mesh& mesh, int64_t nfaces,
                                          uint32_t face_base, const BinArgs& bins, int64_t f0,
                                          float* sv) {
  const bool staged = stage_soup<BLOCK>(mesh, nfaces, f0, sv);
  const int64_t n = f0 + threadIdx.x;
  bool vis = false;
  Setup s{};
  if (n < nfaces) {
    f3 v[3];
    load_face(mesh, n, staged, sv, v);
    vis = face_setup(fr, v, s) && s.botx <= s.topx && s.boty <= s.topy;
  }
  const uint32_t gid = face_base + (uint32_t)n;
  int tx0 = 0, tx1 = -1, ty0 = 0, ty1 = -1;
  if (vis) {
    store_record(bins.rec, gid, s);
    tx0 = s.botx / bins.tile; tx1 = s.topx / bins.tile;
    ty0 = s.boty / bins.tile; ty1 = s.topy / bins.tile;
  }
  const int ntl = vis ? (tx1 - tx0 + 1) * (ty1 - ty0 + 1) : 0;
  const bool big = ntl > bins.big_tiles;
  const unsigned FULL = 0xFFFFFFFFu;
  const int lane = threadIdx.x & 31;
  // big faces: ballot-compacted append to the big-face list
  const unsigned bigmask = __ballot_sync(FULL, big);
  if (bigmask) {
    const int leader = __ffs(bigmask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(bins.big_count, (uint32_t)__popc(bigmask));
    base = __shfl_sync(FULL, base, leader);
    if (big) {
      const uint32_t slot = base + __popc(bigmask & ((1u << lane) - 1u));
      if (slot < bins.big_capacity) bins.big[slot] = gid;
      else atomicOr(bins.status, T3_STATUS_BIG_OVERFLOW);
    }
  }
  // small faces: one append per covered tile, aggregated across the warp
  const int mine = big ? 0 : ntl;
  const int w = tx1 - tx0 + 1;
  for (int k = 0;; k++) {
    const bool want = k < mine;
    const unsigned active = __ballot_sync(FULL, want);
    if (!active) break;
    if (want) {
      const int tile = (ty0 + k / w) * bins.tiles_x + (tx0 + k % w);
      const unsigned grp = __match_any_sync(active, tile);
      const int leader = __ffs(grp) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(bins.count + tile, (uint32_t)__popc(grp));
      base = __shfl_sync(grp, base, leader);
      const uint32_t slot = base + __popc(grp & ((1u << lane) - 1u));
      if (slot < bins.capacity) bins.bins[(size_t)tile * bins.capacity + slot] = gid;
      else atomicOr(bins.status, T3_STATUS_BIN_OVERFLOW);
    }
  }
}


// ---- the tile body -----------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// bounded wait on phase `parity` of an mbarrier; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint32_t limit) {
  for (uint32_t it = 0; it < limit; it++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done) : "r"(bar), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}

struct SmemKeySink {
  unsigned long long* keys;
  int x0, y0;
  __device__ __forceinline__ void operator()(int x, int y, unsigned long long key) const {
    atomicMin(keys + (x - x0) * TS_DYN + (y - y0), key);
  }
  int TS_DYN;
};

// bin entries staged per chunk (16 KB): the dynamic shared memory of a tile
// CTA is TS * TS * 8 bytes of keys + 4 * min(capacity, kQueueMax) bytes
constexpr uint32_t kQueueMax = 4096;
__host__ __device__ __forceinline__ uint32_t queue_entries(uint32_t capacity) {
  return capacity < kQueueMax ? capacity : kQueueMax;
}

// The static shared state of a tile CTA.
template <int TS, int BLOCK>
struct TileShared {
  WarpFaces wfs[BLOCK / 32];
  WarpCols wcs[BLOCK / 32];
  unsigned long long bar;
  int ok;
  int list[TS * TS];
  int count;
};

// One tile of one view: its bin (in chunks) and the big faces rasterised into
// shared-memory keys, then the tile shaded (or, for the learned IBL, its keys
// handed to the network pass).  keys: TS * TS entries, queue: qcap entries
// (a multiple of 4) of dynamic shared memory.  Every thread of the CTA calls it.
template <int TS, int BLOCK, int NL, int MODE, bool TEX = true, int SIG = 0>
__device__ __forceinline__ void tile_body(const DevScene* __restrict__ sc, const BinArgs& bins,
                                          const t3_outputs& out, int tile, TileShared<TS, BLOCK>& sh,
                                          unsigned long long* keys, uint32_t* queue, uint32_t qcap) {
  const t3_frame& fr = sc->frame;
  const int W = fr.width, H = fr.height;
  const int tx = tile % bins.tiles_x, ty = tile / bins.tiles_x;
  const int x0 = tx * TS, y0 = ty * TS;
  const int x1 = min(x0 + TS - 1, W - 1), y1 = min(y0 + TS - 1, H - 1);
  const uint32_t n = min(bins.count[tile], bins.capacity);
  const uint32_t bar_a = smem_u32(&sh.bar);
  const unsigned FULL = 0xFFFFFFFFu;

  if (threadIdx.x == 0) {
    sh.ok = 1;
    sh.count = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar_a), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int i = threadIdx.x; i < TS * TS; i += BLOCK) {
    unsigned long long k = T3_EMPTY_KEY;
    const int x = x0 + i / TS, y = y0 + i % TS;
    if (bins.pre && x <= x1 && y <= y1) k = bins.pre[(int64_t)x * H + y];
    keys[i] = k;
  }
  __syncthreads();

  SmemKeySink sink{keys, x0, y0, TS};
  WarpFaces& wf = sh.wfs[threadIdx.x >> 5];
  const int warp = threadIdx.x >> 5;
  constexpr int NW = BLOCK / 32;
  // T3_STARVE_BIN_COPY (tests of the timeout path): nothing is issued and
  // nothing arrives, so the first wait below runs out
  const bool starve = (fr.flags & T3_STARVE_BIN_COPY) != 0;
  const uint32_t first_limit = fr.wait_limit > 0 ? (uint32_t)fr.wait_limit : (1u << 22);
  const uint32_t* bin = bins.bins + (size_t)tile * bins.capacity;
  uint32_t parity = 0;
  for (uint32_t c0 = 0; c0 < n || (starve && c0 == 0); c0 += qcap) {
    const uint32_t cnt = min(qcap, n - c0);
    // a bulk copy moves 16-byte multiples from a 16-byte aligned address: the
    // bin starts so (capacity % 4 == 0) and chunks start at multiples of qcap
    const uint32_t bytes = ((cnt * 4u) + 15u) & ~15u;
    if (threadIdx.x == 0 && !starve) {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar_a), "r"(bytes) : "memory");
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
          :: "r"(smem_u32(queue)), "l"(bin + c0), "r"(bytes), "r"(bar_a) : "memory");
    }
    if (!mbar_wait(bar_a, parity, first_limit)) {
      sh.ok = 0;
      // let our own copy land before the shared memory is reused (when one was issued)
      if (!starve) mbar_wait(bar_a, parity, 1u << 22);
    }
    parity ^= 1u;
    __syncthreads();
    if (!sh.ok) break;  // block-uniform
    // this chunk's faces, 32 per warp per round (the round count is warp-uniform)
    for (uint32_t base = warp * 32; base < cnt; base += NW * 32) {
      const uint32_t i = base + (threadIdx.x & 31);
      Setup s{};
      uint32_t gid = 0;
      const bool act = i < cnt;
      if (act) {
        gid = queue[i];
        load_record(bins.rec, gid, s);
      }
      warp_raster_spans(wf, sh.wcs[warp], s, act, gid, x0, x1, y0, y1, fr, sink);
    }
    __syncthreads();  // the queue is refilled by the next chunk
  }
  const bool ok = sh.ok != 0;
  if (!ok && threadIdx.x == 0) atomicOr(bins.status, T3_STATUS_TIMEOUT);
  if (ok) {
    // big faces overlapping the tile
    const uint32_t nbig = min(*bins.big_count, bins.big_capacity);
    for (uint32_t base = warp * 32; base < nbig; base += NW * 32) {
      const uint32_t i = base + (threadIdx.x & 31);
      Setup s{};
      uint32_t gid = 0;
      bool act = i < nbig;
      if (act) {
        gid = __ldg(bins.big + i);
        load_record(bins.rec, gid, s);
        act = !(s.botx > x1 || s.topx < x0 || s.boty > y1 || s.topy < y0);
      }
      if (__ballot_sync(FULL, act)) warp_raster_spans(wf, sh.wcs[warp], s, act, gid, x0, x1, y0, y1, fr, sink);
    }
  }
  __syncthreads();

  if constexpr (MODE == T3_LIGHT_IBL_MLP) {
    // the network runs in the fused shading pass: hand the keys to it
    for (int i = threadIdx.x; i < TS * TS; i += BLOCK) {
      const int x = x0 + i / TS, y = y0 + i % TS;
      if (x <= x1 && y <= y1) bins.keys[(int64_t)x * H + y] = ok ? keys[i] : T3_EMPTY_KEY;
    }
  } else {
    // shade the tile: empty pixels at once, covered ones compacted so full warps
    // run the shading (consecutive threads take consecutive y: contiguous memory)
    const V3 bg = background(fr);
    const int lane = threadIdx.x & 31;
    for (int i0 = 0; i0 < TS * TS; i0 += BLOCK) {
      const int i = i0 + threadIdx.x;
      const int x = x0 + i / TS, y = y0 + i % TS;
      bool covered = false;
      if (i < TS * TS && x <= x1 && y <= y1) {
        if (MODE == T3_LIGHT_LAMPS && (!ok || keys[i] == T3_EMPTY_KEY))
          write_empty(fr, out, (int64_t)x * H + y, bg);
        else
          covered = true;
      }
      const unsigned m = __ballot_sync(FULL, covered);
      if (m) {
        int slot = 0;
        if (lane == 0) slot = atomicAdd(&sh.count, __popc(m));
        slot = __shfl_sync(FULL, slot, 0);
        if (covered) sh.list[slot + __popc(m & ((1u << lane) - 1u))] = i;
      }
    }
    __syncthreads();
    const int ncov = sh.count;
    for (int j = threadIdx.x; j < ncov; j += BLOCK) {
      const int i = sh.list[j];
      shade_pixel_from_key<NL, MODE, false, TEX, SIG>(sc, bins.rec, ok ? keys[i] : T3_EMPTY_KEY,
                                                      x0 + i / TS, y0 + i % TS, out);
    }
  }
  __syncthreads();  // the shared state is reused by the CTA's next tile
  if (threadIdx.x == 0) asm volatile("mbarrier.inval.shared::cta.b64 [%0];" :: "r"(bar_a) : "memory");
}

} // namespace t3
