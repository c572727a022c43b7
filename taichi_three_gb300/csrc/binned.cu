// binned.cu -- the binned tile rasteriser with fused deferred shading.
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
//          shared memory under an mbarrier; the warps rasterise the binned
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
#include "t3_raster.cuh"
#include "t3_shading.cuh"

namespace t3 {

// ---- k_bin -------------------------------------------------------------------
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
k_bin(const t3_frame fr, const t3_mesh mesh, int64_t nfaces, uint32_t face_base, BinArgs bins) {
  __shared__ __align__(16) float sv[BLOCK * 9];
  const int64_t f0 = (int64_t)blockIdx.x * BLOCK;
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

// ---- k_tile --------------------------------------------------------------------
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

template <int TS, int BLOCK, int NL, int MODE>
__global__ void __launch_bounds__(BLOCK, BLOCK == 256 ? 3 : 6)
k_tile(const DevScene* __restrict__ sc, BinArgs bins, t3_outputs out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(smem_raw);  // TS*TS
  uint32_t* queue = reinterpret_cast<uint32_t*>(smem_raw + TS * TS * 8);        // capacity
  __shared__ WarpFaces wfs[BLOCK / 32];
  __shared__ WarpCols wcs[BLOCK / 32];
  __shared__ __align__(8) unsigned long long bar;
  __shared__ int s_ok;
  __shared__ int s_list[TS * TS];
  __shared__ int s_count;

  const t3_frame& fr = sc->frame;
  const int W = fr.width, H = fr.height;
  const int tile = blockIdx.x;
  const int tx = tile % bins.tiles_x, ty = tile / bins.tiles_x;
  const int x0 = tx * TS, y0 = ty * TS;
  const int x1 = min(x0 + TS - 1, W - 1), y1 = min(y0 + TS - 1, H - 1);
  const uint32_t n = min(bins.count[tile], bins.capacity);
  const uint32_t bar_a = smem_u32(&bar);
  const unsigned FULL = 0xFFFFFFFFu;

  if (threadIdx.x == 0) {
    s_ok = 1;
    s_count = 0;
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
  // stage this tile's bin with one bulk copy: 16-byte multiples from the
  // 16-byte aligned start of a capacity-sized bin (capacity % 4 == 0)
  const uint32_t bytes = ((n * 4u) + 15u) & ~15u;
  // T3_STARVE_BIN_COPY (tests of the timeout path): nothing is issued and
  // nothing arrives, so the first wait below runs out
  const bool starve = (fr.flags & T3_STARVE_BIN_COPY) != 0;
  const uint32_t first_limit = fr.wait_limit > 0 ? (uint32_t)fr.wait_limit : (1u << 22);
  if (threadIdx.x == 0 && !starve) {
    if (bytes) {
      const uint32_t* src = bins.bins + (size_t)tile * bins.capacity;
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                   :: "r"(bar_a), "r"(bytes) : "memory");
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
          :: "r"(smem_u32(queue)), "l"(src), "r"(bytes), "r"(bar_a) : "memory");
    } else {
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(bar_a) : "memory");
    }
  }
  if (!mbar_wait(bar_a, 0, first_limit)) {
    s_ok = 0;
    // let our own copy land before the shared memory is reused (when one was issued)
    if (!starve) mbar_wait(bar_a, 0, 1u << 22);
  }
  __syncthreads();
  const bool ok = s_ok != 0;
  if (!ok && threadIdx.x == 0) atomicOr(bins.status, T3_STATUS_TIMEOUT);

  SmemKeySink sink{keys, x0, y0, TS};
  WarpFaces& wf = wfs[threadIdx.x >> 5];
  const int warp = threadIdx.x >> 5;
  constexpr int NW = BLOCK / 32;
  if (ok) {
    // binned faces, 32 per warp per round (the round count is warp-uniform)
    for (uint32_t base = warp * 32; base < n; base += NW * 32) {
      const uint32_t i = base + (threadIdx.x & 31);
      Setup s{};
      uint32_t gid = 0;
      const bool act = i < n;
      if (act) {
        gid = queue[i];
        load_record(bins.rec, gid, s);
      }
      warp_raster_spans(wf, wcs[warp], s, act, gid, x0, x1, y0, y1, fr, sink);
    }
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
      if (__ballot_sync(FULL, act)) warp_raster_spans(wf, wcs[warp], s, act, gid, x0, x1, y0, y1, fr, sink);
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
        if (lane == 0) slot = atomicAdd(&s_count, __popc(m));
        slot = __shfl_sync(FULL, slot, 0);
        if (covered) s_list[slot + __popc(m & ((1u << lane) - 1u))] = i;
      }
    }
    __syncthreads();
    const int ncov = s_count;
    for (int j = threadIdx.x; j < ncov; j += BLOCK) {
      const int i = s_list[j];
      shade_pixel_from_key<NL, MODE>(sc, bins.rec, ok ? keys[i] : T3_EMPTY_KEY, x0 + i / TS,
                                     y0 + i % TS, out);
    }
  }
  if (threadIdx.x == 0) asm volatile("mbarrier.inval.shared::cta.b64 [%0];" :: "r"(bar_a) : "memory");
}

cudaError_t launch_bin(const t3_frame& fr, const t3_object& ob, const BinArgs& bins, cudaStream_t st) {
  if (ob.nfaces <= 0) return cudaSuccess;
  constexpr int BLOCK = 256;
  const int64_t grid = (ob.nfaces + BLOCK - 1) / BLOCK;
  k_bin<BLOCK><<<(unsigned)grid, BLOCK, 0, st>>>(fr, ob.mesh, ob.nfaces, (uint32_t)ob.face_base, bins);
  return cudaGetLastError();
}

template <int TS, int BLOCK, int NL, int MODE>
static cudaError_t launch_tile_b(const DevScene* sc, const BinArgs& bins, int ntiles,
                                 const t3_outputs& out, cudaStream_t st) {
  const size_t smem = (size_t)TS * TS * 8 + (size_t)bins.capacity * 4;
  cudaError_t e = cudaFuncSetAttribute(k_tile<TS, BLOCK, NL, MODE>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_tile<TS, BLOCK, NL, MODE><<<ntiles, BLOCK, smem, st>>>(sc, bins, out);
  return cudaGetLastError();
}

template <int TS, int BLOCK, int NL>
static cudaError_t launch_tile_nl(const DevScene* sc, const BinArgs& bins, int ntiles,
                                  const t3_outputs& out, cudaStream_t st) {
  if (bins.light_mode == T3_LIGHT_LAMPS)
    return launch_tile_b<TS, BLOCK, NL, T3_LIGHT_LAMPS>(sc, bins, ntiles, out, st);
  if (bins.light_mode == T3_LIGHT_IBL_MC)
    return launch_tile_b<TS, BLOCK, NL, T3_LIGHT_IBL_MC>(sc, bins, ntiles, out, st);
  if (bins.light_mode == T3_LIGHT_IBL_PREFILTERED)
    return launch_tile_b<TS, BLOCK, NL, T3_LIGHT_IBL_PREFILTERED>(sc, bins, ntiles, out, st);
  if (bins.light_mode == T3_LIGHT_IBL_MLP)  // visibility only: one instance serves every NL
    return launch_tile_b<TS, BLOCK, 2, T3_LIGHT_IBL_MLP>(sc, bins, ntiles, out, st);
  return cudaErrorInvalidValue;
}

template <int TS, int BLOCK>
static cudaError_t launch_tile_t(const DevScene* sc, const BinArgs& bins, int ntiles,
                                 const t3_outputs& out, cudaStream_t st) {
  if (bins.max_lobes <= 2) return launch_tile_nl<TS, BLOCK, 2>(sc, bins, ntiles, out, st);
  return launch_tile_nl<TS, BLOCK, 4>(sc, bins, ntiles, out, st);
}

cudaError_t launch_tile(const DevScene* sc, const BinArgs& bins, int ntiles, const t3_outputs& out,
                        cudaStream_t st) {
  switch (bins.tile) {
  case 8: return launch_tile_t<8, 64>(sc, bins, ntiles, out, st);
  case 16: return launch_tile_t<16, 256>(sc, bins, ntiles, out, st);
  case 32: return launch_tile_t<32, 256>(sc, bins, ntiles, out, st);
  default: return cudaErrorInvalidValue;
  }
}

} // namespace t3
