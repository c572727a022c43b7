// batch_binned.cu -- many views through the binned tile rasteriser: one launch
// bins every view's faces into that view's screen tiles, then one persistent
// launch takes (view, tile) items from a global work counter and rasterises
// and shades each tile in shared memory (t3_binned.cuh).  No reference
// counterpart (the reference renders one Scene per call).
//
// Per view the workspace holds the scene copy, its counters (64 + tiles), the
// big-face list, the 64-byte setup records, the tile bins and, for views with
// particles or lines, a key buffer their direct rasterisers fill first (it
// seeds the tiles, as in the single-view binned frame).  Tile size, threads
// per tile CTA and bin capacity come from t3_batch_config; BatchRenderer's
// autotuner sweeps them.
#include "t3_binned.cuh"

#include <cstring>

namespace t3 {

struct BinView {
  const DevScene* sc;
  BinArgs bins;
  t3_outputs out;
  uint32_t block0[T3_MAX_OBJECTS + 1];  // first bin block of each object (+ end)
  uint32_t tile0;                       // first item of this view's tiles
};

struct BinBatchArgs {
  int32_t nscenes;
  uint32_t qcap;      // bin entries staged per chunk
  uint32_t n_blocks;  // bin blocks of the whole batch
  uint32_t n_tiles;   // tile items of the whole batch
  uint32_t* queue;    // tile item counter (zeroed by the first view's upload)
  BinView v[T3_BATCH_MAX_SCENES];
};

constexpr int kBinBlock = 256;

// the last view whose first item (bin block or tile) is <= g
__device__ __forceinline__ int find_view(const BinBatchArgs& a, uint32_t g, bool tiles) {
  int lo = 0, hi = a.nscenes - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const uint32_t first = tiles ? a.v[mid].tile0 : a.v[mid].block0[0];
    if (first <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(kBinBlock) k_batch_bin(const __grid_constant__ BinBatchArgs a) {
  __shared__ __align__(16) float sv[kBinBlock * 9];
  const uint32_t b = blockIdx.x;
  const int s = find_view(a, b, false);
  const BinView& v = a.v[s];
  int o = 0;
  while (o + 1 < T3_MAX_OBJECTS && v.block0[o + 1] <= b) o++;
  const DevObject& ob = v.sc->obj[o];
  bin_faces<kBinBlock>(v.sc->frame, ob.mesh, ob.nfaces, (uint32_t)ob.face_base, v.bins,
                       (int64_t)(b - v.block0[o]) * kBinBlock, sv);
}

template <int TS, int BLOCK, int NL, bool TEX, int SIG>
__global__ void __launch_bounds__(BLOCK, 768 / BLOCK)
k_batch_tile(const __grid_constant__ BinBatchArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ TileShared<TS, BLOCK> sh;
  __shared__ uint32_t s_item;
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(smem_raw);  // TS*TS
  uint32_t* queue = reinterpret_cast<uint32_t*>(smem_raw + TS * TS * 8);        // one chunk
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(a.queue, 1u);
    __syncthreads();
    const uint32_t t = s_item;
    if (t >= a.n_tiles) break;  // block-uniform
    const BinView& v = a.v[find_view(a, t, true)];
    // ends with a block barrier, so s_item is rewritten only after every thread read it
    tile_body<TS, BLOCK, NL, T3_LIGHT_LAMPS, TEX, SIG>(v.sc, v.bins, v.out, (int)(t - v.tile0), sh, keys,
                                                       queue, a.qcap);
  }
}

// ---- host side -------------------------------------------------------------------

static size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

struct BinLayout {
  size_t scene[T3_BATCH_MAX_SCENES], counters[T3_BATCH_MAX_SCENES], big[T3_BATCH_MAX_SCENES];
  size_t rec[T3_BATCH_MAX_SCENES], bins[T3_BATCH_MAX_SCENES], keys[T3_BATCH_MAX_SCENES];
  int tiles_x[T3_BATCH_MAX_SCENES], tiles_y[T3_BATCH_MAX_SCENES];
  uint32_t capacity[T3_BATCH_MAX_SCENES];
  size_t end;
};

static int resolve(const t3_batch_config& c, int& tile, int& threads) {
  tile = c.tile ? c.tile : 16;
  if (tile != 8 && tile != 16 && tile != 32) return T3_EINVAL;
  threads = c.tile_threads ? c.tile_threads : (tile == 8 ? 64 : 256);
  if (threads != 64 && threads != 128 && threads != 256) return T3_EINVAL;
  if (threads == 64 && tile != 8) return T3_EINVAL;
  if (threads > tile * tile) return T3_EINVAL;
  return T3_OK;
}

static int bin_layout(const t3_scene* scenes, int n, const t3_batch_config& c, BinLayout& L) {
  if (!scenes || n <= 0) return T3_EINVAL;
  if (n > T3_BATCH_MAX_SCENES) return T3_ETOOBIG;
  int tile, threads;
  int r = resolve(c, tile, threads);
  if (r) return r;
  size_t at = 256;  // [0]: the tile item counter
  for (int s = 0; s < n; s++) {
    const t3_scene& sc = scenes[s];
    const t3_frame& fr = sc.frame;
    if (fr.width <= 0 || fr.height <= 0 || fr.width > 4096 || fr.height > 4096) return T3_EINVAL;
    L.tiles_x[s] = (fr.width + tile - 1) / tile;
    L.tiles_y[s] = (fr.height + tile - 1) / tile;
    const int64_t ntiles = (int64_t)L.tiles_x[s] * L.tiles_y[s];
    int64_t cap = c.bin_capacity > 0 ? c.bin_capacity : auto_bin_capacity(sc, tile);
    if (c.bin_capacity < 0) cap *= -c.bin_capacity;
    cap = (cap + 3) & ~(int64_t)3;  // bins start on 16-byte boundaries
    if (cap > (1 << 22)) return T3_ETOOBIG;
    L.capacity[s] = (uint32_t)cap;
    const int64_t faces = total_faces(sc) > 0 ? total_faces(sc) : 1;
    L.scene[s] = at;
    at = a256(at + sizeof(DevScene));
    L.counters[s] = at;
    at = a256(at + 4 * (size_t)(64 + ntiles));
    L.big[s] = at;
    at = a256(at + 4 * (size_t)faces);
    L.rec[s] = at;
    at = a256(at + 64 * (size_t)faces);
    L.bins[s] = at;
    at = a256(at + 4 * (size_t)ntiles * (size_t)cap);
    L.keys[s] = 0;
    if (has_points_or_lines(sc)) {
      L.keys[s] = at;
      at = a256(at + 8 * (size_t)fr.width * (size_t)fr.height);
    }
  }
  L.end = at;
  return T3_OK;
}

int batch_binned_size(const t3_scene* scenes, int n, const t3_batch_config& c, size_t* bytes) {
  static thread_local BinLayout L;
  const int r = bin_layout(scenes, n, c, L);
  if (r) return r;
  *bytes = L.end;
  return T3_OK;
}

// the tile kernel instance: lobe kinds and parameters as constants when every
// view has the same untextured material shape, texture nodes compiled in only
// when a view has one
template <int TS, int BLOCK>
static const void* tile_kernel(int fsig, bool textured, int nl) {
  constexpr int F = T3_SIG_FAST;
  if (!textured && fsig == T3_SIG_PBR) return (const void*)k_batch_tile<TS, BLOCK, 2, false, T3_SIG_PBR | F>;
  if (!textured && fsig == T3_SIG_CLASSIC)
    return (const void*)k_batch_tile<TS, BLOCK, 2, false, T3_SIG_CLASSIC | F>;
  (void)nl;
  return (const void*)k_batch_tile<TS, BLOCK, 4, true, 0>;
}

static const void* pick_tile_kernel(int tile, int threads, int fsig, bool textured, int nl) {
  if (tile == 8) return tile_kernel<8, 64>(fsig, textured, nl);
  if (tile == 16) return threads == 128 ? tile_kernel<16, 128>(fsig, textured, nl)
                                        : tile_kernel<16, 256>(fsig, textured, nl);
  return threads == 128 ? tile_kernel<32, 128>(fsig, textured, nl) : tile_kernel<32, 256>(fsig, textured, nl);
}

int render_batch_binned(const t3_scene* scenes, const t3_outputs* outs, int n, const t3_batch_config& c,
                        void* workspace, size_t workspace_bytes, int32_t* status, cudaStream_t st) {
  static thread_local BinLayout L;
  int r = bin_layout(scenes, n, c, L);
  if (r) return r;
  if (workspace_bytes < L.end) return T3_EINVAL;
  int tile, threads;
  resolve(c, tile, threads);
  if (c.ctas_per_sm < 0 || c.ctas_per_sm > 8) return T3_EINVAL;
  static thread_local BinBatchArgs a;
  static thread_local DevScene ds;
  std::memset(&a, 0, sizeof(a));
  uint8_t* ws = reinterpret_cast<uint8_t*>(workspace);
  a.nscenes = n;
  a.queue = reinterpret_cast<uint32_t*>(ws);
  uint32_t maxcap = 4;
  int nl = 1, fsig = -1;
  bool textured = false;
  uint32_t block = 0, titem = 0;
  cudaError_t e = cudaSuccess;
  for (int s = 0; s < n && e == cudaSuccess; s++) {
    r = make_dev_scene(scenes[s], ds);
    if (r) return r;
    if (ds.lighting.mode != T3_LIGHT_LAMPS) return T3_EUNSUPPORTED;
    if (!outs[s].rgb) return T3_EINVAL;
    nl = max_lobes(ds) > nl ? max_lobes(ds) : nl;
    textured = textured || has_textures(ds) != 0;
    const int sf = fast_signature(ds);
    fsig = fsig < 0 || fsig == sf ? sf : 0;
    DevScene* dst = reinterpret_cast<DevScene*>(ws + L.scene[s]);
    uint32_t* counters = reinterpret_cast<uint32_t*>(ws + L.counters[s]);
    const int ntiles = L.tiles_x[s] * L.tiles_y[s];
    // each view's upload zeroes its counters; the first also the status word
    // and the tile item counter
    e = launch_upload_scene(ds, dst, counters, 64 + ntiles, s == 0 ? status : nullptr, st);
    if (e == cudaSuccess && s == 0) e = cudaMemsetAsync(a.queue, 0, sizeof(uint32_t), st);
    BinView& v = a.v[s];
    v.sc = dst;
    v.out = outs[s];
    BinArgs& b = v.bins;
    b.rec = reinterpret_cast<float4*>(ws + L.rec[s]);
    b.bins = reinterpret_cast<uint32_t*>(ws + L.bins[s]);
    b.count = counters + 64;
    b.big = reinterpret_cast<uint32_t*>(ws + L.big[s]);
    b.big_count = counters + 63;
    b.status = status;
    b.capacity = L.capacity[s];
    b.big_capacity = (uint32_t)(total_faces(scenes[s]) > 0 ? total_faces(scenes[s]) : 1);
    b.tile = tile;
    b.tiles_x = L.tiles_x[s];
    b.tiles_y = L.tiles_y[s];
    b.big_tiles = 16;
    b.max_lobes = max_lobes(ds);
    b.light_mode = T3_LIGHT_LAMPS;
    b.keys = nullptr;
    b.pre = nullptr;
    maxcap = b.capacity > maxcap ? b.capacity : maxcap;
    if (L.keys[s]) {
      // particles and lines: their direct rasterisers into the view's keys,
      // which then seed its tiles
      unsigned long long* k = reinterpret_cast<unsigned long long*>(ws + L.keys[s]);
      const int64_t npix = (int64_t)scenes[s].frame.width * scenes[s].frame.height;
      if (e == cudaSuccess) e = launch_clear(k, npix, st);
      for (int o = 0; o < scenes[s].nobjects && e == cudaSuccess; o++)
        if (is_point_or_line(scenes[s].objects[o].mesh))
          e = launch_raster_point_or_line(scenes[s].frame, scenes[s].objects[o], k, nullptr, st);
      b.pre = k;
    }
    for (int o = 0; o < scenes[s].nobjects; o++) {
      v.block0[o] = block;
      if (!is_point_or_line(scenes[s].objects[o].mesh))
        block += (uint32_t)((scenes[s].objects[o].nfaces + kBinBlock - 1) / kBinBlock);
    }
    for (int o = scenes[s].nobjects; o <= T3_MAX_OBJECTS; o++) v.block0[o] = block;
    v.tile0 = titem;
    titem += (uint32_t)ntiles;
  }
  if (e != cudaSuccess) return T3_ECUDA;
  a.n_blocks = block;
  a.n_tiles = titem;
  a.qcap = queue_entries(maxcap);
  if (a.n_blocks) k_batch_bin<<<a.n_blocks, kBinBlock, 0, st>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) return T3_ECUDA;
  const void* fn = pick_tile_kernel(tile, threads, fsig, textured, nl);
  const size_t smem = (size_t)tile * tile * 8 + (size_t)a.qcap * 4;
  int dev = 0, nsm = 0, occ = 0;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads, smem);
  if (e != cudaSuccess) return T3_ECUDA;
  const int per_sm = c.ctas_per_sm > 0 && c.ctas_per_sm < occ ? c.ctas_per_sm : (occ > 0 ? occ : 1);
  void* args[] = {&a};
  e = cudaLaunchKernel(fn, dim3(nsm * per_sm), dim3(threads), args, smem, st);
  if (e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? T3_OK : T3_ECUDA;
}

} // namespace t3
