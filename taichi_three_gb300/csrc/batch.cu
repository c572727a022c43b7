// batch.cu -- many views rendered by two persistent launches driven by global
// work queues.
//
// A batch is up to T3_BATCH_MAX_SCENES independent frames (own resolution,
// camera, objects, lamps).  Their work is cut into items:
//   raster items  (scene, object, chunk of faces_per_item faces): transform,
//                 cull, clip, setup, cooperative raster into the scene's key
//                 buffer (atomicMin), setup records for shading;
//   shade items   (scene, chunk of pixels_per_item pixels): the deferred
//                 shading pass of that scene's pixels.
// One persistent grid takes every raster item of every scene from a global
// counter, then a second persistent grid takes every shade item the same way:
// the whole batch's rasterisation is one launch, load-balanced across scenes
// of very different sizes, and each phase runs at its own occupancy (the
// raster walk wants many light threads, shading fewer heavy ones).
//
// Faces whose bbox exceeds kBigArea pixels are kept out of the warps' walk and
// rasterised by the whole CTA after its chunk (a CTA-wide stride over the bbox).
// Particle and line objects take no raster items: the direct particle and
// line rasterisers write their fragments into the views' keys after the clear.
#include "t3_raster.cuh"
#include "t3_shading.cuh"

#include <cstring>

namespace t3 {

constexpr int kBatchBlock = 256;
constexpr int kBatchPPT = 4;          // pixels per thread per shading pass
constexpr int kBigArea = 1 << 15;     // bbox pixels above which the CTA rasterises a face together
constexpr int kBigSlots = 64;

struct BatchView {
  const DevScene* sc;
  unsigned long long* keys;
  float4* rec;
  t3_outputs out;
  int64_t npix;
  uint32_t raster_item0, raster_items, shade_item0, shade_items;
};

struct BatchArgs {
  int32_t nscenes;
  int32_t faces_per_item;   // multiple of kBatchBlock
  int32_t pixels_per_item;  // multiple of kBatchBlock * kBatchPPT
  uint32_t n_raster, n_items;
  uint32_t* queue;          // [0] raster item counter, [1] shade item counter
  BatchView v[T3_BATCH_MAX_SCENES];
  uint32_t obj_item0[T3_BATCH_MAX_SCENES][T3_MAX_OBJECTS + 1];  // first item of each object (+ end)
};

struct GlobalSink {
  unsigned long long* keys;
  int64_t H;
  __device__ __forceinline__ void operator()(int x, int y, unsigned long long key) const {
    atomicMin(keys + (int64_t)x * H + y, key);
  }
};

// scene of item g: the last v[s] whose first item is <= g (the views are in
// item order)
__device__ __forceinline__ int find_scene(const BatchArgs& a, uint32_t g, bool shade) {
  int lo = 0, hi = a.nscenes - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const uint32_t first = shade ? a.v[mid].shade_item0 : a.v[mid].raster_item0;
    if (first <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(kBatchBlock, 4) k_batch_raster(const __grid_constant__ BatchArgs a) {
  __shared__ __align__(16) float sv[kBatchBlock * 9];
  __shared__ WarpFaces wfs[kBatchBlock / 32];
  __shared__ WarpCols wcs[kBatchBlock / 32];
  __shared__ uint32_t s_item;
  __shared__ uint32_t s_big[kBigSlots];
  __shared__ int s_nbig;

  for (;;) {
    if (threadIdx.x == 0) {
      s_item = atomicAdd(a.queue, 1u);
      s_nbig = 0;
    }
    __syncthreads();
    const uint32_t g = s_item;
    if (g >= a.n_raster) break;
    const int s = find_scene(a, g, false);
    const BatchView& v = a.v[s];
    const DevScene* sc = v.sc;
    const t3_frame& fr = sc->frame;
    int o = 0;
    while (o + 1 < sc->nobjects && a.obj_item0[s][o + 1] <= g) o++;
    const DevObject& ob = sc->obj[o];
    const int64_t first = (int64_t)(g - a.obj_item0[s][o]) * a.faces_per_item;
    const int64_t last = min(first + a.faces_per_item, ob.nfaces);
    GlobalSink sink{v.keys, fr.height};
    for (int64_t f0 = first; f0 < last; f0 += kBatchBlock) {
      const bool staged = stage_soup<kBatchBlock>(ob.mesh, last, f0, sv);
      const int64_t n = f0 + threadIdx.x;
      Setup st{};
      bool vis = false;
      if (n < last) {
        f3 vv[3];
        load_face(ob.mesh, n, staged, sv, vv);
        vis = face_setup(fr, vv, st) && st.botx <= st.topx && st.boty <= st.topy;
      }
      const uint32_t gid = (uint32_t)(ob.face_base + n);
      if (vis) {
        store_record(v.rec, gid, st);
        const int64_t area = (int64_t)(st.topx - st.botx + 1) * (int64_t)(st.topy - st.boty + 1);
        if (area > kBigArea) {
          const int slot = atomicAdd(&s_nbig, 1);
          if (slot < kBigSlots) {
            s_big[slot] = (uint32_t)n;
            vis = false;
          }
          // beyond the slots the face stays in the warp walk (correct, slower)
        }
      }
      warp_raster_spans(wfs[threadIdx.x >> 5], wcs[threadIdx.x >> 5], st, vis, gid, 0, fr.width - 1, 0,
                        fr.height - 1, fr, sink);
      __syncthreads();  // sv is restaged by the next pass
    }
    // big faces of this chunk: the whole CTA strides over each bbox
    const int nbig = min(s_nbig, kBigSlots);
    const float maxd = (float)fr.maxdepth;
    for (int b = 0; b < nbig; b++) {
      const int64_t n = s_big[b];
      f3 vv[3];
      face_verts(ob.mesh, face_ref(ob.mesh, n), vv);
      Setup st;
      if (!face_setup(fr, vv, st)) continue;  // CTA-uniform
      const int32_t h = st.topy - st.boty + 1;
      const int64_t area = (int64_t)(st.topx - st.botx + 1) * h;
      const uint32_t gid = (uint32_t)(ob.face_base + n);
      for (int64_t k = threadIdx.x; k < area; k += kBatchBlock) {
        const int32_t x = st.botx + (int32_t)(k / h);
        const int32_t y = st.boty + (int32_t)(k - (k / h) * h);
        float wx, wy, wz, sum;
        face_raw_weights(st, xadd((float)x, fr.bias[0]), xadd((float)y, fr.bias[1]), wx, wy, wz, sum);
        f3 wei;
        if (!face_inside(wx, wy, wz, sum, wei)) continue;
        const int32_t d = trunc_i32(xmul(face_depth(st, wei), maxd));
        if (d < fr.maxdepth) sink(x, y, pack_key(d, gid));
      }
    }
    __syncthreads();  // s_item / s_big are rewritten by the next iteration
  }
}

template <int NL, bool TEX, int SIG, bool PLAIN = false>
__global__ void __launch_bounds__(kBatchBlock, 3) k_batch_shade(const __grid_constant__ BatchArgs a) {
  __shared__ int s_list[kBatchBlock * kBatchPPT];
  __shared__ unsigned long long s_key[kBatchBlock * kBatchPPT];
  __shared__ int s_count;
  __shared__ uint32_t s_item;
  for (;;) {
    if (threadIdx.x == 0) {
      s_item = atomicAdd(a.queue + 1, 1u);
      s_count = 0;
    }
    __syncthreads();
    const uint32_t gs = s_item;
    if (gs >= a.n_items - a.n_raster) break;
    const int s = find_scene(a, gs, true);
    const BatchView& v = a.v[s];
    const int64_t base = (int64_t)(gs - v.shade_item0) * a.pixels_per_item;
    for (int64_t p0 = base; p0 < base + a.pixels_per_item && p0 < v.npix; p0 += kBatchBlock * kBatchPPT) {
      shade_block<kBatchBlock, kBatchPPT, NL, T3_LIGHT_LAMPS, false, TEX, SIG, PLAIN>(v.sc, v.keys, v.rec, v.out,
                                                                                v.npix, p0, s_list, &s_count,
                                                                                s_key);
      __syncthreads();
      if (threadIdx.x == 0) s_count = 0;
      __syncthreads();
    }
  }
}

// ---- host side -----------------------------------------------------------------

static size_t align256b(size_t x) { return (x + 255) & ~(size_t)255; }

struct BatchLayout {
  size_t counters, scenes, keys[T3_BATCH_MAX_SCENES], rec[T3_BATCH_MAX_SCENES], end;
  int64_t total_pix;
};

static int64_t scene_faces(const t3_scene& sc) {
  int64_t t = 0;
  for (int o = 0; o < sc.nobjects && o < T3_MAX_OBJECTS; o++) t += sc.objects[o].nfaces;
  return t;
}

static int batch_layout(const t3_scene* scenes, int n, BatchLayout& L) {
  if (!scenes || n <= 0) return T3_EINVAL;
  if (n > T3_BATCH_MAX_SCENES) return T3_ETOOBIG;
  L.counters = 0;
  L.scenes = 256;
  size_t at = L.scenes + align256b(sizeof(DevScene)) * (size_t)n;
  // key buffers back to back: one clear covers them all
  L.total_pix = 0;
  for (int s = 0; s < n; s++) {
    const t3_frame& fr = scenes[s].frame;
    // <= 4096 x 4096: 32 clamped bboxes of a warp's walk sum below 2^31 pixels
    if (fr.width <= 0 || fr.height <= 0 || fr.width > 4096 || fr.height > 4096) return T3_EINVAL;
    L.keys[s] = at + 8 * (size_t)L.total_pix;
    L.total_pix += (int64_t)fr.width * fr.height;
  }
  at = align256b(at + 8 * (size_t)L.total_pix);
  for (int s = 0; s < n; s++) {
    L.rec[s] = at;
    const int64_t t = scene_faces(scenes[s]);
    at = align256b(at + 64 * (size_t)(t > 0 ? t : 1));
  }
  L.end = at;
  return T3_OK;
}

} // namespace t3

using namespace t3;

extern "C" {

int t3_batch_workspace_size(const t3_scene* scenes, int nscenes, const t3_batch_config* config,
                            size_t* bytes) {
  if (!bytes) return T3_EINVAL;
  if (config && config->raster == T3_RASTER_BINNED) return batch_binned_size(scenes, nscenes, *config, bytes);
  if (config && config->raster != T3_RASTER_DIRECT) return T3_EINVAL;
  BatchLayout L;
  const int r = batch_layout(scenes, nscenes, L);
  if (r) return r;
  *bytes = L.end;
  return T3_OK;
}

int t3_render_batch(const t3_scene* scenes, const t3_outputs* outs, int nscenes,
                    const t3_batch_config* cfg, void* workspace, size_t workspace_bytes,
                    int32_t* status, void* stream) {
  if (!scenes || !outs || !workspace || !status) return T3_EINVAL;
  t3_batch_config c{1024, 4096, 0, T3_RASTER_DIRECT, 0, 0, 0};
  if (cfg) c = *cfg;
  if (c.raster == T3_RASTER_BINNED)
    return render_batch_binned(scenes, outs, nscenes, c, workspace, workspace_bytes, status, (cudaStream_t)stream);
  if (c.raster != T3_RASTER_DIRECT) return T3_EINVAL;
  BatchLayout L;
  int r = batch_layout(scenes, nscenes, L);
  if (r) return r;
  if (workspace_bytes < L.end) return T3_EINVAL;
  if (c.faces_per_item <= 0) c.faces_per_item = 1024;
  if (c.pixels_per_item <= 0) c.pixels_per_item = 4096;
  if (c.faces_per_item % kBatchBlock || c.pixels_per_item % (kBatchBlock * kBatchPPT)) return T3_EINVAL;
  if (c.ctas_per_sm < 0 || c.ctas_per_sm > 8) return T3_EINVAL;

  static thread_local BatchArgs a;
  static thread_local DevScene ds;
  std::memset(&a, 0, sizeof(a));
  uint8_t* ws = reinterpret_cast<uint8_t*>(workspace);
  cudaStream_t st = (cudaStream_t)stream;
  a.nscenes = nscenes;
  a.faces_per_item = c.faces_per_item;
  a.pixels_per_item = c.pixels_per_item;
  a.queue = reinterpret_cast<uint32_t*>(ws + L.counters);
  int nl = 1, sig = -1, fsig = -1;
  bool textured = false, plain = true;
  uint32_t item = 0;
  cudaError_t e = cudaSuccess;
  for (int s = 0; s < nscenes && e == cudaSuccess; s++) {
    r = make_dev_scene(scenes[s], ds);
    if (r) return r;
    if (ds.lighting.mode != T3_LIGHT_LAMPS) return T3_EUNSUPPORTED;
    if (!outs[s].rgb) return T3_EINVAL;
    nl = max_lobes(ds) > nl ? max_lobes(ds) : nl;
    textured = textured || has_textures(ds) != 0;
    const int ssig = lobe_signature(ds);
    sig = sig < 0 || sig == ssig ? ssig : 0;
    const int sfast = fast_signature(ds);
    fsig = fsig < 0 || fsig == sfast ? sfast : 0;
    plain = plain && plain_soups(ds);
    DevScene* dst = reinterpret_cast<DevScene*>(ws + L.scenes + align256b(sizeof(DevScene)) * (size_t)s);
    // the first upload also zeroes the queue counters and the status
    e = launch_upload_scene(ds, dst, s == 0 ? a.queue : nullptr, s == 0 ? 2 : 0, s == 0 ? status : nullptr,
                            st);
    BatchView& v = a.v[s];
    v.sc = dst;
    v.keys = reinterpret_cast<unsigned long long*>(ws + L.keys[s]);
    v.rec = reinterpret_cast<float4*>(ws + L.rec[s]);
    v.out = outs[s];
    v.npix = (int64_t)scenes[s].frame.width * scenes[s].frame.height;
    v.raster_item0 = item;
    for (int o = 0; o < scenes[s].nobjects; o++) {
      a.obj_item0[s][o] = item;
      // particles and lines take no raster items: their own rasterisers run
      // after the clear (an object without items is skipped by the item search)
      if (!is_point_or_line(scenes[s].objects[o].mesh))
        item += (uint32_t)((scenes[s].objects[o].nfaces + c.faces_per_item - 1) / c.faces_per_item);
    }
    for (int o = scenes[s].nobjects; o <= T3_MAX_OBJECTS; o++) a.obj_item0[s][o] = item;
    v.raster_items = item - v.raster_item0;
  }
  if (e != cudaSuccess) return T3_ECUDA;
  a.n_raster = item;
  uint32_t sitem = 0;
  for (int s = 0; s < nscenes; s++) {
    a.v[s].shade_item0 = sitem;
    a.v[s].shade_items = (uint32_t)((a.v[s].npix + c.pixels_per_item - 1) / c.pixels_per_item);
    sitem += a.v[s].shade_items;
  }
  a.n_items = a.n_raster + sitem;
  e = launch_clear(reinterpret_cast<unsigned long long*>(ws + L.keys[0]), L.total_pix, st);
  // particles and lines: the direct rasterisers into their view's keys (every
  // fragment is an order-independent packed minimum, so it does not matter
  // that the triangles' persistent launch comes after)
  for (int s = 0; s < nscenes && e == cudaSuccess; s++)
    for (int o = 0; o < scenes[s].nobjects && e == cudaSuccess; o++)
      if (is_point_or_line(scenes[s].objects[o].mesh))
        e = launch_raster_point_or_line(scenes[s].frame, scenes[s].objects[o], a.v[s].keys, nullptr, st);
  if (e != cudaSuccess) return T3_ECUDA;
  int dev = 0, nsm = 0, occ_r = 0, occ_s = 0;
  e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  // the shading instance: lobe kinds as constants when every view shares an
  // untextured signature, texture nodes compiled in only when a view has one
  const void* shade_fn;
  constexpr int F = T3_SIG_FAST;
  if (!textured && fsig == T3_SIG_PBR)
    shade_fn = plain ? (const void*)k_batch_shade<2, false, T3_SIG_PBR | F, true>
                     : (const void*)k_batch_shade<2, false, T3_SIG_PBR | F>;
  else if (!textured && fsig == T3_SIG_CLASSIC)
    shade_fn = plain ? (const void*)k_batch_shade<2, false, T3_SIG_CLASSIC | F, true>
                     : (const void*)k_batch_shade<2, false, T3_SIG_CLASSIC | F>;
  else if (!textured && fsig == T3_SIG_DIFFUSE)
    shade_fn = plain ? (const void*)k_batch_shade<1, false, T3_SIG_DIFFUSE | F, true>
                     : (const void*)k_batch_shade<1, false, T3_SIG_DIFFUSE | F>;
  else if (!textured && sig == T3_SIG_PBR) shade_fn = (const void*)k_batch_shade<2, false, T3_SIG_PBR>;
  else if (!textured && sig == T3_SIG_CLASSIC) shade_fn = (const void*)k_batch_shade<2, false, T3_SIG_CLASSIC>;
  else if (!textured && sig == T3_SIG_DIFFUSE) shade_fn = (const void*)k_batch_shade<1, false, T3_SIG_DIFFUSE>;
  else if (nl <= 2) shade_fn = textured ? (const void*)k_batch_shade<2, true, 0> : (const void*)k_batch_shade<2, false, 0>;
  else shade_fn = textured ? (const void*)k_batch_shade<4, true, 0> : (const void*)k_batch_shade<4, false, 0>;
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_r, (const void*)k_batch_raster, kBatchBlock, 0);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_s, shade_fn, kBatchBlock, 0);
  if (e != cudaSuccess) return T3_ECUDA;
  auto per_sm = [&](int occ) { return c.ctas_per_sm > 0 && c.ctas_per_sm < occ ? c.ctas_per_sm : (occ > 0 ? occ : 1); };
  k_batch_raster<<<nsm * per_sm(occ_r), kBatchBlock, 0, st>>>(a);
  void* args[] = {&a};
  e = cudaLaunchKernel(shade_fn, dim3(nsm * per_sm(occ_s)), dim3(kBatchBlock), args, 0, st);
  if (e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? T3_OK : T3_ECUDA;
}

} // extern "C"
