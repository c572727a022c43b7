// noalloc.cu -- t3_render_noalloc: one frame of the direct rasteriser whose
// scratch memory is a fixed device array inside this library.
//
// Who needs it: code that renders inside a host application which owns the
// GPU's memory and hands the renderer only its input and output buffers -- a
// plug-in or frame callback that must not call cudaMalloc (the host forbids
// allocations in its frame loop, or an allocation there could block or fail
// at an unpredictable moment).  t3_render needs a caller-allocated workspace;
// this entry point needs none.
//
// The scratch (scene copy, counters, large-face queue and the packed depth key
// buffer) lives in `g_noalloc_scratch`, a file-scope __device__ array of
// T3_NOALLOC_SCRATCH_BYTES (17,056,000 bytes, about 16.3 MiB).  Every GPU that loads the library
// holds that array until the process exits.  In host code the array's name is
// only a host-side stand-in, so the first call in each CUDA context (with that
// context current) looks up the array's device address with
// cudaGetSymbolAddress and caches it under the context's unique id: a device
// address belongs to the context that loaded the module, so a caller that
// makes its own contexts, or resets the device (which ends the old context),
// gets a fresh lookup rather than a stale pointer.  Make the first call in a
// context before any stream capture.  Each call clears what must start empty
// (counters, status word, key buffer).  All calls share the one array: calls
// whose work overlaps on the GPU (other streams, other host threads, replays
// of a CUDA graph that captured this call) race on it and must be serialised
// by the caller.
#include <cuda.h>

#include <mutex>

#include "t3_internal.cuh"

namespace t3 {

constexpr size_t kNoallocScene = 0;
constexpr size_t kNoallocCounters = 16384;
static_assert(sizeof(DevScene) <= kNoallocCounters, "scene copy outgrew its scratch region");
constexpr size_t kNoallocBig = kNoallocCounters + 256;
constexpr size_t kNoallocKeys = kNoallocBig + 4 * (size_t)T3_NOALLOC_MAX_BIG_FACES;
constexpr size_t kNoallocBytes = kNoallocKeys + 8 * (size_t)T3_NOALLOC_MAX_PIXELS;
static_assert(kNoallocBytes == T3_NOALLOC_SCRATCH_BYTES, "scratch size in tina3.h is stale");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

static std::mutex g_noalloc_mu;
// device addresses of g_noalloc_scratch, one per CUDA context that has called
// (keyed by cuCtxGetId, which is unique over the process's lifetime)
struct NoallocAddr {
  unsigned long long ctx_id;
  void* ptr;
};
static NoallocAddr g_noalloc_addr[64];
static int g_noalloc_next;  // slot replaced next once the table is full

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

// device address of g_noalloc_scratch in the current context (looked up once per context)
static int noalloc_scratch(void** out) {
  // the two driver calls come through the runtime's entry-point table, so the
  // library itself does not link against the driver library
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    cudaDriverEntryPointQueryResult q1, q2;
    if (!get_current &&
        (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", (void**)&get_current, 12000, cudaEnableDefault,
                                          &q1) != cudaSuccess || q1 != cudaDriverEntryPointSuccess))
      get_current = nullptr;
    if (!get_id &&
        (cudaGetDriverEntryPointByVersion("cuCtxGetId", (void**)&get_id, 12000, cudaEnableDefault, &q2) !=
             cudaSuccess || q2 != cudaDriverEntryPointSuccess))
      get_id = nullptr;
    if (!get_current || !get_id) return T3_ECUDA;
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS) return T3_ECUDA;
  if (!ctx) {
    // no context bound to this thread yet: bind the current device's primary
    // context, as the runtime would on its first call (nothing can be capturing)
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaSetDevice(dev) != cudaSuccess) return T3_ECUDA;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return T3_ECUDA;
  }
  if (get_id(ctx, &id) != CUDA_SUCCESS) return T3_ECUDA;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  for (const NoallocAddr& a : g_noalloc_addr)
    if (a.ptr && a.ctx_id == id) {
      *out = a.ptr;
      return T3_OK;
    }
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return T3_ECUDA;
  NoallocAddr* slot = nullptr;
  for (NoallocAddr& a : g_noalloc_addr)
    if (!a.ptr) { slot = &a; break; }
  if (!slot) {
    slot = &g_noalloc_addr[g_noalloc_next];
    g_noalloc_next = (g_noalloc_next + 1) % 64;
  }
  slot->ctx_id = id;
  slot->ptr = p;
  *out = p;
  return T3_OK;
}

} // namespace t3

using namespace t3;

extern "C" int t3_render_noalloc(const t3_scene* scene, int32_t* status, const t3_outputs* out,
                                 void* stream) {
  if (!scene || !status || !out || !out->rgb) return T3_EINVAL;
  const int64_t npix = (int64_t)scene->frame.width * scene->frame.height;
  if (scene->frame.width <= 0 || scene->frame.height <= 0) return T3_EINVAL;
  if (npix > (int64_t)T3_NOALLOC_MAX_PIXELS) return T3_ETOOBIG;
  static thread_local DevScene ds;
  int r = make_dev_scene(*scene, ds);
  if (r) return r;
  void* base = nullptr;
  r = noalloc_scratch(&base);
  if (r) return r;
  uint8_t* ws = reinterpret_cast<uint8_t*>(base);
  cudaStream_t st = (cudaStream_t)stream;
  DevScene* dsc = reinterpret_cast<DevScene*>(ws + kNoallocScene);
  uint32_t* counters = reinterpret_cast<uint32_t*>(ws + kNoallocCounters);
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(ws + kNoallocKeys);
  cudaError_t e = launch_clear(keys, npix, st, counters, 64, status);
  for (int o = 0; o < scene->nobjects && e == cudaSuccess; o++) {
    BigQueue big;
    big.items = reinterpret_cast<uint32_t*>(ws + kNoallocBig);
    big.capacity = T3_NOALLOC_MAX_BIG_FACES;
    big.count = counters + o;
    big.status = status;
    big.rec = nullptr;
    if (is_point_or_line(scene->objects[o].mesh))
      e = launch_raster_point_or_line(scene->frame, scene->objects[o], keys, nullptr, st);
    else
      e = launch_raster_direct(scene->frame, scene->objects[o], keys, big, 4096, st);
  }
  if (e == cudaSuccess) e = launch_shade(ds, dsc, keys, nullptr, *out, status, st);
  return e == cudaSuccess ? T3_OK : T3_ECUDA;
}
