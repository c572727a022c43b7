// shade.cu -- the deferred interpolate-and-shade pass of the direct path.
//
// TriangleRaster.render_color (tina/core/triangle.py:134-153) with the shader it
// calls inlined (t3_shading.cuh).  One thread per pixel: it decodes the winning
// face from the packed key, recomputes that face's setup and barycentric weights
// exactly as the rasteriser did (so depth_f is bit-exact), interpolates
// position / normal / texcoord, evaluates the material once per pixel, then
// sums the lamps and applies ACES.
#include "t3_shading.cuh"

namespace t3 {

// Copies the scene descriptor (a kernel parameter) into the workspace and zeroes
// the per-frame counters: one launch makes the scene readable by every later
// kernel of the frame, including inside a captured CUDA graph.
__global__ void k_upload_scene(const DevScene sc, DevScene* __restrict__ dst,
                               uint32_t* __restrict__ counters, int ncounters,
                               int32_t* __restrict__ status, unsigned long long* __restrict__ key_tag) {
  // a frame of another layout: the direct frame's keys are no longer known empty
  if (key_tag && blockIdx.x == 0 && threadIdx.x == 0) *key_tag = 0ull;
  // the descriptor is split across blocks: each block copies a 1 KB slice, so
  // the constant-bank reads of the parameter run on many SMs at once
  constexpr int nwords = (int)(sizeof(DevScene) / 4);
  const uint32_t* src = reinterpret_cast<const uint32_t*>(&sc);
  uint32_t* d = reinterpret_cast<uint32_t*>(dst);
  for (int i = blockIdx.x * 256 + threadIdx.x; i < nwords; i += gridDim.x * 256) d[i] = src[i];
  if (blockIdx.x == 0 && threadIdx.x == 0 && status) *status = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ncounters; i += gridDim.x * blockDim.x)
    counters[i] = 0u;
}

cudaError_t launch_upload_scene(const DevScene& sc, DevScene* dst, uint32_t* counters,
                                int ncounters, int32_t* status, cudaStream_t st,
                                unsigned long long* key_tag) {
  constexpr int scene_blocks = (int)((sizeof(DevScene) / 4 + 255) / 256);
  int grid = (ncounters + 255) / 256;
  grid = grid < scene_blocks ? scene_blocks : grid > 64 ? 64 : grid;
  k_upload_scene<<<grid, 256, 0, st>>>(sc, dst, counters, ncounters, status, key_tag);
  return cudaGetLastError();
}

// Each block owns PPT * BLOCK consecutive pixels (shade_block).  The scene
// descriptor is a __grid_constant__ kernel parameter: lamps, materials and
// camera are read through the constant cache (warp-uniform broadcasts), not
// as per-pixel global loads.
template <int BLOCK, int PPT, int NL, int MODE, bool TEX, int SIG, bool PLAIN = false>
__global__ void __launch_bounds__(BLOCK, 3)
k_shade(const __grid_constant__ DevScene sc, const unsigned long long* __restrict__ keys,
        const float4* __restrict__ rec, t3_outputs out, int64_t npix, KeyState reset) {
  __shared__ int s_list[BLOCK * PPT];
  __shared__ unsigned long long s_key[BLOCK * PPT];
  __shared__ int s_count;
  if (threadIdx.x == 0) s_count = 0;
  // the keys are empty once every block has run: mark them so for the next frame
  if (reset.tag_word && blockIdx.x == 0 && threadIdx.x == 0) *reset.tag_word = reset.tag;
  __syncthreads();
  shade_block<BLOCK, PPT, NL, MODE, false, TEX, SIG, PLAIN>(
      &sc, keys, rec, out, npix, (int64_t)blockIdx.x * BLOCK * PPT, s_list, &s_count, s_key,
      reset.tag_word ? const_cast<unsigned long long*>(keys) : nullptr);
}

// the lobe signature shared by every shaded object, when an instance exists
// for it (lines take the line colour and are not shaded); 0 otherwise
int lobe_signature(const DevScene& sc) {
  int sig = -1;
  for (int o = 0; o < sc.nobjects; o++) {
    if (is_wire(sc.obj[o].mesh)) continue;
    const DevMaterial& m = sc.obj[o].mat;
    if (m.nlobes > 2) return 0;
    int s = 0;
    for (int k = 0; k < m.nlobes; k++) s |= m.lobes[k].kind << (8 * k);
    if (sig >= 0 && s != sig) return 0;
    sig = s;
  }
  return sig == T3_SIG_PBR || sig == T3_SIG_CLASSIC || sig == T3_SIG_DIFFUSE ? sig : 0;
}

bool plain_soups(const DevScene& sc) {
  constexpr uint32_t edits = T3_MESH_TRANSFORM | T3_MESH_NOCULL | T3_MESH_FLIP_ORDER | T3_MESH_FLIP_NORMAL |
                             T3_MESH_FLAT_NORMAL | T3_MESH_WIREFRAME | T3_MESH_QUADS;
  for (int o = 0; o < sc.nobjects; o++) {
    const t3_mesh& m = sc.obj[o].mesh;
    if (m.kind != T3_MESH_SOUP || (m.flags & edits)) return false;
    if ((sc.frame.flags & T3_SMOOTHING) && !m.norms) return false;
  }
  return sc.nobjects > 0;
}

int fast_signature(const DevScene& sc) {
  int sig = -1;
  for (int o = 0; o < sc.nobjects; o++) {
    if (is_wire(sc.obj[o].mesh)) continue;
    const int s = sc.obj[o].fast.sig;
    if (s == 0 || (sig >= 0 && s != sig)) return 0;
    sig = s;
  }
  return sig > 0 ? sig : 0;
}

template <int NL, int MODE, bool TEX, int SIG = 0, bool PLAIN = false>
static void launch_shade_t(const DevScene& sc, const unsigned long long* keys, const float4* rec,
                           const t3_outputs& out, int64_t npix, cudaStream_t st, const KeyState& ks) {
  constexpr int BLOCK = 256, PPT = 4;
  const int64_t grid = (npix + BLOCK * PPT - 1) / (BLOCK * PPT);
  if constexpr (MODE == T3_LIGHT_LAMPS && !TEX && SIG == 0) {
    // untextured lamp scenes with one common material shape (on plain soups,
    // an instance whose geometry path is compiled for them), or else one
    // common lobe signature
    const int fsig = fast_signature(sc);
    const bool plain = plain_soups(sc);
    constexpr int F = T3_SIG_FAST;
    if (NL == 2 && fsig == T3_SIG_PBR) {
      if (plain) return launch_shade_t<2, MODE, TEX, T3_SIG_PBR | F, true>(sc, keys, rec, out, npix, st, ks);
      return launch_shade_t<2, MODE, TEX, T3_SIG_PBR | F>(sc, keys, rec, out, npix, st, ks);
    }
    if (NL == 2 && fsig == T3_SIG_CLASSIC) {
      if (plain) return launch_shade_t<2, MODE, TEX, T3_SIG_CLASSIC | F, true>(sc, keys, rec, out, npix, st, ks);
      return launch_shade_t<2, MODE, TEX, T3_SIG_CLASSIC | F>(sc, keys, rec, out, npix, st, ks);
    }
    if (NL == 1 && fsig == T3_SIG_DIFFUSE) {
      if (plain) return launch_shade_t<1, MODE, TEX, T3_SIG_DIFFUSE | F, true>(sc, keys, rec, out, npix, st, ks);
      return launch_shade_t<1, MODE, TEX, T3_SIG_DIFFUSE | F>(sc, keys, rec, out, npix, st, ks);
    }
    const int sig = lobe_signature(sc);
    if (NL == 2 && sig == T3_SIG_PBR) return launch_shade_t<2, MODE, TEX, T3_SIG_PBR>(sc, keys, rec, out, npix, st, ks);
    if (NL == 2 && sig == T3_SIG_CLASSIC)
      return launch_shade_t<2, MODE, TEX, T3_SIG_CLASSIC>(sc, keys, rec, out, npix, st, ks);
    if (NL == 1 && sig == T3_SIG_DIFFUSE)
      return launch_shade_t<1, MODE, TEX, T3_SIG_DIFFUSE>(sc, keys, rec, out, npix, st, ks);
  }
  k_shade<BLOCK, PPT, NL, MODE, TEX, SIG, PLAIN><<<(unsigned)grid, BLOCK, 0, st>>>(sc, keys, rec, out, npix, ks);
}

template <int MODE, bool TEX>
static void launch_shade_m(const DevScene& sc, const unsigned long long* keys, const float4* rec,
                           const t3_outputs& out, int64_t npix, int max_lobes, cudaStream_t st,
                           const KeyState& ks) {
  if (max_lobes <= 1) launch_shade_t<1, MODE, TEX>(sc, keys, rec, out, npix, st, ks);
  else if (max_lobes == 2) launch_shade_t<2, MODE, TEX>(sc, keys, rec, out, npix, st, ks);
  else launch_shade_t<4, MODE, TEX>(sc, keys, rec, out, npix, st, ks);
}

cudaError_t launch_shade(const DevScene& sc_host, const DevScene* sc_dev, const unsigned long long* keys,
                         const float4* rec, const t3_outputs& out, int32_t* status, cudaStream_t st,
                         KeyState reset, MlpRows rows) {
  const t3_frame& fr = sc_host.frame;
  const int64_t npix = (int64_t)fr.width * fr.height;
  const int max_lobes = t3::max_lobes(sc_host), light_mode = sc_host.lighting.mode;
  const bool textured = has_textures(sc_host) != 0;
  if (light_mode == T3_LIGHT_LAMPS && textured)
    launch_shade_m<T3_LIGHT_LAMPS, true>(sc_host, keys, rec, out, npix, max_lobes, st, reset);
  else if (light_mode == T3_LIGHT_LAMPS)
    launch_shade_m<T3_LIGHT_LAMPS, false>(sc_host, keys, rec, out, npix, max_lobes, st, reset);
  else if (light_mode == T3_LIGHT_IBL_MC && textured)
    launch_shade_m<T3_LIGHT_IBL_MC, true>(sc_host, keys, rec, out, npix, max_lobes, st, reset);
  else if (light_mode == T3_LIGHT_IBL_MC)
    launch_shade_m<T3_LIGHT_IBL_MC, false>(sc_host, keys, rec, out, npix, max_lobes, st, reset);
  else if (light_mode == T3_LIGHT_IBL_PREFILTERED && textured)
    launch_shade_m<T3_LIGHT_IBL_PREFILTERED, true>(sc_host, keys, rec, out, npix, max_lobes, st, reset);
  else if (light_mode == T3_LIGHT_IBL_PREFILTERED)
    launch_shade_m<T3_LIGHT_IBL_PREFILTERED, false>(sc_host, keys, rec, out, npix, max_lobes, st, reset);
  else if (light_mode == T3_LIGHT_IBL_MLP)
    return launch_shade_mlp(sc_host, keys, rec, out, status, st, rows, rows.rows ? reset : KeyState());
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

} // namespace t3
