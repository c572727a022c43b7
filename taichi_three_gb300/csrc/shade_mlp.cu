// shade_mlp.cu -- the deferred shading pass with the learned IBL term
// (T3_LIGHT_IBL_MLP): interpolation and material evaluation on the CUDA cores,
// the network on the tensor cores, fused in one persistent kernel.
//
// One persistent CTA per SM holds the packed network in shared memory and
// kMlpGroups independent groups of 128 threads (t3_mlp_group.cuh).  Each
// group walks its own stream of 128-pixel chunks: empty pixels get the sky
// along the view ray at once, covered ones are appended to the group's list.
// Whenever 128 covered pixels are pending (or the stream ends), the group's
// thread t takes list entry t: it interpolates the fragment, evaluates the
// material into the weights of the network's nine outputs, adds emission and
// any lamps, and encodes its Fourier features into row t of the A operand
// chunk by chunk while the group's elected thread issues the layers'
// tcgen05.mma; thread t then reads row t of the result from tensor memory and
// composes the pixel:
//   rgb = emission + lamps + cd * E_d + c1 * S1 + c2 * S2,
// with (E_d, S1, S2) = expm1 of the network outputs, cd the summed Lambert lobe
// weights, c1 / c2 the CookTorrance lobe weight times f0 / (1 - f0) -- the
// expectation of the Monte Carlo estimator of t3_ibl.cuh (linear in the lobe
// weights), with the integrals read from the network instead of sampled.
#include "t3_shading.cuh"
#include "t3_mlp_group.cuh"

namespace t3 {

struct MlpCoeffs {
  V3 cd, c1, c2, base;
  float rough, metal;
};

// lobe weights of one fragment (materials of Lambert, CookTorrance and
// Emission leaves with at most one CookTorrance; checked on the host)
template <int NL, bool TEX, int SIG>
__device__ __forceinline__ void eval_mlp_coeffs(const DevMaterial& mat, const Frag& fg, MlpCoeffs& q) {
  q.cd = q.c1 = q.c2 = q.base = v3(0.f, 0.f, 0.f);
  q.rough = 1.0f;
  q.metal = 0.0f;
#pragma unroll
  for (int k = 0; k < NL; k++) {
    if (k >= mat.nlobes) continue;
    const DevLobe& lb = mat.lobes[k];
    V3 w = v3(1.f, 1.f, 1.f);
    for (int j = 0; j < lb.nfac; j++) {
      const int fj = lb.fac[j];
      const V3 f = eval_value<TEX>(mat, fj & 0xFFFF, fg);
      w = w * ((fj & T3_FAC_ONE_MINUS) ? one_minus(f) : f);
    }
    const int kind = SIG ? sig_kind<SIG>(k) : lb.kind;
    if (kind == T3_OP_LAMBERT) {
      q.cd = q.cd + w;
    } else if (kind == T3_OP_COOK) {
      const V3 f0 = eval_value<TEX>(mat, lb.p1, fg);
      q.rough = eval_value<TEX>(mat, lb.p0, fg).x;
      q.c1 = q.c1 + w * f0;
      q.c2 = q.c2 + w * one_minus(f0);
      q.metal = fminf(1.0f, fmaxf(0.0f, (f0.x + f0.y + f0.z) * (1.0f / 3.0f)));
    } else if (kind == T3_OP_EMISSION) {
      q.base = q.base + w;
    }
  }
}

// raster outputs of an empty pixel and the sky along its view ray
__device__ __forceinline__ void write_sky(const t3_frame& fr, const Env& env, const t3_outputs& out,
                                          int64_t i) {
  const int H = fr.height;
  const int x = (int)(i / H), y = (int)(i - (int64_t)x * H);
  if (out.face_id) out.face_id[i] = -1;
  if (out.depth) out.depth[i] = fr.maxdepth;
  if (out.depth_f) out.depth_f[i] = __int_as_float(0x7f800000);
  store_rgb(fr, out, i, env_sample(env, view_ray(fr, xadd((float)x, fr.bias[0]), xadd((float)y, fr.bias[1]))));
}

template <int NL, bool TEX, int SIG>
__global__ void __launch_bounds__(kMlpGroups * 128, 1)
k_shade_mlp(const __grid_constant__ DevScene scene, const unsigned long long* __restrict__ keys,
            const float4* __restrict__ rec, t3_outputs out, int64_t npix, int32_t* __restrict__ status) {
  const DevScene* sc = &scene;  // read through the constant cache
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t cta_bar;
  __shared__ __align__(8) uint64_t gbar[kMlpGroups][3];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_list[kMlpGroups][256];  // pending covered pixels (< 128 carried + one chunk)
  __shared__ int s_count[kMlpGroups];

  const t3_frame& fr = sc->frame;
  const t3_lighting& lt = sc->lighting;
  const Env env{lt.env, lt.env_w, lt.env_h, lt.env_half};
  const int H = fr.height;
  const int lane = threadIdx.x & 31;
  const int g = threadIdx.x >> 7;
  if (threadIdx.x < kMlpGroups) s_count[threadIdx.x] = 0;
  bool ok = group_cta_begin(sm, &cta_bar, gbar, &tmem_slot, lt.mlp);  // ends with a CTA barrier
  const uint32_t tmem_base = tmem_slot;
  MlpGroup G = group_init(sm, gbar, tmem_base);
  int* list = s_list[g];

  // each group walks its own stream of 128-pixel chunks
  const int64_t nchunks = (npix + 127) / 128;
  const int64_t stride = (int64_t)gridDim.x * kMlpGroups;
  int64_t chunk = (int64_t)blockIdx.x * kMlpGroups + g;
  // the key of this thread's pixel in the next chunk, loaded one chunk ahead
  auto key_of = [&](int64_t c) {
    const int64_t i = c * 128 + G.row;
    return c < nchunks && i < npix ? keys[i] : T3_EMPTY_KEY;
  };
  unsigned long long key = key_of(chunk);
  int pending = 0;
  while (ok) {
    // collect covered pixels until a full tile is pending or the stream ends
    while (pending < 128 && chunk < nchunks) {
      const int64_t i = chunk * 128 + G.row;
      const unsigned long long k = key;
      key = key_of(chunk + stride);
      bool covered = false;
      if (i < npix) {
        if (k == T3_EMPTY_KEY) write_sky(fr, env, out, i);
        else covered = true;
      }
      const unsigned m = __ballot_sync(0xFFFFFFFFu, covered);
      if (m) {
        int slot = 0;
        if (lane == 0) slot = atomicAdd(&s_count[g], __popc(m));
        slot = __shfl_sync(0xFFFFFFFFu, slot, 0);
        if (covered) list[slot + __popc(m & ((1u << lane) - 1u))] = (int)i;
      }
      group_sync(G.id);
      pending = s_count[g];
      group_sync(G.id);  // every thread has read the count before the next appends
      chunk += stride;
    }
    if (pending == 0) break;
    const int n = pending < 128 ? pending : 128;

    // thread row r shades list entry r: geometry, lobe weights, lamps, inputs
    bool mine = false;
    int64_t pix = 0;
    MlpCoeffs q;
    float in[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    q.rough = 1.0f;
    q.metal = 0.0f;
    if (G.row < n) {
      pix = list[G.row];
      const int x = (int)(pix / H), y = (int)(pix - (int64_t)x * H);
      PixelGeom pg;
      const bool hit = pixel_geometry(sc, rec, keys[pix], x, y, out, pg);
      if (hit && pg.flat) {
        store_rgb(fr, out, pix, pg.fg.color);  // a line pixel
      } else if (hit) {
        mine = true;
        eval_mlp_coeffs<NL, TEX, SIG>(pg.ob->mat, pg.fg, q);
        if (lt.nlights > 0) {
          LobeState<NL> L;
          V3 amb, emi;
          eval_material<NL, TEX, SIG>(pg.ob->mat, pg.fg, pg.vdir, L, amb, emi);
          q.base = q.base + lamps_term<NL, SIG>(lt, L, pg.fg, pg.vdir);
        }
        const float nv[6] = {pg.fg.normal.x, pg.fg.normal.y, pg.fg.normal.z, pg.vdir.x, pg.vdir.y, pg.vdir.z};
        mirror_inputs(nv, in);
      } else {
        store_rgb(fr, out, pix, env_sample(env, view_ray(fr, xadd((float)x, fr.bias[0]),
                                                         xadd((float)y, fr.bias[1]))));
      }
    }
    float y[16];
    if (!group_tile(G, in, q.rough, q.metal, y)) {  // group-uniform outcome
      ok = false;
      break;
    }
    if (mine) {
      float e[9];
#pragma unroll
      for (int k = 0; k < 9; k++) e[k] = fmaxf(0.f, __expf(y[k]) - 1.0f);  // outputs are log1p
      const V3 ed = v3(e[0], e[1], e[2]), s1 = v3(e[3], e[4], e[5]), s2 = v3(e[6], e[7], e[8]);
      store_rgb(fr, out, pix, q.base + q.cd * ed + q.c1 * s1 + q.c2 * s2);
    }
    // drop the n entries just shaded (every thread read its entry before the
    // tile's first group barrier)
    const int rest = pending - n;
    const int carry = G.row < rest ? list[n + G.row] : 0;
    group_sync(G.id);
    if (G.row < rest) list[G.row] = carry;
    if (G.row == 0) s_count[g] = rest;
    group_sync(G.id);
    pending = rest;
  }
  if (!ok && status && G.row == 0) atomicOr(status, T3_STATUS_TIMEOUT);
  group_cta_end(tmem_base);
}

template <int NL, bool TEX, int SIG>
static cudaError_t launch_shade_mlp_t(const DevScene& sc, const unsigned long long* keys,
                                      const float4* rec, const t3_outputs& out, int64_t npix,
                                      int32_t* status, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(k_shade_mlp<NL, TEX, SIG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kMlpGroupSmem);
  if (e != cudaSuccess) return e;
  int dev = 0, nsm = 0;
  e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const int64_t nchunks = (npix + 127) / 128;
  const int64_t want = (nchunks + kMlpGroups - 1) / kMlpGroups;
  const int grid = (int)(want < nsm ? want : nsm);
  if (grid <= 0) return cudaSuccess;
  k_shade_mlp<NL, TEX, SIG><<<grid, kMlpGroups * 128, kMlpGroupSmem, st>>>(sc, keys, rec, out, npix, status);
  return cudaGetLastError();
}

cudaError_t launch_shade_mlp(const DevScene& sc, const unsigned long long* keys, const float4* rec,
                             const t3_outputs& out, int32_t* status, cudaStream_t st) {
  const int64_t npix = (int64_t)sc.frame.width * sc.frame.height;
  // untextured PBR scenes take the instance with the lobe kinds as constants
  if (!has_textures(sc) && lobe_signature(sc) == T3_SIG_PBR)
    return launch_shade_mlp_t<2, false, T3_SIG_PBR>(sc, keys, rec, out, npix, status, st);
  if (max_lobes(sc) <= 2) return launch_shade_mlp_t<2, true, 0>(sc, keys, rec, out, npix, status, st);
  return launch_shade_mlp_t<4, true, 0>(sc, keys, rec, out, npix, status, st);
}

} // namespace t3
