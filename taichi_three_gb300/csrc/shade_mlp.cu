// shade_mlp.cu -- the deferred shading pass with the learned IBL term
// (T3_LIGHT_IBL_MLP): interpolation and material evaluation on the CUDA cores,
// the network on the tensor cores.
//
// Two kernels (t3_render and the binned frame):
//   k_mlp_rows  one thread per pixel, many CTAs per SM (like the lamp pass):
//               empty pixels get the sky along the view ray; a covered pixel
//               interpolates its fragment, evaluates the material into the
//               weights of the network's nine outputs, adds emission and any
//               lamps, and appends one 96-byte row (the six mirrored direction
//               coordinates, roughness, metallic, the weights and the pixel
//               index) to a compact list.  It returns the keys it reads to
//               empty, as the lamp pass does.
//   k_mlp_net   one persistent CTA per SM of eight groups of four warps
//               (t3_mlp_group.cuh): each group takes 128 rows at a time,
//               encodes their Fourier features into its A operand chunk by
//               chunk while its leader warp issues the tcgen05.mma, reads the
//               result back from tensor memory and composes the pixel.
// Splitting them lets the gathers of the first run at full occupancy and the
// second hold only the network's state, so each keeps its SM busy.
//
// k_shade_mlp (t3_render_noalloc, which has no room for the row list) does
// both in one persistent kernel: each warp walks its own stream of 32-pixel
// chunks, shading 32 covered pixels as its quarter of a group's tile.
//
// Either way the pixel is
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
__device__ __forceinline__ void eval_mlp_coeffs(const DevObject& ob, const Frag& fg, MlpCoeffs& q) {
  const DevMaterial& mat = ob.mat;
  q.cd = q.c1 = q.c2 = q.base = v3(0.f, 0.f, 0.f);
  q.rough = 1.0f;
  q.metal = 0.0f;
  if constexpr ((SIG & T3_SIG_FAST) != 0) {
    // the PBR shape Mix(Lambert * C, CookTorrance(f0 = F), F) (FastMat): the
    // weights (1 - F) C and F with each parameter evaluated once -- the same
    // products as the loop below forms (1 x a = a, 0 + a = a exactly)
    const V3 c = eval_basic(mat.nodes[ob.fast.node[0]], fg);
    const V3 f = eval_value<false>(mat, ob.fast.node[1], fg);
    q.cd = one_minus(f) * c;
    q.c1 = f * f;
    q.c2 = f * one_minus(f);
    q.rough = eval_basic(mat.nodes[ob.fast.node[2]], fg).x;
    q.metal = fminf(1.0f, fmaxf(0.0f, (f.x + f.y + f.z) * (1.0f / 3.0f)));
    return;
  }
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

constexpr int kFusedGroups = 6, kFusedRing = 3, kFusedWarps = kFusedGroups * 4;
constexpr uint32_t kFusedSmem = mlp_group_smem(kFusedGroups, kFusedRing);

template <int NL, bool TEX, int SIG>
__global__ void __launch_bounds__(kFusedGroups * 128, 1)
k_shade_mlp(const __grid_constant__ DevScene scene, const unsigned long long* __restrict__ keys,
            const float4* __restrict__ rec, t3_outputs out, int64_t npix, int32_t* __restrict__ status) {
  const DevScene* sc = &scene;  // read through the constant cache
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ MlpShared<kFusedGroups> S;
  __shared__ int s_list[kFusedWarps][64];  // each warp's pending covered pixels

  const bool ok = mlp_cta_begin(sm, S, scene.lighting.mlp);  // ends with a CTA barrier
  const uint32_t tmem_base = S.tmem_slot;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (ok) {
    const t3_frame& fr = sc->frame;
    const t3_lighting& lt = sc->lighting;
    const Env env{lt.env, lt.env_w, lt.env_h, lt.env_half};
    const int H = fr.height;
    const int g = warp >> 2;
    MlpWarp W = mlp_warp_init<kFusedGroups, kFusedRing>(sm, S, tmem_base, fr);
    int* list = s_list[warp];
    // this warp's stream: 32-pixel chunks, strided over every warp of the grid
    const int64_t nchunks = (npix + 31) / 32;
    const int64_t stride = (int64_t)gridDim.x * kFusedWarps;
    int64_t chunk = (int64_t)blockIdx.x * kFusedWarps + warp;
    auto key_of = [&](int64_t c) {
      const int64_t i = c * 32 + lane;
      return c < nchunks && i < npix ? keys[i] : T3_EMPTY_KEY;
    };
    unsigned long long key = key_of(chunk);  // loaded one chunk ahead
    int pending = 0;                         // warp-uniform
    for (;;) {
      // empty pixels get the sky at once; covered ones join the list until 32 are pending
      while (pending < 32 && chunk < nchunks) {
        const int64_t i = chunk * 32 + lane;
        const unsigned long long k = key;
        key = key_of(chunk + stride);
        bool covered = false;
        if (i < npix) {
          if (k == T3_EMPTY_KEY) write_sky(fr, env, out, i);
          else covered = true;
        }
        const unsigned m = __ballot_sync(0xFFFFFFFFu, covered);
        if (covered) list[pending + __popc(m & ((1u << lane) - 1u))] = (int)i;
        pending += __popc(m);
        chunk += stride;
      }
      __syncwarp();
      // the group takes another tile while any of its warps has a pixel and
      // none has timed out (both votes give every warp of the group the same answer)
      const bool more = group_any(pending > 0, 1 + g);
      if (group_any(W.err, 1 + g) || !more) break;
      const int n = pending < 32 ? pending : 32;
      const int64_t pix = lane < n ? list[lane] : -1;
      const int carry = lane + 32 < pending ? list[lane + 32] : 0;
      __syncwarp();
      if (lane + 32 < pending) list[lane] = carry;
      pending -= n;

      // this lane's row: geometry, lobe weights, lamps, network inputs
      bool mine = false;
      MlpCoeffs q;
      float in[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      q.rough = 1.0f;
      q.metal = 0.0f;
      if (pix >= 0) {
        const int x = (int)(pix / H), y = (int)(pix - (int64_t)x * H);
        PixelGeom pg;
        const bool hit = pixel_geometry(sc, rec, keys[pix], x, y, out, pg);
        if (hit && pg.flat) {
          store_rgb(fr, out, pix, pg.fg.color);  // a line pixel
        } else if (hit) {
          mine = true;
          eval_mlp_coeffs<NL, TEX, SIG>(*pg.ob, pg.fg, q);
          if (lt.nlights > 0) {
            LobeState<NL> L;
            V3 amb, emi;
            if constexpr ((SIG & T3_SIG_FAST) != 0) eval_material_fast<NL, SIG>(*pg.ob, pg.fg, pg.vdir, L, amb, emi);
            else eval_material<NL, TEX, SIG>(pg.ob->mat, pg.fg, pg.vdir, L, amb, emi);
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
      const bool was_ok = !W.err;
      const bool good = warp_network<kFusedRing>(W, in, q.rough, q.metal, y);
      if (!good) {
        if (was_ok && lane == 0 && status) atomicOr(status, T3_STATUS_TIMEOUT);
      } else if (mine) {
        float e[9];
#pragma unroll
        for (int k = 0; k < 9; k++) e[k] = fmaxf(0.f, __expf(y[k]) - 1.0f);  // outputs are log1p
        const V3 ed = v3(e[0], e[1], e[2]), s1 = v3(e[3], e[4], e[5]), s2 = v3(e[6], e[7], e[8]);
        store_rgb(fr, out, pix, q.base + q.cd * ed + q.c1 * s1 + q.c2 * s2);
      }
    }
    if (!warp_drain(W) && lane == 0 && status) atomicOr(status, T3_STATUS_TIMEOUT);
  }
  if (!ok && threadIdx.x == 0 && status) atomicOr(status, T3_STATUS_TIMEOUT);
  mlp_cta_end(tmem_base);
}

// ---- the two-kernel path --------------------------------------------------------
// One row of the list: 6 x float4.
//   [0] in0..in3   [1] in4 in5 rough metal   [2] cd.xyz c1.x   [3] c1.yz c2.xy
//   [4] c2.z base.xyz   [5] pixel index (int bits), 0, 0, 0
constexpr int kRowVec = 6;

template <int BLOCK, int PPT, int NL, bool TEX, int SIG>
__global__ void __launch_bounds__(BLOCK, 3)
k_mlp_rows(const __grid_constant__ DevScene scene, const unsigned long long* __restrict__ keys,
           const float4* __restrict__ rec, t3_outputs out, int64_t npix, float4* __restrict__ rows,
           uint32_t* __restrict__ nrows, KeyState reset) {
  const DevScene* sc = &scene;
  __shared__ int s_list[BLOCK * PPT];
  __shared__ unsigned long long s_key[BLOCK * PPT];
  __shared__ int s_count;
  const t3_frame& fr = sc->frame;
  const t3_lighting& lt = sc->lighting;
  const Env env{lt.env, lt.env_w, lt.env_h, lt.env_half};
  const int H = fr.height;
  const int lane = threadIdx.x & 31;
  unsigned long long* reset_keys = reset.tag_word ? const_cast<unsigned long long*>(keys) : nullptr;
  if (threadIdx.x == 0) s_count = 0;
  // the keys are empty once every block has run: mark them so for the next frame
  if (reset.tag_word && blockIdx.x == 0 && threadIdx.x == 0) *reset.tag_word = reset.tag;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * BLOCK * PPT;
  // empty pixels get the sky at once; covered ones are compacted with their keys
#pragma unroll
  for (int k = 0; k < PPT; k++) {
    const int local = k * BLOCK + threadIdx.x;
    const int64_t i = base + local;
    bool covered = false;
    unsigned long long key = T3_EMPTY_KEY;
    if (i < npix) {
      key = keys[i];
      if (key == T3_EMPTY_KEY) write_sky(fr, env, out, i);
      else covered = true;
      if (covered && reset_keys) reset_keys[i] = T3_EMPTY_KEY;
    }
    const unsigned m = __ballot_sync(0xFFFFFFFFu, covered);
    if (m) {
      int slot = 0;
      if (lane == 0) slot = atomicAdd(&s_count, __popc(m));
      slot = __shfl_sync(0xFFFFFFFFu, slot, 0);
      if (covered) {
        const int at = slot + __popc(m & ((1u << lane) - 1u));
        s_list[at] = local;
        s_key[at] = key;
      }
    }
  }
  __syncthreads();
  const int n = s_count;
  for (int j0 = 0; j0 < n; j0 += BLOCK) {  // block-uniform trip count: whole warps vote below
    const int j = j0 + threadIdx.x;
    bool have = false;
    int64_t pix = 0;
    MlpCoeffs q;
    float in[6];
    if (j < n) {
      pix = base + s_list[j];
      const int x = (int)(pix / H), y = (int)(pix - (int64_t)x * H);
      PixelGeom pg;
      const bool hit = pixel_geometry(sc, rec, s_key[j], x, y, out, pg);
      if (hit && pg.flat) {
        store_rgb(fr, out, pix, pg.fg.color);  // a line pixel
      } else if (hit) {
        have = true;
        eval_mlp_coeffs<NL, TEX, SIG>(*pg.ob, pg.fg, q);
        if (lt.nlights > 0) {
          LobeState<NL> L;
          V3 amb, emi;
          if constexpr ((SIG & T3_SIG_FAST) != 0) eval_material_fast<NL, SIG>(*pg.ob, pg.fg, pg.vdir, L, amb, emi);
          else eval_material<NL, TEX, SIG>(pg.ob->mat, pg.fg, pg.vdir, L, amb, emi);
          q.base = q.base + lamps_term<NL, SIG>(lt, L, pg.fg, pg.vdir);
        }
        const float nv[6] = {pg.fg.normal.x, pg.fg.normal.y, pg.fg.normal.z, pg.vdir.x, pg.vdir.y, pg.vdir.z};
        mirror_inputs(nv, in);
      } else {
        store_rgb(fr, out, pix, env_sample(env, view_ray(fr, xadd((float)x, fr.bias[0]),
                                                         xadd((float)y, fr.bias[1]))));
      }
    }
    // one global atomic per warp reserves the warp's rows
    const unsigned m = __ballot_sync(0xFFFFFFFFu, have);
    if (m) {
      uint32_t slot = 0;
      if (lane == 0) slot = atomicAdd(nrows, (uint32_t)__popc(m));
      slot = __shfl_sync(0xFFFFFFFFu, slot, 0);
      if (have) {
        float4* r = rows + (size_t)(slot + __popc(m & ((1u << lane) - 1u))) * kRowVec;
        r[0] = make_float4(in[0], in[1], in[2], in[3]);
        r[1] = make_float4(in[4], in[5], q.rough, q.metal);
        r[2] = make_float4(q.cd.x, q.cd.y, q.cd.z, q.c1.x);
        r[3] = make_float4(q.c1.y, q.c1.z, q.c2.x, q.c2.y);
        r[4] = make_float4(q.c2.z, q.base.x, q.base.y, q.base.z);
        r[5] = make_float4(__int_as_float((int)pix), 0.f, 0.f, 0.f);
      }
    }
  }
}

constexpr int kNetGroups = 8, kNetRing = 2;
constexpr uint32_t kNetSmem = mlp_group_smem(kNetGroups, kNetRing);

__global__ void __launch_bounds__(kNetGroups * 128, 1)
k_mlp_net(const __grid_constant__ DevScene scene, const float4* __restrict__ rows,
          const uint32_t* __restrict__ nrows, t3_outputs out, int32_t* __restrict__ status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ MlpShared<kNetGroups> S;
  const bool ok = mlp_cta_begin(sm, S, scene.lighting.mlp);  // ends with a CTA barrier
  const uint32_t tmem_base = S.tmem_slot;
  if (ok) {
    const t3_frame& fr = scene.frame;
    const int g = threadIdx.x >> 7;
    MlpWarp W = mlp_warp_init<kNetGroups, kNetRing>(sm, S, tmem_base, fr);
    const uint32_t n = *nrows;  // written by k_mlp_rows, the previous kernel
    const int64_t ntiles = ((int64_t)n + 127) / 128;
    // every warp of a group walks the same tiles: no vote is needed
    for (int64_t t = (int64_t)blockIdx.x * kNetGroups + g; t < ntiles; t += (int64_t)gridDim.x * kNetGroups) {
      const int64_t row = t * 128 + W.row;
      const bool valid = row < (int64_t)n;
      const float4* r = rows + row * kRowVec;
      const float4 a = valid ? __ldg(r) : make_float4(0.f, 0.f, 0.f, 0.f);
      const float4 b = valid ? __ldg(r + 1) : make_float4(0.f, 0.f, 1.f, 0.f);
      const float in[6] = {a.x, a.y, a.z, a.w, b.x, b.y};
      // the row of the group's next tile, on its way while this one runs
      const int64_t next = (t + (int64_t)gridDim.x * kNetGroups) * 128 + W.row;
      if (next < (int64_t)n) asm volatile("prefetch.global.L1 [%0];" :: "l"(rows + next * kRowVec));
      float y[16];
      const bool was_ok = !W.err;
      if (!warp_network<kNetRing>(W, in, b.z, b.w, y)) {
        if (was_ok && (threadIdx.x & 31) == 0 && status) atomicOr(status, T3_STATUS_TIMEOUT);
      } else if (valid) {
        const float4 c = __ldg(r + 2), d = __ldg(r + 3), e4 = __ldg(r + 4), f = __ldg(r + 5);
        float e[9];
#pragma unroll
        for (int k = 0; k < 9; k++) e[k] = fmaxf(0.f, __expf(y[k]) - 1.0f);  // outputs are log1p
        const V3 cd = v3(c.x, c.y, c.z), c1 = v3(c.w, d.x, d.y), c2 = v3(d.z, d.w, e4.x);
        const V3 base = v3(e4.y, e4.z, e4.w);
        const V3 ed = v3(e[0], e[1], e[2]), s1 = v3(e[3], e[4], e[5]), s2 = v3(e[6], e[7], e[8]);
        store_rgb(fr, out, (int64_t)__float_as_int(f.x), base + cd * ed + c1 * s1 + c2 * s2);
      }
    }
    if (!warp_drain(W) && (threadIdx.x & 31) == 0 && status) atomicOr(status, T3_STATUS_TIMEOUT);
  }
  if (!ok && threadIdx.x == 0 && status) atomicOr(status, T3_STATUS_TIMEOUT);
  mlp_cta_end(tmem_base);
}

static cudaError_t sm_count(int& nsm) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return e;
}

template <int NL, bool TEX, int SIG>
static cudaError_t launch_shade_mlp_t(const DevScene& sc, const unsigned long long* keys,
                                      const float4* rec, const t3_outputs& out, int64_t npix,
                                      int32_t* status, cudaStream_t st, const MlpRows& rows,
                                      const KeyState& reset) {
  int nsm = 0;
  cudaError_t e = sm_count(nsm);
  if (e != cudaSuccess) return e;
  if (rows.rows) {
    constexpr int BLOCK = 256, PPT = 4;
    const int64_t grid = (npix + BLOCK * PPT - 1) / (BLOCK * PPT);
    if (grid <= 0) return cudaSuccess;
    k_mlp_rows<BLOCK, PPT, NL, TEX, SIG><<<(unsigned)grid, BLOCK, 0, st>>>(sc, keys, rec, out, npix, rows.rows,
                                                                         rows.count, reset);
    e = cudaGetLastError();
    if (e == cudaSuccess && rows.split) e = cudaEventRecord(rows.split, st);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_mlp_net, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kNetSmem);
    if (e != cudaSuccess) return e;
    k_mlp_net<<<nsm, kNetGroups * 128, kNetSmem, st>>>(sc, rows.rows, rows.count, out, status);
    return cudaGetLastError();
  }
  e = cudaFuncSetAttribute(k_shade_mlp<NL, TEX, SIG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)kFusedSmem);
  if (e != cudaSuccess) return e;
  const int64_t nchunks = (npix + 31) / 32;
  const int64_t want = (nchunks + kFusedWarps - 1) / kFusedWarps;
  const int grid = (int)(want < nsm ? want : nsm);
  if (grid <= 0) return cudaSuccess;
  k_shade_mlp<NL, TEX, SIG><<<grid, kFusedGroups * 128, kFusedSmem, st>>>(sc, keys, rec, out, npix, status);
  return cudaGetLastError();
}

cudaError_t launch_shade_mlp(const DevScene& sc, const unsigned long long* keys, const float4* rec,
                             const t3_outputs& out, int32_t* status, cudaStream_t st, const MlpRows& rows,
                             const KeyState& reset) {
  const int64_t npix = (int64_t)sc.frame.width * sc.frame.height;
  // untextured PBR scenes take the instance with the lobe kinds as constants,
  // and with each material parameter evaluated once when every object has the
  // PBR material shape.  (A row prepass compiled for plain face soups, as the
  // lamp pass has, rounds some network inputs differently from the one-kernel
  // pass of the allocation-free frame, whose pixels must stay equal to these.)
  if (!has_textures(sc) && fast_signature(sc) == T3_SIG_PBR)
    return launch_shade_mlp_t<2, false, T3_SIG_PBR | T3_SIG_FAST>(sc, keys, rec, out, npix, status, st, rows,
                                                                  reset);
  if (!has_textures(sc) && lobe_signature(sc) == T3_SIG_PBR)
    return launch_shade_mlp_t<2, false, T3_SIG_PBR>(sc, keys, rec, out, npix, status, st, rows, reset);
  if (max_lobes(sc) <= 2) return launch_shade_mlp_t<2, true, 0>(sc, keys, rec, out, npix, status, st, rows, reset);
  return launch_shade_mlp_t<4, true, 0>(sc, keys, rec, out, npix, status, st, rows, reset);
}

} // namespace t3
