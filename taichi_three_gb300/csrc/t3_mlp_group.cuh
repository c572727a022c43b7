// t3_mlp_group.cuh -- the learned-IBL network on the tensor cores for the fused
// shading kernels: groups of four warps per CTA, each group's warps working
// through a 128-row tile without group-wide barriers.
//
// A CTA holds the packed network once (t3_mlp_tc.cuh layout, 70,464 bytes).
// Group g owns TMEM columns [64 g, 64 g + 64) and a ring of two or three 8 KB
// A-chunk buffers; warp q of a group owns rows 32 q .. 32 q + 31 of the group's tile
// (the TMEM lanes its quarter of the SM's lanes can read).  The group's warp 0
// is its leader: its lane 0 issues every tcgen05.mma of the group, so each
// layer's accumulation runs in issue order on one thread.  Per tile:
//   layer 1  the warps encode the 400 inputs in 13 K chunks (half an input
//            coordinate = 32 features, then the 16 tail inputs) into the ring.
//            Warps 1-3 arrive on the buffer's `full` barrier once their 32
//            rows are written and go on to the next chunk; the leader writes
//            its rows, waits for `full`, issues the chunk's MMAs and commits
//            them to the buffer's `empty` barrier, which every warp waits on
//            before rewriting that buffer a ring later; after the last
//            chunk it also commits to `done`.
//   2 .. 4   after `done`, each warp reads its rows of the accumulator
//            (tcgen05.ld), adds the bias and applies ReLU while rounding to
//            BF16 (cvt.rn.relu.bf16x2) into its rows of H (over ring buffers 0
//            and 1); warps 1-3 arrive on `hfull`, and the leader, after it,
//            issues the next layer into the same columns and commits to `done`.
// Only the leader waits for the other warps (on mbarriers, suspended, not
// spinning); the others wait only for the MMAs whose results they read, so
// one warp's gathers and encoding run while another's wait.  The group meets
// at a named barrier once per tile, for the votes on whether to go on.
//
// Every wait is bounded.  A warp whose wait runs out records it and from then
// on skips its waits and outputs but still makes every arrival (a leader
// still issues and commits), so the group's other warps see the protocol
// through; the group stops at its next votes (one on pixels left, one on
// time-outs: every warp of the group gets the same answers, so all of them
// leave the loop together).  Before TMEM is freed every leader waits
// (bounded) for its own last MMAs.
#pragma once

#include "t3_mlp_tc.cuh"

namespace t3 {

constexpr int kMaxRing = 3;                        // A-chunk buffers per group, at most
constexpr uint32_t kGroupBase = 71680;             // kBlob rounded up to 1 KB
constexpr uint32_t kChunkBytes = 128 * 32 * 2;     // 128 rows x 32 BF16
constexpr uint32_t kGroupTmemCols = 512;
constexpr uint32_t kMlpWaitLimit = 1u << 24;       // try_wait rounds of one wait
static_assert(kGroupBase >= kBlob, "packed network overlaps the group areas");
static_assert(2 * kChunkBytes == 128 * 64 * 2, "H spans ring buffers 0 and 1");

// shared memory of a CTA of G groups with RING chunk buffers each (H, 128 x 64
// BF16, lies over buffers 0 and 1)
__host__ __device__ constexpr uint32_t mlp_group_smem(int G, int RING) {
  return kGroupBase + (uint32_t)G * RING * kChunkBytes;
}

// The shared-memory mbarriers of one group.
struct GroupBars {
  uint64_t full[kMaxRing];   // 3 arrivals (warps 1-3): chunk rows written
  uint64_t empty[kMaxRing];  // MMA commit: the chunk's MMAs have read the buffer
  uint64_t hfull;            // 3 arrivals (warps 1-3): H rows written (layer input)
  uint64_t done;             // MMA commit: a layer's accumulator is complete
  uint64_t drain;            // the leader's last commit (used once)
};

template <int G>
struct MlpShared {
  static_assert(G * 64 <= (int)kGroupTmemCols, "TMEM columns");
  GroupBars g[G];
  uint64_t cta_bar;          // the network's bulk copy
  uint32_t tmem_slot;
};

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(bar) : "memory");
}

// true on every thread of the group iff v is true on any thread
__device__ __forceinline__ bool group_any(bool v, int id) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n"
      " bar.red.or.pred p, %2, 128, q;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(r) : "r"((uint32_t)v), "r"(id) : "memory");
  return r != 0;
}

// ---- packed FP32 pairs (f32x2 arithmetic: two lanes' worth per instruction) ----
__device__ __forceinline__ uint64_t f2(float lo, float hi) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void f2_split(uint64_t v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t f2_add(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ uint64_t f2_sub(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ uint64_t f2_mul(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
// BF16 pair of the packed FP32 pair, ReLU applied (low half = low lane)
__device__ __forceinline__ uint32_t bf16x2_relu(uint64_t v) {
  float lo, hi;
  f2_split(v, lo, hi);
  uint32_t r;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}
__device__ __forceinline__ uint32_t bf16x2(uint64_t v) {
  float lo, hi;
  f2_split(v, lo, hi);
  uint32_t r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}

// Half h of coordinate x's Fourier features (packed order of t3_mlp_tc.cuh:
// sines of octaves 4h..4h+3, then their cosines) as 16 BF16 pairs.  The
// double-angle steps s' = (2 s) c, c' = (c - s)(c + s) run on two base phases
// per f32x2 instruction and round exactly as encode_coord's scalar steps, so
// both see the same FP32 features.  st carries the (sin, cos) pairs of the
// base phases (j = 0,1 and 2,3) from half 0 to half 1.
__device__ __forceinline__ void encode_half_bf16(float x, int h, uint64_t st[4], uint32_t out[16]) {
  const float base[4] = {3.141592653589793f, 3.7360043360892607f, 4.442882938158366f, 5.283508001182123f};
  if (h == 0) {
    float s[4], c[4];
#pragma unroll
    for (int j = 0; j < 4; j++) __sincosf(x * base[j], &s[j], &c[j]);
    st[0] = f2(s[0], s[1]);  // sines, j = 0, 1
    st[1] = f2(c[0], c[1]);  // cosines, j = 0, 1
    st[2] = f2(s[2], s[3]);
    st[3] = f2(c[2], c[3]);
  }
  const uint64_t two = f2(2.0f, 2.0f);
#pragma unroll
  for (int o = 0; o < 4; o++) {
    out[o * 2] = bf16x2(st[0]);
    out[o * 2 + 1] = bf16x2(st[2]);
    out[8 + o * 2] = bf16x2(st[1]);
    out[8 + o * 2 + 1] = bf16x2(st[3]);
#pragma unroll
    for (int p = 0; p < 4; p += 2) {
      const uint64_t s = st[p], c = st[p + 1];
      st[p] = f2_mul(f2_mul(two, s), c);
      st[p + 1] = f2_mul(f2_sub(c, s), f2_add(c, s));
    }
  }
}

// tcgen05.ld of 16 columns without the wait (the caller waits once for several)
__device__ __forceinline__ void tc_ld16_async(uint32_t taddr, uint32_t r[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// ---- MMA issue (the leader's lane 0) ---------------------------------------------
// D (TMEM column col of the group) = A (ksteps x K16 of a_off) * W^T; no commit
__device__ __forceinline__ void mma_issue(const unsigned char* sm, uint32_t tmem, uint32_t a_off,
                                          uint32_t a_sbo, uint32_t w_off, uint32_t w_sbo, int ksteps, int N,
                                          bool accumulate_first) {
  const uint32_t a = smem_addr(sm + a_off), w = smem_addr(sm + w_off);
  const uint32_t idesc = tc_idesc(128, N);
  for (int ks = 0; ks < ksteps; ks++)
    tc_mma(tmem, tc_desc(a + ks * 256u, 128u, a_sbo), tc_desc(w + ks * 256u, 128u, w_sbo), idesc,
           (ks > 0 || accumulate_first) ? 1u : 0u);
}

// ---- the group's warps -------------------------------------------------------------
struct MlpWarp {
  unsigned char* sm;  // CTA shared memory (packed network at 0)
  uint32_t tmem;      // the group's first column, this warp's lane quarter
  uint32_t bars;      // shared address of the group's GroupBars
  uint32_t area;      // shared byte offset of the group's ring (and H)
  uint32_t chunk;     // chunks of the group issued so far (ring position)
  uint32_t dph;       // parity of the next `done` completion
  uint32_t hph;       // parity of the next `hfull` completion
  uint32_t limit;     // polls of one wait
  int row;            // this lane's row of the tile
  bool leader;        // warp 0 of the group: issues the group's MMAs
  bool starve;        // issue nothing (tests of the timeout path)
  bool err;           // a wait ran out (warp-uniform)
};

__device__ __forceinline__ uint32_t bar_full(uint32_t bars, int b) { return bars + 8u * b; }
__device__ __forceinline__ uint32_t bar_empty(uint32_t bars, int b) { return bars + 8u * (kMaxRing + b); }
__device__ __forceinline__ uint32_t bar_hfull(uint32_t bars) { return bars + 8u * (2 * kMaxRing); }
__device__ __forceinline__ uint32_t bar_done(uint32_t bars) { return bars + 8u * (2 * kMaxRing + 1); }
__device__ __forceinline__ uint32_t bar_drain(uint32_t bars) { return bars + 8u * (2 * kMaxRing + 2); }

__device__ __forceinline__ void warp_wait(MlpWarp& W, uint32_t bar, uint32_t parity) {
  if (W.err) return;
  const bool ok = mbar_wait_bounded(bar, parity, W.limit);
  W.err = !__all_sync(0xFFFFFFFFu, ok);
}

// The warp's rows are written (shared memory for the MMAs, TMEM reads done).
// Warps 1-3 arrive on `bar`; the leader waits for their three arrivals
// (phase `parity`) and then its lane 0 runs issue().
template <typename Issue>
__device__ __forceinline__ void warp_handoff(MlpWarp& W, uint32_t bar, uint32_t parity, Issue issue) {
  fence_async_smem();
  tc_fence_before();
  __syncwarp();
  if (!W.leader) {
    if ((threadIdx.x & 31) == 0) mbar_arrive(bar);
    return;
  }
  warp_wait(W, bar, parity);
  if ((threadIdx.x & 31) == 0 && !W.starve) {
    tc_fence_after();
    issue();
  }
  __syncwarp();
}

// Layer-1 K chunk k (0..12) of this warp's rows into the next ring buffer.
template <int RING>
__device__ __forceinline__ void warp_chunk(MlpWarp& W, int k, const float in[6], float rough, float metal,
                                           uint64_t st[4]) {
  const uint32_t c = W.chunk++;
  const int b = (int)(c % RING);
  if (c >= (uint32_t)RING) warp_wait(W, bar_empty(W.bars, b), (c / RING - 1) & 1u);
  unsigned char* A = W.sm + W.area + (uint32_t)b * kChunkBytes;
  if (k < 12) {
    uint32_t f[16];
    encode_half_bf16(in[k >> 1], k & 1, st, f);
#pragma unroll
    for (int q = 0; q < 4; q++)
      *reinterpret_cast<uint4*>(A + tc_chunk_off(W.row, 8 * q, 32)) = make_uint4(f[4 * q], f[4 * q + 1],
                                                                                 f[4 * q + 2], f[4 * q + 3]);
  } else {
    // roughness, metallic, zero padding (K = 16 layout)
    float t[8] = {rough, metal, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    *reinterpret_cast<uint4*>(A + tc_chunk_off(W.row, 0, 16)) = pack8_bf16(t);
    *reinterpret_cast<uint4*>(A + tc_chunk_off(W.row, 8, 16)) = make_uint4(0u, 0u, 0u, 0u);
  }
  const uint32_t bars = W.bars, tmem = W.tmem & 0xFFFFu, a_off = W.area + (uint32_t)b * kChunkBytes;
  const unsigned char* sm = W.sm;
  warp_handoff(W, bar_full(bars, b), (c / RING) & 1u, [&] {
    if (k < 12) mma_issue(sm, tmem, a_off, 512u, kW1 + (uint32_t)k * 512u, 6400u, 2, 64, k > 0);
    else mma_issue(sm, tmem, a_off, 256u, kW1 + 6144u, 6400u, 1, 64, true);
    tc_commit(bar_empty(bars, b));
    if (k == 12) tc_commit(bar_done(bars));
  });
}

// bias + ReLU of this warp's rows of the layer output, as BF16 into H
__device__ __forceinline__ void warp_epilogue(MlpWarp& W, uint32_t b_off) {
  const uint64_t* bias = reinterpret_cast<const uint64_t*>(W.sm + b_off);  // FP32 pairs
  unsigned char* Hm = W.sm + W.area;
#pragma unroll
  for (int c = 0; c < 64; c += 16) {
    uint32_t r[16];
    tc_ld16_async(W.tmem + c, r);
    tc_wait_ld();
    uint32_t h[8];
#pragma unroll
    for (int i = 0; i < 8; i++)
      h[i] = bf16x2_relu(f2_add(f2(__uint_as_float(r[2 * i]), __uint_as_float(r[2 * i + 1])), bias[(c >> 1) + i]));
#pragma unroll
    for (int q = 0; q < 2; q++)
      *reinterpret_cast<uint4*>(Hm + tc_chunk_off(W.row, c + 8 * q, 64)) =
          make_uint4(h[4 * q], h[4 * q + 1], h[4 * q + 2], h[4 * q + 3]);
  }
}

// The network for the warp's rows of one tile: in = the row's six direction
// coordinates (already mirrored), rough, metal; rows whose lane has no pixel
// run on whatever they hold.  out[16]: the row's output.  False when a wait
// ran out (now or earlier): the output is then not to be used.
template <int RING>
__device__ __forceinline__ bool warp_network(MlpWarp& W, const float in[6], float rough, float metal,
                                             float out[16]) {
  uint64_t st[4];
#pragma unroll
  for (int k = 0; k < 13; k++) warp_chunk<RING>(W, k, in, rough, metal, st);
  const uint32_t bias_in[3] = {kB1, kB2, kB3};
  const uint32_t w_next[3] = {kW2, kW3, kW4};
  for (int l = 0; l < 3; l++) {
    warp_wait(W, bar_done(W.bars), W.dph);
    W.dph ^= 1u;
    tc_fence_after();
    if (!W.err) warp_epilogue(W, bias_in[l]);
    const uint32_t bars = W.bars, tmem = W.tmem & 0xFFFFu, area = W.area, w = w_next[l];
    const unsigned char* sm = W.sm;
    warp_handoff(W, bar_hfull(bars), W.hph, [&] {
      mma_issue(sm, tmem, area, 1024u, w, 1024u, 4, l == 2 ? 16 : 64, false);
      tc_commit(bar_done(bars));
    });
    W.hph ^= 1u;
  }
  warp_wait(W, bar_done(W.bars), W.dph);
  W.dph ^= 1u;
  tc_fence_after();
  if (W.err) return false;
  uint32_t r[16];
  tc_ld16_async(W.tmem, r);
  tc_wait_ld();
  const float* b4 = reinterpret_cast<const float*>(W.sm + kB4);
#pragma unroll
  for (int i = 0; i < 16; i++) out[i] = __uint_as_float(r[i]) + b4[i];
  return true;
}

// CTA prologue: barriers, TMEM (512 columns, warp 0), bulk copy of the packed
// network.  Returns false (on every thread) if the copy's wait ran out.
template <int G>
__device__ __forceinline__ bool mlp_cta_begin(unsigned char* sm, MlpShared<G>& S, const void* blob) {
  const uint32_t cb = smem_addr(&S.cta_bar);
  if (threadIdx.x == 0) {
    mbar_init(cb, 1);
    for (int g = 0; g < G; g++) {
      const uint32_t bars = smem_addr(&S.g[g]);
      for (int b = 0; b < kMaxRing; b++) {
        mbar_init(bar_full(bars, b), 3);
        mbar_init(bar_empty(bars, b), 1);
      }
      mbar_init(bar_hfull(bars), 3);
      mbar_init(bar_done(bars), 1);
      mbar_init(bar_drain(bars), 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_addr(&S.tmem_slot)), "r"(kGroupTmemCols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(cb), "r"(kBlob) : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        :: "r"(smem_addr(sm)), "l"(blob), "r"(kBlob), "r"(cb) : "memory");
  }
  bool ok = mbar_wait_bounded(cb, 0, kMlpWaitLimit);
  if (!ok) mbar_wait_bounded(cb, 0, kMlpWaitLimit);
  return __syncthreads_and(ok) != 0;
}

template <int G, int RING>
__device__ __forceinline__ MlpWarp mlp_warp_init(unsigned char* sm, MlpShared<G>& S, uint32_t tmem_base,
                                                 const t3_frame& fr) {
  MlpWarp W;
  const int warp = threadIdx.x >> 5, g = warp >> 2, q = warp & 3;
  W.sm = sm;
  W.tmem = tmem_base + (uint32_t)g * 64u + ((uint32_t)(q * 32) << 16);
  W.bars = smem_addr(&S.g[g]);
  W.area = kGroupBase + (uint32_t)g * RING * kChunkBytes;
  W.chunk = 0;
  W.dph = 0;
  W.hph = 0;
  W.limit = fr.wait_limit > 0 ? (uint32_t)fr.wait_limit : kMlpWaitLimit;
  W.row = q * 32 + (threadIdx.x & 31);
  W.leader = q == 0;
  W.starve = (fr.flags & T3_STARVE_NETWORK) != 0;
  W.err = false;
  return W;
}

// A leader's last act: commit (tracking every MMA it issued) and wait for it,
// so no MMA of the group is running when TMEM is freed.  False if that wait
// ran out.
__device__ __forceinline__ bool warp_drain(MlpWarp& W) {
  if (!W.leader) return true;
  if ((threadIdx.x & 31) == 0) tc_commit(bar_drain(W.bars));
  __syncwarp();
  return __all_sync(0xFFFFFFFFu, mbar_wait_bounded(bar_drain(W.bars), 0, kMlpWaitLimit));
}

__device__ __forceinline__ void mlp_cta_end(uint32_t tmem_base) {
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem_base),
                 "r"(kGroupTmemCols) : "memory");
  }
}

} // namespace t3
