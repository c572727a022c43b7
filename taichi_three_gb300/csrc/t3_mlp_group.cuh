// t3_mlp_group.cuh -- the learned-IBL network on the tensor cores for the fused
// shading kernel: several independent 128-row tiles in flight per CTA.
//
// A CTA holds the packed network once (t3_mlp_tc.cuh layout, 70,464 bytes) and
// kMlpGroups groups of 128 threads (4 warps each).  Group g owns TMEM columns
// [64 g, 64 g + 64) of the CTA's 512 -- every layer accumulates into the same
// columns: the epilogue has read a layer's output into registers before the
// next layer's MMAs are issued -- and two 8 KB A-chunk buffers, which together
// hold the hidden operand H of the later layers once the first layer is done.
// The first layer's A operand (128 rows x 400 features) is never materialised
// whole: the group encodes half an input coordinate (32 features, packed
// order of t3_mlp_tc.cuh) at a time into a chunk buffer and its elected thread
// issues that chunk's two K = 16 MMAs; the other buffer is being encoded
// meanwhile.  Each buffer has an mbarrier that tcgen05.commit arrives on, so a
// buffer is rewritten only after the MMAs reading it have completed.  Small
// per-group footprints let six groups share an SM, and groups synchronise with
// named barriers (ids 1..kMlpGroups), so one group's gathers and encoding
// overlap the other groups' MMA round trips.
//
// Every wait is bounded; a group whose wait runs out reports false (after one
// more bounded wait for its own MMAs) and stops.
#pragma once

#include "t3_mlp_tc.cuh"

namespace t3 {

#ifndef T3_MLP_GROUPS
#define T3_MLP_GROUPS 6
#endif
constexpr int kMlpGroups = T3_MLP_GROUPS;        // up to 8 (TMEM: 64 columns each)
constexpr uint32_t kGroupBase = 71680;           // kBlob rounded up to 1 KB
constexpr uint32_t kChunkBytes = 128 * 32 * 2;   // 128 rows x 32 BF16
constexpr uint32_t kGroupBytes = 2 * kChunkBytes;  // A0, A1 (together: H, 128 x 64 BF16)
constexpr uint32_t kMlpGroupSmem = kGroupBase + kMlpGroups * kGroupBytes;
static_assert(kMlpGroups * 64 <= 512, "TMEM holds 512 columns");
static_assert(kMlpGroupSmem + kMlpGroups * 1040 + 64 <= 232448, "shared memory per CTA");
constexpr uint32_t kGroupTmemCols = 512;
static_assert(kGroupBase >= kBlob, "packed network overlaps the group areas");

__device__ __forceinline__ void group_sync(int id) {
  asm volatile("bar.sync %0, 128;" :: "r"(id) : "memory");
}

// true on every thread of the group iff v is true on every thread
__device__ __forceinline__ bool group_and(bool v, int id) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n"
      " bar.red.and.pred p, %2, 128, q;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(r) : "r"((uint32_t)v), "r"(id) : "memory");
  return r != 0;
}

struct MlpGroup {
  unsigned char* sm;   // CTA shared memory (packed network at 0)
  uint32_t tmem;       // TMEM address of this group's first column (lane 0)
  uint32_t bar[3];     // shared addresses: chunk buffer 0, chunk buffer 1, layers
  uint32_t ph[3];      // parity of each barrier's next completion
  int id;              // named barrier id
  int row;             // this thread's row (0..127)
  uint32_t a[2], h;    // shared byte offsets of the chunk buffers and H
};

// One thread polls the mbarrier; the rest of the group sleeps in the named
// barrier that publishes the outcome (polling by every thread would spend the
// issue slots the other groups need).
__device__ __forceinline__ bool group_wait(MlpGroup& G, int b) {
  bool ok = true;
  if (G.row == 0) {
    ok = mbar_wait_bounded(G.bar[b], G.ph[b], 1u << 24);
    if (!ok) mbar_wait_bounded(G.bar[b], G.ph[b], 1u << 24);
  }
  G.ph[b] ^= 1u;
  ok = group_and(ok, G.id);
  tc_fence_after();
  return ok;
}

// Issue (by the group's first thread, after a group barrier): D += A_chunk * W^T
__device__ __forceinline__ void group_issue(const MlpGroup& G, uint32_t a_off, uint32_t a_sbo,
                                            uint32_t w_off, uint32_t w_sbo, int ksteps, int N,
                                            uint32_t col, bool accumulate_first, int commit_bar) {
  const uint32_t a = smem_addr(G.sm + a_off), w = smem_addr(G.sm + w_off);
  const uint32_t idesc = tc_idesc(128, N);
  for (int ks = 0; ks < ksteps; ks++) {
    tc_mma(G.tmem + col, tc_desc(a + ks * 256u, 128u, a_sbo), tc_desc(w + ks * 256u, 128u, w_sbo), idesc,
           (ks > 0 || accumulate_first) ? 1u : 0u);
  }
  tc_commit(G.bar[commit_bar]);
}

// bias + ReLU of this thread's row of the 64 columns at `col`, written as BF16 into H
__device__ __forceinline__ void group_epilogue(const MlpGroup& G, uint32_t col, uint32_t b_off) {
  const uint32_t lane_base = (uint32_t)((threadIdx.x & 96) << 16);  // warp's TMEM lane quarter
  const float4* bias = reinterpret_cast<const float4*>(G.sm + b_off);  // 16-byte aligned
#pragma unroll
  for (int c = 0; c < 64; c += 16) {
    float v[16];
    tc_ld16(G.tmem + lane_base + col + c, v);
#pragma unroll
    for (int i = 0; i < 16; i += 4) {
      const float4 b = bias[(c + i) >> 2];
      v[i] = fmaxf(v[i] + b.x, 0.0f);
      v[i + 1] = fmaxf(v[i + 1] + b.y, 0.0f);
      v[i + 2] = fmaxf(v[i + 2] + b.z, 0.0f);
      v[i + 3] = fmaxf(v[i + 3] + b.w, 0.0f);
    }
    *reinterpret_cast<uint4*>(G.sm + G.h + tc_chunk_off(G.row, c, 64)) = pack8_bf16(v);
    *reinterpret_cast<uint4*>(G.sm + G.h + tc_chunk_off(G.row, c + 8, 64)) = pack8_bf16(v + 8);
  }
}

// Half h of the row's coordinate x as 32 BF16 features in chunk buffer b (K = 32 layout)
__device__ __forceinline__ void group_encode_half(const MlpGroup& G, int b, float x, int h, float st[8]) {
  float f[32];
  encode_half(x, h, st, f);
  unsigned char* A = G.sm + G.a[b];
#pragma unroll
  for (int q = 0; q < 4; q++)
    *reinterpret_cast<uint4*>(A + tc_chunk_off(G.row, 8 * q, 32)) = pack8_bf16(f + 8 * q);
}

// The last 16 inputs (roughness, metallic, zero padding) in chunk buffer b (K = 16 layout)
__device__ __forceinline__ void group_encode_tail(const MlpGroup& G, int b, float rough, float metal) {
  unsigned char* A = G.sm + G.a[b];
  float t[8] = {rough, metal, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  *reinterpret_cast<uint4*>(A + tc_chunk_off(G.row, 0, 16)) = pack8_bf16(t);
  t[0] = t[1] = 0.0f;
  *reinterpret_cast<uint4*>(A + tc_chunk_off(G.row, 8, 16)) = pack8_bf16(t);
}

// The whole network for the group's tile.  `in` = this row's six direction
// coordinates (already mirrored), rough, metal; rows of threads with
// `valid == false` are computed on whatever their buffers hold and ignored.
// out[16] receives the row's output.  Returns false on a timed-out wait.
__device__ __forceinline__ bool group_tile(MlpGroup& G, const float in[6], float rough, float metal,
                                           float out[16]) {
  const bool leader = G.row == 0;
  // layer 1: thirteen K chunks (6 coordinates x 2 halves x 32 features, then
  // the 16 tail inputs), chunk k in buffer k & 1, all into the group's columns
  float st[8];
  for (int k = 0; k < 13; k++) {
    const int b = k & 1;
    if (k >= 2 && !group_wait(G, b)) return false;  // chunk k - 2 has left buffer b
    if (k < 12) group_encode_half(G, b, in[k >> 1], k & 1, st);
    else group_encode_tail(G, b, rough, metal);
    fence_async_smem();
    tc_fence_before();
    group_sync(G.id);
    if (leader) {
      tc_fence_after();
      if (k < 12) group_issue(G, G.a[b], 512u, kW1 + (uint32_t)k * 512u, 6400u, 2, 64, 0, k > 0, b);
      else group_issue(G, G.a[b], 256u, kW1 + 6144u, 6400u, 1, 64, 0, true, b);
    }
  }
  if (!group_wait(G, 1)) return false;  // chunk 11
  if (!group_wait(G, 0)) return false;  // chunk 12: layer 1 complete
  // layers 2-4 read the previous output back (bias + ReLU into H) and overwrite
  // the same columns: each epilogue's TMEM loads complete (tcgen05.wait::ld)
  // before the group barrier that precedes the next issue
  const uint32_t w[3] = {kW2, kW3, kW4};
  const uint32_t bias_in[3] = {kB1, kB2, kB3};
  for (int l = 0; l < 3; l++) {
    group_epilogue(G, 0, bias_in[l]);
    fence_async_smem();
    tc_fence_before();
    group_sync(G.id);
    if (leader) {
      tc_fence_after();
      group_issue(G, G.h, 1024u, w[l], 1024u, 4, l == 2 ? 16 : 64, 0, false, 2);
    }
    if (!group_wait(G, 2)) return false;
  }
  const uint32_t lane_base = (uint32_t)((threadIdx.x & 96) << 16);
  tc_ld16(G.tmem + lane_base, out);
  const float* b4 = reinterpret_cast<const float*>(G.sm + kB4);
#pragma unroll
  for (int i = 0; i < 16; i++) out[i] += b4[i];
  tc_fence_before();
  return true;
}

// CTA prologue: barriers, TMEM (512 columns, warp 0), bulk copy of the packed
// network.  Returns false (on every thread) if the copy's wait ran out.
__device__ __forceinline__ bool group_cta_begin(unsigned char* sm, uint64_t* cta_bar, uint64_t (*gbar)[3],
                                                uint32_t* tmem_slot, const void* blob) {
  const uint32_t cb = smem_addr(cta_bar);
  if (threadIdx.x == 0) {
    mbar_init(cb, 1);
    for (int g = 0; g < kMlpGroups; g++)
      for (int k = 0; k < 3; k++) mbar_init(smem_addr(&gbar[g][k]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_addr(tmem_slot)), "r"(kGroupTmemCols) : "memory");
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
  bool ok = mbar_wait_bounded(cb, 0, 1u << 24);
  if (!ok) mbar_wait_bounded(cb, 0, 1u << 24);
  return __syncthreads_and(ok) != 0;
}

__device__ __forceinline__ MlpGroup group_init(unsigned char* sm, uint64_t (*gbar)[3], uint32_t tmem_base) {
  MlpGroup G;
  const int g = threadIdx.x >> 7;
  G.sm = sm;
  G.tmem = tmem_base + (uint32_t)g * 64u;
  for (int k = 0; k < 3; k++) {
    G.bar[k] = smem_addr(&gbar[g][k]);
    G.ph[k] = 0;
  }
  G.id = 1 + g;
  G.row = threadIdx.x & 127;
  const uint32_t base = kGroupBase + (uint32_t)g * kGroupBytes;
  G.a[0] = base;
  G.a[1] = base + kChunkBytes;
  G.h = base;  // both chunk buffers are free once the first layer has completed
  return G;
}

__device__ __forceinline__ void group_cta_end(uint32_t tmem_base) {
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem_base),
                 "r"(kGroupTmemCols) : "memory");
  }
}

} // namespace t3
