// t3_mlp_tc.cuh -- MLP-IBL inference on the tensor cores, one 128-row tile per
// CTA pass (128 threads, thread t owns row t / TMEM lane t).
//
// Packed network (t3_mlp_pack), staged once per CTA into shared memory with a
// bulk copy (cp.async.bulk):
//   W1 [64 x 400], W2 [64 x 64], W3 [64 x 64], W4 [16 x 64]  BF16, each in the
//   K-major core-matrix layout of t3_tc.cuh (rows = output units), then the
//   FP32 biases b1, b2, b3 (64 each) and b4 (16).
// Per tile: the threads write their rows' features into A [128 x 400] BF16;
// thread 0 issues 25 K=16 MMAs into TMEM columns 0-63; each later layer reads
// the previous layer's ReLU output back from TMEM (tcgen05.ld), writes it as
// BF16 into H [128 x 64], and the next MMAs accumulate into fresh columns
// (64-127, 128-191, 192-207).  The FP32 output row (16 values, 9 used) is left
// in registers of the row's thread.
#pragma once

#include "t3_tc.cuh"
#include "tina3.h"

namespace t3 {

constexpr uint32_t kW1 = 0, kW2 = 51200, kW3 = 59392, kW4 = 67584;
constexpr uint32_t kB1 = 69632, kB2 = 69888, kB3 = 70144, kB4 = 70400, kBlob = 70464;
constexpr uint32_t kA = kBlob;                  // A operand, 128 x 400 BF16
constexpr uint32_t kH = kA + 128 * 400 * 2;     // hidden operand, 128 x 64 BF16
constexpr uint32_t kMlpSmem = kH + 128 * 64 * 2;  // 189248 bytes
constexpr uint32_t kTmemCols = 256;

struct MlpTile {
  uint32_t tmem;    // TMEM base address (lane 0)
  uint32_t mbar;    // shared address of the MMA-completion mbarrier
  uint32_t phase;   // parity of the next completion
  unsigned char* sm;
};

// Fourier features of one input coordinate c (|c| <= 1): s[f] = sin(pi c
// 2^(o + j/4)), co[f] = cos(...), f = 4 o + j, o = 0..7, j = 0..3; one fast
// hardware sin / cos per base phase j (|argument| < 5.3 rad, absolute error
// ~1e-6, far below the BF16 operands' 4e-3), then double-angle steps.  Shared
// by the training-side encoder and the fused shading kernel, so both see the
// same FP32 features.
__device__ __forceinline__ void encode_coord(float c, float s[32], float co[32]) {
  const float base[4] = {3.141592653589793f, 3.7360043360892607f, 4.442882938158366f, 5.283508001182123f};
#pragma unroll
  for (int j = 0; j < 4; j++) {
    float a, b;
    __sincosf(c * base[j], &a, &b);
#pragma unroll
    for (int o = 0; o < 8; o++) {
      s[o * 4 + j] = a;
      co[o * 4 + j] = b;
      const float a2 = 2.0f * a * b, b2 = (b - a) * (b + a);
      a = a2;
      b = b2;
    }
  }
}

// The encoded directions: the normal n and the view direction v entered as its
// mirror image about n, r = reflect(-v, n) = 2 (n . v) n - v -- the same
// information, in the coordinates the specular lobes are centred on.
__device__ __forceinline__ void mirror_inputs(const float nv[6], float in[6]) {
  const float d = nv[0] * nv[3] + nv[1] * nv[4] + nv[2] * nv[5];
  in[0] = nv[0];
  in[1] = nv[1];
  in[2] = nv[2];
  in[3] = 2.0f * d * nv[0] - nv[3];
  in[4] = 2.0f * d * nv[1] - nv[4];
  in[5] = 2.0f * d * nv[2] - nv[5];
}

// Packed K order of the first layer.  Features are produced per input
// coordinate in two halves: half h holds the sines, then the cosines, of
// octaves 4h..4h+3 (16 + 16 features), so a 32-feature K chunk is one half of
// one coordinate.  packed_k1 maps a feature's index in the encoder's order
// (coordinate c: 32 sines, then 32 cosines, f = 4 o + j) to its K position in
// the packed W1 and in the A operand; 8-aligned runs stay 8-aligned and
// contiguous.  The tail (roughness, metallic, padding) keeps its positions.
__host__ __device__ __forceinline__ int packed_k1(int k) {
  if (k >= 384) return k;
  const int c = k >> 6, f = k & 63;
  const bool cosine = f >= 32;
  const int fi = f & 31;
  return c * 64 + (fi >> 4) * 32 + (cosine ? 16 : 0) + (fi & 15);
}

// Half h of coordinate x's features in packed order: out[0..15] = sin, out[16..31]
// = cos of octaves 4h..4h+3 (the same values as encode_coord); st carries the
// (sin, cos) pairs of the four base phases from half 0 to half 1.
__device__ __forceinline__ void encode_half(float x, int h, float st[8], float out[32]) {
  const float base[4] = {3.141592653589793f, 3.7360043360892607f, 4.442882938158366f, 5.283508001182123f};
  if (h == 0) {
#pragma unroll
    for (int j = 0; j < 4; j++) __sincosf(x * base[j], &st[2 * j], &st[2 * j + 1]);
  }
#pragma unroll
  for (int o = 0; o < 4; o++) {
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const float a = st[2 * j], b = st[2 * j + 1];
      out[o * 4 + j] = a;
      out[16 + o * 4 + j] = b;
      st[2 * j] = 2.0f * a * b;
      st[2 * j + 1] = (b - a) * (b + a);
    }
  }
}

// one layer: D[128 x N] (TMEM column col) = A[128 x K] * W^T
__device__ __forceinline__ void mlp_issue_layer(const MlpTile& t, uint32_t a_off, uint32_t w_off, int K,
                                                int N, uint32_t col) {
  const uint32_t a = smem_addr(t.sm + a_off), w = smem_addr(t.sm + w_off);
  const uint32_t sbo = (uint32_t)(K / 8) * 128u;
  const uint32_t idesc = tc_idesc(128, N);
  for (int ks = 0; ks < K / 16; ks++) {
    tc_mma(t.tmem + col, tc_desc(a + ks * 256u, 128u, sbo), tc_desc(w + ks * 256u, 128u, sbo), idesc,
           ks > 0 ? 1u : 0u);
  }
  tc_commit(t.mbar);
}

// waits for the layer's MMAs; false when the bounded wait ran out (after one
// more bounded wait, so no MMA of ours is left running when TMEM is freed)
// (the outcome is agreed by the whole CTA, so every thread takes the same path)
__device__ __forceinline__ bool mlp_wait(MlpTile& t) {
  bool ok = mbar_wait_bounded(t.mbar, t.phase, 1u << 24);
  if (!ok) mbar_wait_bounded(t.mbar, t.phase, 1u << 24);
  ok = __syncthreads_and(ok) != 0;
  t.phase ^= 1u;
  tc_fence_after();
  return ok;
}

// bias + ReLU of this thread's row of D (64 columns at `col`), written as BF16 into H
__device__ __forceinline__ void mlp_hidden_epilogue(const MlpTile& t, uint32_t col, uint32_t b_off) {
  const int row = threadIdx.x;
  const uint32_t lane_base = (uint32_t)((threadIdx.x & ~31) << 16);
  const float* bias = reinterpret_cast<const float*>(t.sm + b_off);
#pragma unroll
  for (int c = 0; c < 64; c += 16) {
    float v[16];
    tc_ld16(t.tmem + lane_base + col + c, v);
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = fmaxf(v[i] + bias[c + i], 0.0f);
    *reinterpret_cast<uint4*>(t.sm + kH + tc_chunk_off(row, c, 64)) = pack8_bf16(v);
    *reinterpret_cast<uint4*>(t.sm + kH + tc_chunk_off(row, c + 8, 64)) = pack8_bf16(v + 8);
  }
}

// Runs the four layers for the tile whose A rows the threads have written.
// out[16] receives this thread's output row.  Returns false on a timed-out wait.
__device__ __forceinline__ bool mlp_tile(MlpTile& t, float out[16]) {
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc_fence_after();
    mlp_issue_layer(t, kA, kW1, 400, 64, 0);
  }
  if (!mlp_wait(t)) return false;
  mlp_hidden_epilogue(t, 0, kB1);
  const uint32_t hid_cols[2] = {64, 128};
  const uint32_t hid_w[2] = {kW2, kW3};
  const uint32_t hid_b[2] = {kB2, kB3};
  for (int l = 0; l < 2; l++) {
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc_fence_after();
      mlp_issue_layer(t, kH, hid_w[l], 64, 64, hid_cols[l]);
    }
    if (!mlp_wait(t)) return false;
    // H is read by the MMAs just completed: overwrite it only after every thread waited
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    mlp_hidden_epilogue(t, hid_cols[l], hid_b[l]);
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc_fence_after();
    mlp_issue_layer(t, kH, kW4, 64, 16, 192);
  }
  if (!mlp_wait(t)) return false;
  const uint32_t lane_base = (uint32_t)((threadIdx.x & ~31) << 16);
  tc_ld16(t.tmem + lane_base + 192, out);
  const float* b4 = reinterpret_cast<const float*>(t.sm + kB4);
#pragma unroll
  for (int i = 0; i < 16; i++) out[i] += b4[i];
  // the next tile's writes to A / H and MMAs into these columns come after this
  tc_fence_before();
  __syncthreads();
  return true;
}

// CTA prologue: barrier, TMEM allocation (warp 0), bulk copy of the packed
// network into shared memory.  Returns false if the copy's wait ran out.
__device__ __forceinline__ bool mlp_begin(MlpTile& t, unsigned char* sm, uint64_t* bar,
                                          uint32_t* tmem_slot, const void* blob) {
  t.sm = sm;
  t.mbar = smem_addr(bar);
  t.phase = 0;
  if (threadIdx.x == 0) {
    mbar_init(t.mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_addr(tmem_slot)), "r"(kTmemCols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  t.tmem = *tmem_slot;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(t.mbar), "r"(kBlob)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        :: "r"(smem_addr(sm)), "l"(blob), "r"(kBlob), "r"(t.mbar) : "memory");
  }
  bool ok = mbar_wait_bounded(t.mbar, 0, 1u << 24);
  if (!ok) mbar_wait_bounded(t.mbar, 0, 1u << 24);  // let the copy land before anything else
  ok = __syncthreads_and(ok) != 0;
  t.phase = 1;
  return ok;
}

__device__ __forceinline__ void mlp_end(const MlpTile& t) {
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(t.tmem), "r"(kTmemCols)
                 : "memory");
  }
}

} // namespace t3
