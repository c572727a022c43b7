// mlp.cu -- the learned IBL term: training-data generation, feature encoding,
// forward / backward / Adam kernels (FP32, CUDA cores) and a reference
// inference path.
//
// What the network predicts.  For the materials built from Lambert and
// CookTorrance lobes (PBR = Mix(Lambert * albedo, CookTorrance(r, f0), f0),
// tina/matr/material.py:701-706) the Monte Carlo IBL estimator of t3_ibl.cuh
// is linear in the lobe weights, and each lobe's expectation separates into
// albedo- and f0-independent integrals:
//   Lambert:      E[env(cos-sampled dir)]                          = E_d(n)
//   CookTorrance: E[F G env] with F = f0 + (1 - f0)(1 - VoH)^5
//                 = f0 * S1(n, v, r) + (1 - f0) * S2(n, v, r),
//                 S1 = E[G env],  S2 = E[(1 - VoH)^5 G env]
// (expectations over each lobe's own sampler).  The network maps
// (n, v, roughness, metallic) to log1p of the nine values (E_d, S1, S2) RGB;
// shading composes them with the pixel's albedo, f0 and lobe weights, so one
// network serves every albedo.
//
// Input encoding (400 floats): for each of the six coordinates of n and of the
// mirrored view direction r = 2 (n . v) n - v (v's information in the frame of
// the specular lobes), sin and cos of pi * c * 2^(o + j/4), o = 0..7, j = 0..3
// (32 frequencies),
// evaluated as one sincos per base phase j followed by double-angle steps;
// then roughness, metallic, and zeros up to 400.
#include "t3_shading.cuh"
#include "t3_mlp_tc.cuh"

namespace t3 {

// ---- training targets -----------------------------------------------------
// E_d on an equirect grid of normals: map[i, j] for the direction of texel
// (i, j) (unspheremap), `spp` cosine samples each.
__global__ void k_irradiance_map(Env env, int mw, int mh, int spp, uint32_t seed, float* __restrict__ map) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= mw * mh) return;
  const int i = idx / mh, j = idx - i * mh;
  // unspheremap(I / (shape - 1)) (tina/skybox.py:31-36)
  const float v = (float)i / (float)(mw - 1), u = (float)j / (float)(mh - 1);
  const float h = u * 2.0f - 1.0f, r = sqrtf(fmaxf(0.0f, 1.0f - h * h));
  float s, c;
  sincospif(2.0f * v, &s, &c);
  const V3 n = v3(r * c, h, -r * s);
  const uint32_t base = rng_base(seed, (uint32_t)idx);
  V3 acc = v3(0.f, 0.f, 0.f);
  for (int k = 0; k < spp; k++) {
    const float xu = rng_draw(base, (uint32_t)k, 1u), xv = rng_draw(base, (uint32_t)k, 2u);
    acc = acc + env_sample(env, normalized(tangent_dir(n, sqrtf(xu), xv)));
  }
  acc = (1.0f / (float)spp) * acc;
  map[idx * 3] = acc.x;
  map[idx * 3 + 1] = acc.y;
  map[idx * 3 + 2] = acc.z;
}

// targets[b] = log1p of (E_d(n) from the irradiance map, S1, S2) at (n, v, r)
__global__ void k_targets(Env env, Env irr, const float* __restrict__ nv, const float* __restrict__ rough,
                          int64_t B, int spp, uint32_t seed, float* __restrict__ tgt) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const V3 n = v3(nv[b * 6], nv[b * 6 + 1], nv[b * 6 + 2]);
  const V3 vdir = v3(nv[b * 6 + 3], nv[b * 6 + 4], nv[b * 6 + 5]);
  const float r2 = rough[b] * rough[b];
  const float a2s = fmaxf(0.0f, r2), a2 = fmaxf(1e-6f, r2), kk = a2 * 0.5f;
  const float gn = 1.0f / (1.0f * (1.0f - a2) + 12.566370614359172f * a2);
  const float NoL = fmaxf(1e-10f, dot(vdir, n));
  const float gl = 1.0f / ((NoL * kk + 1.0f) - kk);
  const V3 rdir = reflect3(v3(-vdir.x, -vdir.y, -vdir.z), n);
  const uint32_t base = rng_base(seed, (uint32_t)b);
  V3 s1 = v3(0.f, 0.f, 0.f), s2 = v3(0.f, 0.f, 0.f);
  for (int k = 0; k < spp; k++) {
    const float xu = rng_draw(base, (uint32_t)k, 1u), xv = rng_draw(base, (uint32_t)k, 2u);
    const float u = sqrtf((1.0f - xu) / (1.0f - xu * (1.0f - a2s)));
    const V3 o = tangent_dir(rdir, u, xv);
    if (dot(o, n) < 0.0f) continue;  // CookTorrance.sample zeroes F below the surface
    const V3 half = normalized(vdir + o);
    const float NoV = fmaxf(1e-10f, dot(o, n));
    const float VoH = fminf(1.0f, fmaxf(1e-10f, dot(half, o)));
    const float g = gl * gn / ((NoV * kk + 1.0f) - kk);
    const float om = 1.0f - VoH, om2 = om * om;
    const V3 e = env_sample(env, o);
    s1 = s1 + g * e;
    s2 = s2 + (g * (om * om2 * om2)) * e;
  }
  const float inv = 1.0f / (float)spp;
  const V3 ed = env_sample(irr, n);
  float* t = tgt + b * 9;
  t[0] = log1pf(fmaxf(0.f, ed.x)); t[1] = log1pf(fmaxf(0.f, ed.y)); t[2] = log1pf(fmaxf(0.f, ed.z));
  t[3] = log1pf(s1.x * inv); t[4] = log1pf(s1.y * inv); t[5] = log1pf(s1.z * inv);
  t[6] = log1pf(s2.x * inv); t[7] = log1pf(s2.y * inv); t[8] = log1pf(s2.z * inv);
}

// ---- encoding --------------------------------------------------------------
__device__ __forceinline__ void encode_features(const float nv[6], float rough, float metal, float* x) {
  float in[6];
  mirror_inputs(nv, in);
#pragma unroll 1
  for (int c = 0; c < 6; c++) {
    float s[32], co[32];
    encode_coord(in[c], s, co);
#pragma unroll
    for (int f = 0; f < 32; f++) {
      x[c * 64 + f] = s[f];
      x[c * 64 + 32 + f] = co[f];
    }
  }
  x[384] = rough;
  x[385] = metal;
#pragma unroll
  for (int k = 386; k < T3_MLP_IN; k++) x[k] = 0.0f;
}

__global__ void k_encode(const float* __restrict__ nv, const float* __restrict__ rough,
                         const float* __restrict__ metal, int64_t B, float* __restrict__ X) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  float in[6];
#pragma unroll
  for (int c = 0; c < 6; c++) in[c] = nv[b * 6 + c];
  encode_features(in, rough[b], metal ? metal[b] : 0.0f, X + b * T3_MLP_IN);
}

// ---- a tiled FP32 GEMM -------------------------------------------------------
// C[M, N] (ldc) = op(A)[M, K] * op(B)[K, N], op = transpose when tA / tB;
// epilogue: + bias[N], then EPI 0 none, 1 ReLU, 2 multiply by (mask > 0)
// (ReLU backward, mask [M, N] with ldc), beta 1 accumulates into C.
// Split-K (gridDim.z > 1, for the weight gradients whose K is the batch):
// block z sums K range [z * kchunk, (z + 1) * kchunk) and adds its partial
// into C with atomicAdd (C zeroed beforehand; EPI 0, no bias, beta 0).
template <int EPI>
__global__ void __launch_bounds__(256)
k_sgemm(int M, int N, int K, const float* __restrict__ A, int lda, bool tA,
        const float* __restrict__ B, int ldb, bool tB, float* __restrict__ C, int ldc,
        const float* __restrict__ bias, const float* __restrict__ mask, float beta, int kchunk) {
  constexpr int TM = 64, TN = 64, TK = 16;
  __shared__ float As[TK][TM + 4];
  __shared__ float Bs[TK][TN + 4];
  const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;  // 16 x 16 threads, 4 x 4 outputs each
  const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
  float acc[4][4] = {};
  for (int k0 = kb; k0 < ke; k0 += TK) {
    for (int e = threadIdx.x; e < TK * TM; e += 256) {
      // transposed operands are read along m (contiguous), the others along k
      const int kk = tA ? e / TM : e % TK, mm = tA ? e % TM : e / TK;
      const int m = m0 + mm, k = k0 + kk;
      float v = 0.0f;
      if (m < M && k < ke) v = tA ? A[(int64_t)k * lda + m] : A[(int64_t)m * lda + k];
      As[kk][mm] = v;
    }
    for (int e = threadIdx.x; e < TK * TN; e += 256) {
      const int kk = tB ? e % TK : e / TN, nn = tB ? e / TK : e % TN;
      const int n = n0 + nn, k = k0 + kk;
      float v = 0.0f;
      if (n < N && k < ke) v = tB ? B[(int64_t)n * ldb + k] : B[(int64_t)k * ldb + n];
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; kk++) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int m = m0 + ty * 4 + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int n = n0 + tx * 4 + j;
      if (n >= N) continue;
      float v = acc[i][j];
      if (gridDim.z > 1) {
        atomicAdd(C + (int64_t)m * ldc + n, v);
        continue;
      }
      if (beta != 0.0f) v += beta * C[(int64_t)m * ldc + n];
      if (bias) v += bias[n];
      if (EPI == 1) v = fmaxf(v, 0.0f);
      if (EPI == 2) v = mask[(int64_t)m * ldc + n] > 0.0f ? v : 0.0f;
      C[(int64_t)m * ldc + n] = v;
    }
  }
}

template <int EPI>
static void sgemm(int M, int N, int K, const float* A, int lda, bool tA, const float* B, int ldb,
                  bool tB, float* C, int ldc, const float* bias, const float* mask, float beta,
                  cudaStream_t st) {
  dim3 grid((N + 63) / 64, (M + 63) / 64);
  k_sgemm<EPI><<<grid, 256, 0, st>>>(M, N, K, A, lda, tA, B, ldb, tB, C, ldc, bias, mask, beta, K);
}

// C = A^T B over a long K (the batch), split into K chunks across ~2 waves of
// blocks; C must be zero.
static void sgemm_splitk(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C,
                         int ldc, cudaStream_t st) {
  const int tiles = ((N + 63) / 64) * ((M + 63) / 64);
  int splits = (304 + tiles - 1) / tiles;
  const int max_splits = (K + 255) / 256;  // at least 256 rows of K per block
  if (splits > max_splits) splits = max_splits;
  if (splits < 1) splits = 1;
  const int kchunk = (((K + splits - 1) / splits) + 15) & ~15;
  splits = (K + kchunk - 1) / kchunk;
  dim3 grid((N + 63) / 64, (M + 63) / 64, splits);
  k_sgemm<0><<<grid, 256, 0, st>>>(M, N, K, A, lda, true, B, ldb, false, C, ldc, nullptr, nullptr, 0.f,
                                   kchunk);
}

// parameter layout (FP32): W1 [400,64] b1 [64] W2 [64,64] b2 W3 [64,64] b3 W4 [64,16] b4 [16]
struct MlpParams {
  const float *W1, *b1, *W2, *b2, *W3, *b3, *W4, *b4;
};
__host__ __device__ inline MlpParams mlp_params(const float* p) {
  MlpParams q;
  q.W1 = p; p += T3_MLP_IN * T3_MLP_HID;
  q.b1 = p; p += T3_MLP_HID;
  q.W2 = p; p += T3_MLP_HID * T3_MLP_HID;
  q.b2 = p; p += T3_MLP_HID;
  q.W3 = p; p += T3_MLP_HID * T3_MLP_HID;
  q.b3 = p; p += T3_MLP_HID;
  q.W4 = p; p += T3_MLP_HID * T3_MLP_OUT;
  q.b4 = p;
  return q;
}
constexpr int64_t kMlpParams = (int64_t)T3_MLP_IN * T3_MLP_HID + 2 * T3_MLP_HID * T3_MLP_HID +
                               T3_MLP_HID * T3_MLP_OUT + 3 * T3_MLP_HID + T3_MLP_OUT;

// loss = mean over the batch and the nine used outputs of (y - t)^2; dY = dloss/dy
__global__ void k_mse(const float* __restrict__ Y, const float* __restrict__ T, int64_t B,
                      float* __restrict__ dY, float* __restrict__ loss) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.0f;
  if (b < B) {
    const float scale = 2.0f / (float)(B * 9);
#pragma unroll
    for (int j = 0; j < T3_MLP_OUT; j++) {
      const float d = j < 9 ? Y[b * T3_MLP_OUT + j] - T[b * 9 + j] : 0.0f;
      dY[b * T3_MLP_OUT + j] = d * scale;
      l += d * d;
    }
  }
  // block sum, one atomic per block
  __shared__ float red[256];
  red[threadIdx.x] = l;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, red[0] / (float)(B * 9));
}

// db[j] = sum_b dY[b, j]
__global__ void k_colsum(const float* __restrict__ dY, int64_t B, int N, float* __restrict__ db) {
  const int j = blockIdx.x;
  float s = 0.0f;
  for (int64_t b = threadIdx.x; b < B; b += blockDim.x) s += dY[b * N + j];
  __shared__ float red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int t = 128; t > 0; t >>= 1) {
    if (threadIdx.x < t) red[threadIdx.x] += red[threadIdx.x + t];
    __syncthreads();
  }
  if (threadIdx.x == 0) db[j] = red[0];
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// ---- reference inference (FP32 CUDA cores, one thread per sample) ----------
__global__ void __launch_bounds__(128)
k_mlp_infer_f32(const float* __restrict__ params, const float* __restrict__ X, int64_t B,
                float* __restrict__ Y) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const MlpParams q = mlp_params(params);
  float h[T3_MLP_HID], h2[T3_MLP_HID];
  const float* x = X + b * T3_MLP_IN;
  for (int j = 0; j < T3_MLP_HID; j++) {
    float s = q.b1[j];
    for (int k = 0; k < T3_MLP_IN; k++) s = fmaf(x[k], q.W1[k * T3_MLP_HID + j], s);
    h[j] = fmaxf(s, 0.0f);
  }
  for (int j = 0; j < T3_MLP_HID; j++) {
    float s = q.b2[j];
    for (int k = 0; k < T3_MLP_HID; k++) s = fmaf(h[k], q.W2[k * T3_MLP_HID + j], s);
    h2[j] = fmaxf(s, 0.0f);
  }
  for (int j = 0; j < T3_MLP_HID; j++) {
    float s = q.b3[j];
    for (int k = 0; k < T3_MLP_HID; k++) s = fmaf(h2[k], q.W3[k * T3_MLP_HID + j], s);
    h[j] = fmaxf(s, 0.0f);
  }
  for (int j = 0; j < T3_MLP_OUT; j++) {
    float s = q.b4[j];
    for (int k = 0; k < T3_MLP_HID; k++) s = fmaf(h[k], q.W4[k * T3_MLP_OUT + j], s);
    Y[b * T3_MLP_OUT + j] = s;
  }
}

// ---- packing for the tensor-core path ----------------------------------------
// blob layout: see t3_mlp_tc.cuh (W^T in the K-major core-matrix layout, BF16)
__global__ void k_mlp_pack(const float* __restrict__ params, unsigned char* __restrict__ blob) {
  const MlpParams q = mlp_params(params);
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  struct L { const float* W; int K, N; uint32_t off; };
  const L layers[4] = {{q.W1, T3_MLP_IN, T3_MLP_HID, kW1}, {q.W2, T3_MLP_HID, T3_MLP_HID, kW2},
                       {q.W3, T3_MLP_HID, T3_MLP_HID, kW3}, {q.W4, T3_MLP_HID, T3_MLP_OUT, kW4}};
  int base = 0;
  for (int l = 0; l < 4; l++) {
    const int n_el = layers[l].K * layers[l].N;
    if (tid >= base && tid < base + n_el) {
      const int e = tid - base, k0 = e / layers[l].N, n = e % layers[l].N;  // W[k0][n]
      const int k = l == 0 ? packed_k1(k0) : k0;  // layer 1 in the packed feature order
      const uint32_t off = layers[l].off + tc_chunk_off(n, k & ~7, layers[l].K) + (k & 7) * 2;
      *reinterpret_cast<__nv_bfloat16*>(blob + off) = __float2bfloat16_rn(layers[l].W[e]);
    }
    base += n_el;
  }
  const float* biases[4] = {q.b1, q.b2, q.b3, q.b4};
  const uint32_t boff[4] = {kB1, kB2, kB3, kB4};
  const int bn[4] = {T3_MLP_HID, T3_MLP_HID, T3_MLP_HID, T3_MLP_OUT};
  for (int l = 0; l < 4; l++) {
    if (tid >= base && tid < base + bn[l])
      reinterpret_cast<float*>(blob + boff[l])[tid - base] = biases[l][tid - base];
    base += bn[l];
  }
}

// standalone tensor-core inference: Y[B, 16] from X[B, 400] (FP32 in, BF16 operands)
__global__ void __launch_bounds__(128, 1)
k_mlp_infer_tc(const unsigned char* __restrict__ blob, const float* __restrict__ X, int64_t B,
               float* __restrict__ Y, int32_t* __restrict__ status) {
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  MlpTile t;
  const bool ok = mlp_begin(t, sm, &bar, &tmem_slot, blob);
  const int64_t ntiles = (B + 127) / 128;
  for (int64_t tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x) {
    const int64_t row = tile * 128 + threadIdx.x;
    for (int k = 0; k < T3_MLP_IN; k += 8) {
      float x[8];
#pragma unroll
      for (int i = 0; i < 8; i++) x[i] = row < B ? X[row * T3_MLP_IN + k + i] : 0.0f;
      *reinterpret_cast<uint4*>(sm + kA + tc_chunk_off(threadIdx.x, packed_k1(k), T3_MLP_IN)) = pack8_bf16(x);
    }
    float out[16];
    if (!mlp_tile(t, out)) {
      if (threadIdx.x == 0) atomicOr(status, T3_STATUS_TIMEOUT);
      break;
    }
    if (row < B) {
#pragma unroll
      for (int i = 0; i < 16; i++) Y[row * T3_MLP_OUT + i] = out[i];
    }
  }
  if (!ok && threadIdx.x == 0) atomicOr(status, T3_STATUS_TIMEOUT);
  mlp_end(t);
}

} // namespace t3

using namespace t3;

static int rc_of(cudaError_t e) { return e == cudaSuccess ? T3_OK : T3_ECUDA; }

extern "C" {

int64_t t3_mlp_param_count(void) { return kMlpParams; }

int t3_mlp_irradiance_map(const void* env, int env_w, int env_h, int env_half, int map_w, int map_h,
                          int spp, uint32_t seed, float* map, void* stream) {
  if (!env || !map || env_w < 2 || env_h < 2 || map_w < 2 || map_h < 2 || spp < 1) return T3_EINVAL;
  const Env e{env, env_w, env_h, env_half};
  const int n = map_w * map_h;
  k_irradiance_map<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(e, map_w, map_h, spp, seed, map);
  return rc_of(cudaGetLastError());
}

int t3_mlp_targets(const void* env, int env_w, int env_h, int env_half, const float* irr_map,
                   int map_w, int map_h, const float* nv, const float* rough, int64_t B, int spp,
                   uint32_t seed, float* targets, void* stream) {
  if (!env || !irr_map || !nv || !rough || !targets || B < 0 || spp < 1) return T3_EINVAL;
  if (B == 0) return T3_OK;
  const Env e{env, env_w, env_h, env_half};
  const Env irr{irr_map, map_w, map_h, 0};
  k_targets<<<(unsigned)((B + 127) / 128), 128, 0, (cudaStream_t)stream>>>(e, irr, nv, rough, B, spp,
                                                                        seed, targets);
  return rc_of(cudaGetLastError());
}

int t3_mlp_encode(const float* nv, const float* rough, const float* metal, int64_t B, float* X,
                  void* stream) {
  if (!nv || !rough || !X || B < 0) return T3_EINVAL;
  if (B == 0) return T3_OK;
  k_encode<<<(unsigned)((B + 127) / 128), 128, 0, (cudaStream_t)stream>>>(nv, rough, metal, B, X);
  return rc_of(cudaGetLastError());
}

// acts: workspace [B, 3*64] of post-ReLU hidden activations; Y [B, 16]
int t3_mlp_forward(const float* params, const float* X, int64_t B, float* acts, float* Y,
                   void* stream) {
  if (!params || !X || !acts || !Y || B <= 0 || B > (1 << 30)) return T3_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  const MlpParams q = mlp_params(params);
  const int M = (int)B, H = T3_MLP_HID;
  float* h1 = acts;
  float* h2 = acts + (int64_t)B * H;
  float* h3 = acts + 2 * (int64_t)B * H;
  sgemm<1>(M, H, T3_MLP_IN, X, T3_MLP_IN, false, q.W1, H, false, h1, H, q.b1, nullptr, 0.f, st);
  sgemm<1>(M, H, H, h1, H, false, q.W2, H, false, h2, H, q.b2, nullptr, 0.f, st);
  sgemm<1>(M, H, H, h2, H, false, q.W3, H, false, h3, H, q.b3, nullptr, 0.f, st);
  sgemm<0>(M, T3_MLP_OUT, H, h3, H, false, q.W4, T3_MLP_OUT, false, Y, T3_MLP_OUT, q.b4, nullptr,
           0.f, st);
  return rc_of(cudaGetLastError());
}

// grads: same layout as params; dbuf: workspace [B, 2*64 + 16]; loss: device float (accumulated)
int t3_mlp_backward(const float* params, const float* X, const float* acts, const float* Y,
                    const float* targets, int64_t B, float* grads, float* dbuf, float* loss,
                    void* stream) {
  if (!params || !X || !acts || !Y || !targets || !grads || !dbuf || !loss || B <= 0) return T3_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  const MlpParams q = mlp_params(params);
  MlpParams g = mlp_params(grads);
  float* gW1 = const_cast<float*>(g.W1); float* gb1 = const_cast<float*>(g.b1);
  float* gW2 = const_cast<float*>(g.W2); float* gb2 = const_cast<float*>(g.b2);
  float* gW3 = const_cast<float*>(g.W3); float* gb3 = const_cast<float*>(g.b3);
  float* gW4 = const_cast<float*>(g.W4); float* gb4 = const_cast<float*>(g.b4);
  const int M = (int)B, H = T3_MLP_HID, O = T3_MLP_OUT;
  const float* h1 = acts;
  const float* h2 = acts + (int64_t)B * H;
  const float* h3 = acts + 2 * (int64_t)B * H;
  float* dY = dbuf;                        // [B, 16]
  float* dA = dbuf + (int64_t)B * O;       // [B, 64]
  float* dB = dA + (int64_t)B * H;         // [B, 64]
  // the weight gradients are accumulated by split-K blocks: start from zero
  if (cudaMemsetAsync(grads, 0, sizeof(float) * (size_t)kMlpParams, st) != cudaSuccess) return T3_ECUDA;
  k_mse<<<(unsigned)((B + 255) / 256), 256, 0, st>>>(Y, targets, B, dY, loss);
  // layer 4
  sgemm_splitk(H, O, M, h3, H, dY, O, gW4, O, st);
  k_colsum<<<O, 256, 0, st>>>(dY, B, O, gb4);
  sgemm<2>(M, H, O, dY, O, false, q.W4, O, true, dA, H, nullptr, h3, 0.f, st);  // dh3 * relu'
  // layer 3
  sgemm_splitk(H, H, M, h2, H, dA, H, gW3, H, st);
  k_colsum<<<H, 256, 0, st>>>(dA, B, H, gb3);
  sgemm<2>(M, H, H, dA, H, false, q.W3, H, true, dB, H, nullptr, h2, 0.f, st);
  // layer 2
  sgemm_splitk(H, H, M, h1, H, dB, H, gW2, H, st);
  k_colsum<<<H, 256, 0, st>>>(dB, B, H, gb2);
  sgemm<2>(M, H, H, dB, H, false, q.W2, H, true, dA, H, nullptr, h1, 0.f, st);
  // layer 1
  sgemm_splitk(T3_MLP_IN, H, M, X, T3_MLP_IN, dA, H, gW1, H, st);
  k_colsum<<<H, 256, 0, st>>>(dA, B, H, gb1);
  return rc_of(cudaGetLastError());
}

int t3_mlp_adam(float* params, const float* grads, float* m, float* v, int64_t n, float lr,
                float beta1, float beta2, float eps, int step, void* stream) {
  if (!params || !grads || !m || !v || n <= 0 || step < 1) return T3_EINVAL;
  const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
  k_adam<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(params, grads, m, v, n, lr,
                                                                      beta1, beta2, eps, c1, c2);
  return rc_of(cudaGetLastError());
}

int64_t t3_mlp_packed_bytes(void) { return kBlob; }

int t3_mlp_pack(const float* params, void* blob, void* stream) {
  if (!params || !blob) return T3_EINVAL;
  const int n = T3_MLP_IN * T3_MLP_HID + 2 * T3_MLP_HID * T3_MLP_HID + T3_MLP_HID * T3_MLP_OUT +
                3 * T3_MLP_HID + T3_MLP_OUT;
  k_mlp_pack<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(params, (unsigned char*)blob);
  return rc_of(cudaGetLastError());
}

int t3_mlp_infer(const void* blob, const float* X, int64_t B, float* Y, int32_t* status, void* stream) {
  if (!blob || !X || !Y || !status || B < 0) return T3_EINVAL;
  if (B == 0) return T3_OK;
  if ((reinterpret_cast<uintptr_t>(blob) & 15) != 0) return T3_EINVAL;
  cudaError_t e = cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kMlpSmem);
  if (e != cudaSuccess) return T3_ECUDA;
  const int64_t ntiles = (B + 127) / 128;
  const int grid = (int)(ntiles < 152 ? ntiles : 152);
  k_mlp_infer_tc<<<grid, 128, kMlpSmem, (cudaStream_t)stream>>>((const unsigned char*)blob, X, B, Y,
                                                               status);
  return rc_of(cudaGetLastError());
}

int t3_mlp_infer_f32(const float* params, const float* X, int64_t B, float* Y, void* stream) {
  if (!params || !X || !Y || B < 0) return T3_EINVAL;
  if (B == 0) return T3_OK;
  k_mlp_infer_f32<<<(unsigned)((B + 127) / 128), 128, 0, (cudaStream_t)stream>>>(params, X, B, Y);
  return rc_of(cudaGetLastError());
}

} // extern "C"
