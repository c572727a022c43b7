// binned.cu -- the single-view binned frame: k_bin over one object's faces,
// then k_tile over the frame's tiles (the bodies are in t3_binned.cuh).
#include "t3_binned.cuh"

namespace t3 {

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK)
k_bin(const t3_frame fr, const t3_mesh mesh, int64_t nfaces, uint32_t face_base, BinArgs bins) {
  __shared__ __align__(16) float sv[BLOCK * 9];
  bin_faces<BLOCK>(fr, mesh, nfaces, face_base, bins, (int64_t)blockIdx.x * BLOCK, sv);
}

template <int TS, int BLOCK, int NL, int MODE>
__global__ void __launch_bounds__(BLOCK, BLOCK == 256 ? 3 : 6)
k_tile(const DevScene* __restrict__ sc, BinArgs bins, t3_outputs out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ TileShared<TS, BLOCK> sh;
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(smem_raw);  // TS*TS
  uint32_t* queue = reinterpret_cast<uint32_t*>(smem_raw + TS * TS * 8);        // one chunk
  tile_body<TS, BLOCK, NL, MODE>(sc, bins, out, blockIdx.x, sh, keys, queue, queue_entries(bins.capacity));
}

cudaError_t launch_bin(const t3_frame& fr, const t3_object& ob, const BinArgs& bins, cudaStream_t st) {
  if (ob.nfaces <= 0) return cudaSuccess;
  constexpr int BLOCK = 256;
  const int64_t grid = (ob.nfaces + BLOCK - 1) / BLOCK;
  k_bin<BLOCK><<<(unsigned)grid, BLOCK, 0, st>>>(fr, ob.mesh, ob.nfaces, (uint32_t)ob.face_base, bins);
  return cudaGetLastError();
}

template <int TS, int BLOCK, int NL, int MODE>
static cudaError_t launch_tile_b(const DevScene* sc, const BinArgs& bins, int ntiles,
                                 const t3_outputs& out, cudaStream_t st) {
  const size_t smem = (size_t)TS * TS * 8 + (size_t)queue_entries(bins.capacity) * 4;
  cudaError_t e = cudaFuncSetAttribute(k_tile<TS, BLOCK, NL, MODE>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_tile<TS, BLOCK, NL, MODE><<<ntiles, BLOCK, smem, st>>>(sc, bins, out);
  return cudaGetLastError();
}

template <int TS, int BLOCK, int NL>
static cudaError_t launch_tile_nl(const DevScene* sc, const BinArgs& bins, int ntiles,
                                  const t3_outputs& out, cudaStream_t st) {
  if (bins.light_mode == T3_LIGHT_LAMPS)
    return launch_tile_b<TS, BLOCK, NL, T3_LIGHT_LAMPS>(sc, bins, ntiles, out, st);
  if (bins.light_mode == T3_LIGHT_IBL_MC)
    return launch_tile_b<TS, BLOCK, NL, T3_LIGHT_IBL_MC>(sc, bins, ntiles, out, st);
  if (bins.light_mode == T3_LIGHT_IBL_PREFILTERED)
    return launch_tile_b<TS, BLOCK, NL, T3_LIGHT_IBL_PREFILTERED>(sc, bins, ntiles, out, st);
  if (bins.light_mode == T3_LIGHT_IBL_MLP)  // visibility only: one instance serves every NL
    return launch_tile_b<TS, BLOCK, 2, T3_LIGHT_IBL_MLP>(sc, bins, ntiles, out, st);
  return cudaErrorInvalidValue;
}

template <int TS, int BLOCK>
static cudaError_t launch_tile_t(const DevScene* sc, const BinArgs& bins, int ntiles,
                                 const t3_outputs& out, cudaStream_t st) {
  if (bins.max_lobes <= 2) return launch_tile_nl<TS, BLOCK, 2>(sc, bins, ntiles, out, st);
  return launch_tile_nl<TS, BLOCK, 4>(sc, bins, ntiles, out, st);
}

cudaError_t launch_tile(const DevScene* sc, const BinArgs& bins, int ntiles, const t3_outputs& out,
                        cudaStream_t st) {
  switch (bins.tile) {
  case 8: return launch_tile_t<8, 64>(sc, bins, ntiles, out, st);
  case 16: return launch_tile_t<16, 256>(sc, bins, ntiles, out, st);
  case 32: return launch_tile_t<32, 256>(sc, bins, ntiles, out, st);
  default: return cudaErrorInvalidValue;
  }
}

} // namespace t3
