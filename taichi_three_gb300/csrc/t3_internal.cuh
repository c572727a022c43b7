// t3_internal.cuh -- library-internal types shared by the kernels and the C ABI
// host code: the device copy of a scene (with materials flattened into lobes),
// the workspace layout, status bits and the launchers.
#pragma once

#include <cstddef>

#include "t3_device.cuh"

namespace t3 {

// device status word bits (OR-ed by kernels, read by t3_read_status)
#define T3_STATUS_BIG_OVERFLOW 1
#define T3_STATUS_BIN_OVERFLOW 2
#define T3_STATUS_TIMEOUT 4

// Large-face queue of the direct rasteriser (and its setup-record buffer).
struct BigQueue {
  uint32_t* items;
  uint32_t capacity;
  uint32_t* count;
  int32_t* status;
  float4* rec;  // setup records per global face id, or nullptr (shading recomputes)
  unsigned long long* fragments = nullptr;  // statistics runs: count of depth reductions
  const float4* vndc = nullptr;  // per-vertex NDC + clip w (indexed meshes and grids), or nullptr
};

// Binned rasteriser state (binned.cu).
struct BinArgs {
  float4* rec;           // setup records, 4 x float4 per global face id
  uint32_t* bins;        // [ntiles, capacity] face ids
  uint32_t* count;       // [ntiles] entries appended (may exceed capacity)
  uint32_t* big;         // big-face ids
  uint32_t* big_count;
  int32_t* status;
  uint32_t capacity;     // entries per tile bin (multiple of 4)
  uint32_t big_capacity;
  int32_t tile;          // tile edge in pixels (8, 16, 32)
  int32_t tiles_x, tiles_y;
  int32_t big_tiles;     // faces touching more tiles than this go to the big list
  int32_t max_lobes;     // largest flattened material of the scene
  int32_t light_mode;    // T3_LIGHT_*
  unsigned long long* keys;  // T3_LIGHT_IBL_MLP: the frame's packed keys, written by the tiles
  // the frame's particle and line fragments (packed keys, rasterised before the
  // tiles), which seed each tile's keys; nullptr when the scene has none
  const unsigned long long* pre;
};

// A material tree flattened into a sum of weighted leaf lobes:
//   brdf = sum_k W_k * leaf_k.brdf,  ambient = sum_k W_k * leaf_k.ambient, ...
// W_k is a product of factor nodes along the path from the root (Mix contributes
// (1 - factor) to its first child and factor to its second, Scale its factor).
// fac[j] = node index | T3_FAC_ONE_MINUS.
#define T3_FAC_ONE_MINUS 0x10000
#define T3_FAC_MIX 0x20000  // the factor comes from a Mix node (a sampling choice)
struct DevLobe {
  int32_t kind;    // T3_OP_LAMBERT / PHONG / COOK / EMISSION
  int32_t nfac;
  int32_t p0, p1;  // PHONG: shineness node; COOK: roughness, fresnel nodes
  int32_t int_pow; // PHONG: integer exponent (>0) when shineness is a Python int
  int32_t fac[T3_MAX_FACTORS];
  int32_t _pad[3];
};

struct DevMaterial {
  int32_t nnodes, nlobes;
  int32_t _pad[2];
  t3_node nodes[T3_MAX_NODES];
  DevLobe lobes[T3_MAX_LOBES];
  t3_texture textures[T3_MAX_TEXTURES];
};

// A material of a known shape, found by the host in the flattened lobes, with
// the node indices of its parameters, so that a shading instance for that
// shape evaluates each parameter once instead of walking the lobes' factors
// (the values, and so the pixels, are the same):
//   T3_SIG_PBR      Mix(Lambert * C, CookTorrance(R, F), F), F a FresnelFactor:
//                   node = {C, F, R}
//   T3_SIG_CLASSIC  Mix(Lambert * C, Phong(M), S): node = {C, S, M}, int_pow
//   T3_SIG_DIFFUSE  Lambert * C: node = {C}
struct FastMat {
  int32_t sig;  // 0: none
  int32_t node[3];
  int32_t int_pow;
  int32_t _pad[3];
};

struct DevObject {
  t3_mesh mesh;
  DevMaterial mat;
  int64_t face_base, nfaces;
  FastMat fast;
};

struct DevScene {
  t3_frame frame;
  t3_lighting lighting;  // lighting.tables is cleared: the tables are copied below
  int32_t nobjects;
  int32_t _pad;
  DevObject obj[T3_MAX_OBJECTS];
  t3_ibl_tables tables;  // T3_LIGHT_IBL_PREFILTERED
};
// the shading kernels read each lamp as two float4 loads
static_assert((offsetof(DevScene, lighting) + offsetof(t3_lighting, lights)) % 16 == 0,
              "lamps must be 16-byte aligned inside DevScene");
static_assert(sizeof(t3_light) % 16 == 0, "t3_light must be a multiple of 16 bytes");


// The direct frame's key buffer between frames.  t3_render keeps, at the start
// of its workspace, a 64-bit tag and a u32 ticket: the shading pass resets
// every key it reads to empty and then stores the frame's tag, so the next
// frame with the same tag (same workspace, layout and size) finds its keys
// already empty and skips the clear; the clear stores 0 (keys not known to be
// empty) once all of its blocks have read the tag.  Every other use of the
// workspace leaves 0 there.
struct KeyState {
  unsigned long long* tag_word = nullptr;  // nullptr: no state kept (always clear)
  uint32_t* ticket = nullptr;              // blocks of the clear that have read the tag
  unsigned long long tag = 0;              // this frame's tag (0: never skip the clear)
  // the host expects the tag to match (the previous frame through this
  // workspace emptied the keys): the clear runs as one block, which still
  // clears every key, slowly, if the tag turns out not to match
  bool likely_empty = false;
};

int flatten_material(const t3_material& in, DevMaterial& out);
// first_ids_free: objects may start at any face id past the previous object's
// last (t3_shade of one object of a protocol frame); otherwise they are
// numbered consecutively from 0 (every frame that indexes setup records by id)
int make_dev_scene(const t3_scene& sc, DevScene& out, bool first_ids_free = false);

cudaError_t launch_raster_particles(const t3_frame& fr, const t3_object& ob, unsigned long long* keys,
                                    unsigned long long* fragments, cudaStream_t st);
cudaError_t launch_raster_wires(const t3_frame& fr, const t3_object& ob, unsigned long long* keys,
                                unsigned long long* fragments, cudaStream_t st);
// objects of the particle and wireframe rasterisers (their own direct kernels
// write the frame's keys in every raster mode)
inline bool is_point_or_line(const t3_mesh& m) {
  return m.kind == T3_MESH_PARTICLES || m.kind == T3_MESH_LINES || (m.flags & T3_MESH_WIREFRAME) != 0;
}
inline cudaError_t launch_raster_point_or_line(const t3_frame& fr, const t3_object& ob, unsigned long long* keys,
                                               unsigned long long* fragments, cudaStream_t st) {
  return ob.mesh.kind == T3_MESH_PARTICLES ? launch_raster_particles(fr, ob, keys, fragments, st)
                                           : launch_raster_wires(fr, ob, keys, fragments, st);
}
cudaError_t launch_vertex_ndc(const t3_frame& fr, const t3_mesh& mesh, int64_t nverts, float4* out,
                              cudaStream_t st);
int64_t mesh_vertex_rows(const t3_mesh& m);  // rows the vertex stage transforms (0: none)
cudaError_t launch_red_min_rate(unsigned long long* buf, int64_t n, int rounds, cudaStream_t st);
cudaError_t launch_clear(unsigned long long* keys, int64_t n, cudaStream_t st, uint32_t* counters = nullptr,
                         int ncounters = 0, int32_t* status = nullptr, KeyState ks = KeyState());
cudaError_t launch_upload_scene(const DevScene& sc, DevScene* dst, uint32_t* counters,
                                int ncounters, int32_t* status, cudaStream_t st,
                                unsigned long long* key_tag = nullptr);
cudaError_t launch_raster_direct(const t3_frame& fr, const t3_object& ob, unsigned long long* keys,
                                 const BigQueue& big, int32_t big_threshold, cudaStream_t st);
// the shading pass; the scene descriptor is passed to the kernels by value
// (sc_dev, its uploaded copy, is kept for kernels that read it from memory)
// reset (lamp and Monte Carlo lighting, and the learned IBL with a row list):
// the pass returns every key it reads to empty and then stores reset.tag in
// *reset.tag_word
// rows (learned IBL): the network pass's row list (96 bytes per pixel of the
// frame) and its counter, zeroed before the pass; without it the one-kernel
// network pass runs
struct MlpRows {
  float4* rows = nullptr;
  uint32_t* count = nullptr;
  cudaEvent_t split = nullptr;  // recorded between the two kernels (timing)
};
cudaError_t launch_shade(const DevScene& sc_host, const DevScene* sc_dev, const unsigned long long* keys,
                         const float4* rec, const t3_outputs& out, int32_t* status, cudaStream_t st,
                         KeyState reset = KeyState(), MlpRows rows = MlpRows());
cudaError_t launch_shade_mlp(const DevScene& sc, const unsigned long long* keys, const float4* rec,
                             const t3_outputs& out, int32_t* status, cudaStream_t st,
                             const MlpRows& rows = MlpRows(), const KeyState& reset = KeyState());
int max_lobes(const DevScene& sc);
// the FastMat shape of a flattened material (fast.sig = 0 when none matches)
void find_fast_material(const DevMaterial& m, FastMat& fast);
// the shape shared by every shaded object of the scene, or 0
int fast_signature(const DevScene& sc);
// every object is a face soup without mesh edits (and with normals when the
// frame smooths): the shading instances that compile the other geometry out
bool plain_soups(const DevScene& sc);
// the lobe kinds (one byte per slot) shared by every shaded object of the
// scene when a specialised shading instance exists for them, else 0
int lobe_signature(const DevScene& sc);
int has_textures(const DevScene& sc);  // any Texture / ChessboardTexture node
int has_points_or_lines(const t3_scene& sc);
int64_t total_faces(const t3_scene& sc);
// the binned rasteriser's automatic entries per tile bin: 8 x faces / tiles + 64
int64_t auto_bin_capacity(const t3_scene& sc, int tile);
// t3_render_batch's binned path (batch_binned.cu): workspace bytes, and the batch
int batch_binned_size(const t3_scene* scenes, int n, const t3_batch_config& c, size_t* bytes);
int render_batch_binned(const t3_scene* scenes, const t3_outputs* outs, int n, const t3_batch_config& c,
                        void* workspace, size_t workspace_bytes, int32_t* status, cudaStream_t st);
cudaError_t launch_bin(const t3_frame& fr, const t3_object& ob, const BinArgs& bins, cudaStream_t st);
cudaError_t launch_tile(const DevScene* sc, const BinArgs& bins, int ntiles, const t3_outputs& out,
                        cudaStream_t st);

} // namespace t3
