/*
 * tina3.h -- C ABI of the GB300 triangle rasteriser + deferred shading library
 * (libtina3.so).  Plain C: device pointers, sizes, an explicit cudaStream_t
 * (passed as void*), no torch types.  Every entry point returns 0 on success or
 * a negative T3_E* code.  Nothing here allocates device memory: callers pass
 * every output and the workspace (sized by t3_workspace_size).
 *
 * The structs below are the descriptors the Tina drop-in layer fills from its
 * Python objects.  All matrices are row-major 4x4 float, M[i][j] = m[4*i + j],
 * exactly as Tina's `Engine.W2V` / `Engine.V2W` fields (tina/core/engine.py:13-14).
 *
 * Image buffers use Tina's field indexing: pixel (x, y) lives at x*H + y
 * (a Taichi field of shape (W, H) is x-major), rgb at 3*(x*H + y).
 */
#ifndef TINA3_H
#define TINA3_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes ------------------------------------------------------- */
#define T3_OK 0
#define T3_EINVAL (-1)       /* bad argument (null pointer, size, enum)        */
#define T3_ECUDA (-2)        /* a CUDA launch or runtime call failed            */
#define T3_EOVERFLOW (-3)    /* a bin / queue capacity was exceeded: retry with
                                a larger capacity (t3_workspace_size)          */
#define T3_ETIMEOUT (-4)     /* a bounded device-side wait gave up               */
#define T3_ETOOBIG (-5)      /* a size exceeds a fixed maximum of this entry     */
#define T3_EUNSUPPORTED (-6) /* a feature combination this build does not run    */

/* ---- fixed maxima ---------------------------------------------------------- */
#define T3_MAX_LIGHTS 16   /* Lighting(maxlights=16), tina/core/lighting.py:26 */
#define T3_MAX_NODES 24    /* material expression nodes per object             */
#define T3_MAX_OBJECTS 8   /* objects per frame                                 */
#define T3_MAXDEPTH (1 << 30) /* Engine.maxdepth, tina/core/engine.py:11        */

/* ---- frame ---------------------------------------------------------------- */
/* flags */
#define T3_CULLING 1    /* TriangleRaster(culling=True)  triangle.py:96-98 */
#define T3_CLIPPING 2   /* TriangleRaster(clipping=True) triangle.py:100-104 */
#define T3_SMOOTHING 4  /* interpolate vertex normals     triangle.py:36-38 */
#define T3_TEXTURING 8  /* interpolate texcoords          triangle.py:44-46 */
#define T3_TONEMAP 16   /* ACES after shading             scene/raster.py:202-203 */
#define T3_WIRE_CLIPPING 32 /* WireframeRaster(clipping=True) wireframe.py:78-81 */
/* t3_shade pixel selection (the three-method raster protocol).  With neither
 * flag every pixel is written.  With one or both, only the selected pixels
 * are written and every other pixel's outputs are left as they are: */
#define T3_SHADE_OWNED 128  /* pixels whose winning face belongs to an object of
                               the scene: TriangleRaster.render_color skips
                               occup == -1 (tina/core/triangle.py:134-139)   */
#define T3_SHADE_EMPTY 256  /* pixels no fragment reached: background colour or
                               the sky (Engine.render_background,
                               tina/core/engine.py:42-49)                    */
/* Test of the timeout path (no reference counterpart): the binned tiles issue
 * no bin copy and wait, wait_limit polls, on a barrier nothing arrives on;
 * every tile then gives up, writes background and sets T3_STATUS_TIMEOUT.  No
 * copy is in flight, so nothing is drained; the next frame is unaffected. */
#define T3_STARVE_BIN_COPY 512
/* The same for the learned-IBL network pass: its leader warps issue no
 * tensor-core operation, so every wait on one (wait_limit polls each) runs
 * out; the pass stops, leaves its covered pixels' colour unwritten and sets
 * T3_STATUS_TIMEOUT.  Nothing was issued, so nothing is drained. */
#define T3_STARVE_NETWORK 1024

typedef struct t3_frame {
  int32_t width, height; /* Engine.res                                      */
  int32_t flags;         /* T3_CULLING | ...                                */
  int32_t maxdepth;      /* 2**30                                           */
  float W2V[16];         /* proj @ view, float32 (engine.py:72-76)          */
  float V2W[16];         /* inv(proj @ view), float32                       */
  float bias[2];         /* pixel-centre offset, (0.5, 0.5) by default      */
  float bgcolor[3];      /* Scene(bgcolor=...) image.fill value             */
  float linecolor[3];    /* WireframeRaster(linecolor=...), wireframe.py:6-20 */
  int32_t wait_limit;    /* polls of the binned tiles' first bounded wait on
                            their bin copy (0: the default, 1 << 22) and of
                            each wait of the learned-IBL network pass on the
                            tensor cores (0: 1 << 24); the waits that let an
                            issued copy or MMA land keep the defaults       */
  int32_t _pad;          /* 184 bytes: keeps t3_scene.lighting.lights 16-byte aligned */
} t3_frame;

/* ---- meshes (the mesh protocol of the tina.mesh package) ----------------------------- */
#define T3_MESH_SOUP 0    /* SimpleMesh: verts [n,3,3], norms [n,3,3], coors [n,3,2]   */
#define T3_MESH_GRID 1    /* MeshGrid:   pos [nx,ny,3], nrm [nx,ny,3], tex [nx,ny,2]   */
#define T3_MESH_INDEXED 2 /* MeshModel / ConnectiveMesh: per-vertex arrays + face indices */
#define T3_MESH_PARTICLES 3 /* SimpleParticles (tina/pars/simple.py) for ParticleRaster
                               (tina/core/particle.py): nfaces = particles,
                               verts = positions [n,3], coors = radii [n],
                               norms = colours [n,3] (nullptr: white)                    */
#define T3_MESH_LINES 4   /* SimpleMesh(npolygon=2) (tina/mesh/simple.py): verts [n,2,3];
                             drawn by the wireframe rasteriser (tina/core/wireframe.py);
                             flags: TRANSFORM, WIREFRAME                                */

/* mesh flags (mesh-edit nodes) */
#define T3_MESH_TRANSFORM 1   /* MeshTransform        tina/mesh/trans.py:23-40 */
#define T3_MESH_NOCULL 2      /* MeshNoCulling        tina/mesh/cull.py:31-58  */
#define T3_MESH_FLIP_ORDER 4  /* MeshFlipCulling      tina/mesh/cull.py:5-28   */
#define T3_MESH_FLIP_NORMAL 8 /* MeshFlipNormal       tina/mesh/cull.py:61-66  */
#define T3_MESH_FLAT_NORMAL 16/* MeshFlatNormal       tina/mesh/norm.py:5-14   */
#define T3_MESH_WIREFRAME 32  /* MeshToWire           tina/mesh/wire.py:5-40:
                                 the object is the polygon edges of the mesh as
                                 lines: line n = corners (n % p, (n+1) % p) of
                                 face n / p, p = 3 (4 for T3_MESH_QUADS, 2 for
                                 T3_MESH_LINES), over the faces after the other
                                 edits (NOCULL doubles them); object nfaces =
                                 lines */
#define T3_MESH_QUADS 64      /* MeshGrid(as_quad=True) tina/mesh/grid.py:23-58:
                                 face f of a T3_MESH_GRID is cell f's quad
                                 (a, b, c, d) = ((i,j), (i+1,j), (i+1,j+1),
                                 (i,j+1)); nfaces = (n-1)^2.  Only drawn through
                                 T3_MESH_WIREFRAME (with T3_MESH_TRANSFORM at
                                 most): a quad is not a triangle raster's face */

typedef struct t3_mesh {
  int32_t kind;        /* T3_MESH_*                                              */
  int32_t flags;       /* T3_MESH_* edit flags                                   */
  int64_t nfaces;      /* faces of the underlying mesh (before NOCULL doubling)  */
  const float* verts;  /* positions (layout per kind)                            */
  const float* norms;  /* normals, may be NULL unless T3_SMOOTHING               */
  const float* coors;  /* texcoords, may be NULL unless T3_TEXTURING             */
  const int32_t* faces;/* INDEXED: corner k of face f reads attribute slot s at
                          faces[f*face_stride + k*corner_stride + s]             */
  int32_t face_stride;   /* 3 (ConnectiveMesh [n,3]) or 9 (MeshModel [n,3,3])    */
  int32_t corner_stride; /* 1 or 3                                              */
  int32_t slot_vert, slot_coor, slot_norm; /* 0,0,0 or 0,1,2 (v, vt, vn)          */
  int32_t grid_nx, grid_ny; /* GRID: vertex counts                               */
  int32_t attr_stride;      /* floats per face in face_attr                      */
  const float* face_attr;   /* per-face material attributes [n, attr_stride]     */
  float trans[16];          /* MeshTransform.trans                                */
  float trans_normal[9];    /* transpose(inv(trans))[:3,:3]                       */
  int32_t nverts;           /* vertex rows of verts (indexed meshes; 0 = unknown)   */
} t3_mesh;

/* ---- materials: an expression tree (tina/matr/material.py, nodes.py) -------- */
/* value nodes */
#define T3_OP_CONST 0    /* v[0..2], width in b (1 or 3)                 nodes.py:42-49 */
#define T3_OP_ATTR 1     /* per-face attribute: a = channel, b = width   (FaceAttr)      */
#define T3_OP_INPUT 2    /* a = 0 pos, 1 color, 2 normal, 3 texcoord     nodes.py:79-96  */
#define T3_OP_FRESNEL 3  /* a = metallic, b = albedo, c = specular       material.py:69-83 */
#define T3_OP_TEXTURE 4  /* a = texcoord node, b = texture slot          nodes.py:99-111 */
#define T3_OP_CHECKER 5  /* a = texcoord, b = size, c = color0,
                            (int)v[0] = color1 node                      nodes.py:114-126 */
/* leaf materials */
#define T3_OP_LAMBERT 16 /*                                              material.py:387-442 */
#define T3_OP_PHONG 17   /* a = shineness                                material.py:445-472 */
#define T3_OP_COOK 18    /* a = roughness, b = fresnel                   material.py:244-384 */
#define T3_OP_EMISSION 19/*                                              material.py:659-681 */
/* combinators */
#define T3_OP_MIX 32     /* a = mat1, b = mat2, c = factor               material.py:86-145 */
#define T3_OP_SCALE 33   /* a = mat, b = factor                          material.py:148-191 */
#define T3_OP_ADD 34     /* a = mat1, b = mat2                           material.py:194-238 */

typedef struct t3_node {
  int32_t op, a, b, c;
  float v[4];
} t3_node;

/* An image texture (advans.py texture_as_field): float32 [w, h, channels],
 * Tina's field indexing [i, j]; sampled at texcoord * (shape - 1) with
 * bilerp (common.py:141-150), the +1 neighbour clamped to the image. */
#define T3_MAX_TEXTURES 4
typedef struct t3_texture {
  const float* data;
  int32_t w, h, channels, _pad; /* channels 1 or 3 */
} t3_texture;

typedef struct t3_material {
  int32_t nnodes; /* used entries of nodes[]                                 */
  int32_t root;   /* index of the root material node                          */
  t3_node nodes[T3_MAX_NODES];
  t3_texture textures[T3_MAX_TEXTURES]; /* referenced by T3_OP_TEXTURE nodes  */
} t3_material;

typedef struct t3_object {
  t3_mesh mesh;
  t3_material material;
  int64_t face_base; /* first global face id of this object                  */
  int64_t nfaces;    /* faces exposed to the raster (x2 for T3_MESH_NOCULL)    */
} t3_object;

/* ---- lighting (tina/core/lighting.py) -------------------------------------- */
typedef struct t3_light {
  float dir[4];   /* xyz, w: 0 directional (normalised dir), 1 point (position) */
  float color[4]; /* rgb, pad                                                    */
} t3_light;

#define T3_LIGHT_LAMPS 0   /* Lighting: emission + ambient + sum of lamps              */
#define T3_LIGHT_IBL_MC 1  /* SkyboxLighting by Monte Carlo over the materials' own
                              importance samplers (material.sample, material.py:
                              124-138, 365-405, 460-472): emission + mean of
                              weight * env(dir) over `spp` samples (+ lamps if any)  */
#define T3_LIGHT_IBL_MLP 2 /* SkyboxLighting by the learned IBL network             */
#define T3_LIGHT_IBL_PREFILTERED 3 /* SkyboxLighting's own lookup of prefiltered maps
                              (tina/core/lighting.py:20-21): Lambert.sample_ibl reads
                              the diffuse map at the normal (material.py:441-442);
                              CookTorrance.sample_ibl (material.py:256-277) reads the
                              two specular maps around its roughness at the mirror
                              direction, lerps them, and scales by f0 * A + B from a
                              bilinear LUT read at (VoH, roughness) in texel units;
                              Mix / Scale weigh their children (material.py:141-145,
                              :187-191); Add sums them; Phong has no lookup
                              (T3_EUNSUPPORTED, as the reference raises)            */

/* Prefiltered IBL tables.  Maps use the environment's equirect layout (texel
 * (i, j) at (i*h + j)*3, FP16 when `half`); the LUT is float [lut_w, lut_h, 2]
 * (A, B), read at (VoH, roughness) without scaling, as the reference does. */
#define T3_IBL_LEVELS 7 /* the environment + the maps of roughness 0.03, 0.08,
                           0.18, 0.35, 0.65, 1.0 (CookTorrance.rough_levels,
                           tina/matr/material.py:252-253)                    */
typedef struct t3_ibl_map {
  const void* data;
  int32_t w, h, half, _pad;
} t3_ibl_map;
typedef struct t3_ibl_tables {
  t3_ibl_map spec[T3_IBL_LEVELS]; /* spec[0] is the environment itself          */
  t3_ibl_map diffuse;             /* Lambert.cook_for_ibl's map                  */
  const float* lut;
  int32_t lut_w, lut_h;           /* at least 2 x 3 texels (the region the lookup reads) */
} t3_ibl_tables;

/* MLP-IBL network (see t3_mlp_*): 400 -> 64 -> 64 -> 64 -> 16 (9 used),
 * ReLU hidden layers, BF16 weights (inference) with FP32 biases. */
#define T3_MLP_IN 400
#define T3_MLP_HID 64
#define T3_MLP_OUT 16

typedef struct t3_lighting {
  int32_t mode;     /* T3_LIGHT_*                                             */
  int32_t nlights;  /* lamps; with an IBL mode they are added to the IBL term  */
  float ambient[4];
  t3_light lights[T3_MAX_LIGHTS];
  /* environment map, Tina's equirect layout (tina/skybox.py:40-145): texel
   * (i, j), i < env_w = 2*res, j < env_h = res, at (i*env_h + j)*3; FP16 when
   * env_half, else FP32 */
  const void* env;
  int32_t env_w, env_h, env_half, spp;
  uint32_t seed;    /* Monte Carlo stream seed                                 */
  int32_t _pad;
  const void* mlp;  /* T3_LIGHT_IBL_MLP: packed network (t3_mlp_pack)         */
  const t3_ibl_tables* tables; /* T3_LIGHT_IBL_PREFILTERED (host memory, read at
                                  the call; the maps it points to are device data) */
} t3_lighting;

/* ---- whole-frame parameters --------------------------------------------- */
typedef struct t3_scene {
  t3_frame frame;
  t3_lighting lighting;
  int32_t nobjects;
  int32_t _pad;
  t3_object objects[T3_MAX_OBJECTS];
} t3_scene;

/* outputs of one frame (device pointers; any may be NULL except rgb)       */
typedef struct t3_outputs {
  float* rgb;        /* [W,H,3] scene.img (post tonemap when T3_TONEMAP)      */
  int32_t* face_id;  /* [W,H] winning global face id, -1 where empty          */
  int32_t* depth;    /* [W,H] Engine.depth (int32(depth_f * 2**30)), maxdepth  */
  float* depth_f;    /* [W,H] the winning fragment's float depth, +inf empty    */
} t3_outputs;

/* raster modes */
#define T3_RASTER_DIRECT 0 /* per-face threads, global packed u64 atomicMin     */
#define T3_RASTER_BINNED 1 /* tile bins + per-tile queues in shared memory       */

/* ---- entry points ------------------------------------------------------- */

/* Version / build probe. */
int t3_version(void);

/* sizeof() of t3_frame, t3_mesh, t3_node, t3_material, t3_object, t3_light,
 * t3_lighting, t3_scene, t3_outputs in that order, for binding-layer layout
 * checks.  Returns the count; writes min(n, count) values when out != NULL. */
int t3_struct_sizes(int64_t* out, int n);

/* Workspace bytes needed by t3_render for this scene at raster mode `mode`
 * with tile edge `tile` (8, 16 or 32) and `bin_capacity` entries per frame
 * for the binned mode (0 = automatic).  Replaces the per-raster fields that
 * TriangleRaster.__init__ allocates (tina/core/triangle.py:16-29).
 * The first 16 bytes of a workspace are state that t3_render keeps between
 * frames (whether the direct frame's depth keys were left empty by the last
 * frame's shading, so that the next frame can skip clearing them): zero them
 * once when the workspace is allocated, and again after using the memory for
 * anything else. */
int t3_workspace_size(const t3_scene* scene, int mode, int tile,
                      int64_t bin_capacity, size_t* bytes);

/* Effective per-tile bin capacity (entries) of the binned rasteriser for this
 * scene at tile edge `tile`; `bin_capacity` 0 selects the automatic size
 * (8 x faces / tiles + 64, rounded up to 32).  No counterpart in the
 * reference, whose rasteriser has no bins. */
int t3_bin_capacity(const t3_scene* scene, int tile, int64_t bin_capacity, int64_t* capacity);

/* Largest per-tile bin count of the last binned frame rendered with this
 * workspace (synchronises `stream`): the capacity a re-render needs after
 * T3_STATUS_BIN_OVERFLOW.  No counterpart in the reference. */
int t3_bin_counts_max(const t3_scene* scene, int tile, int64_t bin_capacity, const void* workspace,
                      size_t workspace_bytes, int64_t* max_count, void* stream);

/* Engine.clear_depth (tina/core/engine.py:68-70) for the packed buffer:
 * depth_id[W*H] = empty key. */
int t3_clear(uint64_t* depth_id, int64_t npixels, void* stream);

/* TriangleRaster.set_object + render_occup (tina/core/triangle.py:72-131)
 * for one object: per-face transform, cull, clip, setup and depth test into
 * the packed buffer key = (uint32(depth) ^ 0x80000000) << 32 | global face id,
 * whose unsigned minimum equals the serial reference's winner (lowest depth,
 * ties to the lowest face id).  `workspace` holds the large-triangle queue.
 * `status` (device int32) receives T3_* codes of device-side overflows. */
int t3_raster(const t3_frame* frame, const t3_object* object,
              uint64_t* depth_id, void* workspace, size_t workspace_bytes,
              int32_t* status, void* stream);

/* TriangleRaster.render_color + Shader + Lighting + ToneMapping
 * (tina/core/triangle.py:134-153, shader.py:119-131, lighting.py:84-98,
 * postp/tonemap.py:10-12) for all objects of the scene.  The workspace (at
 * least t3_workspace_size bytes) receives the device copy of the scene.
 * frame.flags T3_SHADE_OWNED / T3_SHADE_EMPTY restrict the pixels written
 * (one object of a multi-object frame, then the background).
 * Lighting T3_LIGHT_LAMPS and T3_LIGHT_IBL_MC; T3_LIGHT_IBL_MLP returns
 * T3_EUNSUPPORTED here (t3_render runs it and reports its device status). */
int t3_shade(const t3_scene* scene, const uint64_t* depth_id, void* workspace,
             size_t workspace_bytes, const t3_outputs* out, void* stream);

/* Statistics (no reference counterpart): the number of depth reductions
 * (fragments passing the inside and maxdepth tests) the direct rasteriser
 * performs for the scene -- the atomic work of a frame.  Runs clear + raster
 * with a counting instance of the kernels and synchronises the stream.
 * workspace: t3_workspace_size(scene, T3_RASTER_DIRECT, ...) bytes. */
int t3_raster_fragments(const t3_scene* scene, void* workspace, size_t workspace_bytes,
                        int64_t* fragments, void* stream);
/* u64 atomicMin throughput probe: `rounds` reductions on each of n distinct
 * addresses of buf (zeroed or filled by the caller; L2-resident when n * 8
 * is well below the L2 size).  The caller times it. */
int t3_red_min_rate(uint64_t* buf, int64_t n, int rounds, void* stream);

/* Scene.render (tina/scene/raster.py:168-207) for one frame: clear, raster
 * every object (mode T3_RASTER_*), shade, tonemap. */
int t3_render(const t3_scene* scene, int mode, int tile, int64_t bin_capacity,
              void* workspace, size_t workspace_bytes, int32_t* status,
              const t3_outputs* out, void* stream);

/* MeshGrid.pre_compute (tina/mesh/grid.py:27-36): nrm[i,j] =
 * normalize(cross(pos[i+1,j] - pos[i-1,j], pos[i,j+1] - pos[i,j-1])) with
 * clamped neighbours, for a [nx, ny, 3] float grid. */
int t3_grid_normals(const float* pos, float* nrm, int nx, int ny, void* stream);

/* MeshSmoothNormal (tina/mesh/norm.py:17-55) of an indexed mesh (kind
 * T3_MESH_INDEXED, no edit flags): norms_out[v] = normalized(sum, over the
 * faces that use vertex v in face order, of normalized(cross(b - a, c - a))),
 * [nverts, 3] floats, bit-identical to the reference's serial loop; a vertex
 * no face uses gets NaN (the reference's normalized zero vector).  A mesh
 * wrapped by MeshSmoothNormal is then described as the indexed mesh with
 * norms = norms_out and slot_norm = slot_vert.  `workspace` (device, 16-byte
 * aligned) holds t3_smooth_normals_workspace_size bytes. */
int t3_smooth_normals_workspace_size(int64_t nfaces, int64_t nverts, size_t* bytes);
int t3_smooth_normals(const t3_mesh* mesh, int64_t nverts, float* norms_out, void* workspace,
                      size_t workspace_bytes, void* stream);

/* Height-field animation of a grid's positions [nx, ny, 3] (no reference
 * counterpart; the reference's demos animate grids from Python):
 * pos[i, j].z = amp * sin(fx * x + wx * t) * cos(fy * y + wy * t). */
int t3_grid_wave(float* pos, int nx, int ny, float amp, float fx, float fy, float wx, float wy,
                 float t, void* stream);

/* ToneMapping.apply (tina/postp/tonemap.py:10-12): in-place ACES on n floats. */
int t3_tonemap(float* rgb, int64_t n, void* stream);

/* t3_render with timing events: when stage_events is non-NULL, events [0..3]
 * (cudaEvent_t handles, entries may be NULL) are recorded on `stream` at frame
 * start, after the key clear, after the rasteriser and after shading. */
int t3_render_staged(const t3_scene* scene, int mode, int tile, int64_t bin_capacity,
                     void* workspace, size_t workspace_bytes, int32_t* status,
                     const t3_outputs* out, void* stream, void* const* stage_events);
/* The same with nevents = 4 or 5 events; with 5, event [3] is recorded between
 * the learned-IBL shading's two kernels (after the row prepass, before the
 * network kernel) -- for other lighting together with [4] -- and [4] after
 * shading. */
int t3_render_staged_n(const t3_scene* scene, int mode, int tile, int64_t bin_capacity,
                       void* workspace, size_t workspace_bytes, int32_t* status,
                       const t3_outputs* out, void* stream, void* const* stage_events, int nevents);

/* Timing-event helpers for callers without their own CUDA runtime binding. */
int t3_event_create(void** event);
int t3_event_destroy(void* event);
int t3_event_elapsed_ms(void* start, void* end, float* ms); /* waits for `end` */

/* Limits of t3_render_noalloc's built-in scratch array. */
#define T3_NOALLOC_MAX_PIXELS (1u << 21)      /* 2,097,152 px: covers 1920x1080 */
#define T3_NOALLOC_MAX_BIG_FACES (1u << 16)   /* faces with bbox > 4096 px per frame */
/* scene copy (16 KiB) + counters (256 B) + large-face queue + depth keys */
#define T3_NOALLOC_SCRATCH_BYTES \
  (16384u + 256u + 4u * T3_NOALLOC_MAX_BIG_FACES + 8u * T3_NOALLOC_MAX_PIXELS)

/* t3_render (direct mode) for callers that cannot allocate device memory --
 * code running inside a host application that owns the GPU's memory and hands
 * the renderer only its buffers.  No counterpart in the reference, which has
 * no allocation-free entry point.  The caller passes the scene, a device status
 * word and the outputs; the scratch (depth keys, counters, large-face queue,
 * scene copy) is a fixed device array inside the library,
 * T3_NOALLOC_SCRATCH_BYTES (17,056,000 bytes, about 16.3 MiB),
 * held by every GPU that loads the library until the process exits.  Limits:
 * width * height <= T3_NOALLOC_MAX_PIXELS (else T3_ETOOBIG); at most
 * T3_NOALLOC_MAX_BIG_FACES faces with a bbox above 4096 px per frame (more set
 * T3_STATUS_BIG_OVERFLOW in *status and those faces are dropped).  The first
 * call in each CUDA context looks the array's address up and caches it under
 * the context's id (make that call before any stream capture; a new context,
 * or the one made after a device reset, gets its own lookup).  All calls share
 * the array: calls that overlap on the GPU race and must be serialised by the
 * caller, and so must replays of a CUDA graph that captured this call (the
 * graph holds the same array's address).  Calls no cudaMalloc/cudaFree. */
int t3_render_noalloc(const t3_scene* scene, int32_t* status, const t3_outputs* out, void* stream);

/* ---- post-processing of scene.img (images [W, H, 3] float32, pixel x*H + y) ----
 * Blooming.apply (tina/postp/blooming.py:52-75): threshold filter, half-res
 * average, separable Gaussian (radius taps, weights of init_gwei :30-40),
 * bilinear add-back; workspace: t3_bloom_workspace_floats floats. */
int64_t t3_bloom_workspace_floats(int width, int height);
int t3_bloom(float* rgb, int width, int height, float thresh, float factor, float scale, float sigma,
             int radius, float* workspace, int64_t workspace_floats, void* stream);
/* FXAA.apply (tina/postp/fxaa.py:25-68); workspace: t3_fxaa_workspace_floats floats. */
int64_t t3_fxaa_workspace_floats(int width, int height);
int t3_fxaa(float* rgb, int width, int height, float abs_thresh, float rel_thresh, float factor,
            float* workspace, int64_t workspace_floats, void* stream);
/* Accumator.update (tina/util/accumator.py:16-23): acc = acc (1 - 1/count) + src / count. */
int t3_accumulate(float* acc, const float* src, int64_t n, int count, void* stream);

/* ---- batched multi-view rendering ------------------------------------------
 * No reference counterpart: the reference renders one Scene per call
 * (tina/scene/raster.py:168-207).  Up to T3_BATCH_MAX_SCENES independent
 * frames (each its own t3_scene: resolution <= 4096 x 4096, camera, objects,
 * lamps; lighting T3_LIGHT_LAMPS) are rendered by two launches over all of
 * them.  Direct: a persistent launch whose CTAs take (scene, object, face
 * chunk) raster items from a global work queue, then a persistent shading
 * launch over (scene, pixel chunk) items.  Binned: one launch bins every
 * scene's faces into its screen tiles, then a persistent launch takes
 * (scene, tile) items from a global queue and rasterises and shades each
 * tile in shared memory. */
#define T3_BATCH_MAX_SCENES 64

typedef struct t3_batch_config {
  int32_t faces_per_item;   /* direct: faces per raster item, multiple of 256 (0: 1024)    */
  int32_t pixels_per_item;  /* direct: pixels per shading item, multiple of 1024 (0: 4096) */
  int32_t ctas_per_sm;      /* cap on resident CTAs per SM, 1..8 (0: as many as fit)       */
  int32_t raster;           /* T3_RASTER_DIRECT (0) or T3_RASTER_BINNED                    */
  int32_t tile;             /* binned: tile edge 8, 16 or 32 (0: 16)                       */
  int32_t tile_threads;     /* binned: threads per tile CTA, 64 (tile 8 only), 128 or 256
                               (0: 64 for tile 8, else 256)                                */
  int64_t bin_capacity;     /* binned: entries per tile bin in every scene; 0: each scene's
                               automatic size (8 x faces / tiles + 64); -k: k times it    */
} t3_batch_config;

/* Workspace bytes of t3_render_batch for these scenes and this configuration
 * (NULL: the direct defaults). */
int t3_batch_workspace_size(const t3_scene* scenes, int nscenes, const t3_batch_config* config,
                            size_t* bytes);

/* Renders scenes[i] into outs[i] for i < nscenes (every output as t3_render).
 * A binned bin that overflows sets T3_STATUS_BIN_OVERFLOW in *status (its
 * faces are dropped): render again with a larger bin_capacity. */
int t3_render_batch(const t3_scene* scenes, const t3_outputs* outs, int nscenes,
                    const t3_batch_config* config, void* workspace, size_t workspace_bytes,
                    int32_t* status, void* stream);


/* ---- MLP-IBL (learned image-based lighting) -------------------------------
 * The network maps (normal, view direction, roughness, metallic) to log1p of
 * the albedo-independent IBL integrals of the Lambert and CookTorrance lobes
 * (E_d, S1, S2; RGB each) under the method's own Monte Carlo estimator; shading
 * composes them with the pixel's albedo and f0.  No counterpart in the
 * reference (its IBL is a prefiltered-map lookup, material.py:256-320). */
int64_t t3_mlp_param_count(void);   /* FP32 parameters: W1 b1 W2 b2 W3 b3 W4 b4 */
int64_t t3_mlp_packed_bytes(void);  /* bytes of the packed BF16 inference blob  */
/* E_d on an equirect grid of normals (map [map_w, map_h, 3]), spp cosine samples */
int t3_mlp_irradiance_map(const void* env, int env_w, int env_h, int env_half, int map_w, int map_h,
                          int spp, uint32_t seed, float* map, void* stream);
/* training targets [B, 9] = log1p(E_d from the map, S1, S2) at nv [B, 6] (n, v), rough [B] */
int t3_mlp_targets(const void* env, int env_w, int env_h, int env_half, const float* irr_map,
                   int map_w, int map_h, const float* nv, const float* rough, int64_t B, int spp,
                   uint32_t seed, float* targets, void* stream);
/* input features X [B, 400] of (n, v, roughness, metallic) */
int t3_mlp_encode(const float* nv, const float* rough, const float* metal, int64_t B, float* X,
                  void* stream);
/* forward: hidden activations acts [B, 192], outputs Y [B, 16] */
int t3_mlp_forward(const float* params, const float* X, int64_t B, float* acts, float* Y,
                   void* stream);
/* backward of the mean squared error over the 9 used outputs: grads (param
 * layout), dbuf workspace [B, 144], loss (device float, accumulated) */
int t3_mlp_backward(const float* params, const float* X, const float* acts, const float* Y,
                    const float* targets, int64_t B, float* grads, float* dbuf, float* loss,
                    void* stream);
/* one Adam step (bias-corrected) over n parameters */
int t3_mlp_adam(float* params, const float* grads, float* m, float* v, int64_t n, float lr,
                float beta1, float beta2, float eps, int step, void* stream);
/* BF16 inference blob (16-byte aligned, t3_mlp_packed_bytes) from FP32 params */
int t3_mlp_pack(const float* params, void* blob, void* stream);
/* inference on the tensor cores (tcgen05, FP32 accumulate): Y [B, 16] */
int t3_mlp_infer(const void* blob, const float* X, int64_t B, float* Y, int32_t* status, void* stream);
/* FP32 CUDA-core inference of the same network (reference path) */
int t3_mlp_infer_f32(const float* params, const float* X, int64_t B, float* Y, void* stream);

/* Skybox bake of SkyboxLighting's tables (tina/matr/material.py:279-316,
 * :407-438): out [out_w, out_h, 3] float, texel (i, j) = the environment
 * averaged about the direction of its equirect coordinate (i, j) / (shape - 1)
 * (Skybox.unmapcoor, tina/skybox.py:131-135) over `nsamples` directions
 * tangentspace(dir) @ spherical(h, xi) weighted by h, with
 * h = sqrt((1 - xi) / (1 - xi (1 - roughness^2))) (CookTorrance, roughness >= 0)
 * or h = xi (Lambert, roughness < 0); xi from the counter-based stream `seed`. */
int t3_ibl_bake(const void* env, int env_w, int env_h, int env_half, float roughness, int nsamples,
                uint32_t seed, float* out, int out_w, int out_h, void* stream);

/* Reads back the device status word written by the last t3_raster/t3_render
 * (synchronises `stream`). */
int t3_read_status(const int32_t* status, int32_t* host_status, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TINA3_H */
