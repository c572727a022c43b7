// api.cu -- the extern "C" entry points of libtina3.so (declared in include/tina3.h).
//
// Host-side responsibilities: argument checks, flattening each material tree
// into weighted lobes, the workspace layout, and the launch sequence of one
// frame (Scene.render, tina/scene/raster.py:168-207):
//   upload scene + zero counters -> clear keys -> per object: raster (+ big
//   faces) -> shade (+ tonemap).
// No entry point allocates device memory; every buffer is caller-owned.
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "t3_internal.cuh"

namespace t3 {

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

static int is_leaf(int op) {
  return op == T3_OP_LAMBERT || op == T3_OP_PHONG || op == T3_OP_COOK || op == T3_OP_EMISSION;
}
static int is_basic(int op) { return op == T3_OP_CONST || op == T3_OP_ATTR || op == T3_OP_INPUT; }
static int is_leaf_value(int op) { return is_basic(op) || op == T3_OP_TEXTURE || op == T3_OP_CHECKER; }
static int is_value(int op) { return is_leaf_value(op) || op == T3_OP_FRESNEL; }

// Walks the material tree from `node`, multiplying factors along the path.
static int flatten_rec(const t3_material& in, int node, int* fac, int nfac, DevMaterial& out,
                       int depth) {
  if (depth > T3_MAX_NODES) return T3_EINVAL;
  if (node < 0 || node >= in.nnodes) return T3_EINVAL;
  const t3_node& nd = in.nodes[node];
  if (is_leaf(nd.op)) {
    if (out.nlobes >= T3_MAX_LOBES || nfac > T3_MAX_FACTORS) return T3_EUNSUPPORTED;
    DevLobe& lb = out.lobes[out.nlobes++];
    std::memset(&lb, 0, sizeof(lb));
    lb.kind = nd.op;
    lb.nfac = nfac;
    for (int j = 0; j < nfac; j++) lb.fac[j] = fac[j];
    lb.p0 = nd.a;
    lb.p1 = nd.b;
    if (nd.op == T3_OP_PHONG) {
      if (nd.a < 0 || nd.a >= in.nnodes || !is_value(in.nodes[nd.a].op)) return T3_EINVAL;
      const t3_node& mn = in.nodes[nd.a];
      if (mn.op == T3_OP_CONST && mn.c == 1 && mn.v[0] >= 1.0f && mn.v[0] <= 65536.0f)
        lb.int_pow = (int)mn.v[0];
    }
    if (nd.op == T3_OP_COOK) {
      if (nd.a < 0 || nd.a >= in.nnodes || nd.b < 0 || nd.b >= in.nnodes) return T3_EINVAL;
      if (!is_value(in.nodes[nd.a].op) || !is_value(in.nodes[nd.b].op)) return T3_EINVAL;
    }
    return T3_OK;
  }
  int f2[T3_MAX_FACTORS + 2];
  for (int j = 0; j < nfac && j < T3_MAX_FACTORS; j++) f2[j] = fac[j];
  switch (nd.op) {
  case T3_OP_MIX: {
    if (nd.c < 0 || nd.c >= in.nnodes || !is_value(in.nodes[nd.c].op)) return T3_EINVAL;
    if (nfac + 1 > T3_MAX_FACTORS) return T3_EUNSUPPORTED;
    f2[nfac] = nd.c | T3_FAC_ONE_MINUS | T3_FAC_MIX;
    int r = flatten_rec(in, nd.a, f2, nfac + 1, out, depth + 1);
    if (r) return r;
    f2[nfac] = nd.c | T3_FAC_MIX;
    return flatten_rec(in, nd.b, f2, nfac + 1, out, depth + 1);
  }
  case T3_OP_SCALE: {
    if (nd.b < 0 || nd.b >= in.nnodes || !is_value(in.nodes[nd.b].op)) return T3_EINVAL;
    if (nfac + 1 > T3_MAX_FACTORS) return T3_EUNSUPPORTED;
    f2[nfac] = nd.b;
    return flatten_rec(in, nd.a, f2, nfac + 1, out, depth + 1);
  }
  case T3_OP_ADD: {
    int r = flatten_rec(in, nd.a, f2, nfac, out, depth + 1);
    if (r) return r;
    return flatten_rec(in, nd.b, f2, nfac, out, depth + 1);
  }
  default:
    return T3_EINVAL;
  }
}

int flatten_material(const t3_material& in, DevMaterial& out) {
  std::memset(&out, 0, sizeof(out));
  if (in.nnodes <= 0 || in.nnodes > T3_MAX_NODES) return T3_EINVAL;
  // value nodes may only reference earlier value nodes: FRESNEL over leaf
  // values (basic, texture, checker), textures and checkers over basic ones
  for (int i = 0; i < in.nnodes; i++) {
    const t3_node& nd = in.nodes[i];
    if (nd.op == T3_OP_FRESNEL) {
      const int refs[3] = {nd.a, nd.b, nd.c};
      for (int r : refs)
        if (r < 0 || r >= i || !is_leaf_value(in.nodes[r].op)) return T3_EINVAL;
    }
    if (nd.op == T3_OP_TEXTURE) {
      if (nd.a < 0 || nd.a >= i || !is_basic(in.nodes[nd.a].op)) return T3_EINVAL;
      if (nd.b < 0 || nd.b >= T3_MAX_TEXTURES) return T3_EINVAL;
      const t3_texture& t = in.textures[nd.b];
      if (!t.data || t.w < 1 || t.h < 1 || (t.channels != 1 && t.channels != 3)) return T3_EINVAL;
    }
    if (nd.op == T3_OP_CHECKER) {
      const int refs[4] = {nd.a, nd.b, nd.c, (int)nd.v[0]};
      for (int r : refs)
        if (r < 0 || r >= i || !is_basic(in.nodes[r].op)) return T3_EINVAL;
    }
    if (nd.op == T3_OP_ATTR && (nd.a < 0 || (nd.b != 1 && nd.b != 3))) return T3_EINVAL;
    if (nd.op == T3_OP_INPUT && (nd.a < 0 || nd.a > 3)) return T3_EINVAL;
  }
  out.nnodes = in.nnodes;
  for (int i = 0; i < in.nnodes; i++) out.nodes[i] = in.nodes[i];
  for (int t = 0; t < T3_MAX_TEXTURES; t++) out.textures[t] = in.textures[t];
  int fac[T3_MAX_FACTORS];
  return flatten_rec(in, in.root, fac, 0, out, 0);
}

static int check_mesh(const t3_mesh& m, int flags, int64_t nfaces) {
  if (nfaces < 0) return T3_EINVAL;
  if (nfaces == 0) return T3_OK;
  if (!m.verts) return T3_EINVAL;
  if (m.kind == T3_MESH_PARTICLES) return m.coors ? T3_OK : T3_EINVAL;  // positions, radii
  if (m.kind == T3_MESH_LINES) {
    // line soup: only MeshTransform / MeshToWire edits apply, one or two lines per entry
    if (m.flags & ~(T3_MESH_TRANSFORM | T3_MESH_WIREFRAME)) return T3_EINVAL;
    return nfaces <= m.nfaces * ((m.flags & T3_MESH_WIREFRAME) ? 2 : 1) ? T3_OK : T3_EINVAL;
  }
  if (m.flags & T3_MESH_QUADS) {
    // MeshGrid(as_quad=True): drawn only as MeshToWire's lines, under MeshTransform at most
    if (m.kind != T3_MESH_GRID || !(m.flags & T3_MESH_WIREFRAME)) return T3_EUNSUPPORTED;
    if (m.flags & ~(T3_MESH_QUADS | T3_MESH_TRANSFORM | T3_MESH_WIREFRAME)) return T3_EUNSUPPORTED;
  }
  if (m.flags & T3_MESH_WIREFRAME) {
    // MeshToWire: three lines per face of the (NOCULL-doubled) mesh, four per quad
    const int64_t per = (m.flags & T3_MESH_QUADS) ? 4 : 3;
    if (nfaces > m.nfaces * ((m.flags & T3_MESH_NOCULL) ? 2 : 1) * per) return T3_EINVAL;
    flags &= ~(T3_SMOOTHING | T3_TEXTURING);  // lines read positions only
  }
  if ((flags & T3_SMOOTHING) && !(m.flags & T3_MESH_FLAT_NORMAL) && !m.norms) return T3_EINVAL;
  if ((flags & T3_TEXTURING) && !m.coors) return T3_EINVAL;
  if (m.kind == T3_MESH_GRID) {
    if (m.grid_nx < 2 || m.grid_ny < 2) return T3_EINVAL;
  } else if (m.kind == T3_MESH_INDEXED) {
    if (!m.faces || m.face_stride <= 0 || m.corner_stride <= 0) return T3_EINVAL;
  } else if (m.kind != T3_MESH_SOUP) {
    return T3_EINVAL;
  }
  return T3_OK;
}

static int check_frame(const t3_frame& fr) {
  if (fr.width <= 0 || fr.height <= 0 || fr.width > 32768 || fr.height > 32768) return T3_EINVAL;
  if (fr.maxdepth <= 0) return T3_EINVAL;
  return T3_OK;
}

int make_dev_scene(const t3_scene& sc, DevScene& out, bool first_ids_free) {
  std::memset(&out, 0, sizeof(out));
  int r = check_frame(sc.frame);
  if (r) return r;
  if (sc.nobjects < 0 || sc.nobjects > T3_MAX_OBJECTS) return T3_ETOOBIG;
  if (sc.lighting.nlights < 0 || sc.lighting.nlights > T3_MAX_LIGHTS) return T3_ETOOBIG;
  if (sc.lighting.mode == T3_LIGHT_IBL_MC || sc.lighting.mode == T3_LIGHT_IBL_MLP) {
    if (!sc.lighting.env || sc.lighting.env_w < 2 || sc.lighting.env_h < 2) return T3_EINVAL;
    if (sc.lighting.mode == T3_LIGHT_IBL_MC && (sc.lighting.spp < 1 || sc.lighting.spp > (1 << 20)))
      return T3_EINVAL;
    if (sc.lighting.mode == T3_LIGHT_IBL_MLP &&
        (!sc.lighting.mlp || (reinterpret_cast<uintptr_t>(sc.lighting.mlp) & 15) != 0))
      return T3_EINVAL;
  } else if (sc.lighting.mode == T3_LIGHT_IBL_PREFILTERED) {
    const t3_ibl_tables* T = sc.lighting.tables;
    if (!sc.lighting.env || sc.lighting.env_w < 2 || sc.lighting.env_h < 2 || !T) return T3_EINVAL;
    for (int k = 0; k <= T3_IBL_LEVELS; k++) {
      const t3_ibl_map& m = k < T3_IBL_LEVELS ? T->spec[k] : T->diffuse;
      if (!m.data || m.w < 2 || m.h < 2 || (reinterpret_cast<uintptr_t>(m.data) & 3) != 0) return T3_EINVAL;
    }
    if (!T->lut || T->lut_w < 2 || T->lut_h < 2 || (reinterpret_cast<uintptr_t>(T->lut) & 7) != 0)
      return T3_EINVAL;
    out.tables = *T;
  } else if (sc.lighting.mode != T3_LIGHT_LAMPS) {
    return T3_EINVAL;
  }
  out.frame = sc.frame;
  out.lighting = sc.lighting;
  out.lighting.tables = nullptr;  // a host pointer: kernels read out.tables
  out.nobjects = sc.nobjects;
  int64_t total = 0;
  for (int o = 0; o < sc.nobjects; o++) {
    const t3_object& ob = sc.objects[o];
    r = check_mesh(ob.mesh, sc.frame.flags, ob.nfaces);
    if (r) return r;
    if (first_ids_free ? ob.face_base < total : ob.face_base != total) return T3_EINVAL;
    total = ob.face_base + ob.nfaces;
    if (total >= (int64_t)0xFFFFFFFFll) return T3_ETOOBIG;  // ids are uint32 in the key
    out.obj[o].mesh = ob.mesh;
    out.obj[o].face_base = ob.face_base;
    out.obj[o].nfaces = ob.nfaces;
    r = flatten_material(ob.material, out.obj[o].mat);
    if (r) return r;
    find_fast_material(out.obj[o].mat, out.obj[o].fast);
    if (sc.lighting.mode == T3_LIGHT_IBL_PREFILTERED) {
      // Phong has no prefiltered lookup (IMaterial.sample_ibl raises, material.py:39-40)
      for (int k = 0; k < out.obj[o].mat.nlobes; k++)
        if (out.obj[o].mat.lobes[k].kind == T3_OP_PHONG && !is_wire(ob.mesh)) return T3_EUNSUPPORTED;
    }
    if (sc.lighting.mode == T3_LIGHT_IBL_MLP) {
      // the network covers Lambert and one CookTorrance lobe (plus emission)
      int cook = 0;
      for (int k = 0; k < out.obj[o].mat.nlobes; k++) {
        const int kind = out.obj[o].mat.lobes[k].kind;
        if (kind == T3_OP_PHONG) return T3_EUNSUPPORTED;
        cook += kind == T3_OP_COOK;
      }
      if (cook > 1) return T3_EUNSUPPORTED;
    }
    // per-face attribute reads must stay inside the mesh's attribute rows
    for (int i = 0; i < ob.material.nnodes; i++) {
      const t3_node& nd = ob.material.nodes[i];
      if (nd.op != T3_OP_ATTR) continue;
      if (!ob.mesh.face_attr || nd.a + nd.b > ob.mesh.attr_stride) return T3_EINVAL;
    }
  }
  return T3_OK;
}

static bool plain_value(const DevMaterial& m, int i) {
  return i >= 0 && i < m.nnodes && is_basic(m.nodes[i].op);
}

void find_fast_material(const DevMaterial& m, FastMat& f) {
  std::memset(&f, 0, sizeof(f));
  const DevLobe& a = m.lobes[0];
  if (m.nlobes == 1 && a.kind == T3_OP_LAMBERT && a.nfac == 1 && !(a.fac[0] & ~0xFFFF) &&
      plain_value(m, a.fac[0])) {
    f.sig = T3_OP_LAMBERT;  // T3_SIG_DIFFUSE
    f.node[0] = a.fac[0];
    return;
  }
  if (m.nlobes != 2) return;
  const DevLobe& b = m.lobes[1];
  if (a.kind != T3_OP_LAMBERT || a.nfac != 2 || b.nfac != 1) return;
  const int mixf = a.fac[0], col = a.fac[1], mixg = b.fac[0];
  const int F = mixf & 0xFFFF;
  if (mixf != (F | T3_FAC_ONE_MINUS | T3_FAC_MIX) || mixg != (F | T3_FAC_MIX)) return;
  if ((col & ~0xFFFF) || !plain_value(m, col)) return;
  if (b.kind == T3_OP_COOK && F < m.nnodes && m.nodes[F].op == T3_OP_FRESNEL && b.p1 == F &&
      plain_value(m, b.p0)) {
    const t3_node& alb = m.nodes[m.nodes[F].b];
    if (std::memcmp(&alb, &m.nodes[col], sizeof(t3_node)) != 0) return;  // basecolor twice
    f.sig = T3_OP_LAMBERT | (T3_OP_COOK << 8);  // T3_SIG_PBR
    f.node[0] = col;
    f.node[1] = F;
    f.node[2] = b.p0;
  } else if (b.kind == T3_OP_PHONG && plain_value(m, F) && plain_value(m, b.p0)) {
    f.sig = T3_OP_LAMBERT | (T3_OP_PHONG << 8);  // T3_SIG_CLASSIC
    f.node[0] = col;
    f.node[1] = F;
    f.node[2] = b.p0;
    f.int_pow = b.int_pow;
  }
}

int max_lobes(const DevScene& sc) {
  int m = 1;
  for (int o = 0; o < sc.nobjects; o++) m = sc.obj[o].mat.nlobes > m ? sc.obj[o].mat.nlobes : m;
  return m;
}

int has_points_or_lines(const t3_scene& sc) {
  for (int o = 0; o < sc.nobjects && o < T3_MAX_OBJECTS; o++)
    if (is_point_or_line(sc.objects[o].mesh) && sc.objects[o].nfaces > 0) return 1;
  return 0;
}

int64_t mesh_vertex_rows(const t3_mesh& m) {
  if (m.kind == T3_MESH_GRID) return (int64_t)m.grid_nx * m.grid_ny;
  if (m.kind == T3_MESH_INDEXED) return m.nverts > 0 ? m.nverts : 0;
  return 0;
}

int has_textures(const DevScene& sc) {
  for (int o = 0; o < sc.nobjects; o++)
    for (int i = 0; i < sc.obj[o].mat.nnodes; i++)
      if (sc.obj[o].mat.nodes[i].op == T3_OP_TEXTURE || sc.obj[o].mat.nodes[i].op == T3_OP_CHECKER) return 1;
  return 0;
}

static int64_t max_object_faces(const t3_scene& sc) {
  int64_t m = 0;
  for (int o = 0; o < sc.nobjects && o < T3_MAX_OBJECTS; o++)
    if (sc.objects[o].nfaces > m) m = sc.objects[o].nfaces;
  return m;
}

int64_t total_faces(const t3_scene& sc) {
  int64_t t = 0;
  for (int o = 0; o < sc.nobjects && o < T3_MAX_OBJECTS; o++) t += sc.objects[o].nfaces;
  return t;
}

// Workspace layout of one frame (byte offsets, 256-aligned):
//   state     16 bytes kept between frames: the key tag and the clear's ticket
//             (KeyState; zero in a new workspace)
//   scene     DevScene (device copy of the descriptors)
//   counters  uint32[64 + ntiles]: per-object big-face counts, big-list count,
//             tile bin counts -- zeroed by the scene upload every frame
//   big       uint32[big_capacity] big-face ids
//   rec       float4[4 * total_faces] setup records of the visible faces
//   direct:   keys  uint64[W*H] packed (depth, id)
//   binned:   bins  uint32[ntiles * bin_capacity]
//   learned IBL: the network pass's rows, 96 bytes per pixel (their count is
//             counter kMlpRowCounter)
struct Layout {
  size_t scene, counters, big, keys, rec, bins, vtx, mlp, end;
  int ncounters;
  uint32_t big_capacity, bin_capacity;
  int tile, tiles_x, tiles_y;
};

constexpr size_t kStateBytes = 256;  // KeyState's tag (8 bytes) and ticket (4), padded
constexpr int kMlpRowCounter = 62;   // counters[0..T3_MAX_OBJECTS): big faces; [63]: binned big list

// The tag of a direct frame's key buffer: which workspace, layout and frame
// size the empty keys belong to (splitmix64 finaliser over the four values).
static unsigned long long key_tag(const void* ws, size_t keys_at, int64_t npix, size_t end) {
  unsigned long long h = 0x9E3779B97F4A7C15ull;
  const unsigned long long v[4] = {(unsigned long long)(uintptr_t)ws, (unsigned long long)keys_at,
                                   (unsigned long long)npix, (unsigned long long)end};
  for (unsigned long long x : v) {
    h ^= x + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    h ^= h >> 30;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 27;
    h *= 0x94D049BB133111EBull;
    h ^= h >> 31;
  }
  return h ? h : 1ull;
}

static MlpRows mlp_rows(uint8_t* ws, const Layout& L, uint32_t* counters) {
  MlpRows r;
  if (L.mlp) {
    r.rows = reinterpret_cast<float4*>(ws + L.mlp);
    r.count = counters + kMlpRowCounter;
  }
  return r;
}

static KeyState key_state(void* ws, unsigned long long tag) {
  KeyState ks;
  ks.tag_word = reinterpret_cast<unsigned long long*>(ws);
  ks.ticket = reinterpret_cast<uint32_t*>(reinterpret_cast<uint8_t*>(ws) + 8);
  ks.tag = tag;
  return ks;
}

// Host-side record of the workspaces whose last direct frame (issued by this
// process) ended with a shading pass that empties the keys, with that frame's
// tag.  It only picks the size of the next frame's clear; the clear itself
// checks the tag on the device, so a stale entry (a graph replayed out of
// order, a workspace freed and reused) costs time, never correctness.
struct KeyHint {
  const void* ws;
  unsigned long long tag;
};
static std::mutex g_hint_mu;
static KeyHint g_hints[32];
static int g_hint_next;

static bool hint_empty(const void* ws, unsigned long long tag) {
  std::lock_guard<std::mutex> lock(g_hint_mu);
  for (const KeyHint& h : g_hints)
    if (h.ws == ws) return h.tag == tag;
  return false;
}

// tag 0 forgets the workspace
static void hint_set(const void* ws, unsigned long long tag) {
  std::lock_guard<std::mutex> lock(g_hint_mu);
  for (KeyHint& h : g_hints) {
    if (h.ws == ws) {
      h.tag = tag;
      return;
    }
  }
  if (!tag) return;
  g_hints[g_hint_next] = KeyHint{ws, tag};
  g_hint_next = (g_hint_next + 1) % 32;
}

int64_t auto_bin_capacity(const t3_scene& sc, int tile) {
  const int64_t tx = (sc.frame.width + tile - 1) / tile, ty = (sc.frame.height + tile - 1) / tile;
  const int64_t per = 8 * total_faces(sc) / (tx * ty) + 64;
  int64_t cap = per < 64 ? 64 : per > (1 << 16) ? (1 << 16) : per;
  return (cap + 31) & ~(int64_t)31;
}

static int layout_for(const t3_scene& sc, int mode, int tile, int64_t bin_capacity, Layout& L) {
  std::memset(&L, 0, sizeof(L));
  L.scene = kStateBytes;
  L.counters = L.scene + align256(sizeof(DevScene));
  L.tile = tile;
  if (mode == T3_RASTER_BINNED) {
    if (tile != 8 && tile != 16 && tile != 32) return T3_EINVAL;
    L.tiles_x = (sc.frame.width + tile - 1) / tile;
    L.tiles_y = (sc.frame.height + tile - 1) / tile;
    int64_t cap = bin_capacity > 0 ? ((bin_capacity + 3) & ~(int64_t)3) : auto_bin_capacity(sc, tile);
    if (cap > (1 << 20)) return T3_ETOOBIG;
    L.bin_capacity = (uint32_t)cap;
    L.ncounters = 64 + L.tiles_x * L.tiles_y;
  } else if (mode == T3_RASTER_DIRECT) {
    L.ncounters = 64;
  } else {
    return T3_EINVAL;
  }
  int64_t cap = mode == T3_RASTER_BINNED ? total_faces(sc) : max_object_faces(sc);
  if (cap < 1) cap = 1;
  L.big_capacity = (uint32_t)cap;
  L.big = align256(L.counters + 4 * (size_t)L.ncounters);
  const size_t after_big = align256(L.big + 4 * (size_t)cap);
  L.rec = after_big;
  const size_t after_rec = align256(L.rec + 64 * (size_t)(total_faces(sc) > 0 ? total_faces(sc) : 1));
  if (mode == T3_RASTER_BINNED) {
    L.bins = after_rec;
    L.end = align256(L.bins + 4 * (size_t)L.tiles_x * L.tiles_y * L.bin_capacity);
    if (sc.lighting.mode == T3_LIGHT_IBL_MLP || has_points_or_lines(sc)) {
      // particle and line fragments seed the tiles' keys; the tiles hand their
      // keys to the fused network shading pass
      L.keys = L.end;
      L.end = align256(L.keys + 8 * (size_t)sc.frame.width * (size_t)sc.frame.height);
    }
  } else {
    L.keys = after_rec;
    L.end = align256(L.keys + 8 * (size_t)sc.frame.width * (size_t)sc.frame.height);
    // vertex stage outputs (float4 per vertex row) of every indexed / grid object
    L.vtx = L.end;
    size_t vtx = 0;
    for (int o = 0; o < sc.nobjects && o < T3_MAX_OBJECTS; o++)
      vtx += align256(16 * (size_t)mesh_vertex_rows(sc.objects[o].mesh));
    L.end += vtx;
  }
  if (sc.lighting.mode == T3_LIGHT_IBL_MLP) {
    L.mlp = L.end;
    L.end = align256(L.mlp + 96 * (size_t)sc.frame.width * (size_t)sc.frame.height);
  }
  return T3_OK;
}

static int cuda_rc(cudaError_t e) { return e == cudaSuccess ? T3_OK : T3_ECUDA; }

} // namespace t3

using namespace t3;

extern "C" {

int t3_version(void) { return 8; }

// sizeof of every ABI struct, for binding-layer layout checks.
int t3_struct_sizes(int64_t* out, int n) {
  const int64_t s[] = {(int64_t)sizeof(t3_frame),    (int64_t)sizeof(t3_mesh),
                       (int64_t)sizeof(t3_node),     (int64_t)sizeof(t3_material),
                       (int64_t)sizeof(t3_object),   (int64_t)sizeof(t3_light),
                       (int64_t)sizeof(t3_lighting), (int64_t)sizeof(t3_scene),
                       (int64_t)sizeof(t3_outputs)};
  const int k = (int)(sizeof(s) / sizeof(s[0]));
  if (!out) return k;
  for (int i = 0; i < n && i < k; i++) out[i] = s[i];
  return k;
}

int t3_workspace_size(const t3_scene* scene, int mode, int tile, int64_t bin_capacity,
                      size_t* bytes) {
  if (!scene || !bytes) return T3_EINVAL;
  int r = check_frame(scene->frame);
  if (r) return r;
  if (scene->nobjects < 0 || scene->nobjects > T3_MAX_OBJECTS) return T3_ETOOBIG;
  Layout L;
  r = layout_for(*scene, mode, tile, bin_capacity, L);
  if (r) return r;
  *bytes = L.end;
  return T3_OK;
}

int t3_bin_capacity(const t3_scene* scene, int tile, int64_t bin_capacity, int64_t* capacity) {
  if (!scene || !capacity) return T3_EINVAL;
  Layout L;
  int r = layout_for(*scene, T3_RASTER_BINNED, tile, bin_capacity, L);
  if (r) return r;
  *capacity = L.bin_capacity;
  return T3_OK;
}

int t3_clear(uint64_t* depth_id, int64_t npixels, void* stream) {
  if (!depth_id || npixels < 0) return T3_EINVAL;
  return cuda_rc(launch_clear(reinterpret_cast<unsigned long long*>(depth_id), npixels,
                              (cudaStream_t)stream));
}

int t3_raster(const t3_frame* frame, const t3_object* object, uint64_t* depth_id, void* workspace,
              size_t workspace_bytes, int32_t* status, void* stream) {
  if (!frame || !object || !depth_id || !workspace || !status) return T3_EINVAL;
  int r = check_frame(*frame);
  if (r) return r;
  r = check_mesh(object->mesh, frame->flags, object->nfaces);
  if (r) return r;
  // workspace: one counter + the big-face queue of this object
  const size_t need = 256 + sizeof(uint32_t) * (size_t)(object->nfaces > 0 ? object->nfaces : 1);
  if (workspace_bytes < need) return T3_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  if (is_point_or_line(object->mesh))  // ParticleRaster / WireframeRaster
    return cuda_rc(launch_raster_point_or_line(*frame, *object,
                                               reinterpret_cast<unsigned long long*>(depth_id), nullptr, st));
  uint8_t* ws = reinterpret_cast<uint8_t*>(workspace);
  BigQueue big;
  big.count = reinterpret_cast<uint32_t*>(ws);
  big.items = reinterpret_cast<uint32_t*>(ws + 256);
  big.capacity = (uint32_t)(object->nfaces > 0 ? object->nfaces : 1);
  big.status = status;
  big.rec = nullptr;
  cudaError_t e = cudaMemsetAsync(big.count, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return T3_ECUDA;
  return cuda_rc(launch_raster_direct(*frame, *object, reinterpret_cast<unsigned long long*>(depth_id),
                                      big, 128, st));
}

int t3_shade(const t3_scene* scene, const uint64_t* depth_id, void* workspace,
             size_t workspace_bytes, const t3_outputs* out, void* stream) {
  if (!scene || !depth_id || !out || !out->rgb || !workspace) return T3_EINVAL;
  if (workspace_bytes < kStateBytes + align256(sizeof(DevScene))) return T3_EINVAL;
  // the network pass reports timeouts through a status word: t3_render has one
  if (scene->lighting.mode == T3_LIGHT_IBL_MLP) return T3_EUNSUPPORTED;
  static thread_local DevScene ds;
  int r = make_dev_scene(*scene, ds, true);
  if (r) return r;
  // the shading kernel takes the scene by value; the workspace is not written
  return cuda_rc(launch_shade(ds, reinterpret_cast<DevScene*>(reinterpret_cast<uint8_t*>(workspace) + kStateBytes),
                              reinterpret_cast<const unsigned long long*>(depth_id), nullptr, *out, nullptr,
                              (cudaStream_t)stream));
}

int t3_render(const t3_scene* scene, int mode, int tile, int64_t bin_capacity, void* workspace,
              size_t workspace_bytes, int32_t* status, const t3_outputs* out, void* stream) {
  return t3_render_staged(scene, mode, tile, bin_capacity, workspace, workspace_bytes, status, out,
                          stream, nullptr);
}

int t3_render_staged(const t3_scene* scene, int mode, int tile, int64_t bin_capacity,
                     void* workspace, size_t workspace_bytes, int32_t* status,
                     const t3_outputs* out, void* stream, void* const* stage_events) {
  return t3_render_staged_n(scene, mode, tile, bin_capacity, workspace, workspace_bytes, status, out, stream,
                            stage_events, 4);
}

int t3_render_staged_n(const t3_scene* scene, int mode, int tile, int64_t bin_capacity,
                       void* workspace, size_t workspace_bytes, int32_t* status,
                       const t3_outputs* out, void* stream, void* const* stage_events, int nevents) {
  if (!scene || !workspace || !status || !out || !out->rgb) return T3_EINVAL;
  if (stage_events && nevents != 4 && nevents != 5) return T3_EINVAL;
  static thread_local DevScene ds;
  int r = make_dev_scene(*scene, ds);
  if (r) return r;
  Layout L;
  r = layout_for(*scene, mode, tile, bin_capacity, L);
  if (r) return r;
  if (workspace_bytes < L.end) return T3_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  uint8_t* ws = reinterpret_cast<uint8_t*>(workspace);
  uint32_t* counters = reinterpret_cast<uint32_t*>(ws + L.counters);
  DevScene* dsc = reinterpret_cast<DevScene*>(ws + L.scene);
  auto mark = [&](int k) -> cudaError_t {
    if (!stage_events || !stage_events[k]) return cudaSuccess;
    return cudaEventRecord((cudaEvent_t)stage_events[k], st);
  };
  // with five events: [3] between the learned-IBL shading's two kernels
  const int last = stage_events && nevents == 5 ? 4 : 3;
  auto rows_of = [&]() {
    MlpRows r = mlp_rows(ws, L, counters);
    if (last == 4) r.split = (cudaEvent_t)stage_events[3];
    return r;
  };
  cudaError_t e = mark(0);
  if (mode == T3_RASTER_DIRECT) {
    // the shading kernels take the scene by value: no device copy is needed,
    // and the clear also zeroes the counters and the status
    unsigned long long* keys = reinterpret_cast<unsigned long long*>(ws + L.keys);
    const int64_t npix = (int64_t)scene->frame.width * scene->frame.height;
    // the keys a previous frame's shading emptied are not cleared again; the
    // lamp and Monte Carlo shading passes empty them for the next frame
    KeyState ks = key_state(ws, key_tag(ws, L.keys, npix, L.end));
    ks.likely_empty = hint_empty(ws, ks.tag);
    hint_set(ws, 0ull);
    if (e == cudaSuccess) e = launch_clear(keys, npix, st, counters, L.ncounters, status, ks);
    if (e == cudaSuccess) e = mark(1);
    size_t vtx = L.vtx;
    for (int o = 0; o < scene->nobjects && e == cudaSuccess; o++) {
      BigQueue big;
      big.items = reinterpret_cast<uint32_t*>(ws + L.big);
      big.capacity = L.big_capacity;
      big.count = counters + o;
      big.status = status;
      big.rec = reinterpret_cast<float4*>(ws + L.rec);
      if (is_point_or_line(scene->objects[o].mesh)) {
        e = launch_raster_point_or_line(scene->frame, scene->objects[o], keys, nullptr, st);
        continue;
      }
      const int64_t nv = mesh_vertex_rows(scene->objects[o].mesh);
      if (nv > 0 && scene->objects[o].nfaces > 0) {
        float4* out = reinterpret_cast<float4*>(ws + vtx);
        e = launch_vertex_ndc(scene->frame, scene->objects[o].mesh, nv, out, st);
        big.vndc = out;
        vtx += align256(16 * (size_t)nv);
      }
      if (e == cudaSuccess) e = launch_raster_direct(scene->frame, scene->objects[o], keys, big, 4096, st);
    }
    if (e == cudaSuccess) e = mark(2);
    if (e == cudaSuccess)
      e = launch_shade(ds, dsc, keys, reinterpret_cast<const float4*>(ws + L.rec), *out, status, st, ks,
                       rows_of());
    // every shading pass of a direct frame returns the keys to empty
    if (e == cudaSuccess) hint_set(ws, ks.tag);
  } else {
    hint_set(ws, 0ull);
    if (e == cudaSuccess)
      e = launch_upload_scene(ds, dsc, counters, L.ncounters, status, st,
                              reinterpret_cast<unsigned long long*>(ws));
    BinArgs b;
    b.rec = reinterpret_cast<float4*>(ws + L.rec);
    b.bins = reinterpret_cast<uint32_t*>(ws + L.bins);
    b.count = counters + 64;
    b.big = reinterpret_cast<uint32_t*>(ws + L.big);
    b.big_count = counters + 63;
    b.status = status;
    b.capacity = L.bin_capacity;
    b.big_capacity = L.big_capacity;
    b.tile = L.tile;
    b.tiles_x = L.tiles_x;
    b.tiles_y = L.tiles_y;
    b.big_tiles = 16;
    b.max_lobes = max_lobes(ds);
    b.light_mode = ds.lighting.mode;
    b.keys = ds.lighting.mode == T3_LIGHT_IBL_MLP ? reinterpret_cast<unsigned long long*>(ws + L.keys)
                                                  : nullptr;
    b.pre = nullptr;
    if (e == cudaSuccess) e = mark(1);
    if (has_points_or_lines(*scene)) {
      // particles and lines take the direct rasterisers into the frame's keys,
      // which then seed the tiles (every fragment is an order-independent
      // minimum, so the result equals the direct path's)
      unsigned long long* gk = reinterpret_cast<unsigned long long*>(ws + L.keys);
      const int64_t npix = (int64_t)scene->frame.width * scene->frame.height;
      if (e == cudaSuccess) e = launch_clear(gk, npix, st, nullptr, 0, nullptr);
      for (int o = 0; o < scene->nobjects && e == cudaSuccess; o++)
        if (is_point_or_line(scene->objects[o].mesh))
          e = launch_raster_point_or_line(scene->frame, scene->objects[o], gk, nullptr, st);
      b.pre = gk;
    }
    for (int o = 0; o < scene->nobjects && e == cudaSuccess; o++)
      if (!is_point_or_line(scene->objects[o].mesh)) e = launch_bin(scene->frame, scene->objects[o], b, st);
    if (e == cudaSuccess) e = mark(2);
    if (e == cudaSuccess) e = launch_tile(dsc, b, L.tiles_x * L.tiles_y, *out, st);
    if (e == cudaSuccess && b.keys)
      e = launch_shade(ds, dsc, b.keys, b.rec, *out, status, st, KeyState(), rows_of());
  }
  if (e == cudaSuccess && last == 4 && !(ds.lighting.mode == T3_LIGHT_IBL_MLP && L.mlp)) e = mark(3);
  if (e == cudaSuccess) e = mark(last);
  return cuda_rc(e);
}

int t3_raster_fragments(const t3_scene* scene, void* workspace, size_t workspace_bytes, int64_t* fragments,
                        void* stream) {
  if (!scene || !workspace || !fragments) return T3_EINVAL;
  static thread_local DevScene ds;
  int r = make_dev_scene(*scene, ds);
  if (r) return r;
  Layout L;
  r = layout_for(*scene, T3_RASTER_DIRECT, 16, 0, L);
  if (r) return r;
  if (workspace_bytes < L.end) return T3_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  uint8_t* ws = reinterpret_cast<uint8_t*>(workspace);
  uint32_t* counters = reinterpret_cast<uint32_t*>(ws + L.counters);
  unsigned long long* count = reinterpret_cast<unsigned long long*>(counters + 62);  // 8-byte aligned
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(ws + L.keys);
  const int64_t npix = (int64_t)scene->frame.width * scene->frame.height;
  // a full clear (tag 0), which also marks the keys as not known to be empty
  hint_set(ws, 0ull);
  cudaError_t e = launch_clear(keys, npix, st, counters, L.ncounters, nullptr, key_state(ws, 0ull));
  for (int o = 0; o < scene->nobjects && e == cudaSuccess; o++) {
    BigQueue big;
    big.items = reinterpret_cast<uint32_t*>(ws + L.big);
    big.capacity = L.big_capacity;
    big.count = counters + o;
    big.status = reinterpret_cast<int32_t*>(counters + 61);
    big.rec = nullptr;
    big.fragments = count;
    if (is_point_or_line(scene->objects[o].mesh))
      e = launch_raster_point_or_line(scene->frame, scene->objects[o], keys, count, st);
    else
      e = launch_raster_direct(scene->frame, scene->objects[o], keys, big, 4096, st);
  }
  unsigned long long host = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&host, count, sizeof(host), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return T3_ECUDA;
  *fragments = (int64_t)host;
  return T3_OK;
}

int t3_red_min_rate(uint64_t* buf, int64_t n, int rounds, void* stream) {
  if (!buf || n <= 0 || rounds <= 0) return T3_EINVAL;
  return cuda_rc(launch_red_min_rate(reinterpret_cast<unsigned long long*>(buf), n, rounds,
                                     (cudaStream_t)stream));
}

int t3_bin_counts_max(const t3_scene* scene, int tile, int64_t bin_capacity, const void* workspace,
                      size_t workspace_bytes, int64_t* max_count, void* stream) {
  if (!scene || !workspace || !max_count) return T3_EINVAL;
  Layout L;
  int r = layout_for(*scene, T3_RASTER_BINNED, tile, bin_capacity, L);
  if (r) return r;
  if (workspace_bytes < L.end) return T3_EINVAL;
  const int ntiles = L.tiles_x * L.tiles_y;
  uint32_t* counts = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)ntiles);
  if (!counts) return T3_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  const uint8_t* ws = reinterpret_cast<const uint8_t*>(workspace);
  cudaError_t e = cudaMemcpyAsync(counts, ws + L.counters + 64 * sizeof(uint32_t),
                                  sizeof(uint32_t) * (size_t)ntiles, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  int64_t m = 0;
  for (int i = 0; i < ntiles && e == cudaSuccess; i++) m = counts[i] > m ? counts[i] : m;
  free(counts);
  if (e != cudaSuccess) return T3_ECUDA;
  *max_count = m;
  return T3_OK;
}

int t3_event_create(void** event) {
  if (!event) return T3_EINVAL;
  cudaEvent_t ev;
  if (cudaEventCreate(&ev) != cudaSuccess) return T3_ECUDA;
  *event = (void*)ev;
  return T3_OK;
}

int t3_event_destroy(void* event) {
  if (!event) return T3_EINVAL;
  return cuda_rc(cudaEventDestroy((cudaEvent_t)event));
}

int t3_event_elapsed_ms(void* start, void* end, float* ms) {
  if (!start || !end || !ms) return T3_EINVAL;
  if (cudaEventSynchronize((cudaEvent_t)end) != cudaSuccess) return T3_ECUDA;
  return cuda_rc(cudaEventElapsedTime(ms, (cudaEvent_t)start, (cudaEvent_t)end));
}

int t3_read_status(const int32_t* status, int32_t* host_status, void* stream) {
  if (!status || !host_status) return T3_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(host_status, status, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return cuda_rc(e);
}

} // extern "C"
