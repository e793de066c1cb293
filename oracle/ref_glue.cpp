// ref_glue.cpp - runs the reference's own shader functions on the CPU.
//
// TEST INFRASTRUCTURE ONLY: compiled by oracle/ref_shaders.py into
// oracle/_ref/libref_shaders.so, once per (stage, variant), around the
// transformed text of one shader of the reference checkout
// (vulkan/radixsort-vulkan/shader/*.comp, included as REF_SHADER_FILE).  The
// shader's function bodies are compiled as written; this file supplies
//   * a shim with the GLSL names they use (uint, vec3/vec4, findMSB, min/max,
//     gl_GlobalInvocationID / gl_WorkGroupSize / gl_NumWorkGroups), and
//   * one extern "C" entry per variant that points the shader's buffer
//     globals at the caller's arrays, sets its uniforms, and runs main() as a
//     single invocation with a stride of 1 (every grid-stride loop then visits
//     its indices in order; a racy write keeps the last writer in index
//     order), plus the host steps of main.rs:60-170 the stage needs.
// Nothing here restates the shader arithmetic: that is the point of the pin.

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

namespace {

// ---- GLSL shim -----------------------------------------------------------
typedef uint32_t uint;
struct GlUvec3 {
  uint x, y, z;
};
GlUvec3 gl_GlobalInvocationID{0, 0, 0};
GlUvec3 gl_WorkGroupSize{1, 1, 1};
GlUvec3 gl_NumWorkGroups{1, 1, 1};

struct vec3 {
  float v[3];
  float& operator[](int i) { return v[i]; }
};
struct vec4 {
  float v[4];
  float& operator[](int i) { return v[i]; }
};

// GLSL findMSB: index of the highest set bit, -1 for 0; for a negative int,
// the highest clear bit.
inline int findMSB(uint32_t x) { return x == 0 ? -1 : 31 - __builtin_clz(x); }
inline int findMSB(int32_t x) { return findMSB(x < 0 ? ~static_cast<uint32_t>(x) : static_cast<uint32_t>(x)); }
inline int findMSB(uint64_t x) { return x == 0 ? -1 : 63 - __builtin_clzll(x); }
using std::max;
using std::min;

// Always-zero high bits of a code in its word (2 for 30-bit codes in 32 bits,
// 1 for 63-bit codes in 64), used by the D2 patches.
int ref_unused_bits = 2;

// Every third bit of a 63-bit code, for the 64-bit extension of octree.comp's
// corner decode (the reference has 32-bit codes only).  A plain bit loop.
inline float ref_third_bits64(int64_t m) {
  const uint64_t v = static_cast<uint64_t>(m);
  uint32_t q = 0;
  for (int k = 0; k < 21; ++k) q |= static_cast<uint32_t>((v >> (3 * k)) & 1u) << k;
  return static_cast<float>(q);
}

// Octree depth of a prefix length under the variant's rule.
#ifdef REF_PATCH_D2
#define REF_DEPTH(p) ((int(p) - ref_unused_bits) / 3)
#else
#define REF_DEPTH(p) (int(p) / 3)
#endif
// First (bottom) octree slot of radix node k under the D3 patch.
#define REF_BASE(k) ((k) == 0 ? 0 : int(node_offsets[k]) - int(rt_node_counts[k]) + 1)

#define main ref_shader_main
#include REF_SHADER_FILE
#undef main

}  // namespace

#ifdef REF_PATCH_W64
typedef uint64_t RefKey;
static constexpr int kCodeBits = 63;
#else
typedef uint32_t RefKey;
static constexpr int kCodeBits = 30;
#endif

// ---- morton.comp: k_ComputeMortonCode over pts float[n][4] ----------------
#ifdef REF_STAGE_MORTON
extern "C" void REF_SYM(const float* pts, uint32_t n_pts, float mn, float rg, uint32_t* keys) {
  data = (decltype(data))pts;
  morton_keys = keys;
  n = n_pts;
  min_coord = mn;
  range = rg;
  ref_shader_main();
}
#endif

// ---- unique.comp: k_CountUnique in place; returns n_unique ----------------
#ifdef REF_STAGE_UNIQUE
extern "C" uint32_t REF_SYM(RefKey* k, uint32_t n_keys) {
  keys = (decltype(keys))k;
  n = n_keys;
  n_unique = 0;
  ref_shader_main();
  return n_unique;
}
#endif

// ---- build_radix_tree.comp over m nodes (codes has m + 1 entries) ---------
// The host zero-initialises every tree buffer (main.rs:97-104), so parent[0]
// stays 0.  has_leaf_* are `bool` buffers in this shader; returned as u8.
// With the unpatched direction (D1) a node can scatter its parent link to
// parent[m], one past the end of the buffer: the shader runs over zeroed
// copies with spare room, and the first m entries are returned.
#ifdef REF_STAGE_TREE
extern "C" void REF_SYM(const RefKey* c, int32_t m, uint8_t* prefix, uint8_t* hll, uint8_t* hlr, int32_t* left,
                        int32_t* par) {
  if (m <= 0) return;
  const size_t cap = (size_t)m + 64;
  std::vector<uint8_t> p(cap, 0);
  std::vector<int32_t> lc(cap, 0), pa(cap, 0);
  std::unique_ptr<bool[]> l(new bool[cap]()), r(new bool[cap]());
  codes = (decltype(codes))c;
  n = m;
  prefix_n = p.data();
  has_leaf_left = l.get();
  has_leaf_right = r.get();
  left_child = (decltype(left_child))lc.data();
  parent = (decltype(parent))pa.data();
  ref_shader_main();
  for (int32_t i = 0; i < m; ++i) {
    prefix[i] = p[i];
    hll[i] = l[i] ? 1 : 0;
    hlr[i] = r[i] ? 1 : 0;
    left[i] = lc[i];
    par[i] = pa[i];
  }
}
#endif

// ---- edge_count.comp: countEdges over n_brt_nodes nodes -------------------
#ifdef REF_STAGE_EDGE
extern "C" void REF_SYM(const uint8_t* prefix, const int32_t* par, uint32_t* edge, uint32_t m, int unused_bits) {
  prefix_n = (decltype(prefix_n))prefix;
  parent = (decltype(parent))par;
  edge_count = edge;
  n_brt_nodes = m;
  ref_unused_bits = unused_bits;
  ref_shader_main();
}
#endif

// ---- partial_sum.comp: k_PartialSum of data[first, last) ------------------
#ifdef REF_STAGE_PSUM
extern "C" void REF_SYM(const int32_t* in, uint32_t first_, uint32_t last_, int32_t* out) {
  data = (decltype(data))in;
  d_first = (decltype(d_first))out;
  first = first_;
  last = last_;
  ref_shader_main();
}
#endif

// ---- octree.comp: root setup (main.rs:140-153), make, then link -----------
// out: 64-byte std430 nodes (children, corner, cell_size, masks, pad), n_out
// of them.  The shader writes into a zeroed array of OctNode::new() values
// (octree.rs:45-55) with 64 spare nodes past n_out, as a literal D3 layout
// can write past the last slot.
#ifdef REF_STAGE_OCTREE
struct RefOctOut {
  int32_t children[8];
  float corner[4];
  float cell_size;
  int32_t child_node_mask;
  int32_t child_leaf_mask;
  int32_t pad;
};
static_assert(sizeof(RefOctOut) == 64, "std430 node stride");

extern "C" void REF_SYM(RefOctOut* out, uint32_t n_out, const uint32_t* offsets, const uint32_t* counts,
                        const RefKey* c, const uint8_t* prefix, const int32_t* parents, const int32_t* left,
                        const uint8_t* hll, const uint8_t* hlr, float mn, float rg, int32_t m, int unused_bits) {
  std::vector<OctNode> nodes((size_t)n_out + 64);
  std::memset(nodes.data(), 0, nodes.size() * sizeof(OctNode));
  oct_nodes = nodes.data();
  node_offsets = (decltype(node_offsets))offsets;
  rt_node_counts = (decltype(rt_node_counts))counts;
  codes = (decltype(codes))c;
  rt_prefixN = (decltype(rt_prefixN))prefix;
  rt_parents = (decltype(rt_parents))parents;
  rt_leftChild = (decltype(rt_leftChild))left;
  rt_hasLeafLeft = (decltype(rt_hasLeafLeft))hll;
  rt_hasLeafRight = (decltype(rt_hasLeafRight))hlr;
  min_coord = mn;
  range = rg;
  n_brt_nodes = m;
  ref_unused_bits = unused_bits;
  // main.rs:142-151: root level and prefix from the first code, corner decoded
  // by the shader's own morton32_to_xyz, cell = range.
  const int root_level = (m > 0) ? REF_DEPTH(prefix[0]) : 0;
  const RefKey root_prefix = c[0] >> (kCodeBits - 3 * root_level);
  morton32_to_xyz(nodes[0].corner, root_prefix << (kCodeBits - 3 * root_level), mn, rg);
  nodes[0].cell_size = rg;
  ref_shader_main();  // k_MakeOctNodes for every radix node
#ifdef REF_RUN_LINK
  // D8: the link pass, commented out of main(), runs after make completes.
  for (int i = 0; i < m; ++i) k_LinkLeafNodes(i);
#endif
  for (uint32_t s = 0; s < n_out; ++s) {
    RefOctOut& o = out[s];
    const OctNode& nd = nodes[s];
    std::memcpy(o.children, nd.children, sizeof(o.children));
    std::memcpy(o.corner, nd.corner.v, sizeof(o.corner));
    o.cell_size = nd.cell_size;
    o.child_node_mask = nd.child_node_mask;
    o.child_leaf_mask = nd.child_leaf_mask;
    o.pad = 0;
  }
}
#endif
