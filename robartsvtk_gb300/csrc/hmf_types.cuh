// hmf_types.cuh -- plain data types and launch constants shared by the
// kernels (hmf_kernels.cuh, hmf_flow_tma.cuh, hmf_tree_bulk.cuh) and the host
// code of the solver context.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace hmf {

constexpr int kMaxVertices = 64;

// Per non-root vertex, one iteration parity (flows ping-pong between two sets
// because a CTA reads flows of its neighbours' tiles).
struct FlowVertex {
  const float* px_in;
  const float* py_in;
  const float* pz_in;
  float* px_out;
  float* py_out;
  float* pz_out;
  const float* sink;    // own sink flow, previous iteration
  const float* inc;     // parent's sink (or the source flow), previous iteration
  const float* label;   // own label, previous iteration
  const float* smooth;  // per-voxel smoothness or nullptr (S == 1)
  float* div;           // out: divergence of the projected flows
  float alpha;
  int pad_;
};

struct Geometry {
  int vx, vy, vz;
  int pitch;        // floats per row (vx rounded up to a multiple of 4)
  long long plane;  // pitch * vy
  long long vol;    // plane * vz (elements per array, padding included)
};

struct FlowParams {
  float step;  // StepSize
  float icc;   // 1.0f / CC, computed in float as the reference host does
  int zchunk;  // planes per CTA
  int tiles_x;
};

// Post-order tree table for the per-voxel sweep; entries 0..n-1, root last.
struct TreeEntry {
  float* sink;          // sink flow (root: source flow), read
  float* label;         // nullptr for the root, read
  float* sink_out;      // where the sweep writes the new sink (== sink in a solve)
  float* label_out;     // where it writes the new label (== label in a solve)
  const float* div;     // nullptr for the root
  const float* data;    // leaves: data term (capacity)
  int parent;           // entry index of the parent, -1 for the root
  int first_kid;        // into TreeTable::kids
  int n_kids;
  float inv_kids;       // 1.0f / (kids + 1) for branches, 1.0f / kids for the root
};

// Directed acyclic graphs (hmf_create_dag; kernels in hmf_dag.cuh): nodes as
// entries in the rooted DAG's forward-iterator order, the root at entry 0.
constexpr int kMaxDagEdges = 256;

struct DagEntry {
  float* sink;        // the root: its source flow
  float* inc;         // own source buffer (nullptr for the root)
  float* label;       // nullptr for the root
  const float* div;   // nullptr for the root
  const float* data;  // leaves: data term
  float k;            // branches: 1 / (weighted children + 1)
  int leaf;
  int first_in, n_in;    // in-edges (parents) in edge order
  int first_out, n_out;  // out-edges (children) in edge order
};

struct DagTable {
  int n;  // entries (the root included)
  int n_leaves;
  float cc, icc, shift;  // shift = 1 / (CC * the root's weighted children)
  int leaves[kMaxVertices];  // entry indices, forward order
  int in_parent[kMaxDagEdges];
  float in_wup[kMaxDagEdges], in_wdown[kMaxDagEdges];
  int out_child[kMaxDagEdges];
  float out_w[kMaxDagEdges];
  DagEntry e[kMaxVertices];
};

// The graph of dag_bulk_n_kernel<N> (N <= 8 entries, no repeated edge), in
// kernel parameters: entry e's staged arrays, its parents as a bit mask with
// per-pair weights, and its parents in in-edge order for the push-down sum.
constexpr int kDagRegMax = 8;
struct DagRegParams {
  float* sink[kDagRegMax];  // entry 0: the root's source
  float* inc[kDagRegMax];
  float* label[kDagRegMax];
  const float* div[kDagRegMax];
  const float* data[kDagRegMax];
  float k[kDagRegMax];                    // branch reset weights
  float wup[kDagRegMax][kDagRegMax];      // [child][parent] push-up weight
  float wdown_ord[kDagRegMax][kDagRegMax];  // [child][j] push-down weight of its j-th in-edge
  int parent_ord[kDagRegMax][kDagRegMax];   // [child][j] parent entry of its j-th in-edge
  int n_in[kDagRegMax];
  unsigned pmask[kDagRegMax];  // bit p: entry p is a parent
  unsigned leaf_mask;
  float cc, icc, shift;
};

struct TreeTable {
  int n;
  int n_leaves;
  float cc;
  float icc;
  float root_init;  // 1.0f / CC
  int kids[kMaxVertices];
  int leaves[kMaxVertices];  // entry indices of the leaves in DFS pre-order
  TreeEntry e[kMaxVertices];
};

constexpr int kTmaBoxX = 36;   // box width: 16-byte aligned start plus 32 lanes plus 1
constexpr int kTmaRows = 32;   // window rows
constexpr int kTmaPlane = kTmaBoxX * kTmaRows;        // floats per staged array plane
// Two rings.  The z flow of plane k+1 is needed one step early (the divergence
// of plane k), everything else only in its own step, so the main ring (px, py,
// sink, label, parent sink, smoothness) has 3 slots and the pz ring 4.  Plane
// k + kTmaMainLead (main ring) and pz of plane k + 1 + kTmaPzLead are issued
// in step k, after its first CTA barrier, kTmaMainLead / kTmaPzLead steps
// before their first use.  The leads may rise to the slot counts (main) and
// the slot count less one (pz); on a GB300 at 256^3 a lead of 3 on both rings
// measured 0.9 % slower per iteration than 2, and 3 on either ring alone
// within 0.2 %, so both stay at 2.
constexpr int kTmaMainArrays = 6;
constexpr int kTmaMainSlots = 3;
constexpr int kTmaPzSlots = 4;
constexpr int kTmaMainLead = 2;
constexpr int kTmaPzLead = 2;
static_assert(kTmaMainLead >= 1 && kTmaMainLead <= kTmaMainSlots, "main-ring lead");
static_assert(kTmaPzLead >= 1 && kTmaPzLead <= kTmaPzSlots - 1, "pz-ring lead");
constexpr int kTmaMaxOutX = 28;
constexpr int kTmaMaxOutY = 27;
constexpr int kTmaThreads = 256;
constexpr int kTmaSmemBytes =
                              (kTmaMainSlots * kTmaMainArrays + kTmaPzSlots) * kTmaPlane * 4 +
                              (3 * 256 + 2 * 256) * 4 + 64;

// Shape of flow_tma_kernel<W>: W warps of 4 register rows, a window of 32
// columns x 4W rows (the TMA box is kTmaBoxX x 4W), 28 x (4W - 5) outputs.
// W = 8: two CTAs per SM (~108 KB of shared memory each); W = 16: one CTA of
// 16 warps per SM (~208 KB), half the halo rows per output.
template <int W>
struct FlowTmaShape {
  static constexpr int kRows = 4 * W;
  static constexpr int kThreads = 32 * W;
  static constexpr int kPlane = kTmaBoxX * kRows;
  static constexpr int kMaxOutY = kRows - 5;
  static constexpr int kCtasPerSm = W <= 8 ? 2 : 1;
  static constexpr int kSmemBytes = (kTmaMainSlots * kTmaMainArrays + kTmaPzSlots) * kPlane * 4 + 5 * kThreads * 4 + 64;
};
static_assert(FlowTmaShape<8>::kSmemBytes == kTmaSmemBytes, "the 32-row shape keeps its layout");
static_assert(FlowTmaShape<16>::kSmemBytes <= 227 * 1024, "the 64-row shape fits one SM's shared memory");

struct FlowVertexTMA {  // 64-byte aligned through its CUtensorMap members
  CUtensorMap flow_in[2][3];  // [parity][axis]: flows read in iterations of that parity
  CUtensorMap sink, label, inc, smooth;
  float* flow_out[2][3];      // [parity][axis]: flows written in iterations of that parity
  float* div;
  float alpha;
  int has_smooth;
};

// One volume of a solve (a batch holds several of different sizes).
struct FlowVolume {
  Geometry G;
  int tiles_x;  // windows across x
  int out_x;    // output columns per window (<= 28)
  int out_y;    // output rows per window (<= 27)
  int zchunk;   // planes per window column
};

// One CTA's work: a window column (tile, z chunk) of one volume; the vertex is
// blockIdx.x % n_vertices.
struct FlowItem {
  int vol;
  int tile;
  int zc;
  int pad_;
};

struct FlowTmaParams {
  float step;
  float icc;
  int parity;
  int n_vertices;     // non-root vertices: units = n_vertices * n_items
  int n_items;        // work items of this launch (from `items`)
  int units_per_cta;  // grid.x = ceil(units / units_per_cta)
  const FlowVolume* vols;
  const FlowItem* items;
  int* error_flag;
  unsigned long long wait_limit_ns;  // bound of every copy wait (kTmaWaitLimitNs unless a caller sets it)
};

// Compile-time flag passed to generic lambdas (kernel specialisations).
template <bool B>
struct BoolTag {
  static constexpr bool value = B;
};

// Default bound of every mbarrier wait of the copy pipelines; a wait that
// runs out sets the error flag instead of hanging.  The flow kernels take
// their bound as a parameter (hmf_set_wait_limit); the drain after a
// time-out always uses this one.
constexpr uint64_t kTmaWaitLimitNs = 500000000ull;  // 0.5 s: far beyond any healthy copy

}  // namespace hmf
