// hmf_capi.cu -- the C ABI of include/hmf.h: solver context, device memory
// plan, input staging and the launch sequence of one solve.
//
// Reference counterparts:
//  - buffer plan      vtkHierarchicalMaxFlowSegmentation.cxx:711-905 (host) and
//                     vtkCudaHierarchicalMaxFlowSegmentation.cxx:513-538 (device)
//  - initialisation   vtkCudaHierarchicalMaxFlowSegmentation.cxx:478-667
//  - iteration loop   vtkCudaHierarchicalMaxFlowSegmentation.cxx:669-716
// The reference pages buffers between host and device when the GPU is short
// of memory; here the whole state is resident (it fits in HBM for every
// workload this library targets) and allocated once per context.
//
// A context holds one or more volumes (a batch) of possibly different sizes
// that share one label tree and one set of parameters.  Every per-vertex array
// is one allocation holding the volumes back to back, each volume a pitched
// block; the per-voxel kernels (initialisation, tree sweep) run once over the
// whole concatenation and the flow kernel over a table of (volume, window)
// work items, so a batch costs the same two launches per iteration as a
// single volume.
//
// A context made by hmf_create_dag solves the directed-acyclic-graph problem
// of vtkCudaDirectedAcyclicGraphMaxFlowSegmentation instead: the same flow
// kernel (each node's "inc" is its own source buffer), then dag_sweep_kernel
// (hmf_dag.cuh) per iteration.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/hmf.h"
#include "hmf_ctx.hpp"
#include "hmf_dag.cuh"
#include "hmf_flow_tma.cuh"
#include "hmf_kernels.cuh"
#include "hmf_tree_bulk.cuh"

namespace {

thread_local std::string g_create_error;

// Largest extent along one axis: row pitches (rounded up to 4 floats) and the
// kernels' per-axis coordinates stay within int.
constexpr int kMaxDim = 1 << 30;

constexpr int kTX = 32, kTY = 8;
constexpr int kPipelineIterations = 32;  // iterations per replayed graph of a pipelined solve (even)
constexpr int kTuneIterations = 8;      // iterations of each solve the autotuner times
constexpr int kMaxFlowUnits = 64;       // units (window-vertex marches) one flow CTA may take
constexpr int kTreeThreads = 256;

}  // namespace

namespace hmfi {

int fail(hmf_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  else g_create_error = msg;
  return code;
}

int cuda_fail(hmf_ctx* c, cudaError_t e, const char* what) {
  return fail(c, e == cudaErrorMemoryAllocation ? HMF_ERR_OUT_OF_MEMORY : HMF_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

std::string device_pointer_problem(const void* p) {
  if (!p) return "";
  cudaPointerAttributes a{};
  const cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return std::string("not a CUDA address (") + cudaGetErrorString(e) + ")";
  }
  if (a.type == cudaMemoryTypeManaged) return "";
  if (a.type != cudaMemoryTypeDevice) return "host memory passed as device memory (HMF_DEVICE)";
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return "no current CUDA device";
  if (a.device != dev)
    return "memory of CUDA device " + std::to_string(a.device) + ", but the call runs on device " +
           std::to_string(dev);
  return "";
}

int check_device_pointer(hmf_ctx* c, const void* p, const char* what) {
  const std::string why = device_pointer_problem(p);
  return why.empty() ? HMF_OK : fail(c, HMF_ERR_INVALID_ARGUMENT, std::string(what) + ": " + why);
}

int build_tree(hmf_ctx* c, const int* par, int n) {
  if (!par) return fail(c, HMF_ERR_TREE, "tree parent array is NULL");
  if (n < 2) return fail(c, HMF_ERR_TREE, "the tree needs a root and at least one leaf");
  if (n > hmf::kMaxVertices)
    return fail(c, HMF_ERR_TREE, "trees of more than " + std::to_string(hmf::kMaxVertices) +
                                     " vertices are not supported");
  c->n = n;
  c->parent.assign(par, par + n);
  c->kids.assign(n, {});
  c->root = -1;
  for (int v = 0; v < n; ++v) {
    const int p = par[v];
    if (p < 0) {
      if (c->root >= 0) return fail(c, HMF_ERR_TREE, "the tree has more than one root");
      c->root = v;
    } else if (p >= n || p == v) {
      return fail(c, HMF_ERR_TREE, "tree parent id out of range");
    } else {
      c->kids[p].push_back(v);
    }
  }
  if (c->root < 0) return fail(c, HMF_ERR_TREE, "the tree has no root");
  std::vector<char> seen(n, 0);
  std::vector<int> stack{c->root};
  while (!stack.empty()) {
    const int v = stack.back();
    stack.pop_back();
    if (seen[v]) return fail(c, HMF_ERR_TREE, "the tree has a cycle");
    seen[v] = 1;
    c->preorder.push_back(v);
    for (int k = (int)c->kids[v].size() - 1; k >= 0; --k) stack.push_back(c->kids[v][k]);
  }
  if ((int)c->preorder.size() != n) return fail(c, HMF_ERR_TREE, "the tree is not connected");
  for (int v : c->preorder)
    if (c->kids[v].empty()) c->leaves.push_back(v);
  // post-order: children (in order) before their parent
  std::vector<std::pair<int, int>> st{{c->root, 0}};
  while (!st.empty()) {
    auto& top = st.back();
    if (top.second < (int)c->kids[top.first].size()) {
      const int kid = c->kids[top.first][top.second++];
      st.push_back({kid, 0});
    } else {
      c->postorder.push_back(top.first);
      st.pop_back();
    }
  }
  return HMF_OK;
}

// A rooted DAG (vtkRootedDirectedAcyclicGraph.cxx:145-243): one vertex
// without parents, every vertex reachable, no cycle.  Levels are longest
// paths from the root; the forward order visits them level by level, a child
// entered from a parent one level up, children in edge order
// (vtkRootedDirectedAcyclicGraphForwardIterator.cxx:95-120).  Parent and child
// counts are weighted as vtkDirectedAcyclicGraphMaxFlowSegmentation.cxx:928-995
// computes them.
int build_dag(hmf_ctx* c, int n, int n_edges, const int* ep, const int* ec, const float* ew) {
  if (!ep || !ec) return fail(c, HMF_ERR_TREE, "edge arrays are NULL");
  if (n < 2 || n_edges < 1) return fail(c, HMF_ERR_TREE, "the graph needs a root, a leaf and an edge");
  if (n > hmf::kMaxVertices)
    return fail(c, HMF_ERR_TREE, "graphs of more than " + std::to_string(hmf::kMaxVertices) +
                                     " vertices are not supported");
  if (n_edges > hmf::kMaxDagEdges)
    return fail(c, HMF_ERR_TREE, "graphs of more than " + std::to_string(hmf::kMaxDagEdges) +
                                     " edges are not supported");
  c->dag = true;
  c->n = n;
  c->e_parent.assign(ep, ep + n_edges);
  c->e_child.assign(ec, ec + n_edges);
  c->e_weighted = ew != nullptr;
  c->e_weight.assign(n_edges, 1.0f);
  if (ew) c->e_weight.assign(ew, ew + n_edges);
  c->in_e.assign(n, {});
  c->out_e.assign(n, {});
  for (int e = 0; e < n_edges; ++e) {
    if (ep[e] < 0 || ep[e] >= n || ec[e] < 0 || ec[e] >= n || ep[e] == ec[e])
      return fail(c, HMF_ERR_TREE, "edge vertex out of range");
    if (ew && !(ew[e] > 0.0f && ew[e] < INFINITY)) return fail(c, HMF_ERR_TREE, "edge weights must be positive");
    c->out_e[ep[e]].push_back(e);
    c->in_e[ec[e]].push_back(e);
  }
  c->root = -1;
  for (int v = 0; v < n; ++v)
    if (c->in_e[v].empty()) {
      if (c->root >= 0) return fail(c, HMF_ERR_TREE, "the graph has more than one root");
      c->root = v;
    }
  if (c->root < 0) return fail(c, HMF_ERR_TREE, "the graph has no root");
  std::vector<int> indeg(n), topo{c->root}, level(n, 0);
  for (int v = 0; v < n; ++v) indeg[v] = (int)c->in_e[v].size();
  for (size_t i = 0; i < topo.size(); ++i)
    for (int e : c->out_e[topo[i]]) {
      const int k = ec[e];
      level[k] = std::max(level[k], level[topo[i]] + 1);
      if (--indeg[k] == 0) topo.push_back(k);
    }
  if ((int)topo.size() != n) return fail(c, HMF_ERR_TREE, "the graph has a cycle or an unreachable vertex");
  std::vector<char> seen(n, 0);
  c->preorder.assign(1, c->root);
  seen[c->root] = 1;
  for (size_t i = 0; i < c->preorder.size(); ++i) {
    const int v = c->preorder[i];
    for (int e : c->out_e[v]) {
      const int k = ec[e];
      if (level[k] != level[v] + 1 || seen[k]) continue;
      seen[k] = 1;
      c->preorder.push_back(k);
    }
  }
  c->kids.assign(n, {});
  c->parent.assign(n, -1);
  for (int v = 0; v < n; ++v) {
    for (int e : c->out_e[v]) c->kids[v].push_back(ec[e]);
    if (!c->in_e[v].empty()) c->parent[v] = ep[c->in_e[v][0]];
  }
  c->leaves.clear();
  for (int v : c->preorder)
    if (c->kids[v].empty()) c->leaves.push_back(v);
  c->n_parents.assign(n, 0.0f);
  for (int v = 0; v < n; ++v)
    for (int e : c->in_e[v]) c->n_parents[v] += c->e_weighted ? c->e_weight[e] : 1.0f;
  c->wkids.assign(n, 0.0f);
  for (int v = 0; v < n; ++v)
    for (int e : c->out_e[v]) {
      const float t = (float)((c->e_weighted ? (double)c->e_weight[e] : 1.0) / c->n_parents[ec[e]]);
      c->wkids[v] += t * t;
    }
  return HMF_OK;
}

// Device memory plan: per non-root vertex 9 arrays (sink, label, div, two
// sets of three flow components), the root's source flow; every array holds
// all volumes.
int allocate_state(hmf_ctx* c) {
  const size_t arr = round_up((size_t)c->total * sizeof(float), 256);
  const int nonroot = c->n - 1;
  const int nvol = (int)c->vols.size();
  c->arena_bytes = arr * (size_t)((c->dag ? 10 : 9) * nonroot + 1) + 4096;
  CK(cudaMalloc(&c->arena, c->arena_bytes), "cudaMalloc(state)");
  // Every write the solver's work depends on is queued on the context's own
  // stream: the legacy stream's cudaMemset/cudaMemcpy are not ordered with
  // non-blocking streams, so a zeroing queued there could land after a
  // solve's first writes.
  CK(cudaMemsetAsync(c->arena, 0, c->arena_bytes, c->stream), "cudaMemsetAsync(state)");
  char* p = c->arena;
  auto take = [&]() {
    float* r = reinterpret_cast<float*>(p);
    p += arr;
    return r;
  };
  c->sink.assign(c->n, nullptr);
  c->label.assign(c->n, nullptr);
  c->div.assign(c->n, nullptr);
  c->inc.assign(c->n, nullptr);
  for (int s = 0; s < 2; ++s) {
    c->fx[s].assign(c->n, nullptr);
    c->fy[s].assign(c->n, nullptr);
    c->fz[s].assign(c->n, nullptr);
  }
  for (int v = 0; v < c->n; ++v) {
    c->sink[v] = take();
    if (v == c->root) continue;
    c->label[v] = take();
    c->div[v] = take();
    if (c->dag) c->inc[v] = take();
    for (int s = 0; s < 2; ++s) {
      c->fx[s][v] = take();
      c->fy[s][v] = take();
      c->fz[s][v] = take();
    }
  }
  CK(cudaMalloc(&c->d_flow[0], sizeof(hmf::FlowVertex) * hmf::kMaxVertices * 2), "cudaMalloc(tables)");
  c->d_flow[1] = c->d_flow[0] + hmf::kMaxVertices;
  CK(cudaMalloc(&c->d_tma, sizeof(hmf::FlowVertexTMA) * (size_t)nvol * nonroot), "cudaMalloc(tma table)");
  CK(cudaMalloc(&c->d_fvol, sizeof(hmf::FlowVolume) * nvol), "cudaMalloc(volume table)");
  CK(cudaMalloc(&c->d_tree, sizeof(hmf::TreeTable)), "cudaMalloc(tree table)");
  if (c->dag) CK(cudaMalloc(&c->d_dag, sizeof(hmf::DagTable)), "cudaMalloc(graph table)");
  CK(cudaMalloc(&c->d_smooth_list, sizeof(float*) * hmf::kMaxVertices), "cudaMalloc(smooth list)");
  CK(cudaMalloc(&c->d_error, sizeof(int)), "cudaMalloc(error flag)");
  CK(cudaMemsetAsync(c->d_error, 0, sizeof(int), c->stream), "cudaMemsetAsync(error flag)");
  return HMF_OK;
}

// Output rows of one flow window of the context's shape.
int flow_max_out_y(const hmf_ctx* c) { return 4 * c->flow_warps - 5; }

// Flow-kernel work plan for a given z-chunk length: windows of at most
// 28 x (4W - 5) outputs spread evenly over each volume, z split into chunks
// of `zchunk` planes.  Items enumerate volume, then z chunk, then window, so that windows
// that share halos run side by side.
int plan_flow(hmf_ctx* c, int zchunk) {
  c->h_fvol.assign(c->vols.size(), hmf::FlowVolume{});
  c->h_items.clear();
  for (size_t b = 0; b < c->vols.size(); ++b) {
    const auto& V = c->vols[b];
    hmf::FlowVolume& F = c->h_fvol[b];
    F.G.vx = V.vx;
    F.G.vy = V.vy;
    F.G.vz = V.vz;
    F.G.pitch = V.pitch;
    F.G.plane = V.plane;
    F.G.vol = V.vol;
    const int nx = (V.vx + hmf::kTmaMaxOutX - 1) / hmf::kTmaMaxOutX;
    const int ny = (V.vy + flow_max_out_y(c) - 1) / flow_max_out_y(c);
    F.out_x = (V.vx + nx - 1) / nx;
    F.out_y = (V.vy + ny - 1) / ny;
    F.tiles_x = nx;
    F.zchunk = std::min(zchunk, V.vz);
    const int chunks = (V.vz + F.zchunk - 1) / F.zchunk;
    for (int zc = 0; zc < chunks; ++zc)
      for (int t = 0; t < nx * ny; ++t) c->h_items.push_back(hmf::FlowItem{(int)b, t, zc, 0});
  }
  c->n_items = (int)c->h_items.size();
  c->zchunk = zchunk;
  if (c->d_items) cudaFree(c->d_items);
  c->d_items = nullptr;
  CK(cudaMalloc(&c->d_items, sizeof(hmf::FlowItem) * c->h_items.size()), "cudaMalloc(work items)");
  // on the context's stream (ordered before its launches), completed before
  // the host tables can change again
  CK(cudaMemcpyAsync(c->d_items, c->h_items.data(), sizeof(hmf::FlowItem) * c->h_items.size(),
                     cudaMemcpyHostToDevice, c->stream),
     "cudaMemcpyAsync(work items)");
  CK(cudaMemcpyAsync(c->d_fvol, c->h_fvol.data(), sizeof(hmf::FlowVolume) * c->h_fvol.size(), cudaMemcpyHostToDevice,
                     c->stream),
     "cudaMemcpyAsync(volume table)");
  CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize(work items)");
  return HMF_OK;
}

// Default z chunk.  A CTA marches its chunk's planes plus three halo planes,
// so long chunks waste less; but the windows of one wave of CTAs share their
// halo planes, parent sinks and smoothness images with the windows of the
// next wave only while those planes are still in L2, and a wave's L2
// footprint grows with its chunk length (~7 MB per plane for two CTAs per
// SM).  Measured on GB300: chunks of ~48 planes are fastest while a z chunk
// takes at most a few waves; when it takes many (the windows of a wave cover
// about one row of the volume, so every row boundary is crossed between
// waves) ~24 planes are, up to 2.2x faster than whole-volume chunks.  Within
// that cap the chunk count minimises waves x (planes + 3 halo + ~4 planes'
// worth of per-CTA set-up): small volumes get short chunks, so that their
// few windows still spread over the SMs.  Chunks are balanced (the deepest
// volume cut into equal chunks).
int default_zchunk(const hmf_ctx* c) {
  const int oy = flow_max_out_y(c);
  const long long slots = std::max(1, c->sm_count) * (c->flow_warps <= 8 ? 2LL : 1LL);  // flow CTAs per SM
  long long per_chunk = 0;                                  // CTAs of one z chunk of the largest volume
  int maxz = 1;
  for (const auto& V : c->vols) {
    per_chunk = std::max(per_chunk, (long long)((V.vx + hmf::kTmaMaxOutX - 1) / hmf::kTmaMaxOutX) *
                                        ((V.vy + oy - 1) / oy) * (c->n - 1));
    maxz = std::max(maxz, V.vz);
  }
  // a wave covers about one row of windows only when one volume's chunk
  // takes many waves (a batch of small volumes puts whole volumes in a wave)
  // A pipelined single volume drains its slab pipeline at every replayed
  // graph's end and overlaps slabs within it; there chunks of up to 64 planes
  // measured faster (256^3 tree4: 1.164 ms per iteration at 64 planes against
  // 1.185 at 43).
  const bool pipelined = c->pipeline && c->vols.size() == 1 && !c->dag;
  const int cap = per_chunk > 8 * slots ? 24 : (pipelined ? 64 : 48);
  int best_z = 1;
  double best = 1e300;
  for (int chunks = 1; chunks <= maxz; ++chunks) {
    const int z = (maxz + chunks - 1) / chunks;
    if (z > cap) continue;
    long long ctas = 0;
    for (const auto& V : c->vols) {
      const int zv = std::min(z, V.vz);
      ctas += (long long)((V.vx + hmf::kTmaMaxOutX - 1) / hmf::kTmaMaxOutX) *
              ((V.vy + oy - 1) / oy) * ((V.vz + zv - 1) / zv) * (c->n - 1);
    }
    const double cost = (double)((ctas + slots - 1) / slots) * (double)(z + 7);
    if (cost < best) best = cost, best_z = z;  // ties keep the longer chunk
  }
  return best_z;
}

// cuTensorMapEncodeTiled, fetched through the runtime so that the library
// needs no link-time dependency on the driver library.
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// 3-D map of one pitched volume block, box = one window plane of 36 columns
// and `rows` rows.
int encode_plane_map(hmf_ctx* c, CUtensorMap* m, const float* base, const hmf_ctx::Volume& V, int rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return fail(c, HMF_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
  const cuuint64_t dims[3] = {(cuuint64_t)V.vx, (cuuint64_t)V.vy, (cuuint64_t)V.vz};
  const cuuint64_t strides[2] = {(cuuint64_t)V.pitch * 4, (cuuint64_t)V.plane * 4};
  if (rows <= 0) rows = 4 * c->flow_warps;
  const cuuint32_t box[3] = {(cuuint32_t)hmf::kTmaBoxX, (cuuint32_t)rows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(c, HMF_ERR_CUDA, "cuTensorMapEncodeTiled failed with " + std::to_string((int)r));
  return HMF_OK;
}

// Inputs as device arrays over the concatenation: the data term of each leaf
// and one smoothness array per group of vertices that use the same image in
// every volume.  A single dense, 16-byte aligned device input is used in
// place; everything else is copied into pitched staging blocks.

int stage_inputs(hmf_ctx* c, cudaStream_t s, Staged& out) {
  const size_t arr = round_up((size_t)c->total * sizeof(float), 256);
  const int nvol = (int)c->vols.size();
  // smoothness groups: vertices whose (pointer, where) agree in every volume
  std::map<std::vector<std::pair<const float*, int>>, int> group_of_key;
  std::vector<std::vector<std::pair<const float*, int>>> groups;
  std::vector<int> group(c->n, -1);
  for (int v = 0; v < c->n; ++v) {
    if (v == c->root) continue;
    std::vector<std::pair<const float*, int>> key;
    bool any = false;
    for (int b = 0; b < nvol; ++b) {
      key.push_back({c->smooth[b][v].ptr, c->smooth[b][v].ptr ? c->smooth[b][v].where : 0});
      any = any || c->smooth[b][v].ptr;
    }
    if (!any) continue;
    auto it = group_of_key.find(key);
    if (it == group_of_key.end()) {
      it = group_of_key.emplace(key, (int)groups.size()).first;
      groups.push_back(key);
    }
    group[v] = it->second;
  }
  const bool single = nvol == 1;
  const auto& V0 = c->vols[0];
  auto borrowable = [&](const float* p, int where) {
    return single && where == HMF_DEVICE && V0.pitch == V0.vx && (reinterpret_cast<uintptr_t>(p) % 16) == 0;
  };
  size_t need = 0;
  for (int l : c->leaves)
    if (!borrowable(c->data[0][l].ptr, c->data[0][l].where)) need += arr;
  for (auto& g : groups)
    if (!borrowable(g[0].first, g[0].second)) need += arr;
  if (need > c->staging_bytes) {
    if (c->staging) cudaFree(c->staging);
    c->staging = nullptr;
    c->staging_bytes = 0;
    CK(cudaMalloc(&c->staging, need), "cudaMalloc(input staging)");
    CK(cudaMemsetAsync(c->staging, 0, need, s), "cudaMemsetAsync(input staging)");
    c->staging_bytes = need;
  }
  char* p = c->staging;
  // one array over the concatenation from per-volume sources (null: left as is)
  auto stage = [&](const std::vector<std::pair<const float*, int>>& src, const float** res) -> int {
    if (borrowable(src[0].first, src[0].second)) {
      *res = src[0].first;
      return HMF_OK;
    }
    float* dst = reinterpret_cast<float*>(p);
    p += arr;
    for (int b = 0; b < nvol; ++b) {
      if (!src[b].first) continue;
      const auto& V = c->vols[b];
      const cudaMemcpyKind kind = src[b].second == HMF_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
      if (V.pitch == V.vx) {  // unpadded rows: one linear copy (a 2-D copy moves row by row)
        CK(cudaMemcpyAsync(dst + V.off, src[b].first, (size_t)V.vol * sizeof(float), kind, s),
           "cudaMemcpyAsync(input)");
        continue;
      }
      CK(cudaMemcpy2DAsync(dst + V.off, (size_t)V.pitch * sizeof(float), src[b].first, (size_t)V.vx * sizeof(float),
                           (size_t)V.vx * sizeof(float), (size_t)V.vy * V.vz, kind, s),
         "cudaMemcpy2DAsync(input)");
    }
    *res = dst;
    return HMF_OK;
  };
  out.data.assign(c->n, nullptr);
  out.smooth.assign(c->n, nullptr);
  for (int l : c->leaves) {
    std::vector<std::pair<const float*, int>> src;
    for (int b = 0; b < nvol; ++b) src.push_back({c->data[b][l].ptr, c->data[b][l].where});
    int rc = stage(src, &out.data[l]);
    if (rc) return rc;
  }
  out.distinct.assign(groups.size(), nullptr);
  for (size_t g = 0; g < groups.size(); ++g) {
    int rc = stage(groups[g], &out.distinct[g]);
    if (rc) return rc;
  }
  for (int v = 0; v < c->n; ++v)
    if (group[v] >= 0) out.smooth[v] = out.distinct[group[v]];
  return HMF_OK;
}

int launch_flow_tma(hmf_ctx* c, int parity, cudaStream_t s) { return launch_flow_tma_with(c, c->d_tma, parity, s); }

namespace {
__global__ void request_stall_kernel(int* error_flag) { atomicOr(error_flag, hmf::kStallRequest); }
}  // namespace

int maybe_request_stall(hmf_ctx* c, int kind, cudaStream_t s) {
  if (c->stall_kind != kind) return HMF_OK;
  c->stall_kind = -1;
  request_stall_kernel<<<1, 1, 0, s>>>(c->d_error);
  CK(cudaGetLastError(), "request_stall_kernel launch");
  return HMF_OK;
}

int launch_flow_tma_with(hmf_ctx* c, const hmf::FlowVertexTMA* table, int parity, cudaStream_t s) {
  return launch_flow_tma_items(c, table, parity, 0, c->n_items, s);
}

int launch_flow_tma_items(hmf_ctx* c, const hmf::FlowVertexTMA* table, int parity, int first_item, int n_items,
                          cudaStream_t s) {
  hmf::FlowTmaParams fp;
  fp.step = c->step;
  fp.icc = 1.0f / c->cc;
  fp.parity = parity;
  fp.n_vertices = c->n - 1;
  fp.n_items = n_items;
  fp.units_per_cta = c->flow_units;
  fp.vols = c->d_fvol;
  fp.items = c->d_items + first_item;
  fp.error_flag = c->d_error;
  fp.wait_limit_ns = c->wait_limit_ns;
  if (int rc = maybe_request_stall(c, HMF_STALL_FLOW, s)) return rc;
  const long long units = (long long)n_items * (c->n - 1);
  const dim3 grid((unsigned)((units + c->flow_units - 1) / c->flow_units), 1, 1);
  const bool multi = c->flow_units > 1;
  if (c->flow_warps == 16) {
    if (multi)
      hmf::flow_tma_kernel<16, true>
          <<<grid, hmf::FlowTmaShape<16>::kThreads, hmf::FlowTmaShape<16>::kSmemBytes, s>>>(table, fp);
    else
      hmf::flow_tma_kernel<16, false>
          <<<grid, hmf::FlowTmaShape<16>::kThreads, hmf::FlowTmaShape<16>::kSmemBytes, s>>>(table, fp);
  } else {
    if (multi)
      hmf::flow_tma_kernel<8, true><<<grid, hmf::FlowTmaShape<8>::kThreads, hmf::FlowTmaShape<8>::kSmemBytes, s>>>(table, fp);
    else
      hmf::flow_tma_kernel<8, false><<<grid, hmf::FlowTmaShape<8>::kThreads, hmf::FlowTmaShape<8>::kSmemBytes, s>>>(table, fp);
  }
  CK(cudaGetLastError(), "flow_tma_kernel launch");
  ++c->launches;
  return HMF_OK;
}

int launch_flow(hmf_ctx* c, int parity, cudaStream_t s) {
  if (c->use_tma) return launch_flow_tma(c, parity, s);
  // shared-memory ring flow kernel: single volumes only (checked at create)
  const auto& V = c->vols[0];
  hmf::Geometry G{V.vx, V.vy, V.vz, V.pitch, V.plane, V.vol};
  hmf::FlowParams fp;
  fp.step = c->step;
  fp.icc = 1.0f / c->cc;
  fp.tiles_x = (G.vx + kTX - 1) / kTX;
  const int tiles = fp.tiles_x * ((G.vy + kTY - 1) / kTY);
  const int nonroot = c->n - 1;
  // enough CTAs for a few waves; split z into chunks when the xy tiling is small
  const long long target = (long long)c->sm_count * 8;
  int chunks = 1;
  if ((long long)tiles * nonroot < target)
    chunks = (int)std::min<long long>((target + (long long)tiles * nonroot - 1) / ((long long)tiles * nonroot),
                                      std::max(1, G.vz / 8));
  fp.zchunk = (G.vz + chunks - 1) / chunks;
  chunks = (G.vz + fp.zchunk - 1) / fp.zchunk;
  dim3 grid(tiles, chunks, nonroot), block(kTX, kTY);
  hmf::flow_kernel<kTX, kTY><<<grid, block, hmf::FlowTile<kTX, kTY>::SMEM_BYTES, s>>>(c->d_flow[parity], G, fp);
  CK(cudaGetLastError(), "flow_kernel launch");
  ++c->launches;
  return HMF_OK;
}

int tree_grid(hmf_ctx* c) {
  const long long blocks = (c->geo.vol + kTreeThreads - 1) / kTreeThreads;
  return (int)std::min<long long>(blocks, (long long)c->sm_count * 16);
}

// The convergence log's device view (the arena of hmf_set_convergence_log).
hmf::GapLog gap_view(const hmf_ctx* c, int t) {
  hmf::GapLog g{};
  unsigned int* base = reinterpret_cast<unsigned int*>(c->d_gap);
  g.base = base;
  g.t = t;
  g.max_bits = base + 2;
  g.sum = reinterpret_cast<double*>(c->d_gap + round_up(8 + 4 * (size_t)c->gap_cap, 8));
  g.capacity = c->gap_cap;
  g.vx = c->vols[0].vx;
  g.pitch = c->vols.size() == 1 && c->vols[0].pitch != c->vols[0].vx ? c->vols[0].pitch : 0;
  return g;
}

size_t gap_bytes(int cap) { return round_up(8 + 4 * (size_t)cap, 8) + 8 * (size_t)cap; }

// The sweep over the elements [0, G.vol) of `table`'s arrays.
int launch_tree_bulk_geo(hmf_ctx* c, const hmf::TreeTable* table, const hmf::Geometry& G, cudaStream_t s,
                         bool gap_log, int gap_t) {
  const int smem = hmf::tree_bulk_smem_bytes(c->n);
  const int vc = hmf::tree_bulk_chunk(c->n);
  const long long chunks = (G.vol + vc - 1) / vc;
  const int per_sm = std::max(1, (227 * 1024) / (smem + 4096));
  const int grid = (int)std::min<long long>(chunks, (long long)c->sm_count * per_sm);
  if (int rc = maybe_request_stall(c, HMF_STALL_SWEEP, s)) return rc;
  const hmf::GapLog gap = gap_log ? gap_view(c, gap_t) : hmf::GapLog{};
  switch (c->n) {
#define HMF_TREE_N(N)                                                                        \
  case N:                                                                                    \
    if (gap_log)                                                                             \
      hmf::tree_bulk_n_kernel<N, true><<<grid, vc / 4, smem, s>>>(table, G, c->d_error, gap); \
    else                                                                                     \
      hmf::tree_bulk_n_kernel<N, false><<<grid, vc / 4, smem, s>>>(table, G, c->d_error);    \
    break;
    HMF_TREE_N(2) HMF_TREE_N(3) HMF_TREE_N(4) HMF_TREE_N(5) HMF_TREE_N(6) HMF_TREE_N(7) HMF_TREE_N(8)
    HMF_TREE_N(9) HMF_TREE_N(10) HMF_TREE_N(11) HMF_TREE_N(12) HMF_TREE_N(13) HMF_TREE_N(14) HMF_TREE_N(15)
    HMF_TREE_N(16)
#undef HMF_TREE_N
    default:
      hmf::tree_bulk_kernel<<<grid, vc / 4, smem, s>>>(table, G, c->d_error, gap);
  }
  CK(cudaGetLastError(), "tree_bulk_kernel launch");
  ++c->launches;
  return HMF_OK;
}

int launch_tree_bulk_with(hmf_ctx* c, const hmf::TreeTable* table, cudaStream_t s, bool gap_log, int gap_t) {
  return launch_tree_bulk_geo(c, table, c->geo, s, gap_log, gap_t);
}

// Grid of the per-voxel DAG kernels: as many blocks as are resident at once.
int dag_grid(hmf_ctx* c, const void* kernel, size_t smem) {
  int per = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, hmf::kDagThreads, smem) != cudaSuccess || per < 1)
    per = 1;
  const long long blocks = (c->geo.vol + hmf::kDagThreads - 1) / hmf::kDagThreads;
  return (int)std::max<long long>(1, std::min<long long>(blocks, (long long)c->sm_count * per));
}

int launch_dag_sweep(hmf_ctx* c, cudaStream_t s) {
  if (!c->dag_simple)
    if (int rc = maybe_request_stall(c, HMF_STALL_SWEEP, s)) return rc;
  if (!c->dag_simple && !c->dag_generic && c->dag_reg_ok) {
    const int smem = hmf::dag_bulk_n_smem_bytes(c->n);
    const long long chunks = (c->geo.vol + hmf::kDagNVc - 1) / hmf::kDagNVc;
    auto launch = [&](auto kernel) {
      int per = 1;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, hmf::kDagNVc, smem) != cudaSuccess || per < 1)
        per = 1;
      const int grid = (int)std::max<long long>(1, std::min<long long>(chunks, (long long)c->sm_count * per));
      kernel<<<grid, hmf::kDagNVc, smem, s>>>(c->h_dagreg, c->geo.vol, c->dag_last ? 1 : 0, c->d_error);
    };
    switch (c->n) {
      case 2: launch(hmf::dag_bulk_n_kernel<2>); break;
      case 3: launch(hmf::dag_bulk_n_kernel<3>); break;
      case 4: launch(hmf::dag_bulk_n_kernel<4>); break;
      case 5: launch(hmf::dag_bulk_n_kernel<5>); break;
      case 6: launch(hmf::dag_bulk_n_kernel<6>); break;
      case 7: launch(hmf::dag_bulk_n_kernel<7>); break;
      default: launch(hmf::dag_bulk_n_kernel<8>); break;
    }
    CK(cudaGetLastError(), "dag_bulk_n_kernel launch");
    ++c->launches;
    return HMF_OK;
  }
  if (!c->dag_simple) {
    const int A = hmf::dag_bulk_arrays(c->n, (int)c->leaves.size());
    const int vc = hmf::dag_bulk_chunk(A);
    const int smem = hmf::dag_bulk_smem_bytes(A);
    int per = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, hmf::dag_bulk_kernel, vc, smem) != cudaSuccess || per < 1)
      per = 1;
    const long long chunks = (c->geo.vol + vc - 1) / vc;
    const int grid = (int)std::max<long long>(1, std::min<long long>(chunks, (long long)c->sm_count * per));
    hmf::dag_bulk_kernel<<<grid, vc, smem, s>>>(c->d_dag, c->geo.vol, c->dag_last ? 1 : 0, c->d_error);
    CK(cudaGetLastError(), "dag_bulk_kernel launch");
    ++c->launches;
    return HMF_OK;
  }
  const size_t smem = 4 * (size_t)c->n * hmf::kDagThreads * sizeof(float);
  hmf::dag_sweep_kernel<<<dag_grid(c, (const void*)hmf::dag_sweep_kernel, smem), hmf::kDagThreads, smem, s>>>(
      c->d_dag, c->geo.vol, c->dag_last ? 1 : 0);
  CK(cudaGetLastError(), "dag_sweep_kernel launch");
  ++c->launches;
  return HMF_OK;
}

int launch_tree(hmf_ctx* c, cudaStream_t s) {
  if (c->dag) return launch_dag_sweep(c, s);
  if (c->tree_kind == 0) return launch_tree_bulk_with(c, c->d_tree, s, c->gap_on, c->gap_t);
  if (c->tree_kind == 1) {
    const size_t smem4 = 4 * (size_t)c->n * hmf::kTree4Threads * sizeof(float4);
    const long long quads = c->geo.vol / 4;
    const int grid = (int)std::min<long long>((quads + hmf::kTree4Threads - 1) / hmf::kTree4Threads,
                                              (long long)c->sm_count * 32);
    hmf::tree4_kernel<<<grid, hmf::kTree4Threads, smem4, s>>>(c->d_tree, c->geo);
    CK(cudaGetLastError(), "tree4_kernel launch");
    ++c->launches;
    return HMF_OK;
  }
  const size_t smem = 3 * (size_t)c->n * kTreeThreads * sizeof(float);
  hmf::tree_kernel<<<tree_grid(c), kTreeThreads, smem, s>>>(c->d_tree, c->geo);
  CK(cudaGetLastError(), "tree_kernel launch");
  ++c->launches;
  return HMF_OK;
}

int record_iteration(hmf_ctx* c, int parity, cudaStream_t s) {
  int rc = launch_flow(c, parity, s);
  if (rc) return rc;
  return launch_tree(c, s);
}

// ---- z-slab pipeline of the replayed iterations ---------------------------
// With the pipeline on (hmf_set_pipeline) a single volume's iteration is cut
// at the flow plan's z chunks into slabs: the flow launch of a slab runs its
// chunk's work items, the sweep launch of a slab its planes' elements, each
// a graph node with only the dependencies the stencil needs --
//   sweep(t, k) after flow(t, k-1 .. k+1): the flows of the neighbouring
//     slabs read this slab's halo planes of sinks and labels, which the sweep
//     replaces;
//   flow(t+1, k) after sweep(t, k-1 .. k+1): it reads those planes' new
//     sinks and labels, and it overwrites the flow set that flow(t, k +- 1)
//     read as halo (both before those sweeps).
// So the sweeps of some slabs run beside the flows of others (the flow
// kernel leaves HBM bandwidth unused, the sweep needs little besides it),
// and the next iteration's first slabs start before this one's last.  The
// arithmetic is unchanged: results are bit-identical.
// A flow launch reads planes zs - 2 .. ze + 2 of its chunk [zs, ze), so the
// dependencies above reach only the neighbouring slabs when every slab but
// the last has at least 3 planes; with shorter chunks the pipeline is off.
//
// A batch is cut into groups of consecutive volumes instead (about equal in
// voxels): a group's flow items and its elements are contiguous, and groups
// share nothing, so each group's launches depend only on the group's own
// previous launch, and the groups' flows and sweeps overlap freely.
constexpr int kBatchGroups = 6;

bool pipeline_active(const hmf_ctx* c) {
  if (!c->pipeline || c->dag || !c->use_tma || c->tree_kind != 0 || c->semantics != HMF_SEMANTICS_REF_CUDA ||
      c->n_items <= 0 || c->h_fvol.empty())
    return false;
  if (c->vols.size() > 1) return true;
  return c->h_fvol[0].zchunk >= 3;
}

// Per-segment sweep tables: the solver's table with every array pointer
// moved to the segment's first element (its inputs may move between solves,
// so they are written before every pipelined solve, into the array the
// graphs point at).
int upload_slab_tables(hmf_ctx* c, cudaStream_t s) {
  const int K = c->n_slabs;
  c->h_tree_slabs.assign(K, c->h_tree);
  for (int k = 0; k < K; ++k) {
    const long long base = c->seg_base[k];
    hmf::TreeTable& T = c->h_tree_slabs[k];
    for (int e = 0; e < T.n; ++e) {
      hmf::TreeEntry& E = T.e[e];
      if (E.sink) E.sink += base;
      if (E.label) E.label += base;
      if (E.sink_out) E.sink_out += base;
      if (E.label_out) E.label_out += base;
      if (E.div) E.div += base;
      if (E.data) E.data += base;
    }
  }
  CK(cudaMemcpyAsync(c->d_tree_slabs, c->h_tree_slabs.data(), sizeof(hmf::TreeTable) * K, cudaMemcpyHostToDevice, s),
     "cudaMemcpyAsync(slab tables)");
  return HMF_OK;
}

// Segments of the current plan (one per z chunk of a single volume, or
// groups of a batch's volumes), their tables' device array, streams and
// events (made when the graphs are captured).
int prepare_slabs(hmf_ctx* c, cudaStream_t s) {
  c->seg_first_item.clear();
  c->seg_items.clear();
  c->seg_base.clear();
  c->slab_geo.clear();
  if (c->vols.size() == 1) {
    const auto& V = c->vols[0];
    const int zc = c->h_fvol[0].zchunk;
    const int K = (V.vz + zc - 1) / zc;
    const int per = c->n_items / K;  // windows of one z chunk
    for (int k = 0; k < K; ++k) {
      const long long z0 = (long long)k * zc, z1 = std::min<long long>(V.vz, z0 + zc);
      c->seg_first_item.push_back(k * per);
      c->seg_items.push_back(per);
      c->seg_base.push_back(z0 * V.plane);
      c->slab_geo.push_back(c->geo);
      c->slab_geo.back().vol = (z1 - z0) * V.plane;
    }
    c->seg_neighbours = 1;
  } else {
    // work items per volume (plan_flow enumerates them volume by volume)
    std::vector<int> items(c->vols.size(), 0);
    for (const auto& it : c->h_items) ++items[it.vol];
    const int nv = (int)c->vols.size();
    const int G = std::min(nv, kBatchGroups);
    long long done = 0;
    int b = 0, item = 0;
    for (int g = 0; g < G && b < nv; ++g) {
      const long long goal = (c->total * (g + 1)) / G;  // elements up to the end of this group
      const int b0 = b, i0 = item;
      const int later = G - 1 - g;  // groups after this one, one volume each at least
      long long elems = 0;
      do {
        elems += c->vols[b].vol;
        item += items[b];
        ++b;
      } while (b < nv - later && (g == G - 1 || done + elems < goal));
      c->seg_first_item.push_back(i0);
      c->seg_items.push_back(item - i0);
      c->seg_base.push_back(c->vols[b0].off);
      c->slab_geo.push_back(c->geo);
      c->slab_geo.back().vol = elems;
      done += elems;
    }
    c->seg_neighbours = 0;
  }
  const int K = (int)c->seg_base.size();
  // Every graph of one plan (captured one after another once the plan's
  // graphs were dropped) points at the same table array, so it is
  // reallocated only when the segment count changes.
  if (!c->d_tree_slabs || c->n_slabs != K) {
    if (c->d_tree_slabs) cudaFree(c->d_tree_slabs);
    c->d_tree_slabs = nullptr;
    CK(cudaMalloc(&c->d_tree_slabs, sizeof(hmf::TreeTable) * K), "cudaMalloc(slab tables)");
  }
  c->n_slabs = K;
  if (int rc = upload_slab_tables(c, s)) return rc;
  while ((int)c->slab_streams.size() < K) {
    cudaStream_t st = nullptr;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate(slab)");
    c->slab_streams.push_back(st);
    cudaEvent_t ef = nullptr, es = nullptr;
    CK(cudaEventCreateWithFlags(&ef, cudaEventDisableTiming), "cudaEventCreate(slab)");
    CK(cudaEventCreateWithFlags(&es, cudaEventDisableTiming), "cudaEventCreate(slab)");
    c->slab_ev_flow.push_back(ef);
    c->slab_ev_sweep.push_back(es);
  }
  return HMF_OK;
}

// Records n_iter iterations as slab nodes on the slab streams, forked from
// and joined back to c->stream (which is being captured).
int record_slab_iterations(hmf_ctx* c, int n_iter) {
  const int K = c->n_slabs;
  cudaStream_t origin = c->stream;
  CK(cudaEventRecord(c->ev_join, origin), "cudaEventRecord(fork)");
  for (int k = 0; k < K; ++k) CK(cudaStreamWaitEvent(c->slab_streams[k], c->ev_join, 0), "cudaStreamWaitEvent(fork)");
  for (int t = 0; t < n_iter; ++t) {
    for (int k = 0; k < K; ++k) {
      cudaStream_t st = c->slab_streams[k];
      if (t > 0)  // sweep(t-1, k) precedes on this stream
        for (int j = std::max(0, k - c->seg_neighbours); j <= std::min(K - 1, k + c->seg_neighbours); ++j)
          if (j != k) CK(cudaStreamWaitEvent(st, c->slab_ev_sweep[j], 0), "cudaStreamWaitEvent(sweep)");
      if (int rc = launch_flow_tma_items(c, c->d_tma, t & 1, c->seg_first_item[k], c->seg_items[k], st)) return rc;
      CK(cudaEventRecord(c->slab_ev_flow[k], st), "cudaEventRecord(flow)");
    }
    for (int k = 0; k < K; ++k) {
      cudaStream_t st = c->slab_streams[k];
      for (int j = std::max(0, k - c->seg_neighbours); j <= std::min(K - 1, k + c->seg_neighbours); ++j)
        if (j != k) CK(cudaStreamWaitEvent(st, c->slab_ev_flow[j], 0), "cudaStreamWaitEvent(flow)");
      if (int rc = launch_tree_bulk_geo(c, c->d_tree_slabs + k, c->slab_geo[k], st, c->gap_on, t)) return rc;
      CK(cudaEventRecord(c->slab_ev_sweep[k], st), "cudaEventRecord(sweep)");
    }
  }
  for (int k = 0; k < K; ++k) CK(cudaStreamWaitEvent(origin, c->slab_ev_sweep[k], 0), "cudaStreamWaitEvent(join)");
  return HMF_OK;
}

// The convergence log's base advances by the graph's iterations after its
// last sweep.
int record_gap_advance(hmf_ctx* c, int n_iter) {
  if (!c->gap_on) return HMF_OK;
  hmf::gap_advance_kernel<<<1, 1, 0, c->stream>>>(reinterpret_cast<unsigned int*>(c->d_gap), n_iter);
  CK(cudaGetLastError(), "gap_advance_kernel launch");
  return HMF_OK;
}

int capture(hmf_ctx* c, int n_iter, cudaGraphExec_t* out) {
  cudaGraph_t g = nullptr;
  const bool slabs = pipeline_active(c);
  if (slabs)
    if (int rc = prepare_slabs(c, c->stream)) return rc;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
  long long before = c->launches;
  int rc = HMF_OK;
  if (slabs) rc = record_slab_iterations(c, n_iter);
  else
    for (int i = 0; i < n_iter && rc == HMF_OK; ++i) {
      c->gap_t = i;
      rc = record_iteration(c, i & 1, c->stream);
    }
  c->gap_t = 0;
  if (!rc) rc = record_gap_advance(c, n_iter);
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  c->launches = before;
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphInstantiate");
  return HMF_OK;
}

void drop_graphs(hmf_ctx* c) {
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->graph_pair) cudaGraphExecDestroy(c->graph_pair);
  if (c->graph_one) cudaGraphExecDestroy(c->graph_one);
  if (c->graph_many) cudaGraphExecDestroy(c->graph_many);
  c->graph_pair = c->graph_one = c->graph_many = nullptr;
}

int timed(hmf_ctx* c, int kind, cudaStream_t s, int (*fn)(hmf_ctx*, cudaStream_t, int), int arg) {
  if (!c->timing) return fn(c, s, arg);
  CK(cudaEventRecord(c->ev_t0, s), "cudaEventRecord");
  int rc = fn(c, s, arg);
  if (rc) return rc;
  CK(cudaEventRecord(c->ev_t1, s), "cudaEventRecord");
  CK(cudaEventSynchronize(c->ev_t1), "cudaEventSynchronize");
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, c->ev_t0, c->ev_t1), "cudaEventElapsedTime");
  c->kind_ms[kind] += ms;
  c->kind_count[kind] += 1;
  return HMF_OK;
}

// The graph table of dag_sweep_kernel / dag_init_kernel: entries in forward
// order (root first), weights as the reference's tasks hold them
// (vtkCudaDirectedAcyclicGraphMaxFlowSegmentation.cxx:394-692, 957-1037):
// push-down and label weight = edge weight, else 1/#parents; push-up weight =
// that divided by the parent's weighted children (+1 for a branch); branch
// reset weight 1/(weighted children + 1); root shift 1/(CC * weighted children).
int prepare_dag_table(hmf_ctx* c, cudaStream_t s, const Staged& in) {
  hmf::DagTable& T = c->h_dag;
  std::memset(&T, 0, sizeof(T));
  std::vector<int> ent(c->n, -1);
  for (int i = 0; i < c->n; ++i) ent[c->preorder[i]] = i;
  T.n = c->n;
  T.cc = c->cc;
  T.icc = 1.0f / c->cc;
  T.shift = (float)(1.0 / (double)(c->cc * c->wkids[c->root]));
  auto wdown = [&](int e) {
    return c->e_weighted ? c->e_weight[e] : (float)(1.0 / (double)c->in_e[c->e_child[e]].size());
  };
  int pin = 0, pout = 0;
  for (int i = 0; i < c->n; ++i) {
    const int v = c->preorder[i];
    hmf::DagEntry& E = T.e[i];
    E.sink = c->sink[v];
    E.leaf = c->kids[v].empty() && v != c->root;
    if (v != c->root) {
      E.inc = c->inc[v];
      E.label = c->label[v];
      E.div = c->div[v];
      E.data = E.leaf ? in.data[v] : nullptr;
      E.k = (float)(1.0 / ((double)c->wkids[v] + 1.0));
    }
    if (E.leaf) T.leaves[T.n_leaves++] = i;
    E.first_in = pin;
    for (int e : c->in_e[v]) {
      const int p = c->e_parent[e];
      const float W = c->e_weighted ? c->e_weight[e] : (float)(1.0 / (double)c->in_e[v].size());
      T.in_parent[pin] = ent[p];
      T.in_wdown[pin] = wdown(e);
      T.in_wup[pin] = p == c->root ? W / c->wkids[p] : W / (c->wkids[p] + 1.0f);
      ++pin;
    }
    E.n_in = pin - E.first_in;
    E.first_out = pout;
    for (int e : c->out_e[v]) {
      T.out_child[pout] = ent[c->e_child[e]];
      T.out_w[pout] = wdown(e);
      ++pout;
    }
    E.n_out = pout - E.first_out;
  }
  CK(cudaMemcpyAsync(c->d_dag, &T, sizeof(T), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(graph table)");
  // the same graph as kernel parameters of dag_bulk_n_kernel (small graphs
  // whose edges are all distinct)
  hmf::DagRegParams& R = c->h_dagreg;
  std::memset(&R, 0, sizeof(R));
  c->dag_reg_ok = c->n <= hmf::kDagRegMax;
  for (int i = 0; i < c->n && c->dag_reg_ok; ++i) {
    const hmf::DagEntry& E = T.e[i];
    R.sink[i] = E.sink;
    R.inc[i] = E.inc;
    R.label[i] = E.label;
    R.div[i] = E.div;
    R.data[i] = E.data;
    R.k[i] = E.k;
    if (E.leaf) R.leaf_mask |= 1u << i;
    R.n_in[i] = E.n_in;
    for (int j = 0; j < E.n_in; ++j) {
      const int p = T.in_parent[E.first_in + j];
      if ((R.pmask[i] >> p) & 1u) c->dag_reg_ok = false;  // a repeated edge
      R.pmask[i] |= 1u << p;
      R.wup[i][p] = T.in_wup[E.first_in + j];
      R.wdown_ord[i][j] = T.in_wdown[E.first_in + j];
      R.parent_ord[i][j] = p;
    }
  }
  R.cc = T.cc;
  R.icc = T.icc;
  R.shift = T.shift;
  return HMF_OK;
}

int prepare_tables(hmf_ctx* c, cudaStream_t s, const Staged& in) {
  const int nvol = (int)c->vols.size();
  const int nonroot = c->n - 1;
  // shared-memory ring flow kernel tables (one volume), one per parity
  std::vector<hmf::FlowVertex>& fv = c->h_flow;
  fv.assign(2 * hmf::kMaxVertices, hmf::FlowVertex{});
  int slot = 0;
  for (int v : c->preorder) {
    if (v == c->root) continue;
    for (int par = 0; par < 2; ++par) {
      hmf::FlowVertex& f = fv[par * hmf::kMaxVertices + slot];
      f.px_in = c->fx[par][v];
      f.py_in = c->fy[par][v];
      f.pz_in = c->fz[par][v];
      f.px_out = c->fx[par ^ 1][v];
      f.py_out = c->fy[par ^ 1][v];
      f.pz_out = c->fz[par ^ 1][v];
      f.sink = c->sink[v];
      f.inc = c->dag ? c->inc[v] : c->sink[c->parent[v]];
      f.label = c->label[v];
      f.smooth = in.smooth[v];
      f.div = c->div[v];
      f.alpha = (float)c->alpha[v];  // stored as float, as the reference does (.cxx:692)
    }
    ++slot;
  }
  CK(cudaMemcpyAsync(c->d_flow[0], fv.data(), sizeof(hmf::FlowVertex) * fv.size(), cudaMemcpyHostToDevice, s),
     "cudaMemcpyAsync(flow table)");
  if (c->use_tma) {
    std::vector<hmf::FlowVertexTMA>& tv = c->h_tma;
    tv.assign((size_t)nvol * nonroot, hmf::FlowVertexTMA{});
    for (int b = 0; b < nvol; ++b) {
      const auto& V = c->vols[b];
      int j = 0;
      for (int v : c->preorder) {
        if (v == c->root) continue;
        hmf::FlowVertexTMA& f = tv[(size_t)b * nonroot + j++];
        std::memset(&f, 0, sizeof(f));
        int rc = HMF_OK;
        for (int par = 0; par < 2 && !rc; ++par) {
          rc = encode_plane_map(c, &f.flow_in[par][0], c->fx[par][v] + V.off, V);
          if (!rc) rc = encode_plane_map(c, &f.flow_in[par][1], c->fy[par][v] + V.off, V);
          if (!rc) rc = encode_plane_map(c, &f.flow_in[par][2], c->fz[par][v] + V.off, V);
          f.flow_out[par][0] = c->fx[par ^ 1][v] + V.off;
          f.flow_out[par][1] = c->fy[par ^ 1][v] + V.off;
          f.flow_out[par][2] = c->fz[par ^ 1][v] + V.off;
        }
        if (!rc) rc = encode_plane_map(c, &f.sink, c->sink[v] + V.off, V);
        if (!rc) rc = encode_plane_map(c, &f.label, c->label[v] + V.off, V);
        if (!rc) rc = encode_plane_map(c, &f.inc, (c->dag ? c->inc[v] : c->sink[c->parent[v]]) + V.off, V);
        const bool has_s = in.smooth[v] && c->smooth[b][v].ptr;
        if (!rc && has_s) rc = encode_plane_map(c, &f.smooth, in.smooth[v] + V.off, V);
        if (rc) return rc;
        f.has_smooth = has_s;
        f.div = c->div[v] + V.off;
        f.alpha = (float)c->alpha[v];
      }
    }
    CK(cudaMemcpyAsync(c->d_tma, tv.data(), sizeof(hmf::FlowVertexTMA) * tv.size(), cudaMemcpyHostToDevice, s),
       "cudaMemcpyAsync(tma table)");
  }
  if (c->dag) {
    int rc = prepare_dag_table(c, s, in);
    if (rc) return rc;
  } else {
  hmf::TreeTable& tt = c->h_tree;
  std::memset(&tt, 0, sizeof(tt));
  std::vector<int> entry(c->n, -1);
  for (int i = 0; i < c->n; ++i) entry[c->postorder[i]] = i;
  tt.n = c->n;
  tt.n_leaves = (int)c->leaves.size();
  tt.cc = c->cc;
  tt.icc = 1.0f / c->cc;
  tt.root_init = 1.0f / c->cc;
  int kpos = 0;
  for (int i = 0; i < c->n; ++i) {
    const int v = c->postorder[i];
    hmf::TreeEntry& E = tt.e[i];
    E.sink = E.sink_out = c->sink[v];
    E.label = E.label_out = v == c->root ? nullptr : c->label[v];
    E.div = v == c->root ? nullptr : c->div[v];
    E.data = in.data[v];
    E.parent = v == c->root ? -1 : entry[c->parent[v]];
    E.first_kid = kpos;
    E.n_kids = (int)c->kids[v].size();
    for (int k : c->kids[v]) tt.kids[kpos++] = entry[k];
    const int nk = E.n_kids;
    E.inv_kids = nk == 0 ? 0.0f : (v == c->root ? 1.0f / (float)nk : 1.0f / (float)(nk + 1));
  }
  for (size_t j = 0; j < c->leaves.size(); ++j) tt.leaves[j] = entry[c->leaves[j]];
  CK(cudaMemcpyAsync(c->d_tree, &tt, sizeof(tt), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(tree table)");
  }
  c->n_smooth_list = (int)in.distinct.size();
  c->h_smooth_list = in.distinct;
  if (!in.distinct.empty())
    CK(cudaMemcpyAsync(c->d_smooth_list, c->h_smooth_list.data(), sizeof(float*) * in.distinct.size(),
                       cudaMemcpyHostToDevice, s),
       "cudaMemcpyAsync(smooth list)");
  return HMF_OK;
}

int do_init(hmf_ctx* c, cudaStream_t s, int) {
  if (c->dag) {
    const size_t smem = (size_t)c->n * hmf::kDagThreads * sizeof(float);
    hmf::dag_init_kernel<<<dag_grid(c, (const void*)hmf::dag_init_kernel, smem), hmf::kDagThreads, smem, s>>>(
        c->d_dag, c->geo.vol);
    CK(cudaGetLastError(), "dag_init_kernel launch");
    ++c->launches;
    return HMF_OK;
  }
  const size_t smem = (size_t)c->n * kTreeThreads * sizeof(float);
  hmf::init_kernel<<<tree_grid(c), kTreeThreads, smem, s>>>(c->d_tree, c->geo, c->d_smooth_list,
                                                           c->n_smooth_list,
                                                           c->semantics == HMF_SEMANTICS_REF_CPU,
                                                           c->d_error);
  CK(cudaGetLastError(), "init_kernel launch");
  ++c->launches;
  return HMF_OK;
}

int do_flow(hmf_ctx* c, cudaStream_t s, int parity) { return launch_flow(c, parity, s); }
int do_tree(hmf_ctx* c, cudaStream_t s, int) { return launch_tree(c, s); }
int do_refcpu(hmf_ctx* c, cudaStream_t s, int) {
  hmf::refcpu_kernel<<<tree_grid(c), kTreeThreads, 0, s>>>(c->d_tree, c->geo, c->iterations);
  CK(cudaGetLastError(), "refcpu_kernel launch");
  ++c->launches;
  return HMF_OK;
}

// The dynamic shared-memory limit is a per-device property of the function,
// shared by every context: it is always set to what the largest supported
// tree needs, so that no context lowers it below another's requirement.
int configure_kernels(hmf_ctx* c) {
  CK(cudaFuncSetAttribute(hmf::flow_kernel<kTX, kTY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          hmf::FlowTile<kTX, kTY>::SMEM_BYTES),
     "cudaFuncSetAttribute(flow_kernel)");
  const int tree_smem = 3 * hmf::kMaxVertices * kTreeThreads * (int)sizeof(float);
  CK(cudaFuncSetAttribute(hmf::tree_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, tree_smem),
     "cudaFuncSetAttribute(tree_kernel)");
  CK(cudaFuncSetAttribute(hmf::init_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          hmf::kMaxVertices * kTreeThreads * (int)sizeof(float)),
     "cudaFuncSetAttribute(init_kernel)");
  CK(cudaFuncSetAttribute(hmf::flow_tma_kernel<8, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          hmf::FlowTmaShape<8>::kSmemBytes),
     "cudaFuncSetAttribute(flow_tma_kernel)");
  CK(cudaFuncSetAttribute(hmf::flow_tma_kernel<16, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          hmf::FlowTmaShape<16>::kSmemBytes),
     "cudaFuncSetAttribute(flow_tma_kernel)");
  CK(cudaFuncSetAttribute(hmf::flow_tma_kernel<8, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          hmf::FlowTmaShape<8>::kSmemBytes),
     "cudaFuncSetAttribute(flow_tma_kernel)");
  CK(cudaFuncSetAttribute(hmf::flow_tma_kernel<16, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          hmf::FlowTmaShape<16>::kSmemBytes),
     "cudaFuncSetAttribute(flow_tma_kernel)");
  CK(cudaFuncSetAttribute(hmf::tree4_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          4 * hmf::kTree4MaxVertices * hmf::kTree4Threads * (int)sizeof(float4)),
     "cudaFuncSetAttribute(tree4_kernel)");
  CK(cudaFuncSetAttribute(hmf::tree_bulk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          128 + hmf::kTreeBulkSmemBudget),
     "cudaFuncSetAttribute(tree_bulk_kernel)");
#define HMF_TREE_N_ATTR(N)                                                                           \
  CK(cudaFuncSetAttribute(hmf::tree_bulk_n_kernel<N, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                          hmf::tree_bulk_smem_bytes(N)),                                             \
     "cudaFuncSetAttribute(tree_bulk_n_kernel)");                                                    \
  CK(cudaFuncSetAttribute(hmf::tree_bulk_n_kernel<N, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                          hmf::tree_bulk_smem_bytes(N)),                                             \
     "cudaFuncSetAttribute(tree_bulk_n_kernel)");
  HMF_TREE_N_ATTR(2) HMF_TREE_N_ATTR(3) HMF_TREE_N_ATTR(4) HMF_TREE_N_ATTR(5) HMF_TREE_N_ATTR(6)
  HMF_TREE_N_ATTR(7) HMF_TREE_N_ATTR(8) HMF_TREE_N_ATTR(9) HMF_TREE_N_ATTR(10) HMF_TREE_N_ATTR(11)
  HMF_TREE_N_ATTR(12) HMF_TREE_N_ATTR(13) HMF_TREE_N_ATTR(14) HMF_TREE_N_ATTR(15) HMF_TREE_N_ATTR(16)
#undef HMF_TREE_N_ATTR
  CK(cudaFuncSetAttribute(hmf::dag_sweep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          4 * hmf::kMaxVertices * hmf::kDagThreads * (int)sizeof(float)),
     "cudaFuncSetAttribute(dag_sweep_kernel)");
#define HMF_DAG_N_ATTR(N)                                                                    \
  CK(cudaFuncSetAttribute(hmf::dag_bulk_n_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                          hmf::dag_bulk_n_smem_bytes(N)),                                    \
     "cudaFuncSetAttribute(dag_bulk_n_kernel)");
  HMF_DAG_N_ATTR(2) HMF_DAG_N_ATTR(3) HMF_DAG_N_ATTR(4) HMF_DAG_N_ATTR(5) HMF_DAG_N_ATTR(6)
  HMF_DAG_N_ATTR(7) HMF_DAG_N_ATTR(8)
#undef HMF_DAG_N_ATTR
  CK(cudaFuncSetAttribute(hmf::dag_bulk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          128 + hmf::kDagBulkSmemBudget),
     "cudaFuncSetAttribute(dag_bulk_kernel)");
  CK(cudaFuncSetAttribute(hmf::dag_init_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          hmf::kMaxVertices * hmf::kDagThreads * (int)sizeof(float)),
     "cudaFuncSetAttribute(dag_init_kernel)");
  return HMF_OK;
}

bool valid_vertex(const hmf_ctx* c, int v) { return c && v >= 0 && v < c->n; }
bool valid_volume(const hmf_ctx* c, int b) { return c && b >= 0 && b < (int)c->vols.size(); }

int check_error_flag(hmf_ctx* c) {
  int flag = 0;
  CK(cudaMemcpyAsync(&flag, c->d_error, sizeof(int), cudaMemcpyDeviceToHost, c->stream),
     "cudaMemcpyAsync(error flag)");
  CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize(error flag)");
  return decode_error_flag(c, flag);
}

int decode_error_flag(hmf_ctx* c, int flag) {
  flag &= ~hmf::kStallRequest;  // a stall request no kernel took
  if (flag & 4) return fail(c, HMF_ERR_CUDA, "shared-memory staging area misaligned; results are invalid");
  if (flag & 2) return fail(c, HMF_ERR_CUDA, "an asynchronous-copy wait timed out; results are invalid");
  if (flag & 1)
    return fail(c, HMF_ERR_INVALID_ARGUMENT,
                "Data prior and smoothness must be non-negative (the solve ran on invalid input)");
  if (flag & 8) return fail(c, HMF_ERR_INVALID_ARGUMENT, "a ground-truth class index is not a leaf index");
  return HMF_OK;
}

int copy_out(hmf_ctx* c, int b, const float* src, float* out, int where, void* stream) {
  if (!out) return fail(c, HMF_ERR_INVALID_ARGUMENT, "output pointer is NULL");
  if (where != HMF_HOST && where != HMF_DEVICE) return fail(c, HMF_ERR_INVALID_ARGUMENT, "bad `where`");
  DeviceGuard dg(c->device);
  if (where == HMF_DEVICE)
    if (int rc = check_device_pointer(c, out, "output")) return rc;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const auto& V = c->vols[b];
  const cudaMemcpyKind kind = where == HMF_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  if (V.pitch == V.vx) {  // unpadded rows: one linear copy
    CK(cudaMemcpyAsync(out, src + V.off, (size_t)V.vol * sizeof(float), kind, s), "cudaMemcpyAsync(output)");
  } else {
    CK(cudaMemcpy2DAsync(out, (size_t)V.vx * sizeof(float), src + V.off, (size_t)V.pitch * sizeof(float),
                         (size_t)V.vx * sizeof(float), (size_t)V.vy * V.vz, kind, s),
       "cudaMemcpy2DAsync(output)");
  }
  if (where == HMF_HOST) {  // the error flag rides on the same stream: one synchronisation
    if (!c->h_error) CK(cudaMallocHost(&c->h_error, sizeof(int)), "cudaMallocHost(error flag)");
    CK(cudaMemcpyAsync(c->h_error, c->d_error, sizeof(int), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync(error flag)");
    CK(cudaStreamSynchronize(s), "cudaStreamSynchronize(output)");
    return decode_error_flag(c, *c->h_error);
  }
  return HMF_OK;
}

// Cache of tuned flow plans (window warps, z chunk), keyed by the work
// shape: SM count, tree (vertex count and the children count of every
// vertex in pre-order), semantics and the volume sizes, each axis rounded up
// to a multiple of 16 (sizes in one bucket share window counts within one
// and the same z-chunk choices).  Process-wide; with HMF_AUTOTUNE_CACHE set
// to a file path it is also read from and appended to that file (one
// "key warps zchunk" line per tuned shape), so later processes reuse it.
struct TunedPlan {
  int warps, zchunk, units;
};
std::mutex g_tune_mutex;
std::map<std::string, TunedPlan> g_tune_cache;
bool g_tune_file_read = false;

std::string tune_key(const hmf_ctx* c) {
  std::string k = std::to_string(c->sm_count) + "/" + std::to_string(c->semantics) + "/n" + std::to_string(c->n) + ":";
  for (int v : c->preorder) k += std::to_string(c->kids[v].size()) + ",";
  for (const auto& V : c->vols)
    k += "/" + std::to_string((V.vx + 15) / 16 * 16) + "x" + std::to_string((V.vy + 15) / 16 * 16) + "x" +
         std::to_string((V.vz + 15) / 16 * 16);
  return k;
}

// with g_tune_mutex held
void tune_file_read() {
  if (g_tune_file_read) return;
  g_tune_file_read = true;
  const char* path = std::getenv("HMF_AUTOTUNE_CACHE");
  if (!path || !*path) return;
  FILE* f = std::fopen(path, "r");
  if (!f) return;
  char line[4200], key[4096];
  while (std::fgets(line, sizeof(line), f)) {
    int w = 0, z = 0, u = 1;  // lines written before the units field read as one unit per CTA
    if (std::sscanf(line, "%4095s %d %d %d", key, &w, &z, &u) >= 3 && (w == 8 || w == 16) && z >= 1 && u >= 1 &&
        u <= kMaxFlowUnits)
      g_tune_cache[key] = TunedPlan{w, z, u};
  }
  std::fclose(f);
}

// with g_tune_mutex held
void tune_file_append(const std::string& key, const TunedPlan& t) {
  const char* path = std::getenv("HMF_AUTOTUNE_CACHE");
  if (!path || !*path) return;
  FILE* f = std::fopen(path, "a");
  if (!f) return;
  std::fprintf(f, "%s %d %d %d\n", key.c_str(), t.warps, t.zchunk, t.units);
  std::fclose(f);
}

int begin_solve_with(hmf_ctx* c, cudaStream_t user, Staged& staged, StateLoader load, void* arg);

int begin_solve(hmf_ctx* c, cudaStream_t user, Staged& staged) { return begin_solve_with(c, user, staged, nullptr, nullptr); }

int begin_solve_with(hmf_ctx* c, cudaStream_t user, Staged& staged, StateLoader load, void* arg) {
  for (size_t b = 0; b < c->vols.size(); ++b)
    for (int l : c->leaves)
      if (!c->data[b][l].ptr) return fail(c, HMF_ERR_MISSING_INPUT, "Missing data prior for leaf node.");
  cudaStream_t s = c->stream;
  c->launches = 0;
  for (int k = 0; k < 3; ++k) c->kind_ms[k] = 0, c->kind_count[k] = 0;
  c->solved = false;
  c->continuable = false;
  // order after the caller's queued work
  CK(cudaEventRecord(c->ev_join, user), "cudaEventRecord(join)");
  CK(cudaStreamWaitEvent(s, c->ev_join, 0), "cudaStreamWaitEvent(join)");
  CK(cudaMemsetAsync(c->d_error, 0, sizeof(int), s), "cudaMemsetAsync(error flag)");
  int rc = stage_inputs(c, s, staged);
  if (!rc) rc = prepare_tables(c, s, staged);
  if (rc) return rc;
  c->st_data = staged.data;
  c->st_smooth = staged.smooth;
  if (load) return load(c, s, arg);  // a continued solve: the caller's state replaces the initialisation
  // flows of parity 0 start at zero
  const size_t bytes = (size_t)c->total * sizeof(float);
  for (int v = 0; v < c->n; ++v) {
    if (v == c->root) continue;
    CK(cudaMemsetAsync(c->fx[0][v], 0, bytes, s), "cudaMemsetAsync(flows)");
    CK(cudaMemsetAsync(c->fy[0][v], 0, bytes, s), "cudaMemsetAsync(flows)");
    CK(cudaMemsetAsync(c->fz[0][v], 0, bytes, s), "cudaMemsetAsync(flows)");
  }
  return timed(c, 2, s, do_init, 0);
}

int end_solve(hmf_ctx* c, cudaStream_t user) {
  CK(cudaEventRecord(c->ev_join, c->stream), "cudaEventRecord(done)");
  CK(cudaStreamWaitEvent(user, c->ev_join, 0), "cudaStreamWaitEvent(done)");
  c->solved = true;
  return HMF_OK;
}

}  // namespace hmfi

using namespace hmfi;

namespace {

// The common part of hmf_create_batch and hmf_create_dag: volumes, the graph
// (`build`), device, stream, state, kernel attributes and the flow plan.
template <class BuildGraph>
int create_context(hmf_ctx** out, int n_volumes, const int* dims, int semantics, int device, BuildGraph build,
                   bool device_state = true) {
  g_create_error.clear();
  if (!out) return fail(nullptr, HMF_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  if (n_volumes < 1 || !dims) return fail(nullptr, HMF_ERR_INVALID_ARGUMENT, "a batch needs at least one volume");
  for (int b = 0; b < n_volumes; ++b) {
    if (dims[3 * b] <= 0 || dims[3 * b + 1] <= 0 || dims[3 * b + 2] <= 0)
      return fail(nullptr, HMF_ERR_INVALID_ARGUMENT, "volume dimensions must be positive");
    if (dims[3 * b] > kMaxDim || dims[3 * b + 1] > kMaxDim || dims[3 * b + 2] > kMaxDim)
      return fail(nullptr, HMF_ERR_INVALID_ARGUMENT, "volume dimensions above 2^30 are not supported");
  }
  if (semantics != HMF_SEMANTICS_REF_CUDA && semantics != HMF_SEMANTICS_REF_CPU)
    return fail(nullptr, HMF_ERR_INVALID_ARGUMENT, "unknown semantics");
  hmf_ctx* c = new hmf_ctx();
  c->device = device;
  c->semantics = semantics;
  long long off = 0;
  for (int b = 0; b < n_volumes; ++b) {
    hmf_ctx::Volume V;
    V.vx = dims[3 * b];
    V.vy = dims[3 * b + 1];
    V.vz = dims[3 * b + 2];
    V.pitch = (V.vx + 3) / 4 * 4;
    V.plane = (long long)V.pitch * V.vy;
    V.vol = V.plane * V.vz;
    if (device_state && V.vol >= (1LL << 31)) {  // the flow kernel addresses a volume's elements with 32-bit offsets
      g_create_error = "volumes of 2^31 or more elements (rows padded to 4 floats) are not supported";
      delete c;
      return HMF_ERR_INVALID_ARGUMENT;
    }
    V.off = off;
    off += V.vol;  // a multiple of 4: every block starts 16-byte aligned
    c->vols.push_back(V);
  }
  c->total = off;
  const auto& V0 = c->vols[0];
  c->geo.vx = V0.vx;
  c->geo.vy = V0.vy;
  c->geo.vz = V0.vz;
  c->geo.pitch = n_volumes == 1 ? V0.pitch : 0;
  c->geo.plane = V0.plane;
  c->geo.vol = c->total;
  int rc = build(c);
  if (rc) {
    g_create_error = c->err;
    delete c;
    return rc;
  }
  // a DAG vertex without AddSmoothnessScalar has alpha 0: the CUDA DAG class
  // reads its scalar map with operator[] (vtkCudaDirectedAcyclicGraphMaxFlowSegmentation.cxx:365)
  c->alpha.assign(c->n, c->dag ? 0.0 : 1.0);
  if (const char* e = std::getenv("HMF_DAG_KERNEL")) {
    c->dag_simple = std::strcmp(e, "simple") == 0;
    c->dag_generic = std::strcmp(e, "generic") == 0;
  }
  // Kernel selection.  HMF_FLOW_KERNEL=ring / HMF_TREE_KERNEL=quad|scalar select
  // the simpler kernels (same results), for comparisons.
  if (const char* e = std::getenv("HMF_FLOW_KERNEL")) c->use_tma = std::strcmp(e, "ring") != 0 || n_volumes > 1;
  c->tree_kind = 0;
  if (const char* e = std::getenv("HMF_TREE_KERNEL")) {
    if (std::strcmp(e, "quad") == 0 && c->n <= hmf::kTree4MaxVertices) c->tree_kind = 1;
    if (std::strcmp(e, "scalar") == 0) c->tree_kind = 2;
  }
  c->data.assign(n_volumes, std::vector<hmf_ctx::Input>(c->n));
  c->smooth.assign(n_volumes, std::vector<hmf_ctx::Input>(c->n));
  {
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || device < 0 || device >= ndev) {
      g_create_error = e != cudaSuccess ? std::string("no CUDA device: ") + cudaGetErrorString(e)
                                        : std::string("CUDA device index out of range");
      delete c;
      return HMF_ERR_CUDA;
    }
    DeviceGuard dg(device);
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, device);
    if (e == cudaSuccess) c->sm_count = prop.multiProcessorCount;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev_t0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev_t1);
    if (e != cudaSuccess) {
      g_create_error = std::string("CUDA setup failed: ") + cudaGetErrorString(e);
      hmf_destroy(c);
      return HMF_ERR_CUDA;
    }
    if (!device_state) {  // an out-of-core context: its blocks hold the device state
      *out = c;
      return HMF_OK;
    }
    rc = allocate_state(c);
    if (!rc) rc = configure_kernels(c);
    if (!rc) {
      int z = 0;
      {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        tune_file_read();
        auto it = g_tune_cache.find(tune_key(c));
        if (it != g_tune_cache.end()) {
          c->flow_warps = it->second.warps;
          c->flow_units = it->second.units;
          z = it->second.zchunk;
        }
      }
      rc = plan_flow(c, z ? z : default_zchunk(c));
    }
    if (rc) {
      g_create_error = c->err;
      hmf_destroy(c);
      return rc;
    }
  }
  *out = c;
  return HMF_OK;
}

}  // namespace

namespace hmfi {

int solve_with(hmf_ctx* c, cudaStream_t user, StateLoader load, void* arg) {
  DeviceGuard dg(c->device);
  cudaStream_t s = c->stream;
  Staged staged;
  int rc = begin_solve_with(c, user, staged, load, arg);
  if (rc) return rc;
  c->gap_logged = 0;
  if (c->gap_on && c->semantics == HMF_SEMANTICS_REF_CUDA) {
    if (c->gap_cap < c->iterations) {  // a longer log: new arena, graphs re-captured with it
      drop_graphs(c);
      if (c->d_gap) cudaFree(c->d_gap);
      c->d_gap = nullptr;
      c->gap_cap = 0;
      const int cap = std::max(c->iterations, 64);
      CK(cudaMalloc(&c->d_gap, gap_bytes(cap)), "cudaMalloc(convergence log)");
      c->gap_cap = cap;
    }
    CK(cudaMemsetAsync(c->d_gap, 0, gap_bytes(c->gap_cap), s), "cudaMemsetAsync(convergence log)");
    c->gap_logged = c->iterations;
  }
  if (c->semantics == HMF_SEMANTICS_REF_CPU) {
    rc = timed(c, 1, s, do_refcpu, 0);
    if (rc) return rc;
  } else if (c->timing || c->stall_kind >= 0) {
    for (int it = 0; it < c->iterations; ++it) {
      c->dag_last = c->dag && it == c->iterations - 1;
      c->gap_t = it;  // the log's base stays 0 on this path
      rc = timed(c, 0, s, do_flow, it & 1);
      if (!rc) rc = timed(c, 1, s, do_tree, 0);
      c->dag_last = false;
      c->gap_t = 0;
      if (rc) return rc;
    }
  } else {
    if (!c->graph_pair) {
      rc = capture(c, 2, &c->graph_pair);
      if (!rc) rc = capture(c, 1, &c->graph_one);
      // a pipelined solve replays several iterations per graph, so that the
      // pipeline drains (at a graph's end) rarely
      if (!rc && pipeline_active(c)) rc = capture(c, kPipelineIterations, &c->graph_many);
      if (rc) return rc;
    }
    // a DAG's last iteration runs fewer tasks: launched on its own
    const int graphed = c->dag ? std::max(0, c->iterations - 1) : c->iterations;
    const long long per_iter = pipeline_active(c) ? 2LL * c->n_slabs : 2;
    if (pipeline_active(c))
      if (int rc2 = upload_slab_tables(c, s)) return rc2;
    int it0 = 0;
    if (c->graph_many)
      for (; it0 + kPipelineIterations <= graphed; it0 += kPipelineIterations) {
        CK(cudaGraphLaunch(c->graph_many, s), "cudaGraphLaunch");
        c->launches += per_iter * kPipelineIterations;
      }
    for (int it = it0; it + 1 < graphed; it += 2) {
      CK(cudaGraphLaunch(c->graph_pair, s), "cudaGraphLaunch");
      c->launches += 2 * per_iter;
    }
    if ((graphed - it0) & 1) {
      CK(cudaGraphLaunch(c->graph_one, s), "cudaGraphLaunch");
      c->launches += per_iter;
    }
    if (c->dag && c->iterations > 0) {
      rc = launch_flow(c, graphed & 1, s);
      c->dag_last = true;
      if (!rc) rc = launch_tree(c, s);
      c->dag_last = false;
      if (rc) return rc;
    }
  }
  // final flows live in set (iterations & 1); nothing else depends on parity
  // (REF_CPU leaves the flows at zero in set 0)
  c->flow_parity = c->semantics == HMF_SEMANTICS_REF_CUDA ? (c->iterations & 1) : 0;
  c->continuable = true;
  return end_solve(c, user);
}

}  // namespace hmfi

extern "C" {

int hmf_create_batch(hmf_ctx** out, int n_volumes, const int* dims, const int* parent, int n_nodes,
                     int semantics, int device) {
  return create_context(out, n_volumes, dims, semantics, device,
                        [&](hmf_ctx* c) { return build_tree(c, parent, n_nodes); });
}

int hmf_create_dag(hmf_ctx** out, int vx, int vy, int vz, int n_nodes, int n_edges, const int* edge_parent,
                   const int* edge_child, const float* edge_weight, int semantics, int device) {
  if (semantics == HMF_SEMANTICS_REF_CPU) {
    g_create_error = "REF_CPU semantics is not available for graphs: the reference CPU class reads past its "
                     "flow buffers (vtkMaxFlowSegmentationUtilities.cxx:197-200)";
    if (out) *out = nullptr;
    return HMF_ERR_INVALID_ARGUMENT;
  }
  const int dims[3] = {vx, vy, vz};
  return create_context(out, 1, dims, semantics, device, [&](hmf_ctx* c) {
    return build_dag(c, n_nodes, n_edges, edge_parent, edge_child, edge_weight);
  });
}

int hmf_create(hmf_ctx** out, int vx, int vy, int vz, const int* parent, int n_nodes, int semantics,
               int device) {
  const int dims[3] = {vx, vy, vz};
  return hmf_create_batch(out, 1, dims, parent, n_nodes, semantics, device);
}

int hmf_create_paged(hmf_ctx** out, int vx, int vy, int vz, const int* parent, int n_nodes, int semantics,
                     int device, double max_gpu_usage) {
  const int dims[3] = {vx, vy, vz};
  hmf_ctx* c = nullptr;
  int rc = create_context(&c, 1, dims, semantics, device, [&](hmf_ctx* k) { return build_tree(k, parent, n_nodes); },
                          false);
  if (rc) {
    if (out) *out = nullptr;
    return rc;
  }
  rc = paged_setup(c, max_gpu_usage);
  if (rc) {
    g_create_error = c->err;
    hmf_destroy(c);
    *out = nullptr;
    return rc;
  }
  *out = c;
  return HMF_OK;
}

int hmf_destroy(hmf_ctx* c) {
  if (!c) return HMF_OK;
  DeviceGuard dg(c->device);
  paged_free(c);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->graph_pair) cudaGraphExecDestroy(c->graph_pair);
  if (c->graph_one) cudaGraphExecDestroy(c->graph_one);
  if (c->graph_many) cudaGraphExecDestroy(c->graph_many);
  if (c->d_tree_slabs) cudaFree(c->d_tree_slabs);
  for (auto st : c->slab_streams) cudaStreamDestroy(st);
  for (auto ev : c->slab_ev_flow) cudaEventDestroy(ev);
  for (auto ev : c->slab_ev_sweep) cudaEventDestroy(ev);
  if (c->arena) cudaFree(c->arena);
  if (c->staging) cudaFree(c->staging);
  if (c->d_flow[0]) cudaFree(c->d_flow[0]);
  if (c->d_tma) cudaFree(c->d_tma);
  if (c->d_fvol) cudaFree(c->d_fvol);
  if (c->d_items) cudaFree(c->d_items);
  if (c->d_tree) cudaFree(c->d_tree);
  if (c->d_dag) cudaFree(c->d_dag);
  if (c->d_smooth_list) cudaFree(c->d_smooth_list);
  if (c->d_error) cudaFree(c->d_error);
  if (c->h_error) cudaFreeHost(c->h_error);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  if (c->ev_t0) cudaEventDestroy(c->ev_t0);
  if (c->ev_t1) cudaEventDestroy(c->ev_t1);
  adjoint_free(c);
  fp64_free(c);
  if (c->d_post) cudaFree(c->d_post);
  if (c->d_gap) cudaFree(c->d_gap);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return HMF_OK;
}

int hmf_batch_set_data(hmf_ctx* c, int volume, int node, const float* data, int where) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (!valid_volume(c, volume)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "volume index out of range");
  if (!valid_vertex(c, node)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "vertex id out of range");
  if (where != HMF_HOST && where != HMF_DEVICE) return fail(c, HMF_ERR_INVALID_ARGUMENT, "bad `where`");
  if (!c->kids[node].empty())
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "data terms are only used for leaves");
  if (where == HMF_DEVICE && data) {
    DeviceGuard dg(c->device);
    if (int rc = check_device_pointer(c, data, "data term")) return rc;
  }
  c->data[volume][node] = {data, where};
  return HMF_OK;
}

int hmf_set_data(hmf_ctx* c, int node, const float* data, int where) {
  return hmf_batch_set_data(c, 0, node, data, where);
}

int hmf_batch_set_smoothness(hmf_ctx* c, int volume, int node, const float* smooth, int where) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (!valid_volume(c, volume)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "volume index out of range");
  if (!valid_vertex(c, node)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "vertex id out of range");
  if (where != HMF_HOST && where != HMF_DEVICE) return fail(c, HMF_ERR_INVALID_ARGUMENT, "bad `where`");
  if (node == c->root) return fail(c, HMF_ERR_INVALID_ARGUMENT, "the root has no smoothness term");
  if (where == HMF_DEVICE && smooth) {
    DeviceGuard dg(c->device);
    if (int rc = check_device_pointer(c, smooth, "smoothness image")) return rc;
  }
  c->smooth[volume][node] = {smooth, where};
  return HMF_OK;
}

int hmf_set_smoothness(hmf_ctx* c, int node, const float* smooth, int where) {
  return hmf_batch_set_smoothness(c, 0, node, smooth, where);
}

int hmf_set_smoothness_scalar(hmf_ctx* c, int node, double alpha) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (!valid_vertex(c, node)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "vertex id out of range");
  if (!(alpha >= 0.0)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "Cannot use a negative smoothness value.");
  c->alpha[node] = alpha;
  return HMF_OK;
}

int hmf_set_params(hmf_ctx* c, int iterations, float step_size, float cc) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  const float step = std::min(1.0f, std::max(0.0f, step_size));
  const float ccc = std::min(1.0f, std::max(0.0f, cc));
  if (step != c->step || ccc != c->cc) {
    // the captured iteration graphs hold StepSize and 1/CC as kernel arguments
    DeviceGuard dg(c->device);
    drop_graphs(c);
  }
  c->iterations = std::max(0, iterations);
  c->step = step;
  c->cc = ccc;
  return HMF_OK;
}

int hmf_solve(hmf_ctx* c, void* stream) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  DeviceGuard dg(c->device);
  cudaStream_t user = reinterpret_cast<cudaStream_t>(stream);
  if (c->pg) return paged_solve(c, user);
  return solve_with(c, user, nullptr, nullptr);
}

namespace {
// StateLoader of hmf_solve_continue: the state is the last run's, in place;
// the replayed iterations start from flow set 0, so flows left in set 1 by
// an odd iteration count move there first (device copies, exact).
int continue_state(hmf_ctx* c, cudaStream_t s, void*) {
  if (c->flow_parity == 0) return HMF_OK;
  const size_t bytes = (size_t)c->total * sizeof(float);
  for (int v = 0; v < c->n; ++v) {
    if (v == c->root) continue;
    CK(cudaMemcpyAsync(c->fx[0][v], c->fx[1][v], bytes, cudaMemcpyDeviceToDevice, s), "cudaMemcpyAsync(flows)");
    CK(cudaMemcpyAsync(c->fy[0][v], c->fy[1][v], bytes, cudaMemcpyDeviceToDevice, s), "cudaMemcpyAsync(flows)");
    CK(cudaMemcpyAsync(c->fz[0][v], c->fz[1][v], bytes, cudaMemcpyDeviceToDevice, s), "cudaMemcpyAsync(flows)");
  }
  c->flow_parity = 0;
  return HMF_OK;
}
}  // namespace

int hmf_solve_continue(hmf_ctx* c, void* stream) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (c->dag)
    return fail(c, HMF_ERR_INVALID_ARGUMENT,
                "graphs (hmf_create_dag) cannot continue: their last iteration runs fewer tasks");
  // the adjoint and the autotuner leave other state in the solver's arrays
  // (neither runs on an out-of-core context)
  if (!c->solved || !c->continuable)
    return fail(c, HMF_ERR_STATE, "hmf_solve_continue follows hmf_solve or hmf_solve_continue");
  DeviceGuard dg(c->device);
  // out of core: the state is the host copy the last solve ended in
  if (c->pg) return paged_solve(c, reinterpret_cast<cudaStream_t>(stream), true);
  return solve_with(c, reinterpret_cast<cudaStream_t>(stream), continue_state, nullptr);
}

int hmf_autotune(hmf_ctx* c, void* stream) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (int rc = refuse_paged(c, "hmf_autotune")) return rc;
  if (!c->use_tma || c->semantics != HMF_SEMANTICS_REF_CUDA) return HMF_OK;
  const int saved_iters = c->iterations;
  const bool saved_timing = c->timing;
  int maxz = 1;
  for (const auto& V : c->vols) maxz = std::max(maxz, V.vz);
  TunedPlan best{c->flow_warps, c->zchunk, c->flow_units};
  double best_ms = 1e30;
  int rc = HMF_OK;
  DeviceGuard dg(c->device);
  cudaStream_t user = reinterpret_cast<cudaStream_t>(stream);
  // Each candidate is timed as the solve runs it (graph replay, the slab
  // pipeline when on): a warm solve captures the plan's graphs, two more are
  // timed with events on the caller's stream and the faster counts.  The
  // solves run kTuneIterations iterations, more when the default plan does
  // them in under 2 ms (small volumes), so that launch jitter does not pick
  // the plan; a candidate must beat the incumbent by 1 % to replace it (the
  // default plan is timed first).  Candidates, for each window shape
  // (32 x 32 and 32 x 64): the default plan's chunk, then 16, 24, 32, 48, 64,
  // 96, ... up to the longest volume, one unit per CTA; then the best of
  // those with 2 and 4 units (window-vertex marches) per CTA.
  c->timing = false;
  c->iterations = kTuneIterations;
  auto time_plan = [&](int w, int z, int u, float* ms) -> int {
    c->flow_warps = w;
    c->flow_units = u;
    drop_graphs(c);
    int r = plan_flow(c, z);
    if (!r) r = hmf_solve(c, stream);
    *ms = 1e30f;
    for (int rep = 0; rep < 2 && !r; ++rep) {
      cudaError_t e = cudaEventRecord(c->ev_t0, user);
      if (e == cudaSuccess) r = hmf_solve(c, stream);
      if (!r && e == cudaSuccess) e = cudaEventRecord(c->ev_t1, user);
      if (!r && e == cudaSuccess) e = cudaEventSynchronize(c->ev_t1);
      float t = 1e30f;
      if (!r && e == cudaSuccess) e = cudaEventElapsedTime(&t, c->ev_t0, c->ev_t1);
      if (!r && e != cudaSuccess) r = cuda_fail(c, e, "autotune timing");
      *ms = std::min(*ms, t);
    }
    return r;
  };
  auto consider = [&](float ms, const TunedPlan& p) {
    if (ms < best_ms * 0.99) best_ms = ms, best = p;
  };
  {
    float ms = 0;
    c->flow_warps = 8;
    rc = time_plan(8, default_zchunk(c), 1, &ms);
    if (!rc && ms < 2.0f)
      c->iterations = std::min(kTuneIterations * 32, (int)(kTuneIterations * std::ceil(2.0f / std::max(ms, 0.01f))));
  }
  for (int w : {8, 16}) {
    if (rc) break;
    c->flow_warps = w;
    const int z_default = default_zchunk(c);
    for (int i = -1; rc == HMF_OK; ++i) {
      const int z = i < 0 ? z_default : std::min((i & 1 ? 24 : 16) << (i >> 1), maxz);
      float ms = 0;
      rc = time_plan(w, z, 1, &ms);
      if (rc) break;
      consider(ms, TunedPlan{w, z, 1});
      if (i >= 0 && z >= maxz) break;
    }
  }
  for (int u : {2, 4}) {
    if (rc) break;
    float ms = 0;
    rc = time_plan(best.warps, best.zchunk, u, &ms);
    if (!rc) consider(ms, TunedPlan{best.warps, best.zchunk, u});
  }
  c->iterations = saved_iters;
  c->timing = saved_timing;
  c->solved = false;
  c->flow_warps = best.warps;
  c->flow_units = best.units;
  if (rc) return rc;
  drop_graphs(c);
  rc = plan_flow(c, best.zchunk);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  const std::string key = tune_key(c);
  g_tune_cache[key] = best;
  tune_file_append(key, best);
  return HMF_OK;
}

int hmf_set_pipeline(hmf_ctx* c, int enabled) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (int rc = refuse_paged(c, "hmf_set_pipeline")) return rc;
  if ((enabled != 0) == c->pipeline) return HMF_OK;
  DeviceGuard dg(c->device);
  drop_graphs(c);
  c->pipeline = enabled != 0;
  return HMF_OK;
}

int hmf_get_pipeline(const hmf_ctx* c) { return c ? (pipeline_active(c) ? 1 : 0) : HMF_ERR_INVALID_ARGUMENT; }

int hmf_set_flow_window(hmf_ctx* c, int rows) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (int rc = refuse_paged(c, "hmf_set_flow_window")) return rc;
  if (rows != 0 && rows != 32 && rows != 64)
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "flow window rows must be 32 or 64 (0: default)");
  DeviceGuard dg(c->device);
  drop_graphs(c);
  c->flow_warps = rows == 64 ? 16 : 8;
  return plan_flow(c, default_zchunk(c));
}

int hmf_get_flow_window(const hmf_ctx* c) { return c ? 4 * c->flow_warps : HMF_ERR_INVALID_ARGUMENT; }

int hmf_set_flow_units(hmf_ctx* c, int units) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (int rc = refuse_paged(c, "hmf_set_flow_units")) return rc;
  if (units < 0 || units > kMaxFlowUnits)
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "units per flow CTA must lie in [0, 64]");
  DeviceGuard dg(c->device);
  drop_graphs(c);  // the captured launches carry the grid
  c->flow_units = units ? units : 1;
  return HMF_OK;
}

int hmf_get_flow_units(const hmf_ctx* c) { return c ? c->flow_units : HMF_ERR_INVALID_ARGUMENT; }

int hmf_set_zchunk(hmf_ctx* c, int z) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (int rc = refuse_paged(c, "hmf_set_zchunk")) return rc;
  if (z < 0) return fail(c, HMF_ERR_INVALID_ARGUMENT, "the z chunk must be >= 0 (0: default plan)");
  DeviceGuard dg(c->device);
  drop_graphs(c);
  int maxz = 1;
  for (const auto& V : c->vols) maxz = std::max(maxz, V.vz);
  return plan_flow(c, z ? std::min(z, maxz) : default_zchunk(c));
}

int hmf_get_zchunk(const hmf_ctx* c) { return c ? c->zchunk : HMF_ERR_INVALID_ARGUMENT; }

int hmf_set_convergence_log(hmf_ctx* c, int enabled) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (int rc = refuse_paged(c, "hmf_set_convergence_log")) return rc;
  if (enabled) {
    if (c->dag) return fail(c, HMF_ERR_INVALID_ARGUMENT, "the convergence log is for label trees (hmf_create)");
    if (c->semantics != HMF_SEMANTICS_REF_CUDA)
      return fail(c, HMF_ERR_INVALID_ARGUMENT, "the convergence log needs REF_CUDA semantics");
    if (c->tree_kind != 0)
      return fail(c, HMF_ERR_INVALID_ARGUMENT, "the convergence log runs in the staged sweep kernels only");
    if (c->vols.size() > 1)
      for (const auto& V : c->vols)
        if (V.pitch != V.vx)
          return fail(c, HMF_ERR_INVALID_ARGUMENT,
                      "the convergence log of a batch needs every volume's VX to be a multiple of 4");
  }
  if ((enabled != 0) == c->gap_on) return HMF_OK;
  DeviceGuard dg(c->device);
  drop_graphs(c);  // the captured sweeps differ
  c->gap_on = enabled != 0;
  return HMF_OK;
}

int hmf_get_convergence(hmf_ctx* c, double* max_change, double* mean_change, int capacity) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (int rc = refuse_paged(c, "hmf_get_convergence")) return rc;
  if (capacity < 0) return fail(c, HMF_ERR_INVALID_ARGUMENT, "capacity must be >= 0");
  const int n = std::min(capacity, c->gap_logged);
  if (n == 0) return c->gap_logged;
  DeviceGuard dg(c->device);
  const hmf::GapLog g = gap_view(c, 0);
  std::vector<unsigned int> bits(n);
  std::vector<double> sums(n);
  CK(cudaMemcpyAsync(bits.data(), g.max_bits, 4 * (size_t)n, cudaMemcpyDeviceToHost, c->stream),
     "cudaMemcpyAsync(convergence log)");
  CK(cudaMemcpyAsync(sums.data(), g.sum, 8 * (size_t)n, cudaMemcpyDeviceToHost, c->stream),
     "cudaMemcpyAsync(convergence log)");
  CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize(convergence log)");
  double voxels = 0;
  for (const auto& V : c->vols) voxels += (double)V.vx * V.vy * V.vz;
  const double count = voxels * (double)(c->n - 1);
  for (int i = 0; i < n; ++i) {
    float f;
    std::memcpy(&f, &bits[i], 4);
    if (max_change) max_change[i] = f;
    if (mean_change) mean_change[i] = sums[i] / count;
  }
  return c->gap_logged;
}

int hmf_set_wait_limit(hmf_ctx* c, long long limit_ns) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (int rc = refuse_paged(c, "hmf_set_wait_limit")) return rc;
  if (limit_ns < 0) return fail(c, HMF_ERR_INVALID_ARGUMENT, "the wait limit must be >= 0 (0: default)");
  const unsigned long long v = limit_ns ? (unsigned long long)limit_ns : hmf::kTmaWaitLimitNs;
  if (v == c->wait_limit_ns) return HMF_OK;
  DeviceGuard dg(c->device);
  drop_graphs(c);  // the captured launches carry the old bound
  c->wait_limit_ns = v;
  return HMF_OK;
}

int hmf_inject_wait_stall(hmf_ctx* c, int kernel) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (int rc = refuse_paged(c, "hmf_inject_wait_stall")) return rc;
  if (kernel < -1 || kernel > HMF_STALL_REVERSE_SWEEP) return fail(c, HMF_ERR_INVALID_ARGUMENT, "unknown kernel");
  c->stall_kind = kernel;
  return HMF_OK;
}

int hmf_batch_get_labels(hmf_ctx* c, int volume, int node, float* out, int where, void* stream) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (!valid_volume(c, volume)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "volume index out of range");
  if (!valid_vertex(c, node) || node == c->root)
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "labels exist for non-root vertices only");
  if (!c->solved) return fail(c, HMF_ERR_STATE, "hmf_solve has not run");
  if (c->pg) return paged_copy_out(c, true, node, out, where, stream);
  return copy_out(c, volume, c->label[node], out, where, stream);
}

int hmf_get_labels(hmf_ctx* c, int node, float* out, int where, void* stream) {
  return hmf_batch_get_labels(c, 0, node, out, where, stream);
}

int hmf_batch_get_sink(hmf_ctx* c, int volume, int node, float* out, int where, void* stream) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (!valid_volume(c, volume)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "volume index out of range");
  if (!valid_vertex(c, node)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "vertex id out of range");
  if (!c->solved) return fail(c, HMF_ERR_STATE, "hmf_solve has not run");
  if (c->pg) return paged_copy_out(c, false, node, out, where, stream);
  return copy_out(c, volume, c->sink[node], out, where, stream);
}

int hmf_get_sink(hmf_ctx* c, int node, float* out, int where, void* stream) {
  return hmf_batch_get_sink(c, 0, node, out, where, stream);
}

int hmf_num_volumes(const hmf_ctx* c) { return c ? (int)c->vols.size() : HMF_ERR_INVALID_ARGUMENT; }

int hmf_leaf_order(const hmf_ctx* c, int* out, int cap) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  const int nl = (int)c->leaves.size();
  for (int i = 0; i < nl && i < cap && out; ++i) out[i] = c->leaves[i];
  return nl;
}

size_t hmf_device_bytes(const hmf_ctx* c) {
  if (!c) return 0;
  if (c->pg) return paged_bytes(c);
  return c->arena_bytes + c->staging_bytes + adjoint_bytes(c) + fp64_bytes(c) + sizeof(hmf::FlowVertex) * hmf::kMaxVertices * 2 +
         sizeof(hmf::FlowVertexTMA) * c->vols.size() * (c->n - 1) + sizeof(hmf::TreeTable) +
         sizeof(hmf::FlowItem) * c->h_items.size();
}

int hmf_set_timing(hmf_ctx* c, int enabled) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  c->timing = enabled != 0;
  return HMF_OK;
}

int hmf_get_stats(const hmf_ctx* c, long long* launches, double* avg_ms, int n_kinds) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (launches) *launches = c->launches;
  for (int k = 0; k < n_kinds && k < 3 && avg_ms; ++k)
    avg_ms[k] = c->kind_count[k] ? c->kind_ms[k] / (double)c->kind_count[k] : 0.0;
  return HMF_OK;
}

const char* hmf_last_error(const hmf_ctx* c) { return c ? c->err.c_str() : g_create_error.c_str(); }

}  // extern "C"

// ---------------------------------------------------------------------------
// hmf_solve_noalloc: the solve above with every device buffer carved out of
// one static array of this library instead of cudaMalloc, for callers that
// must not allocate device memory (see include/hmf.h).
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocBytes = HMF_NOALLOC_SCRATCH_BYTES;
constexpr int kNoAllocMaxDevices = 64;

// Held on every GPU that loads this library, until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of g_noalloc_scratch in the current context.  In host code
// the symbol itself is only a stand-in, so the address is looked up on every
// call (no allocation), with the device current, and handed to the kernels:
// a cached address would outlive a cudaDeviceReset, after which the module
// (and the array) are loaded again elsewhere.
std::mutex g_noalloc_mutex;

int noalloc_fail(int code, const char* msg) {
  g_create_error = msg;
  return code;
}

int noalloc_cuda_fail(cudaError_t e, const char* what) {
  g_create_error = std::string(what) + ": " + cudaGetErrorString(e);
  return HMF_ERR_CUDA;
}

#define NCK(call, what)                                     \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return noalloc_cuda_fail(e_, what); \
  } while (0)

int noalloc_setup(int device, unsigned char** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (device < 0 || device >= kNoAllocMaxDevices)
    return noalloc_fail(HMF_ERR_CUDA, "device ordinal beyond the supported range");
  void* p = nullptr;
  NCK(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(scratch)");
  NCK(cudaFuncSetAttribute(hmf::flow_kernel<kTX, kTY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           hmf::FlowTile<kTX, kTY>::SMEM_BYTES),
      "cudaFuncSetAttribute(flow_kernel)");
  NCK(cudaFuncSetAttribute(hmf::tree_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           3 * hmf::kMaxVertices * kTreeThreads * (int)sizeof(float)),
      "cudaFuncSetAttribute(tree_kernel)");
  NCK(cudaFuncSetAttribute(hmf::init_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           hmf::kMaxVertices * kTreeThreads * (int)sizeof(float)),
      "cudaFuncSetAttribute(init_kernel)");
  *out = static_cast<unsigned char*>(p);
  return HMF_OK;
}

// Fixed-size tree bookkeeping (no heap): children in increasing id order,
// DFS pre-order leaves, post-order entries with the root last.
struct NoAllocTree {
  int n = 0, root = -1, n_leaves = 0;
  int parent[hmf::kMaxVertices];
  int n_kids[hmf::kMaxVertices];
  int kids[hmf::kMaxVertices][hmf::kMaxVertices];
  int preorder[hmf::kMaxVertices];
  int postorder[hmf::kMaxVertices];
  int leaves[hmf::kMaxVertices];
};

int noalloc_tree(const int* par, int n, NoAllocTree& t) {
  if (!par || n < 2) return noalloc_fail(HMF_ERR_TREE, "the tree needs a root and at least one leaf");
  if (n > hmf::kMaxVertices) return noalloc_fail(HMF_ERR_TREE, "the tree has too many vertices");
  t.n = n;
  for (int v = 0; v < n; ++v) t.n_kids[v] = 0;
  for (int v = 0; v < n; ++v) {
    const int p = par[v];
    t.parent[v] = p;
    if (p < 0) {
      if (t.root >= 0) return noalloc_fail(HMF_ERR_TREE, "the tree has more than one root");
      t.root = v;
    } else if (p >= n || p == v) {
      return noalloc_fail(HMF_ERR_TREE, "tree parent id out of range");
    } else {
      t.kids[p][t.n_kids[p]++] = v;
    }
  }
  if (t.root < 0) return noalloc_fail(HMF_ERR_TREE, "the tree has no root");
  int stack[hmf::kMaxVertices], top = 0, count = 0;
  bool seen[hmf::kMaxVertices] = {};
  stack[top++] = t.root;
  while (top) {
    const int v = stack[--top];
    if (seen[v]) return noalloc_fail(HMF_ERR_TREE, "the tree has a cycle");
    seen[v] = true;
    t.preorder[count++] = v;
    for (int k = t.n_kids[v] - 1; k >= 0; --k) {
      if (top >= hmf::kMaxVertices) return noalloc_fail(HMF_ERR_TREE, "the tree has a cycle");
      stack[top++] = t.kids[v][k];
    }
  }
  if (count != n) return noalloc_fail(HMF_ERR_TREE, "the tree is not connected");
  for (int i = 0; i < n; ++i)
    if (t.n_kids[t.preorder[i]] == 0) t.leaves[t.n_leaves++] = t.preorder[i];
  int vst[hmf::kMaxVertices], kst[hmf::kMaxVertices], depth = 0, m = 0;
  vst[0] = t.root;
  kst[0] = 0;
  depth = 1;
  while (depth) {
    const int v = vst[depth - 1];
    if (kst[depth - 1] < t.n_kids[v]) {
      const int kid = t.kids[v][kst[depth - 1]++];
      vst[depth] = kid;
      kst[depth] = 0;
      ++depth;
    } else {
      t.postorder[m++] = v;
      --depth;
    }
  }
  return HMF_OK;
}

}  // namespace

extern "C" int hmf_solve_noalloc(int vx, int vy, int vz, const int* parent, int n_nodes, int semantics,
                                 const float* const* data, const float* const* smooth, const double* alpha,
                                 int iterations, float step_size, float cc, float* const* labels,
                                 void* stream) {
  if (vx <= 0 || vy <= 0 || vz <= 0)
    return noalloc_fail(HMF_ERR_INVALID_ARGUMENT, "volume dimensions must be positive");
  if (vx > kMaxDim || vy > kMaxDim || vz > kMaxDim)
    return noalloc_fail(HMF_ERR_INVALID_ARGUMENT, "volume dimensions above 2^30 are not supported");
  if (semantics != HMF_SEMANTICS_REF_CUDA && semantics != HMF_SEMANTICS_REF_CPU)
    return noalloc_fail(HMF_ERR_INVALID_ARGUMENT, "unknown semantics");
  if (!data) return noalloc_fail(HMF_ERR_MISSING_INPUT, "Missing data prior for leaf node.");
  NoAllocTree t;
  int rc = noalloc_tree(parent, n_nodes, t);
  if (rc) return rc;
  for (int j = 0; j < t.n_leaves; ++j)
    if (!data[t.leaves[j]]) return noalloc_fail(HMF_ERR_MISSING_INPUT, "Missing data prior for leaf node.");
  for (int v = 0; v < t.n; ++v)
    if (alpha && v != t.root && !(alpha[v] >= 0.0))
      return noalloc_fail(HMF_ERR_INVALID_ARGUMENT, "Cannot use a negative smoothness value.");
  {  // the caller's buffers the kernels and copies will touch
    std::vector<const void*> bufs;
    for (int j = 0; j < t.n_leaves; ++j) bufs.push_back(data[t.leaves[j]]);
    for (int v = 0; v < t.n; ++v)
      if (v != t.root) {
        if (smooth) bufs.push_back(smooth[v]);
        if (labels) bufs.push_back(labels[v]);
      }
    for (const void* q : bufs) {
      const std::string why = device_pointer_problem(q);
      if (!why.empty()) return noalloc_fail(HMF_ERR_INVALID_ARGUMENT, ("hmf_solve_noalloc: " + why).c_str());
    }
  }
  iterations = std::max(0, iterations);
  step_size = std::min(1.0f, std::max(0.0f, step_size));
  cc = std::min(1.0f, std::max(0.0f, cc));

  hmf::Geometry G;
  G.vx = vx;
  G.vy = vy;
  G.vz = vz;
  G.pitch = (vx + 3) / 4 * 4;
  G.plane = (long long)G.pitch * vy;
  G.vol = G.plane * vz;

  // distinct smoothness images
  const float* distinct[hmf::kMaxVertices];
  int slot_of[hmf::kMaxVertices];
  int n_distinct = 0;
  for (int v = 0; v < t.n; ++v) {
    slot_of[v] = -1;
    if (v == t.root || !smooth || !smooth[v]) continue;
    int s = 0;
    while (s < n_distinct && distinct[s] != smooth[v]) ++s;
    if (s == n_distinct) distinct[n_distinct++] = smooth[v];
    slot_of[v] = s;
  }

  // scratch plan: tables, then state arrays, then pitched input copies
  const size_t arr = round_up((size_t)G.vol * sizeof(float), 256);
  const size_t tables = round_up(sizeof(hmf::FlowVertex) * hmf::kMaxVertices * 2, 256) +
                        round_up(sizeof(hmf::TreeTable), 256) + round_up(sizeof(float*) * hmf::kMaxVertices, 256) +
                        256;
  const size_t n_arrays = (size_t)9 * (t.n - 1) + 1 + t.n_leaves + n_distinct;
  if ((size_t)G.vol > (kNoAllocBytes / sizeof(float)) || n_arrays > kNoAllocBytes / arr ||
      tables + n_arrays * arr > kNoAllocBytes)
    return noalloc_fail(HMF_ERR_INVALID_ARGUMENT,
                        "problem too large for hmf_solve_noalloc: its state exceeds the 64 MiB static scratch "
                        "array; use hmf_create / hmf_solve");

  int device = 0;
  NCK(cudaGetDevice(&device), "cudaGetDevice");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  // the call stages its tables from this frame and waits for its stream:
  // nothing of it can be recorded into a graph
  cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
  NCK(cudaStreamIsCapturing(s, &capturing), "cudaStreamIsCapturing");
  if (capturing != cudaStreamCaptureStatusNone)
    return noalloc_fail(HMF_ERR_INVALID_ARGUMENT, "hmf_solve_noalloc cannot run inside a stream capture");
  unsigned char* base = nullptr;
  rc = noalloc_setup(device, &base);
  if (rc) return rc;
  int sm_count = 0;
  NCK(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device), "cudaDeviceGetAttribute");

  unsigned char* p = base;
  auto* d_flow = reinterpret_cast<hmf::FlowVertex*>(p);
  p += round_up(sizeof(hmf::FlowVertex) * hmf::kMaxVertices * 2, 256);
  auto* d_tree = reinterpret_cast<hmf::TreeTable*>(p);
  p += round_up(sizeof(hmf::TreeTable), 256);
  auto* d_smooth_list = reinterpret_cast<const float**>(p);
  p += round_up(sizeof(float*) * hmf::kMaxVertices, 256);
  int* d_error = reinterpret_cast<int*>(p);
  p += 256;
  auto take = [&]() {
    float* r = reinterpret_cast<float*>(p);
    p += arr;
    return r;
  };
  float* sink[hmf::kMaxVertices] = {};
  float* label[hmf::kMaxVertices] = {};
  float* div[hmf::kMaxVertices] = {};
  float* fl[2][3][hmf::kMaxVertices] = {};
  for (int v = 0; v < t.n; ++v) {
    sink[v] = take();
    if (v == t.root) continue;
    label[v] = take();
    div[v] = take();
    for (int par = 0; par < 2; ++par)
      for (int a = 0; a < 3; ++a) fl[par][a][v] = take();
  }
  const float* d_data[hmf::kMaxVertices] = {};
  const float* d_distinct[hmf::kMaxVertices] = {};
  for (int j = 0; j < t.n_leaves; ++j) d_data[t.leaves[j]] = take();
  for (int k = 0; k < n_distinct; ++k) d_distinct[k] = take();
  const size_t used = (size_t)(p - base);

  // everything this call uses starts at zero
  NCK(cudaMemsetAsync(base, 0, used, s), "cudaMemsetAsync(scratch)");
  const size_t row = (size_t)vx * sizeof(float), prow = (size_t)G.pitch * sizeof(float);
  for (int j = 0; j < t.n_leaves; ++j)
    NCK(cudaMemcpy2DAsync(const_cast<float*>(d_data[t.leaves[j]]), prow, data[t.leaves[j]], row, row,
                          (size_t)vy * vz, cudaMemcpyDeviceToDevice, s),
        "cudaMemcpy2DAsync(data)");
  for (int k = 0; k < n_distinct; ++k)
    NCK(cudaMemcpy2DAsync(const_cast<float*>(d_distinct[k]), prow, distinct[k], row, row, (size_t)vy * vz,
                          cudaMemcpyDeviceToDevice, s),
        "cudaMemcpy2DAsync(smoothness)");

  // tables, built on the host stack and staged by the (pageable) copies
  hmf::FlowVertex fv[2 * hmf::kMaxVertices];
  std::memset(fv, 0, sizeof(fv));
  int slot = 0;
  for (int i = 0; i < t.n; ++i) {
    const int v = t.preorder[i];
    if (v == t.root) continue;
    for (int par = 0; par < 2; ++par) {
      hmf::FlowVertex& f = fv[par * hmf::kMaxVertices + slot];
      f.px_in = fl[par][0][v];
      f.py_in = fl[par][1][v];
      f.pz_in = fl[par][2][v];
      f.px_out = fl[par ^ 1][0][v];
      f.py_out = fl[par ^ 1][1][v];
      f.pz_out = fl[par ^ 1][2][v];
      f.sink = sink[v];
      f.inc = sink[t.parent[v]];
      f.label = label[v];
      f.smooth = slot_of[v] >= 0 ? d_distinct[slot_of[v]] : nullptr;
      f.div = div[v];
      f.alpha = alpha ? (float)alpha[v] : 1.0f;
    }
    ++slot;
  }
  static_assert(sizeof(hmf::TreeTable) < 16384, "tree table size");
  hmf::TreeTable tt;
  std::memset(&tt, 0, sizeof(tt));
  int entry[hmf::kMaxVertices];
  for (int i = 0; i < t.n; ++i) entry[t.postorder[i]] = i;
  tt.n = t.n;
  tt.n_leaves = t.n_leaves;
  tt.cc = cc;
  tt.icc = 1.0f / cc;
  tt.root_init = 1.0f / cc;
  int kpos = 0;
  for (int i = 0; i < t.n; ++i) {
    const int v = t.postorder[i];
    hmf::TreeEntry& E = tt.e[i];
    E.sink = E.sink_out = sink[v];
    E.label = E.label_out = v == t.root ? nullptr : label[v];
    E.div = v == t.root ? nullptr : div[v];
    E.data = d_data[v];
    E.parent = v == t.root ? -1 : entry[t.parent[v]];
    E.first_kid = kpos;
    E.n_kids = t.n_kids[v];
    for (int k = 0; k < t.n_kids[v]; ++k) tt.kids[kpos++] = entry[t.kids[v][k]];
    const int nk = E.n_kids;
    E.inv_kids = nk == 0 ? 0.0f : (v == t.root ? 1.0f / (float)nk : 1.0f / (float)(nk + 1));
  }
  for (int j = 0; j < t.n_leaves; ++j) tt.leaves[j] = entry[t.leaves[j]];
  NCK(cudaMemcpyAsync(d_flow, fv, sizeof(fv), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(flow table)");
  NCK(cudaMemcpyAsync(d_tree, &tt, sizeof(tt), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(tree table)");
  if (n_distinct)
    NCK(cudaMemcpyAsync(d_smooth_list, d_distinct, sizeof(float*) * n_distinct, cudaMemcpyHostToDevice, s),
        "cudaMemcpyAsync(smooth list)");

  // initialisation and iterations, as hmf_solve queues them
  const long long tblocks = (G.vol + kTreeThreads - 1) / kTreeThreads;
  const int tgrid = (int)std::min<long long>(tblocks, (long long)sm_count * 16);
  hmf::init_kernel<<<tgrid, kTreeThreads, (size_t)t.n * kTreeThreads * sizeof(float), s>>>(
      d_tree, G, d_smooth_list, n_distinct, semantics == HMF_SEMANTICS_REF_CPU, d_error);
  NCK(cudaGetLastError(), "init_kernel launch");
  if (semantics == HMF_SEMANTICS_REF_CPU) {
    hmf::refcpu_kernel<<<tgrid, kTreeThreads, 0, s>>>(d_tree, G, iterations);
    NCK(cudaGetLastError(), "refcpu_kernel launch");
  } else {
    hmf::FlowParams fp;
    fp.step = step_size;
    fp.icc = 1.0f / cc;
    fp.tiles_x = (vx + kTX - 1) / kTX;
    const int tiles = fp.tiles_x * ((vy + kTY - 1) / kTY);
    const int nonroot = t.n - 1;
    const long long target = (long long)sm_count * 8;
    int chunks = 1;
    if ((long long)tiles * nonroot < target)
      chunks = (int)std::min<long long>((target + (long long)tiles * nonroot - 1) / ((long long)tiles * nonroot),
                                        std::max(1, vz / 8));
    fp.zchunk = (vz + chunks - 1) / chunks;
    chunks = (vz + fp.zchunk - 1) / fp.zchunk;
    const dim3 fgrid(tiles, chunks, nonroot), fblock(kTX, kTY);
    const size_t tsmem = 3 * (size_t)t.n * kTreeThreads * sizeof(float);
    for (int it = 0; it < iterations; ++it) {
      hmf::flow_kernel<kTX, kTY><<<fgrid, fblock, hmf::FlowTile<kTX, kTY>::SMEM_BYTES, s>>>(
          d_flow + (it & 1) * hmf::kMaxVertices, G, fp);
      NCK(cudaGetLastError(), "flow_kernel launch");
      hmf::tree_kernel<<<tgrid, kTreeThreads, tsmem, s>>>(d_tree, G);
      NCK(cudaGetLastError(), "tree_kernel launch");
    }
  }
  if (labels) {
    for (int v = 0; v < t.n; ++v) {
      if (v == t.root || !labels[v]) continue;
      NCK(cudaMemcpy2DAsync(labels[v], row, label[v], prow, row, (size_t)vy * vz, cudaMemcpyDeviceToDevice, s),
          "cudaMemcpy2DAsync(labels)");
    }
  }
  // the flag is read on the caller's stream, so the wait covers that stream
  // only (a plain cudaMemcpy would wait for every blocking stream)
  int flag = 0;
  NCK(cudaMemcpyAsync(&flag, d_error, sizeof(int), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync(error flag)");
  NCK(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  if (flag)
    return noalloc_fail(HMF_ERR_INVALID_ARGUMENT,
                        "Data prior and smoothness must be non-negative (the solve ran on invalid input)");
  return HMF_OK;
}
