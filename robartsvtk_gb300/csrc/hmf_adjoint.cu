// hmf_adjoint.cu -- hmf_solve_adjoint and the gradient getters of
// include/hmf.h (no counterpart in the reference, which only solves forward).
//
// Forward: the solver's own kernels (flow_tma_kernel, tree_bulk_kernel) run
// over tables that read the state x_t from one state slot and write x_{t+1}
// into another, so keeping a state costs no copy.  Which slots, and which
// states are recomputed later, is the schedule (hmf_schedule.hpp): every
// state kept when HBM holds T + 1 slots; a fixed checkpoint interval k when
// the caller asks for one (ceil(T/k) checkpoint slots + k segment slots);
// otherwise the schedule with the fewest forward iterations over the slots
// that fit.  Recomputed states are bit-identical to the first pass (same
// kernels, same inputs).  One backward step per iteration, from the last to
// the first: adj_sweep_kernel (trees of up to 8 vertices; adj_tree_kernel
// beyond) reverses the sink/label sweep of all vertices, and
// adj_flow_tma_kernel reverses the flow step of every vertex
// (HMF_ADJOINT_KERNEL=chain selects adj_tree_kernel and the unfused
// per-vertex kernels of hmf_adjoint.cuh instead; same results).  Memory:
// the schedule's slots of 6(n-1)+1 arrays, plus 7n float arrays (+11 for
// the unfused kernels) and one double array per leaf; the second set of flow
// adjoints uses the solver's second flow set.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "hmf_adjoint.cuh"
#include "hmf_adjoint_flow.cuh"
#include "hmf_adjoint_sweep.cuh"
#include "hmf_ctx.hpp"
#include "hmf_schedule.hpp"

using namespace hmfi;

namespace {

constexpr int kAdjThreads = 256;
constexpr int kAdjTemps = 11;  // g, ppx, ppy, ppz, m, Fm, F2b, qx, qy, qz, dbo

}  // namespace

struct AdjointState {
  int iterations = 0;
  int A = 0;          // arrays per state slot
  long long arr = 0;  // floats per array (multiple of 64)
  int n_slots = 0;
  AdjSchedule sched;
  std::vector<int> fwd_table;  // per action: index of its forward tables (forward actions)
  int n_pairs = 0;             // distinct (read slot, write slot) pairs of the forward actions
  char* arena = nullptr;
  size_t bytes = 0;
  float* slots = nullptr;             // n_slots state slots
  // [v*arr] sweep part of the sinks' / labels' adjoint.  The sweep reverse
  // reads and writes them voxel by voxel (every read of a voxel before its
  // write, in the same thread), so the old and new parts share one array:
  // sb[1] == sb[0], ub[1] == ub[0].
  float* sb[2] = {nullptr, nullptr};
  float* ub[2] = {nullptr, nullptr};
  float* gb = nullptr;                // [v*arr] adjoint of g of the flow reverse
  float* dbp = nullptr;               // [v*arr]
  // Adjoint of the flows, two sets (the reverse flow kernel reads one and
  // writes the other: its windows read halos their neighbours write).  Set 0
  // is Pb [(v*3 + axis)*arr]; set 1 is the solver's second flow set, idle
  // while the adjoint runs (the forward iterations use the state slots).
  float* Pb = nullptr;
  int pb_par = 0;                     // the set holding the current adjoint of the flows
  float* tmp = nullptr;               // kAdjTemps arrays
  double* Db = nullptr;               // [leaf index * arr]
  int* truth = nullptr;               // dense class indices
  double* scal = nullptr;             // [0] loss, [1 + v] alpha gradient
  const float** d_ctx = nullptr;      // solver arrays in slot order (null: not copied)
  hmf::AdjTree* d_tree = nullptr;
  // forward tables per (read slot, write slot) pair
  hmf::FlowVertexTMA* d_tflow = nullptr;  // [pair][n-1]
  hmf::TreeTable* d_ttree = nullptr;      // [pair]
  int table_cap = 0;
  std::vector<hmf::FlowVertexTMA> h_tflow;
  std::vector<hmf::TreeTable> h_ttree;
  // reverse flow kernel: tables per state slot, its own window plan
  hmf::AdjFlowVertex* d_aflow = nullptr;  // [slot][n-1]
  int aflow_cap = 0;
  std::vector<hmf::AdjFlowVertex> h_aflow;
  hmf::FlowVolume* d_avol = nullptr;
  hmf::FlowItem* d_aitems = nullptr;
  int n_aitems = 0, aitems_cap = 0;
  hmf::FlowVolume h_avol{};
  std::vector<hmf::FlowItem> h_aitems;
  bool chain = false;  // unfused per-vertex reverse kernels and the scalar sweep reverse
  bool done = false;
  double loss = 0.0;
  std::vector<double> alpha_grad;
  hmf::AdjTree h_tree{};
  std::vector<const float*> h_ctx;
};

namespace {

// state-slot array index of the sink of vertex v (non-root j-th in id order)
int slot_base(const hmf_ctx* c, int v) {
  if (v == c->root) return hmf::kAdjPerVertex * (c->n - 1);
  int j = 0;
  for (int u = 0; u < v; ++u) j += u != c->root;
  return hmf::kAdjPerVertex * j;
}

float* slot_ptr(const AdjointState* S, int slot) { return S->slots + (size_t)slot * S->A * S->arr; }
float* slot_array(const AdjointState* S, int slot, int index) {
  return slot_ptr(S, slot) + (size_t)index * S->arr;
}

int grid_for(const hmf_ctx* c, long long n) {
  return (int)std::max<long long>(1, std::min<long long>((n + kAdjThreads - 1) / kAdjThreads, (long long)c->sm_count * 16));
}

int plan(hmf_ctx* c, int T, int k_req) {
  AdjointState* S = c->adj;
  const long long arr = (long long)round_up((size_t)c->total, 64);
  const int A = hmf::kAdjPerVertex * (c->n - 1) + 1;
  const size_t slot_bytes = (size_t)A * arr * sizeof(float);
  const int L = (int)c->leaves.size();
  const int temps = S->chain ? kAdjTemps : 0;  // scratch of the unfused reverse kernels only
  const size_t fixed = ((size_t)(7 * c->n + temps) * arr) * sizeof(float) + (size_t)L * arr * sizeof(double) +
                       (size_t)arr * sizeof(int) + 4096;
  // state slots that fit: the caller's byte budget, else 85% of the free
  // device memory (the held arena is reusable); the caller's slot cap
  double budget = (double)c->adj_max_bytes;
  if (budget <= 0.0) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) free_b = 0;
    budget = 0.85 * (double)(free_b + S->bytes);
  }
  long long fit = budget > (double)fixed ? (long long)((budget - (double)fixed) / (double)slot_bytes) : 0;
  if (c->adj_max_slots > 0) fit = std::min<long long>(fit, c->adj_max_slots);
  if (k_req > 0) {
    S->sched = schedule_fixed(T, k_req);
    if (c->adj_max_slots > 0 && S->sched.slots > c->adj_max_slots) {
      char msg[160];
      std::snprintf(msg, sizeof(msg), "checkpoint interval %d needs %d state slots, more than the %d allowed",
                    k_req, S->sched.slots, c->adj_max_slots);
      return fail(c, HMF_ERR_OUT_OF_MEMORY, msg);
    }
  } else if (T > 0 && fit >= (long long)T + 1) {
    S->sched = schedule_fixed(T, T);  // every state kept
  } else if (!schedule_fewest(T, (int)std::min<long long>(fit, INT32_MAX), &S->sched)) {
    char msg[200];
    std::snprintf(msg, sizeof(msg),
                  "%lld state slots of %.1f MB fit in the adjoint's device memory budget; %d iterations need more",
                  fit, (double)slot_bytes / 1048576.0, T);
    return fail(c, HMF_ERR_OUT_OF_MEMORY, msg);
  }
  const int n_slots = S->sched.slots;
  // forward tables per distinct (read slot, write slot) pair
  {
    std::vector<int> pair_id((size_t)n_slots * n_slots, -1);
    S->fwd_table.assign(S->sched.actions.size(), -1);
    S->n_pairs = 0;
    for (size_t i = 0; i < S->sched.actions.size(); ++i) {
      const AdjAction& x = S->sched.actions[i];
      if (x.kind != kActForward) continue;
      int& id = pair_id[(size_t)x.a * n_slots + x.b];
      if (id < 0) id = S->n_pairs++;
      S->fwd_table[i] = id;
    }
  }
  const size_t need = (size_t)n_slots * slot_bytes + fixed;
  if (need > S->bytes) {
    if (S->arena) cudaFree(S->arena);
    S->arena = nullptr;
    S->bytes = 0;
    CK(cudaMalloc(&S->arena, need), "cudaMalloc(adjoint state)");
    CK(cudaMemsetAsync(S->arena, 0, need, c->stream), "cudaMemsetAsync(adjoint state)");
    S->bytes = need;
  }
  S->iterations = T;
  S->A = A;
  S->arr = arr;
  S->n_slots = n_slots;
  char* p = S->arena;
  auto takef = [&](size_t arrays) {
    float* r = reinterpret_cast<float*>(p);
    p += arrays * arr * sizeof(float);
    return r;
  };
  S->slots = takef((size_t)n_slots * A);
  S->sb[0] = S->sb[1] = takef(c->n);
  S->ub[0] = S->ub[1] = takef(c->n);
  S->gb = takef(c->n);
  S->dbp = takef(c->n);
  S->Pb = takef(3 * (size_t)c->n);
  S->tmp = temps ? takef(temps) : nullptr;
  S->Db = reinterpret_cast<double*>(p);
  p += (size_t)L * arr * sizeof(double);
  S->truth = reinterpret_cast<int*>(p);
  if (S->n_pairs > S->table_cap) {
    if (S->d_tflow) cudaFree(S->d_tflow);
    if (S->d_ttree) cudaFree(S->d_ttree);
    S->d_tflow = nullptr;
    S->d_ttree = nullptr;
    S->table_cap = 0;
    CK(cudaMalloc(&S->d_tflow, sizeof(hmf::FlowVertexTMA) * (size_t)S->n_pairs * (c->n - 1)),
       "cudaMalloc(adjoint flow tables)");
    CK(cudaMalloc(&S->d_ttree, sizeof(hmf::TreeTable) * (size_t)S->n_pairs), "cudaMalloc(adjoint tree tables)");
    S->table_cap = S->n_pairs;
  }
  if (n_slots > S->aflow_cap) {
    if (S->d_aflow) cudaFree(S->d_aflow);
    S->d_aflow = nullptr;
    S->aflow_cap = 0;
    CK(cudaMalloc(&S->d_aflow, sizeof(hmf::AdjFlowVertex) * (size_t)n_slots * (c->n - 1)),
       "cudaMalloc(adjoint reverse tables)");
    S->aflow_cap = n_slots;
  }
  return HMF_OK;
}

float* pb_array(const AdjointState* S, const hmf_ctx* c, int parity, int v, int axis) {
  if (parity == 0) return S->Pb + ((size_t)v * 3 + axis) * S->arr;
  return axis == 0 ? c->fx[1][v] : axis == 1 ? c->fy[1][v] : c->fz[1][v];  // null for the root (no flows)
}

// Windows of at most 27 x 27 outputs spread evenly over the volume; z chunk:
// the one that minimises waves x planes marched per CTA, with one CTA per SM
// and the five halo planes the reverse chain reaches (3 low, 2 high) -- the
// work of a wave is set by its longest CTA, so a last, partial wave costs as
// much as a full one.
int plan_reverse(hmf_ctx* c, cudaStream_t s) {
  AdjointState* S = c->adj;
  const auto& V = c->vols[0];
  hmf::FlowVolume& F = S->h_avol;
  F.G = c->geo;
  const int nx = (V.vx + hmf::kAfMaxOut - 1) / hmf::kAfMaxOut;
  const int ny = (V.vy + hmf::kAfMaxOut - 1) / hmf::kAfMaxOut;
  F.out_x = (V.vx + nx - 1) / nx;
  F.out_y = (V.vy + ny - 1) / ny;
  F.tiles_x = nx;
  const long long per_chunk = (long long)nx * ny * (c->n - 1);
  const int slots = std::max(1, c->sm_count);
  int best_z = V.vz;
  double best = 1e300;
  for (int z = V.vz; z >= 4; --z) {
    const long long chunks = (V.vz + z - 1) / z;
    const long long waves = (per_chunk * chunks + slots - 1) / slots;
    const double cost = (double)waves * (double)(z + 5);
    if (cost < best) best = cost, best_z = z;
  }
  F.zchunk = std::min(best_z, V.vz);
  const int chunks = (V.vz + F.zchunk - 1) / F.zchunk;
  S->h_aitems.clear();
  for (int zc = 0; zc < chunks; ++zc)
    for (int t = 0; t < nx * ny; ++t) S->h_aitems.push_back(hmf::FlowItem{0, t, zc, 0});
  S->n_aitems = (int)S->h_aitems.size();
  if (!S->d_avol) CK(cudaMalloc(&S->d_avol, sizeof(hmf::FlowVolume)), "cudaMalloc(reverse volume table)");
  if (S->n_aitems > S->aitems_cap) {
    if (S->d_aitems) cudaFree(S->d_aitems);
    S->d_aitems = nullptr;
    S->aitems_cap = 0;
    CK(cudaMalloc(&S->d_aitems, sizeof(hmf::FlowItem) * S->n_aitems), "cudaMalloc(reverse work items)");
    S->aitems_cap = S->n_aitems;
  }
  CK(cudaMemcpyAsync(S->d_avol, &F, sizeof(F), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(reverse volume table)");
  CK(cudaMemcpyAsync(S->d_aitems, S->h_aitems.data(), sizeof(hmf::FlowItem) * S->n_aitems, cudaMemcpyHostToDevice,
                     s),
     "cudaMemcpyAsync(reverse work items)");
  return HMF_OK;
}

// Reverse-kernel tables, one per state slot (the state before the iteration).
int build_reverse_tables(hmf_ctx* c, const Staged& staged, cudaStream_t s) {
  AdjointState* S = c->adj;
  const int nv = c->n - 1, n_slots = S->n_slots;
  const auto& V = c->vols[0];
  const int rows = hmf::kAfBoxY;
  S->h_aflow.assign((size_t)n_slots * nv, hmf::AdjFlowVertex{});
  for (int sl = 0; sl < n_slots; ++sl) {
    int j = 0;
    for (int v = 0; v < c->n; ++v) {
      if (v == c->root) continue;
      hmf::AdjFlowVertex& f = S->h_aflow[(size_t)sl * nv + j++];
      std::memset(&f, 0, sizeof(f));
      const int base = slot_base(c, v), pbase = slot_base(c, c->parent[v]);
      int rc = encode_plane_map(c, &f.px, slot_array(S, sl, base + hmf::kAdjPx), V, rows);
      if (!rc) rc = encode_plane_map(c, &f.py, slot_array(S, sl, base + hmf::kAdjPy), V, rows);
      if (!rc) rc = encode_plane_map(c, &f.pz, slot_array(S, sl, base + hmf::kAdjPz), V, rows);
      if (!rc) rc = encode_plane_map(c, &f.s, slot_array(S, sl, base + hmf::kAdjSink), V, rows);
      if (!rc) rc = encode_plane_map(c, &f.c, slot_array(S, sl, pbase + hmf::kAdjSink), V, rows);
      if (!rc) rc = encode_plane_map(c, &f.u, slot_array(S, sl, base + hmf::kAdjLabel), V, rows);
      const bool has_s = staged.smooth[v] && c->smooth[0][v].ptr;
      if (!rc && has_s) rc = encode_plane_map(c, &f.smooth, staged.smooth[v], V, rows);
      for (int par = 0; par < 2 && !rc; ++par)
        for (int ax = 0; ax < 3 && !rc; ++ax) {
          rc = encode_plane_map(c, &f.pb[par][ax], pb_array(S, c, par, v, ax), V, rows);
          f.pb_out[par][ax] = pb_array(S, c, par ^ 1, v, ax);
        }
      if (!rc) rc = encode_plane_map(c, &f.dbp, S->dbp + (size_t)v * S->arr, V, rows);
      if (rc) return rc;
      f.has_smooth = has_s;
      f.gb = S->gb + (size_t)v * S->arr;
      f.alpha_grad = S->scal + 1 + v;
      f.alpha = (float)c->alpha[v];  // stored as float, as the reference does (.cxx:692)
    }
  }
  CK(cudaMemcpyAsync(S->d_aflow, S->h_aflow.data(), sizeof(hmf::AdjFlowVertex) * S->h_aflow.size(),
                     cudaMemcpyHostToDevice, s),
     "cudaMemcpyAsync(adjoint reverse tables)");
  return HMF_OK;
}

int copy_state(hmf_ctx* c, float* slot, bool to_slot, cudaStream_t s) {
  const AdjointState* S = c->adj;
  const dim3 grid((unsigned)std::min<long long>((S->arr / 4 + kAdjThreads - 1) / kAdjThreads, 1024), (unsigned)S->A);
  hmf::adj_state_copy_kernel<<<grid, kAdjThreads, 0, s>>>(S->d_ctx, slot, S->arr, to_slot ? 1 : 0);
  CK(cudaGetLastError(), "adj_state_copy_kernel launch");
  ++c->launches;
  return HMF_OK;
}

// Tables of a forward iteration from slot a to slot b (the same for every
// iteration t): the flow kernel reads the flows, sinks and labels of slot a
// and writes the flows and divergence of slot b; the sweep reads slot a's
// sinks and labels and b's divergence and writes b's sinks and labels.
int build_transition_tables(hmf_ctx* c, const Staged& staged, cudaStream_t s) {
  AdjointState* S = c->adj;
  const int P = S->n_pairs, nv = c->n - 1;
  const auto& V = c->vols[0];
  S->h_tflow.assign((size_t)P * nv, hmf::FlowVertexTMA{});
  S->h_ttree.assign((size_t)P, hmf::TreeTable{});
  std::vector<char> done((size_t)P, 0);
  for (size_t i = 0; i < S->sched.actions.size(); ++i) {
    const int pr = S->fwd_table[i];
    if (pr < 0 || done[pr]) continue;
    done[pr] = 1;
    const int a = S->sched.actions[i].a, b = S->sched.actions[i].b;
    int j = 0;
    for (int v : c->preorder) {
      if (v == c->root) continue;
      hmf::FlowVertexTMA& f = S->h_tflow[(size_t)pr * nv + j++];
      std::memset(&f, 0, sizeof(f));
      const int base = slot_base(c, v), pbase = slot_base(c, c->parent[v]);
      int rc = HMF_OK;
      for (int ax = 0; ax < 3 && !rc; ++ax) {
        rc = encode_plane_map(c, &f.flow_in[0][ax], slot_array(S, a, base + hmf::kAdjPx + ax), V);
        f.flow_in[1][ax] = f.flow_in[0][ax];
        f.flow_out[0][ax] = f.flow_out[1][ax] = slot_array(S, b, base + hmf::kAdjPx + ax);
      }
      if (!rc) rc = encode_plane_map(c, &f.sink, slot_array(S, a, base + hmf::kAdjSink), V);
      if (!rc) rc = encode_plane_map(c, &f.label, slot_array(S, a, base + hmf::kAdjLabel), V);
      if (!rc) rc = encode_plane_map(c, &f.inc, slot_array(S, a, pbase + hmf::kAdjSink), V);
      const bool has_s = staged.smooth[v] && c->smooth[0][v].ptr;
      if (!rc && has_s) rc = encode_plane_map(c, &f.smooth, staged.smooth[v], V);
      if (rc) return rc;
      f.has_smooth = has_s;
      f.div = slot_array(S, b, base + hmf::kAdjDiv);
      f.alpha = (float)c->alpha[v];  // stored as float, as the reference does (.cxx:692)
    }
    hmf::TreeTable& tt = S->h_ttree[pr];
    tt = c->h_tree;  // the solver's own table: tree, constants, data terms
    for (int i = 0; i < c->n; ++i) {
      const int v = c->postorder[i];
      hmf::TreeEntry& E = tt.e[i];
      const int base = slot_base(c, v);
      E.sink = slot_array(S, a, base + hmf::kAdjSink);
      E.sink_out = slot_array(S, b, base + hmf::kAdjSink);
      if (v == c->root) continue;
      E.label = slot_array(S, a, base + hmf::kAdjLabel);
      E.label_out = slot_array(S, b, base + hmf::kAdjLabel);
      E.div = slot_array(S, b, base + hmf::kAdjDiv);
    }
  }
  if (P > 0) {
    CK(cudaMemcpyAsync(S->d_tflow, S->h_tflow.data(), sizeof(hmf::FlowVertexTMA) * S->h_tflow.size(),
                       cudaMemcpyHostToDevice, s),
       "cudaMemcpyAsync(adjoint flow tables)");
    CK(cudaMemcpyAsync(S->d_ttree, S->h_ttree.data(), sizeof(hmf::TreeTable) * S->h_ttree.size(),
                       cudaMemcpyHostToDevice, s),
       "cudaMemcpyAsync(adjoint tree tables)");
  }
  return HMF_OK;
}

// one forward iteration with the tables of pair `pair`
int forward_iteration(hmf_ctx* c, int pair, cudaStream_t s) {
  AdjointState* S = c->adj;
  int rc = launch_flow_tma_with(c, S->d_tflow + (size_t)pair * (c->n - 1), 0, s);
  if (!rc) rc = launch_tree_bulk_with(c, S->d_ttree + pair, s);
  return rc;
}

int prepare_adjoint_tables(hmf_ctx* c, const Staged& staged, cudaStream_t s) {
  AdjointState* S = c->adj;
  const int n = c->n;
  // solver arrays in slot order (flows of set 0, where a solve starts); the
  // divergence is not copied (a slot-0 divergence is never read)
  S->h_ctx.assign((size_t)S->A, nullptr);
  for (int v = 0; v < n; ++v) {
    const int b = slot_base(c, v);
    S->h_ctx[b + hmf::kAdjSink] = c->sink[v];
    if (v == c->root) continue;
    S->h_ctx[b + hmf::kAdjLabel] = c->label[v];
    S->h_ctx[b + hmf::kAdjPx] = c->fx[0][v];
    S->h_ctx[b + hmf::kAdjPy] = c->fy[0][v];
    S->h_ctx[b + hmf::kAdjPz] = c->fz[0][v];
  }
  if (!S->d_ctx)
    CK(cudaMalloc(&S->d_ctx, sizeof(float*) * (hmf::kAdjPerVertex * hmf::kMaxVertices + 1)), "cudaMalloc(adjoint tables)");
  if (!S->d_tree) CK(cudaMalloc(&S->d_tree, sizeof(hmf::AdjTree)), "cudaMalloc(adjoint tree)");
  CK(cudaMemcpyAsync(S->d_ctx, S->h_ctx.data(), sizeof(float*) * S->h_ctx.size(), cudaMemcpyHostToDevice, s),
     "cudaMemcpyAsync(adjoint tables)");
  hmf::AdjTree& T = S->h_tree;
  std::memset(&T, 0, sizeof(T));
  T.n = n;
  T.root = c->root;
  T.cc = c->cc;
  T.icc = 1.0f / c->cc;
  T.step = c->step;
  int kpos = 0;
  for (int v = 0; v < n; ++v) {
    T.parent[v] = c->parent[v];
    T.first_kid[v] = kpos;
    T.n_kids[v] = (int)c->kids[v].size();
    for (int k : c->kids[v]) T.kids[kpos++] = k;
    const int nk = T.n_kids[v];
    T.inv_kids[v] = nk == 0 ? 0.0f : (v == c->root ? 1.0f / (float)nk : 1.0f / (float)(nk + 1));
    T.sbase[v] = slot_base(c, v);
    T.data[v] = staged.data[v];
  }
  // flow part of each sink adjoint, in the order the vertices' flow steps
  // are reversed (id order): own (+) and children's (-) contributions
  int q = 0;
  for (int w = 0; w < n; ++w) {
    T.comb_first[w] = q;
    for (int v = 0; v < n; ++v) {
      if (v == c->root) continue;
      if (v == w) T.comb_v[q] = v, T.comb_sign[q++] = 1;
      if (c->parent[v] == w) T.comb_v[q] = v, T.comb_sign[q++] = -1;
    }
  }
  T.comb_first[n] = q;
  for (int k = 0; k < n; ++k) T.preorder[k] = c->preorder[k];
  for (size_t j = 0; j < c->leaves.size(); ++j) T.Db[c->leaves[j]] = S->Db + j * S->arr;
  CK(cudaMemcpyAsync(S->d_tree, &T, sizeof(T), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(adjoint tree)");
  return HMF_OK;
}

int backward_step(hmf_ctx* c, const Staged& staged, int slotA, int slotB, int cur, cudaStream_t s) {
  AdjointState* S = c->adj;
  const long long arr = S->arr;
  const int n = c->n;
  const hmf::Geometry G = c->geo;
  const float* stA = slot_ptr(S, slotA);
  hmf::AdjSweep W;
  W.stA = stA;
  W.stB = slot_ptr(S, slotB);
  W.arr = arr;
  W.sbn = S->sb[cur];
  W.ubn = S->ub[cur];
  W.gbn = S->gb;
  W.sbo = S->sb[cur ^ 1];
  W.ubo = S->ub[cur ^ 1];
  W.dbp = S->dbp;
  if (S->chain || n > hmf::kSwMaxN) {
    const long long blocks = (G.vol + hmf::kAdjTreeThreads - 1) / hmf::kAdjTreeThreads;
    const int grid = (int)std::min<long long>(blocks, (long long)c->sm_count * 8);
    const size_t smem = 5 * (size_t)n * hmf::kAdjTreeThreads * sizeof(float);
    hmf::adj_tree_kernel<<<grid, hmf::kAdjTreeThreads, smem, s>>>(S->d_tree, G, W);
    CK(cudaGetLastError(), "adj_tree_kernel launch");
  } else {
    const int smem = hmf::adj_sweep_smem_bytes(n);
    const long long chunks = (G.vol + hmf::kSwVc - 1) / hmf::kSwVc;
    const int per_sm = std::max(1, (227 * 1024) / (smem + (int)sizeof(hmf::AdjTree) + 1024));
    const int grid = (int)std::min<long long>(chunks, (long long)c->sm_count * per_sm);
    bool pre = true;  // vertex ids in pre-order: the sink pass runs in id order
    for (int k = 0; k < n; ++k) pre = pre && c->preorder[k] == k;
    bool flat = c->root == 0;  // every other vertex a leaf of root 0: parents known at compile time
    for (int v = 1; v < n; ++v) flat = flat && c->parent[v] == 0;
    if (int rc = maybe_request_stall(c, HMF_STALL_REVERSE_SWEEP, s)) return rc;
    switch (n * 4 + (flat ? 2 : pre ? 1 : 0)) {
#define HMF_SWEEP_CASE(N)                                                                                  \
  case 4 * N:                                                                                              \
    hmf::adj_sweep_kernel<N, false, false><<<grid, hmf::kSwVc, smem, s>>>(S->d_tree, G, W, c->d_error);    \
    break;                                                                                                 \
  case 4 * N + 1:                                                                                          \
    hmf::adj_sweep_kernel<N, true, false><<<grid, hmf::kSwVc, smem, s>>>(S->d_tree, G, W, c->d_error);     \
    break;                                                                                                 \
  case 4 * N + 2:                                                                                          \
    hmf::adj_sweep_kernel<N, true, true><<<grid, hmf::kSwVc, smem, s>>>(S->d_tree, G, W, c->d_error);      \
    break;
      HMF_SWEEP_CASE(2) HMF_SWEEP_CASE(3) HMF_SWEEP_CASE(4) HMF_SWEEP_CASE(5)
      HMF_SWEEP_CASE(6) HMF_SWEEP_CASE(7) HMF_SWEEP_CASE(8)
#undef HMF_SWEEP_CASE
    }
    CK(cudaGetLastError(), "adj_sweep_kernel launch");
  }
  ++c->launches;
  if (!S->chain) {
    hmf::AdjFlowParams fp;
    fp.step = c->step;
    fp.icc = 1.0f / c->cc;
    fp.parity = S->pb_par;
    fp.n_vertices = n - 1;
    fp.vols = S->d_avol;
    fp.items = S->d_aitems;
    fp.error_flag = c->d_error;
    fp.wait_limit_ns = c->wait_limit_ns;
    if (int rc = maybe_request_stall(c, HMF_STALL_REVERSE_FLOW, s)) return rc;
    const dim3 grid((unsigned)S->n_aitems * (unsigned)(n - 1));
    hmf::adj_flow_tma_kernel<<<grid, hmf::kAfThreads, hmf::kAfSmemBytes, s>>>(
        S->d_aflow + (size_t)slotA * (n - 1), fp);
    CK(cudaGetLastError(), "adj_flow_tma_kernel launch");
    ++c->launches;
    S->pb_par ^= 1;
    return HMF_OK;
  }
  hmf::AdjParams P;
  P.G = G;
  P.step = c->step;
  P.icc = 1.0f / c->cc;
  const int grid = grid_for(c, G.vol);
  for (int v = 0; v < n; ++v) {
    if (v == c->root) continue;
    const int b = slot_base(c, v), pb = slot_base(c, c->parent[v]);
    hmf::AdjVertex V;
    std::memset(&V, 0, sizeof(V));
    V.s = stA + (size_t)(b + hmf::kAdjSink) * arr;
    V.u = stA + (size_t)(b + hmf::kAdjLabel) * arr;
    V.px = stA + (size_t)(b + hmf::kAdjPx) * arr;
    V.py = stA + (size_t)(b + hmf::kAdjPy) * arr;
    V.pz = stA + (size_t)(b + hmf::kAdjPz) * arr;
    V.c = stA + (size_t)pb * arr;
    V.smooth = c->smooth[0][v].ptr ? staged.smooth[v] : nullptr;
    V.alpha = (float)c->alpha[v];  // stored as float, as the reference does (.cxx:692)
    float* t = S->tmp;
    V.g = t + 0 * arr;
    V.ppx = t + 1 * arr;
    V.ppy = t + 2 * arr;
    V.ppz = t + 3 * arr;
    V.m = t + 4 * arr;
    V.Fm = t + 5 * arr;
    V.F2b = t + 6 * arr;
    V.qx = t + 7 * arr;
    V.qy = t + 8 * arr;
    V.qz = t + 9 * arr;
    V.dbo = t + 10 * arr;
    V.Pbx = pb_array(S, c, S->pb_par, v, 0);
    V.Pby = pb_array(S, c, S->pb_par, v, 1);
    V.Pbz = pb_array(S, c, S->pb_par, v, 2);
    V.dbp = S->dbp + (size_t)v * arr;
    V.gb = S->gb + (size_t)v * arr;
    V.alpha_grad = S->scal + 1 + v;
    hmf::adj_grad_kernel<<<grid, kAdjThreads, 0, s>>>(V, P);
    hmf::adj_flow_kernel<<<grid, kAdjThreads, 0, s>>>(V, P);
    hmf::adj_mult_kernel<<<grid, kAdjThreads, 0, s>>>(V, P);
    hmf::adj_descent_kernel<<<grid, kAdjThreads, 0, s>>>(V, P);
    hmf::adj_gsum_kernel<<<grid, kAdjThreads, 0, s>>>(V, P);
    hmf::adj_oldflow_kernel<<<grid, kAdjThreads, 0, s>>>(V, P);
    CK(cudaGetLastError(), "adjoint flow kernels launch");
    c->launches += 6;
  }
  return HMF_OK;
}

}  // namespace

namespace hmfi {

void adjoint_free(hmf_ctx* c) {
  if (!c || !c->adj) return;
  AdjointState* S = c->adj;
  if (S->arena) cudaFree(S->arena);
  if (S->d_ctx) cudaFree(S->d_ctx);
  if (S->d_tree) cudaFree(S->d_tree);
  if (S->d_tflow) cudaFree(S->d_tflow);
  if (S->d_ttree) cudaFree(S->d_ttree);
  if (S->d_aflow) cudaFree(S->d_aflow);
  if (S->d_avol) cudaFree(S->d_avol);
  if (S->d_aitems) cudaFree(S->d_aitems);
  if (S->scal) cudaFree(S->scal);
  delete S;
  c->adj = nullptr;
}

size_t adjoint_bytes(const hmf_ctx* c) {
  if (!c || !c->adj) return 0;
  const AdjointState* S = c->adj;
  return S->bytes + (size_t)S->table_cap * ((c->n - 1) * sizeof(hmf::FlowVertexTMA) + sizeof(hmf::TreeTable)) +
         (size_t)S->aflow_cap * (c->n - 1) * sizeof(hmf::AdjFlowVertex);
}

}  // namespace hmfi

extern "C" {

int hmf_solve_adjoint(hmf_ctx* c, const int* truth, int where, int checkpoint_every, double eps, double* loss,
                      void* stream) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (int rc = refuse_paged(c, "hmf_solve_adjoint")) return rc;
  if (c->vols.size() != 1) return fail(c, HMF_ERR_INVALID_ARGUMENT, "the adjoint supports single-volume contexts");
  if (c->dag) return fail(c, HMF_ERR_INVALID_ARGUMENT, "the adjoint is defined for trees (hmf_create), not graphs");
  if (c->semantics != HMF_SEMANTICS_REF_CUDA)
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "the adjoint is defined for the REF_CUDA semantics");
  if (!truth) return fail(c, HMF_ERR_INVALID_ARGUMENT, "ground-truth pointer is NULL");
  if (where != HMF_HOST && where != HMF_DEVICE) return fail(c, HMF_ERR_INVALID_ARGUMENT, "bad `where`");
  if (!(eps > 0.0) || !(eps < 1.0)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "eps must lie in (0, 1)");
  if (checkpoint_every < 0) return fail(c, HMF_ERR_INVALID_ARGUMENT, "checkpoint interval must be >= 0");
  DeviceGuard dg(c->device);
  if (where == HMF_DEVICE)
    if (int rc = check_device_pointer(c, truth, "ground truth")) return rc;
  if (!c->adj) c->adj = new AdjointState();
  AdjointState* S = c->adj;
  S->done = false;
  cudaStream_t user = reinterpret_cast<cudaStream_t>(stream);
  cudaStream_t s = c->stream;
  const int T = c->iterations;
  const int n = c->n;
  if (!S->scal) CK(cudaMalloc(&S->scal, sizeof(double) * (1 + hmf::kMaxVertices)), "cudaMalloc(adjoint scalars)");
  // per-device function attribute: always the largest tree's requirement
  CK(cudaFuncSetAttribute(hmf::adj_tree_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          5 * hmf::kMaxVertices * hmf::kAdjTreeThreads * (int)sizeof(float)),
     "cudaFuncSetAttribute(adj_tree_kernel)");
  CK(cudaFuncSetAttribute(hmf::adj_flow_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, hmf::kAfSmemBytes),
     "cudaFuncSetAttribute(adj_flow_tma_kernel)");

#define HMF_SWEEP_ATTR(N)                                                                                  \
  CK(cudaFuncSetAttribute(hmf::adj_sweep_kernel<N, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                          hmf::adj_sweep_smem_bytes(N)),                                                     \
     "cudaFuncSetAttribute(adj_sweep_kernel)");                                                              \
  CK(cudaFuncSetAttribute(hmf::adj_sweep_kernel<N, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                          hmf::adj_sweep_smem_bytes(N)),                                                     \
     "cudaFuncSetAttribute(adj_sweep_kernel)");                                                              \
  CK(cudaFuncSetAttribute(hmf::adj_sweep_kernel<N, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,   \
                          hmf::adj_sweep_smem_bytes(N)),                                                     \
     "cudaFuncSetAttribute(adj_sweep_kernel)");
  HMF_SWEEP_ATTR(2) HMF_SWEEP_ATTR(3) HMF_SWEEP_ATTR(4) HMF_SWEEP_ATTR(5)
  HMF_SWEEP_ATTR(6) HMF_SWEEP_ATTR(7) HMF_SWEEP_ATTR(8)
#undef HMF_SWEEP_ATTR
  {
    const char* e = std::getenv("HMF_ADJOINT_KERNEL");
    S->chain = e && std::strcmp(e, "chain") == 0;
  }
  int rc = plan(c, T, checkpoint_every);
  if (rc) return rc;
  Staged staged;
  rc = begin_solve(c, user, staged);  // stages the inputs and runs the initialisation
  if (!rc) rc = prepare_adjoint_tables(c, staged, s);
  if (!rc) rc = build_transition_tables(c, staged, s);
  if (!rc) rc = plan_reverse(c, s);
  if (!rc && !S->chain) rc = build_reverse_tables(c, staged, s);
  if (rc) return rc;
  const long long arr = S->arr;
  const auto& V0 = c->vols[0];
  const size_t dense = (size_t)V0.vx * V0.vy * V0.vz;
  CK(cudaMemcpyAsync(S->truth, truth, dense * sizeof(int),
                     where == HMF_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s),
     "cudaMemcpyAsync(truth)");
  // zero the adjoints (sb, ub, gb, dbp and the first Pb set are contiguous; the
  // second set is written before it is read) and accumulators
  CK(cudaMemsetAsync(S->sb[0], 0, (size_t)7 * n * arr * sizeof(float), s), "cudaMemsetAsync(adjoints)");
  S->pb_par = 0;
  CK(cudaMemsetAsync(S->Db, 0, c->leaves.size() * arr * sizeof(double), s), "cudaMemsetAsync(gradients)");
  CK(cudaMemsetAsync(S->scal, 0, sizeof(double) * (1 + hmf::kMaxVertices), s), "cudaMemsetAsync(scalars)");

  // ---- the schedule: x_0 into slot 0, then forward iterations, the loss
  // where x_T is reached (it seeds the label adjoints of the leaves) and the
  // backward steps from T-1 down to 0, with recomputations in between
  rc = copy_state(c, slot_ptr(S, 0), true, s);
  int cur = 0;
  for (size_t i = 0; i < S->sched.actions.size() && !rc; ++i) {
    const AdjAction& x = S->sched.actions[i];
    if (x.kind == kActForward) {
      rc = forward_iteration(c, S->fwd_table[i], s);
    } else if (x.kind == kActBackward) {
      rc = backward_step(c, staged, x.a, x.b, cur, s);
      cur ^= 1;
    } else {
      // the final sinks and labels into the solver's arrays (hmf_get_labels / _sink)
      rc = copy_state(c, slot_ptr(S, x.a), false, s);
      if (rc) break;
      hmf::AdjLoss Lo;
      std::memset(&Lo, 0, sizeof(Lo));
      Lo.n_leaves = (int)c->leaves.size();
      for (int j = 0; j < Lo.n_leaves; ++j) {
        Lo.u[j] = slot_array(S, x.a, slot_base(c, c->leaves[j]) + hmf::kAdjLabel);
        Lo.ub[j] = S->ub[0] + (size_t)c->leaves[j] * arr;
      }
      Lo.n_voxels = (double)dense;
      Lo.eps = eps;
      hmf::adj_loss_kernel<<<grid_for(c, c->geo.vol), kAdjThreads, 0, s>>>(Lo, S->truth, c->geo, S->scal,
                                                                          c->d_error);
      CK(cudaGetLastError(), "adj_loss_kernel launch");
      ++c->launches;
    }
  }
  if (rc) return rc;
  // ---- initial sinks: min over the leaves of D
  {
    hmf::AdjInit I;
    std::memset(&I, 0, sizeof(I));
    I.n_leaves = (int)c->leaves.size();
    for (int j = 0; j < I.n_leaves; ++j) {
      I.data[j] = staged.data[c->leaves[j]];
      I.Db[j] = S->Db + (size_t)j * arr;
    }
    I.sb = S->sb[cur];
    I.gb = S->gb;
    I.arr = arr;
    I.n = n;
    hmf::adj_init_kernel<<<grid_for(c, c->geo.vol), kAdjThreads, 0, s>>>(S->d_tree, I, c->geo);
    CK(cudaGetLastError(), "adj_init_kernel launch");
    ++c->launches;
  }
  std::vector<double> scal(1 + hmf::kMaxVertices, 0.0);
  CK(cudaMemcpyAsync(scal.data(), S->scal, sizeof(double) * scal.size(), cudaMemcpyDeviceToHost, s),
     "cudaMemcpyAsync(adjoint scalars)");
  CK(cudaStreamSynchronize(s), "cudaStreamSynchronize(adjoint)");
  rc = end_solve(c, user);
  if (rc) return rc;
  rc = check_error_flag(c);
  if (rc) return rc;
  S->loss = scal[0];
  S->alpha_grad.assign(scal.begin() + 1, scal.begin() + 1 + n);
  S->done = true;
  if (loss) *loss = S->loss;
  return HMF_OK;
}

int hmf_get_data_gradient(hmf_ctx* c, int leaf, double* out, int where, void* stream) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (!valid_vertex(c, leaf) || !c->kids[leaf].empty())
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "data gradients exist for leaves only");
  if (!out) return fail(c, HMF_ERR_INVALID_ARGUMENT, "output pointer is NULL");
  if (where != HMF_HOST && where != HMF_DEVICE) return fail(c, HMF_ERR_INVALID_ARGUMENT, "bad `where`");
  if (!c->adj || !c->adj->done) return fail(c, HMF_ERR_STATE, "hmf_solve_adjoint has not run");
  DeviceGuard dg(c->device);
  if (where == HMF_DEVICE)
    if (int rc = check_device_pointer(c, out, "data gradient output")) return rc;
  const AdjointState* S = c->adj;
  const int j = (int)(std::find(c->leaves.begin(), c->leaves.end(), leaf) - c->leaves.begin());
  const auto& V = c->vols[0];
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  CK(cudaMemcpy2DAsync(out, (size_t)V.vx * sizeof(double), S->Db + (size_t)j * S->arr,
                       (size_t)V.pitch * sizeof(double), (size_t)V.vx * sizeof(double), (size_t)V.vy * V.vz,
                       where == HMF_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s),
     "cudaMemcpy2DAsync(data gradient)");
  if (where == HMF_HOST) CK(cudaStreamSynchronize(s), "cudaStreamSynchronize(data gradient)");
  return HMF_OK;
}

int hmf_get_alpha_gradient(hmf_ctx* c, double* out, int n) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (!out) return fail(c, HMF_ERR_INVALID_ARGUMENT, "output pointer is NULL");
  if (!c->adj || !c->adj->done) return fail(c, HMF_ERR_STATE, "hmf_solve_adjoint has not run");
  for (int v = 0; v < n && v < c->n; ++v) out[v] = c->adj->alpha_grad[v];
  return c->n;
}

int hmf_get_adjoint_plan(const hmf_ctx* c, int* checkpoint_every, int* recomputed_segments) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (!c->adj) return HMF_ERR_STATE;
  if (checkpoint_every) *checkpoint_every = c->adj->sched.k;
  if (recomputed_segments) *recomputed_segments = c->adj->sched.recomputed_segments;
  return HMF_OK;
}

int hmf_set_adjoint_memory(hmf_ctx* c, long long max_bytes, int max_state_slots) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (max_bytes < 0 || max_state_slots < 0)
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "adjoint memory limits must be >= 0 (0: no limit)");
  c->adj_max_bytes = max_bytes;
  c->adj_max_slots = max_state_slots;
  return HMF_OK;
}

int hmf_get_adjoint_schedule(const hmf_ctx* c, int* state_slots, long long* forward_iterations,
                             long long* backward_steps) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (!c->adj) return HMF_ERR_STATE;
  const AdjSchedule& sc = c->adj->sched;
  if (state_slots) *state_slots = sc.slots;
  if (forward_iterations) *forward_iterations = sc.forward;
  if (backward_steps) {
    long long nb = 0;
    for (const auto& x : sc.actions) nb += x.kind == kActBackward;
    *backward_steps = nb;
  }
  return HMF_OK;
}

long long hmf_adjoint_schedule(int iterations, int state_slots, int checkpoint_every, int* actions,
                               long long capacity) {
  if (iterations < 0 || checkpoint_every < 0 || capacity < 0 || (capacity > 0 && !actions))
    return HMF_ERR_INVALID_ARGUMENT;
  AdjSchedule sc;
  if (checkpoint_every > 0) sc = schedule_fixed(iterations, checkpoint_every);
  else if (!schedule_fewest(iterations, state_slots, &sc)) return HMF_ERR_OUT_OF_MEMORY;
  const long long n = (long long)sc.actions.size();
  for (long long i = 0; i < n && i < capacity; ++i) {
    actions[4 * i + 0] = sc.actions[i].kind;
    actions[4 * i + 1] = sc.actions[i].t;
    actions[4 * i + 2] = sc.actions[i].a;
    actions[4 * i + 3] = sc.actions[i].b;
  }
  return n;
}

}  // extern "C"
