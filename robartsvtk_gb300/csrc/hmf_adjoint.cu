// hmf_adjoint.cu -- hmf_solve_adjoint and the gradient getters of
// include/hmf.h (no counterpart in the reference, which only solves forward).
//
// Forward: the solver's own kernels (flow_tma_kernel / tree_bulk_kernel),
// one iteration at a time, with the state (flows, sinks, labels) copied into
// a checkpoint slot every k iterations.  Backward: segment by segment from
// the last, the segment's states are recomputed from its checkpoint with the
// same forward kernels (bit-identical to the first pass) and kept in segment
// slots, then the backward steps of hmf_adjoint.cuh run from the last
// iteration of the segment to its first.  With k >= iterations (the default
// when HBM holds every state) nothing is recomputed: the forward pass keeps
// all states.  Memory: (ceil(T/k) + k + 1) state slots of 5(n-1)+1 arrays
// each, plus 8n + 11 float arrays and one double array per leaf.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "hmf_adjoint.cuh"
#include "hmf_ctx.hpp"

using namespace hmfi;

namespace {

constexpr int kAdjThreads = 256;
constexpr int kAdjTemps = 11;  // g, ppx, ppy, ppz, m, Fm, F2b, qx, qy, qz, dbo

}  // namespace

struct AdjointState {
  int k = 0, iterations = 0;
  int A = 0;           // arrays per state slot
  long long arr = 0;   // floats per array (multiple of 64)
  int n_ckpt = 0, n_seg = 0;
  bool has_fin = false;
  char* arena = nullptr;
  size_t bytes = 0;
  float* ckpt = nullptr;  // n_ckpt slots: states 0, k, 2k, ...
  float* seg = nullptr;   // n_seg slots: states a+1 .. b of the segment [a, b)
  float* fin = nullptr;   // the final state, restored after a recomputing backward pass
  float* sb[2] = {nullptr, nullptr};  // [v*arr] sink adjoints (ping-pong)
  float* ub[2] = {nullptr, nullptr};  // [v*arr] label adjoints
  float* dbp = nullptr;               // [v*arr]
  float* Pb = nullptr;                // [(3v+axis)*arr]
  float* tmp = nullptr;               // kAdjTemps arrays
  double* Db = nullptr;               // [leaf index * arr]
  int* truth = nullptr;               // dense class indices
  double* scal = nullptr;             // [0] loss, [1 + v] alpha gradient
  const float** d_ctx = nullptr;      // [parity * A + j] solver array j
  hmf::AdjTree* d_tree = nullptr;
  bool done = false;
  double loss = 0.0;
  std::vector<double> alpha_grad;
  hmf::AdjTree h_tree{};
  std::vector<const float*> h_ctx;
};

namespace {

// state-slot array index of the sink of vertex v (non-root j-th in id order)
int slot_base(const hmf_ctx* c, int v) {
  if (v == c->root) return 5 * (c->n - 1);
  int j = 0;
  for (int u = 0; u < v; ++u) j += u != c->root;
  return 5 * j;
}

float* slot_ptr(const AdjointState* S, float* base, int slot) { return base + (size_t)slot * S->A * S->arr; }

int grid_for(const hmf_ctx* c, long long n) {
  return (int)std::max<long long>(1, std::min<long long>((n + kAdjThreads - 1) / kAdjThreads, (long long)c->sm_count * 16));
}

int plan(hmf_ctx* c, int T, int k_req) {
  AdjointState* S = c->adj;
  const long long arr = (long long)round_up((size_t)c->total, 64);
  const int A = 5 * (c->n - 1) + 1;
  const size_t slot_bytes = (size_t)A * arr * sizeof(float);
  const int L = (int)c->leaves.size();
  const size_t fixed = ((size_t)(8 * c->n + kAdjTemps) * arr) * sizeof(float) + (size_t)L * arr * sizeof(double) +
                       (size_t)arr * sizeof(int) + 4096;
  int k = k_req;
  if (k <= 0) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) free_b = 0;
    const size_t held = S->bytes;  // reusable
    const double budget = 0.85 * (double)(free_b + held);
    k = (double)(T + 1) * slot_bytes + fixed <= budget ? std::max(T, 1)
                                                       : std::max(1, (int)std::ceil(std::sqrt((double)T)));
  }
  k = std::max(1, std::min(k, std::max(T, 1)));
  const int n_ckpt = std::max(1, (T + k - 1) / k);
  const int n_seg = k;
  const bool has_fin = n_ckpt > 1;
  const size_t need = (size_t)(n_ckpt + n_seg + (has_fin ? 1 : 0)) * slot_bytes + fixed;
  if (need > S->bytes) {
    if (S->arena) cudaFree(S->arena);
    S->arena = nullptr;
    S->bytes = 0;
    CK(cudaMalloc(&S->arena, need), "cudaMalloc(adjoint state)");
    CK(cudaMemset(S->arena, 0, need), "cudaMemset(adjoint state)");
    S->bytes = need;
  }
  S->k = k;
  S->iterations = T;
  S->A = A;
  S->arr = arr;
  S->n_ckpt = n_ckpt;
  S->n_seg = n_seg;
  S->has_fin = has_fin;
  char* p = S->arena;
  auto takef = [&](size_t arrays) {
    float* r = reinterpret_cast<float*>(p);
    p += arrays * arr * sizeof(float);
    return r;
  };
  S->ckpt = takef((size_t)n_ckpt * A);
  S->seg = takef((size_t)n_seg * A);
  S->fin = has_fin ? takef(A) : nullptr;
  for (int q = 0; q < 2; ++q) S->sb[q] = takef(c->n);
  for (int q = 0; q < 2; ++q) S->ub[q] = takef(c->n);
  S->dbp = takef(c->n);
  S->Pb = takef(3 * (size_t)c->n);
  S->tmp = takef(kAdjTemps);
  S->Db = reinterpret_cast<double*>(p);
  p += (size_t)L * arr * sizeof(double);
  S->truth = reinterpret_cast<int*>(p);
  return HMF_OK;
}

int copy_state(hmf_ctx* c, float* slot, int parity, bool to_slot, cudaStream_t s) {
  const AdjointState* S = c->adj;
  const dim3 grid((unsigned)std::min<long long>((S->arr / 4 + kAdjThreads - 1) / kAdjThreads, 1024), (unsigned)S->A);
  hmf::adj_state_copy_kernel<<<grid, kAdjThreads, 0, s>>>(S->d_ctx + (size_t)parity * S->A, slot, S->arr,
                                                          to_slot ? 1 : 0);
  CK(cudaGetLastError(), "adj_state_copy_kernel launch");
  ++c->launches;
  return HMF_OK;
}

int forward_iteration(hmf_ctx* c, int parity, cudaStream_t s) {
  int rc = launch_flow(c, parity, s);
  if (!rc) rc = launch_tree(c, s);
  return rc;
}

int prepare_adjoint_tables(hmf_ctx* c, const Staged& staged, cudaStream_t s) {
  AdjointState* S = c->adj;
  const int n = c->n;
  // solver arrays in slot order, per flow parity
  S->h_ctx.assign(2 * (size_t)S->A, nullptr);
  for (int par = 0; par < 2; ++par) {
    const float** t = S->h_ctx.data() + (size_t)par * S->A;
    for (int v = 0; v < n; ++v) {
      const int b = slot_base(c, v);
      t[b + hmf::kAdjSink] = c->sink[v];
      if (v == c->root) continue;
      t[b + hmf::kAdjLabel] = c->label[v];
      t[b + hmf::kAdjPx] = c->fx[par][v];
      t[b + hmf::kAdjPy] = c->fy[par][v];
      t[b + hmf::kAdjPz] = c->fz[par][v];
    }
  }
  if (!S->d_ctx) CK(cudaMalloc(&S->d_ctx, sizeof(float*) * 2 * (5 * hmf::kMaxVertices + 1)), "cudaMalloc(adjoint tables)");
  if (!S->d_tree) CK(cudaMalloc(&S->d_tree, sizeof(hmf::AdjTree)), "cudaMalloc(adjoint tree)");
  CK(cudaMemcpyAsync(S->d_ctx, S->h_ctx.data(), sizeof(float*) * S->h_ctx.size(), cudaMemcpyHostToDevice, s),
     "cudaMemcpyAsync(adjoint tables)");
  hmf::AdjTree& T = S->h_tree;
  std::memset(&T, 0, sizeof(T));
  T.n = n;
  T.root = c->root;
  T.cc = c->cc;
  T.icc = 1.0f / c->cc;
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
  for (int k = 0; k < n; ++k) T.preorder[k] = c->preorder[k];
  for (size_t j = 0; j < c->leaves.size(); ++j) T.Db[c->leaves[j]] = S->Db + j * S->arr;
  CK(cudaMemcpyAsync(S->d_tree, &T, sizeof(T), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(adjoint tree)");
  return HMF_OK;
}

int backward_step(hmf_ctx* c, const Staged& staged, const float* stA, const float* stB, int cur, cudaStream_t s) {
  AdjointState* S = c->adj;
  const long long arr = S->arr;
  const int n = c->n;
  const hmf::Geometry G = c->geo;
  hmf::AdjSweep W;
  W.stA = stA;
  W.stB = stB;
  W.arr = arr;
  W.sbn = S->sb[cur];
  W.ubn = S->ub[cur];
  W.sbo = S->sb[cur ^ 1];
  W.ubo = S->ub[cur ^ 1];
  W.dbp = S->dbp;
  {
    const long long blocks = (G.vol + hmf::kAdjTreeThreads - 1) / hmf::kAdjTreeThreads;
    const int grid = (int)std::min<long long>(blocks, (long long)c->sm_count * 8);
    const size_t smem = 5 * (size_t)n * hmf::kAdjTreeThreads * sizeof(float);
    hmf::adj_tree_kernel<<<grid, hmf::kAdjTreeThreads, smem, s>>>(S->d_tree, G, W);
    CK(cudaGetLastError(), "adj_tree_kernel launch");
    ++c->launches;
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
    V.Pbx = S->Pb + (size_t)(3 * v + 0) * arr;
    V.Pby = S->Pb + (size_t)(3 * v + 1) * arr;
    V.Pbz = S->Pb + (size_t)(3 * v + 2) * arr;
    V.dbp = S->dbp + (size_t)v * arr;
    V.sbo = S->sb[cur ^ 1] + (size_t)v * arr;
    V.sbo_par = S->sb[cur ^ 1] + (size_t)c->parent[v] * arr;
    V.ubo = S->ub[cur ^ 1] + (size_t)v * arr;
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
  if (S->scal) cudaFree(S->scal);
  delete S;
  c->adj = nullptr;
}

size_t adjoint_bytes(const hmf_ctx* c) { return c && c->adj ? c->adj->bytes : 0; }

}  // namespace hmfi

extern "C" {

int hmf_solve_adjoint(hmf_ctx* c, const int* truth, int where, int checkpoint_every, double eps, double* loss,
                      void* stream) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (c->vols.size() != 1) return fail(c, HMF_ERR_INVALID_ARGUMENT, "the adjoint supports single-volume contexts");
  if (c->semantics != HMF_SEMANTICS_REF_CUDA)
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "the adjoint is defined for the REF_CUDA semantics");
  if (!truth) return fail(c, HMF_ERR_INVALID_ARGUMENT, "ground-truth pointer is NULL");
  if (where != HMF_HOST && where != HMF_DEVICE) return fail(c, HMF_ERR_INVALID_ARGUMENT, "bad `where`");
  if (!(eps > 0.0) || !(eps < 1.0)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "eps must lie in (0, 1)");
  if (checkpoint_every < 0) return fail(c, HMF_ERR_INVALID_ARGUMENT, "checkpoint interval must be >= 0");
  DeviceGuard dg(c->device);
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
  int rc = plan(c, T, checkpoint_every);
  if (rc) return rc;
  Staged staged;
  rc = begin_solve(c, user, staged);
  if (!rc) rc = prepare_adjoint_tables(c, staged, s);
  if (rc) return rc;
  const long long arr = S->arr;
  const auto& V0 = c->vols[0];
  const size_t dense = (size_t)V0.vx * V0.vy * V0.vz;
  CK(cudaMemcpyAsync(S->truth, truth, dense * sizeof(int),
                     where == HMF_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s),
     "cudaMemcpyAsync(truth)");
  // zero the adjoints and the accumulators (sb, ub, dbp and Pb are contiguous)
  CK(cudaMemsetAsync(S->sb[0], 0, (size_t)8 * n * arr * sizeof(float), s), "cudaMemsetAsync(adjoints)");
  CK(cudaMemsetAsync(S->Db, 0, c->leaves.size() * arr * sizeof(double), s), "cudaMemsetAsync(gradients)");
  CK(cudaMemsetAsync(S->scal, 0, sizeof(double) * (1 + hmf::kMaxVertices), s), "cudaMemsetAsync(scalars)");

  // ---- forward pass with checkpoints; the last segment keeps every state
  const int k = S->k;
  const int a_last = T > 0 ? ((T - 1) / k) * k : 0;
  rc = copy_state(c, slot_ptr(S, S->ckpt, 0), 0, true, s);
  for (int it = 0; it < T && !rc; ++it) {
    if (it > 0 && it % k == 0) rc = copy_state(c, slot_ptr(S, S->ckpt, it / k), it & 1, true, s);
    if (!rc) rc = forward_iteration(c, it & 1, s);
    if (!rc && it + 1 > a_last) rc = copy_state(c, slot_ptr(S, S->seg, it - a_last), (it + 1) & 1, true, s);
  }
  if (rc) return rc;
  // ---- loss on the final labels; it seeds the label adjoints of the leaves
  {
    hmf::AdjLoss Lo;
    std::memset(&Lo, 0, sizeof(Lo));
    Lo.n_leaves = (int)c->leaves.size();
    for (int j = 0; j < Lo.n_leaves; ++j) {
      Lo.u[j] = c->label[c->leaves[j]];
      Lo.ub[j] = S->ub[0] + (size_t)c->leaves[j] * arr;
    }
    Lo.n_voxels = (double)dense;
    Lo.eps = eps;
    hmf::adj_loss_kernel<<<grid_for(c, c->geo.vol), kAdjThreads, 0, s>>>(Lo, S->truth, c->geo, S->scal, c->d_error);
    CK(cudaGetLastError(), "adj_loss_kernel launch");
    ++c->launches;
  }
  if (S->has_fin) rc = copy_state(c, S->fin, T & 1, true, s);
  // ---- backward, segment by segment
  int cur = 0;
  for (int a = a_last; a >= 0 && T > 0 && !rc; a -= k) {
    const int b = std::min(a + k, T);
    if (a != a_last) {
      rc = copy_state(c, slot_ptr(S, S->ckpt, a / k), 0, false, s);
      for (int j = 1; j <= b - a && !rc; ++j) {
        rc = forward_iteration(c, (j - 1) & 1, s);
        if (!rc) rc = copy_state(c, slot_ptr(S, S->seg, j - 1), j & 1, true, s);
      }
    }
    for (int it = b - 1; it >= a && !rc; --it) {
      const float* stA = it == a ? slot_ptr(S, S->ckpt, a / k) : slot_ptr(S, S->seg, it - a - 1);
      const float* stB = slot_ptr(S, S->seg, it - a);
      rc = backward_step(c, staged, stA, stB, cur, s);
      cur ^= 1;
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
    I.arr = arr;
    I.n = n;
    hmf::adj_init_kernel<<<grid_for(c, c->geo.vol), kAdjThreads, 0, s>>>(I, c->geo);
    CK(cudaGetLastError(), "adj_init_kernel launch");
    ++c->launches;
  }
  if (S->has_fin) rc = copy_state(c, S->fin, T & 1, false, s);
  if (rc) return rc;
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
  if (checkpoint_every) *checkpoint_every = c->adj->k;
  if (recomputed_segments) *recomputed_segments = c->adj->n_ckpt - 1;
  return HMF_OK;
}

}  // extern "C"
