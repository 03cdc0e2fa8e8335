// hmf_paged.cu -- out-of-core solve (hmf_create_paged): the solver state of
// the whole volume lives in pinned host memory and the device iterates it
// block by block.
//
// The reference pages whole-volume buffers between host and device when they
// do not all fit in MaxGPUUsage of the GPU's memory: it acquires what fits
// (CUDA_GetGPUBuffers, CUDA_hierarchicalmaxflow.cu:33-60), simulates one
// iteration to learn each buffer's next use
// (vtkCudaHierarchicalMaxFlowSegmentation.cxx:884-1038) and, before every
// pass, moves the buffers the pass needs onto the GPU, evicting the one used
// furthest in the future (GetGPUBuffersV2, :1088-1294).  Every iteration then
// crosses the host link once per paged buffer.
//
// Here the unit of residency is a block of z-planes of every array, and the
// link is crossed once per k iterations (temporal blocking): one iteration's
// new state at plane z reads the old state at planes z-2 .. z+2 only, so a
// block of T planes iterated k times on its own (its faces taking the
// volume-face rules) is exact on every plane at least 2k planes from a face
// that lies inside the volume -- 2k + 1 on the high-z side, whose first step
// forms the old divergence of the top plane without the z-flow of the plane
// beyond it.  The volume is covered by overlapping blocks, each owning the
// planes it computes exactly; a round loads every block's planes from the
// host state, runs k iterations with the in-core kernels (same arithmetic:
// results identical to the in-core solve) and stores the owned planes back.
//
// Pipelining: three block contexts take the blocks in turn, each on its own
// stream, so that one block's planes come in over the link while another
// iterates and a third's go out (the two copy directions run concurrently).
// The host state is double-buffered -- round r reads copy (r-1)&1 and writes
// copy r&1 -- so a block's store never waits for a neighbour's load of the
// same round; across rounds a block's load waits only for the stores of the
// three blocks whose owned planes it covers, and a store for the loads of the
// previous round that read what it overwrites.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "hmf_ctx.hpp"

namespace {

constexpr int kBlockContexts = 3;  // blocks in flight: loading, iterating, storing

// One copy of the host state: per vertex the sink; per non-root vertex the
// label and the three flows; dense VX*VY*VZ floats each (pinned).  The
// divergence is not kept: the flow step forms the old divergence from the
// flows and writes the new one before the sweep reads it.
struct HostState {
  char* mem = nullptr;
  size_t bytes = 0;
  std::vector<float*> sink, label, fx, fy, fz;
};

}  // namespace

struct PagedState {
  double usage = 0.75;      // fraction of the device's memory (MaxGPUUsage)
  int forced_planes = 0;    // hmf_set_paged_plan (0: from the budget)
  int forced_iterations = 0;
  int inputs_mode = HMF_PAGED_INPUTS_AUTO;

  // plan of the last solve
  int block_planes = 0, round_iterations = 0, halo = 0;
  std::vector<int> starts, owned;  // per block: first plane, first owned plane
  int rounds = 0;
  bool inputs_on_device = false;
  long long link_bytes = 0;  // bytes between host and device in the last solve
  int final_copy = 0;        // host state copy holding the final state

  hmf_ctx* blk[kBlockContexts] = {};
  int n_blk = 0;
  int blk_planes = 0;  // planes the block contexts were created for
  cudaStream_t st[kBlockContexts] = {};
  std::vector<cudaEvent_t> ev_loaded[2], ev_stored[2];  // [host copy loaded from / stored into][block]
  cudaEvent_t ev_end[kBlockContexts] = {};

  HostState host[2];
  // pinned copies of pageable host inputs
  char* inputs = nullptr;
  size_t input_bytes = 0;
  // device copies of the inputs when they stay resident (HMF_PAGED_INPUTS_DEVICE)
  char* d_inputs = nullptr;
  size_t d_input_bytes = 0;
  // error flag of every block solve of the last solve (pinned)
  int* flags = nullptr;
  int flag_cap = 0, n_flags = 0;
};

namespace hmfi {

namespace {

// Iterations per round, at most: a round moves each plane of ~5 arrays per
// vertex across the host link and back, an iteration ~12 per vertex through
// HBM, and the link runs at ~0.03 of HBM bandwidth, so longer rounds pay off
// until the halo (2k + 1 planes a side) eats the block: with k = (T - 4) / 8
// the halo takes about half of T.  Measured at 256^3 tree4 with 96-plane
// blocks: 8 iterations per round 290 ms per 96 iterations, 11 272 ms.
constexpr int kMaxRoundIterations = 12;
constexpr size_t kBlockFixedBytes = 16u << 20;  // tables, graphs and alignment of one block context

struct BlockLoad {
  const HostState* H;
  cudaEvent_t loaded;
  int first;        // first plane of the block
  long long plane;  // elements per dense plane
  long long* bytes;
};

// Copies `planes` planes between a pitched array of a block context and a
// dense host array.
int copy_planes(hmf_ctx* c, float* dst, size_t dpitch, const float* src, size_t spitch, int vx, int vy,
                int planes, cudaMemcpyKind kind, cudaStream_t s) {
  const size_t row = (size_t)vx * sizeof(float);
  if (dpitch == row && spitch == row) {
    CK(cudaMemcpyAsync(dst, src, row * vy * planes, kind, s), "cudaMemcpyAsync(paged state)");
  } else {
    CK(cudaMemcpy2DAsync(dst, dpitch, src, spitch, row, (size_t)vy * planes, kind, s),
       "cudaMemcpy2DAsync(paged state)");
  }
  return HMF_OK;
}

// StateLoader of a continued block solve: the block's planes of the host
// state into its sinks, labels and parity-0 flows.
int load_block(hmf_ctx* b, cudaStream_t s, void* arg) {
  hmf_ctx* c = b;
  const BlockLoad& L = *static_cast<const BlockLoad*>(arg);
  const HostState& H = *L.H;
  const auto& V = b->vols[0];
  const size_t dp = (size_t)V.pitch * sizeof(float), sp = (size_t)V.vx * sizeof(float);
  const long long off = (long long)L.first * L.plane;
  long long n = 0;
  for (int v = 0; v < b->n; ++v) {
    if (int rc = copy_planes(c, b->sink[v], dp, H.sink[v] + off, sp, V.vx, V.vy, V.vz, cudaMemcpyHostToDevice, s))
      return rc;
    ++n;
    if (v == b->root) continue;
    const float* src[4] = {H.label[v], H.fx[v], H.fy[v], H.fz[v]};
    float* dst[4] = {b->label[v], b->fx[0][v], b->fy[0][v], b->fz[0][v]};
    for (int a = 0; a < 4; ++a)
      if (int rc = copy_planes(c, dst[a], dp, src[a] + off, sp, V.vx, V.vy, V.vz, cudaMemcpyHostToDevice, s))
        return rc;
    n += 4;
  }
  *L.bytes += n * (long long)V.vz * L.plane * (long long)sizeof(float);
  CK(cudaEventRecord(L.loaded, s), "cudaEventRecord(block loaded)");
  return HMF_OK;
}

// The owned planes [z0, z1) of a solved block into a host state copy: sinks,
// labels and the flows of set `parity` (after the last round too, so that a
// continued solve starts from them).
int store_block(hmf_ctx* c, PagedState& P, HostState& H, hmf_ctx* b, int first, int z0, int z1, int parity,
                long long plane, cudaStream_t s) {
  const auto& V = b->vols[0];
  const size_t dp = (size_t)V.vx * sizeof(float), sp = (size_t)V.pitch * sizeof(float);
  const int planes = z1 - z0;
  if (planes <= 0) return HMF_OK;
  const long long hoff = (long long)z0 * plane, boff = (long long)(z0 - first) * V.plane;
  long long n = 0;
  for (int v = 0; v < b->n; ++v) {
    if (int rc = copy_planes(c, H.sink[v] + hoff, dp, b->sink[v] + boff, sp, V.vx, V.vy, planes,
                             cudaMemcpyDeviceToHost, s))
      return rc;
    ++n;
    if (v == b->root) continue;
    if (int rc = copy_planes(c, H.label[v] + hoff, dp, b->label[v] + boff, sp, V.vx, V.vy, planes,
                             cudaMemcpyDeviceToHost, s))
      return rc;
    ++n;
    const float* src[3] = {b->fx[parity][v], b->fy[parity][v], b->fz[parity][v]};
    float* dst[3] = {H.fx[v], H.fy[v], H.fz[v]};
    for (int a = 0; a < 3; ++a)
      if (int rc = copy_planes(c, dst[a] + hoff, dp, src[a] + boff, sp, V.vx, V.vy, planes, cudaMemcpyDeviceToHost, s))
        return rc;
    n += 3;
  }
  P.link_bytes += n * (long long)planes * plane * (long long)sizeof(float);
  return HMF_OK;
}

void free_blocks(PagedState& P) {
  for (auto& b : P.blk)
    if (b) {
      hmf_destroy(b);
      b = nullptr;
    }
  P.n_blk = 0;
  P.blk_planes = 0;
}

// Device bytes of one plane of a block context: 9 arrays per non-root vertex
// and the root's (hmf_create's state) plus the inputs it stages.
size_t plane_bytes(const hmf_ctx* c, int staged_inputs) {
  const auto& V = c->vols[0];
  return (size_t)V.pitch * V.vy * sizeof(float) * (size_t)(9 * (c->n - 1) + 1 + staged_inputs);
}

// The host state copy `H`: sinks, labels and flows (the same layout in every
// solve, so that a continued solve reads the last one's).
int host_state(hmf_ctx* c, HostState& H, size_t arr) {
  const size_t n_arrays = (size_t)5 * (c->n - 1) + 1;
  if (H.bytes < n_arrays * arr) {
    if (H.mem) cudaFreeHost(H.mem);
    H.mem = nullptr;
    H.bytes = 0;
    CK(cudaMallocHost(&H.mem, n_arrays * arr), "cudaMallocHost(paged state)");
    H.bytes = n_arrays * arr;
  }
  char* p = H.mem;
  auto take = [&]() {
    float* r = reinterpret_cast<float*>(p);
    p += arr;
    return r;
  };
  H.sink.assign(c->n, nullptr);
  H.label.assign(c->n, nullptr);
  H.fx.assign(c->n, nullptr);
  H.fy.assign(c->n, nullptr);
  H.fz.assign(c->n, nullptr);
  for (int v = 0; v < c->n; ++v) {
    H.sink[v] = take();
    if (v == c->root) continue;
    H.label[v] = take();
    H.fx[v] = take();
    H.fy[v] = take();
    H.fz[v] = take();
  }
  return HMF_OK;
}

int ensure_events(hmf_ctx* c, std::vector<cudaEvent_t>& evs, int n) {
  while ((int)evs.size() < n) {
    cudaEvent_t e = nullptr;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate(paged)");
    evs.push_back(e);
  }
  return HMF_OK;
}

}  // namespace

int paged_setup(hmf_ctx* c, double max_gpu_usage) {
  if (c->dag) return fail(c, HMF_ERR_INVALID_ARGUMENT, "out-of-core solves are for label trees");
  if (!(max_gpu_usage >= 0.0)) max_gpu_usage = 0.0;
  auto* P = new PagedState();
  c->pg = P;
  P->usage = std::min(1.0, max_gpu_usage);
  for (int i = 0; i < kBlockContexts; ++i) {
    CK(cudaStreamCreateWithFlags(&P->st[i], cudaStreamNonBlocking), "cudaStreamCreate(paged)");
    CK(cudaEventCreateWithFlags(&P->ev_end[i], cudaEventDisableTiming), "cudaEventCreate(paged)");
  }
  return HMF_OK;
}

void paged_free(hmf_ctx* c) {
  PagedState* P = c->pg;
  if (!P) return;
  for (auto s : P->st)
    if (s) cudaStreamSynchronize(s);
  free_blocks(*P);
  for (int i = 0; i < kBlockContexts; ++i) {
    if (P->st[i]) cudaStreamDestroy(P->st[i]);
    if (P->ev_end[i]) cudaEventDestroy(P->ev_end[i]);
  }
  for (int q = 0; q < 2; ++q) {
    for (auto e : P->ev_loaded[q]) cudaEventDestroy(e);
    for (auto e : P->ev_stored[q]) cudaEventDestroy(e);
    if (P->host[q].mem) cudaFreeHost(P->host[q].mem);
  }
  if (P->inputs) cudaFreeHost(P->inputs);
  if (P->d_inputs) cudaFree(P->d_inputs);
  if (P->flags) cudaFreeHost(P->flags);
  delete P;
  c->pg = nullptr;
}

size_t paged_bytes(const hmf_ctx* c) {
  size_t n = c->pg->inputs_on_device ? c->pg->d_input_bytes : 0;
  for (auto b : c->pg->blk)
    if (b) n += hmf_device_bytes(b);
  return n;
}

int paged_solve(hmf_ctx* c, cudaStream_t user, bool cont) {
  PagedState& P = *c->pg;
  const auto& V = c->vols[0];
  for (int l : c->leaves)
    if (!c->data[0][l].ptr) return fail(c, HMF_ERR_MISSING_INPUT, "Missing data prior for leaf node.");
  c->solved = false;
  c->continuable = false;
  // Host copy q of round r: rounds write copy (r + o) & 1 and read the other
  // one; a continued solve's first round reads the copy the last solve
  // ended in (o = that copy ^ 1) instead of initialising its blocks.
  const int o = cont ? (P.final_copy ^ 1) : 0;
  const long long plane = (long long)V.vx * V.vy;
  const size_t arr = (size_t)plane * V.vz * sizeof(float);

  // ---- inputs: the distinct input arrays, where they are, where blocks read them
  std::vector<const float*> in_data(c->n, nullptr), in_smooth(c->n, nullptr);
  std::vector<int> w_data(c->n, HMF_HOST), w_smooth(c->n, HMF_HOST);
  for (int l : c->leaves) in_data[l] = c->data[0][l].ptr, w_data[l] = c->data[0][l].where;
  for (int v = 0; v < c->n; ++v)
    if (v != c->root && c->smooth[0][v].ptr) in_smooth[v] = c->smooth[0][v].ptr, w_smooth[v] = c->smooth[0][v].where;
  std::vector<const float*> host_src;  // distinct host inputs
  auto note_host = [&](const float* p, int w) {
    if (p && w == HMF_HOST && std::find(host_src.begin(), host_src.end(), p) == host_src.end()) host_src.push_back(p);
  };
  for (int l : c->leaves) note_host(in_data[l], w_data[l]);
  for (int v = 0; v < c->n; ++v) note_host(in_smooth[v], w_smooth[v]);
  int staged_inputs = (int)c->leaves.size();
  {
    std::vector<const float*> distinct;
    for (int v = 0; v < c->n; ++v)
      if (in_smooth[v] && std::find(distinct.begin(), distinct.end(), in_smooth[v]) == distinct.end())
        distinct.push_back(in_smooth[v]);
    staged_inputs += (int)distinct.size();
  }

  // ---- plan: block thickness T from the budget, k iterations per round
  const bool cpu = c->semantics == HMF_SEMANTICS_REF_CPU;
  size_t free_b = 0, total_b = 0;
  CK(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
  const size_t budget = (size_t)(P.usage * (double)total_b);
  const size_t host_in_bytes = arr * host_src.size();
  // host inputs stay on the device for the whole solve when they take at most
  // a quarter of the budget (or when asked): the blocks then read them in
  // place instead of over the link every round
  const bool dev_inputs = !host_src.empty() &&
                          (P.inputs_mode == HMF_PAGED_INPUTS_DEVICE ||
                           (P.inputs_mode == HMF_PAGED_INPUTS_AUTO && 4 * host_in_bytes <= budget));
  int T = P.forced_planes;
  if (T <= 0) {
    const size_t per_plane = plane_bytes(c, staged_inputs);
    const size_t fixed = kBlockContexts * kBlockFixedBytes + (dev_inputs ? host_in_bytes : 0);
    if (budget <= fixed + kBlockContexts * per_plane)
      return fail(c, HMF_ERR_OUT_OF_MEMORY, "MaxGPUUsage leaves no room for three blocks of planes");
    T = (int)std::min<size_t>((size_t)V.vz, (budget - fixed) / (kBlockContexts * per_plane));
  }
  T = std::min(T, V.vz);
  // a block context addresses its elements with 32-bit offsets
  T = (int)std::min<long long>(T, ((1LL << 31) - 1) / ((long long)V.pitch * V.vy));
  if (T < 1) return fail(c, HMF_ERR_INVALID_ARGUMENT, "one plane of the volume holds 2^31 elements or more");
  int k;
  if (cpu) {
    k = c->iterations;  // per-voxel iterations (REF_CPU): no halo, one round
  } else if (T >= V.vz) {
    // one block, no halo: one round unless the plan asks for several
    k = P.forced_iterations > 0 ? std::min(P.forced_iterations, c->iterations) : c->iterations;
  } else {
    k = P.forced_iterations > 0 ? P.forced_iterations : std::min(kMaxRoundIterations, (T - 4) / 8);
    k = std::min(k, c->iterations);
    if (k < 1 && c->iterations > 0)
      return fail(c, HMF_ERR_OUT_OF_MEMORY, "MaxGPUUsage holds fewer than 12 planes per block");
  }
  // the flow step recomputes the old divergence from the stored flows, which
  // at a block's top plane lacks the z-flow above it: one more halo plane
  const int halo = (T >= V.vz || cpu || k == 0) ? 0 : 2 * k + 1;
  const int nb = hmf_paged_layout(V.vz, T, halo, nullptr, nullptr, 0);
  if (nb < 0)
    return fail(c, HMF_ERR_INVALID_ARGUMENT,
                "block planes must be at least four times the halo (2 x iterations per round + 1)");
  // A block from the budget is as thick as the budget allows; the same
  // number of blocks also covers the volume with thinner ones, which iterate
  // fewer planes twice (the halos): take the thinnest (the block count does
  // not grow as T does).
  if (P.forced_planes <= 0 && halo > 0 && nb > 1) {
    int lo = 4 * halo, hi = T;
    while (lo < hi) {
      const int mid = lo + (hi - lo) / 2;
      const int n_mid = hmf_paged_layout(V.vz, mid, halo, nullptr, nullptr, 0);
      if (n_mid > 0 && n_mid <= nb) hi = mid;
      else lo = mid + 1;
    }
    T = lo;
  }
  P.starts.assign(nb, 0);
  P.owned.assign(nb, 0);
  if (hmf_paged_layout(V.vz, T, halo, P.starts.data(), P.owned.data(), nb) != nb)
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "block layout");
  std::vector<int> round_iters;
  if (c->iterations == 0 || k == 0) round_iters.push_back(0);
  for (int left = c->iterations; k > 0 && left > 0; left -= k) round_iters.push_back(std::min(k, left));
  P.block_planes = T;
  P.round_iterations = k;
  P.halo = halo;
  P.rounds = (int)round_iters.size();
  P.link_bytes = 0;
  P.final_copy = (P.rounds - 1 + o) & 1;

  // ---- memory: block contexts, the inputs, the host state, the error flags
  const int nc = std::min(kBlockContexts, nb);
  if (P.blk_planes != T || P.n_blk < nc) {
    free_blocks(P);
    for (int i = 0; i < nc; ++i) {
      int rc = hmf_create(&P.blk[i], V.vx, V.vy, T, c->parent.data(), c->n, c->semantics, c->device);
      if (rc) {
        free_blocks(P);
        return fail(c, rc, std::string("block context: ") + hmf_last_error(nullptr));
      }
    }
    P.n_blk = nc;
    P.blk_planes = T;
  }
  CK(cudaEventRecord(c->ev_join, user), "cudaEventRecord(join)");
  for (int i = 0; i < kBlockContexts; ++i)
    CK(cudaStreamWaitEvent(P.st[i], c->ev_join, 0), "cudaStreamWaitEvent(join)");
  // a continued solve reads the host copy the last solve's blocks stored on
  // every stream, whatever its layout was: each stream waits for all of it
  if (cont)
    for (int i = 0; i < kBlockContexts; ++i)
      for (int q = 0; q < kBlockContexts; ++q)
        CK(cudaStreamWaitEvent(P.st[i], P.ev_end[q], 0), "cudaStreamWaitEvent(last solve)");
  // Host inputs: on the device for the whole solve, or from pinned memory
  // (the caller's, when already pinned, else a pinned copy) every round.
  std::vector<const float*> host_dst(host_src.size(), nullptr);
  if (dev_inputs) {
    if (host_in_bytes > P.d_input_bytes) {
      for (auto s : P.st) CK(cudaStreamSynchronize(s), "cudaStreamSynchronize(paged inputs)");
      if (P.d_inputs) cudaFree(P.d_inputs);
      P.d_inputs = nullptr;
      P.d_input_bytes = 0;
      CK(cudaMalloc(&P.d_inputs, host_in_bytes), "cudaMalloc(paged inputs)");
      P.d_input_bytes = host_in_bytes;
    }
    for (size_t i = 0; i < host_src.size(); ++i) {
      host_dst[i] = reinterpret_cast<const float*>(P.d_inputs + i * arr);
      CK(cudaMemcpyAsync(const_cast<float*>(host_dst[i]), host_src[i], arr, cudaMemcpyHostToDevice, P.st[0]),
         "cudaMemcpyAsync(paged inputs)");
    }
    P.link_bytes += (long long)host_in_bytes;
    CK(cudaEventRecord(P.ev_end[0], P.st[0]), "cudaEventRecord(inputs)");
    for (int i = 1; i < kBlockContexts; ++i)
      CK(cudaStreamWaitEvent(P.st[i], P.ev_end[0], 0), "cudaStreamWaitEvent(inputs)");
  } else if (!host_src.empty()) {
    std::vector<size_t> copy;  // pageable inputs: copied into pinned memory
    for (size_t i = 0; i < host_src.size(); ++i) {
      cudaPointerAttributes a;
      if (cudaPointerGetAttributes(&a, host_src[i]) == cudaSuccess && a.type == cudaMemoryTypeHost)
        host_dst[i] = host_src[i];
      else
        copy.push_back(i);
      cudaGetLastError();
    }
    if (!copy.empty()) {
      // the previous solve's copies read the pinned buffer, which the host
      // rewrites here: they are done once its streams are
      for (auto s : P.st) CK(cudaStreamSynchronize(s), "cudaStreamSynchronize(paged inputs)");
      if (arr * copy.size() > P.input_bytes) {
        if (P.inputs) cudaFreeHost(P.inputs);
        P.inputs = nullptr;
        P.input_bytes = 0;
        CK(cudaMallocHost(&P.inputs, arr * copy.size()), "cudaMallocHost(paged inputs)");
        P.input_bytes = arr * copy.size();
      }
      for (size_t q = 0; q < copy.size(); ++q) {
        host_dst[copy[q]] = reinterpret_cast<const float*>(P.inputs + q * arr);
        std::memcpy(const_cast<float*>(host_dst[copy[q]]), host_src[copy[q]], arr);
      }
    }
  }
  P.inputs_on_device = dev_inputs;
  auto route = [&](const float* p, int w, int* where) -> const float* {
    *where = w;
    if (!p || w != HMF_HOST) return p;
    const size_t i = std::find(host_src.begin(), host_src.end(), p) - host_src.begin();
    if (dev_inputs) *where = HMF_DEVICE;
    return host_dst[i];
  };
  for (int l : c->leaves) in_data[l] = route(in_data[l], w_data[l], &w_data[l]);
  for (int v = 0; v < c->n; ++v) in_smooth[v] = route(in_smooth[v], w_smooth[v], &w_smooth[v]);
  const int link_inputs = dev_inputs ? 0 : (int)host_src.size();  // inputs the blocks read over the link

  // one round of a fresh solve writes copy 0 only
  for (int q = 0; q < (P.rounds > 1 || cont ? 2 : 1); ++q)
    if (int rc = host_state(c, P.host[q], arr)) return rc;
  for (int q = 0; q < 2; ++q) {
    if (int rc = ensure_events(c, P.ev_loaded[q], nb)) return rc;
    if (int rc = ensure_events(c, P.ev_stored[q], nb)) return rc;
  }
  const int n_flags = P.rounds * nb;
  if (P.flag_cap < n_flags) {
    for (auto s : P.st) CK(cudaStreamSynchronize(s), "cudaStreamSynchronize(paged flags)");
    if (P.flags) cudaFreeHost(P.flags);
    P.flags = nullptr;
    P.flag_cap = 0;
    CK(cudaMallocHost(&P.flags, sizeof(int) * n_flags), "cudaMallocHost(paged flags)");
    P.flag_cap = n_flags;
  }
  for (int i = 0; i < n_flags; ++i) P.flags[i] = 0;
  P.n_flags = n_flags;
  for (int i = 0; i < nc; ++i) {
    hmf_ctx* b = P.blk[i];
    for (int v = 0; v < c->n; ++v)
      if (v != c->root) hmf_set_smoothness_scalar(b, v, c->alpha[v]);
    b->timing = c->timing;
  }

  // ---- rounds: round r reads host copy (r + 1 + o) & 1 and writes copy (r + o) & 1
  long long launches = 0;
  double kind_ms[3] = {0, 0, 0};
  long long kind_count[3] = {0, 0, 0};
  int flag_i = 0;
  for (int r = 0; r < P.rounds; ++r) {
    const int kr = round_iters[r];
    const int out_q = (r + o) & 1, in_q = (r + 1 + o) & 1;
    HostState& out = P.host[out_q];
    const HostState& in = P.host[in_q];
    const bool loads = r > 0 || cont;
    for (int j = 0; j < nb; ++j) {
      const int slot = j % nc;
      hmf_ctx* b = P.blk[slot];
      cudaStream_t s = P.st[slot];
      const long long off = (long long)P.starts[j] * plane;
      for (int l : c->leaves) {
        int rc = hmf_set_data(b, l, in_data[l] + off, w_data[l]);
        if (rc) return fail(c, rc, std::string("block input: ") + b->err);
      }
      for (int v = 0; v < c->n; ++v) {
        if (v == c->root) continue;
        int rc = hmf_set_smoothness(b, v, in_smooth[v] ? in_smooth[v] + off : nullptr, w_smooth[v]);
        if (rc) return fail(c, rc, std::string("block input: ") + b->err);
      }
      hmf_set_params(b, kr, c->step, c->cc);
      // a block's planes hold the owned planes of its neighbours and itself:
      // its load follows their stores of the previous round (a continued
      // solve's first round follows all of the last solve: joined above)
      const int lo = std::max(0, j - 1), hi = std::min(nb - 1, j + 1);
      if (r > 0)
        for (int m = lo; m <= hi; ++m)
          CK(cudaStreamWaitEvent(s, P.ev_stored[in_q][m], 0), "cudaStreamWaitEvent(stored)");
      int rc;
      if (!loads) {
        rc = solve_with(b, s, nullptr, nullptr);
      } else {
        BlockLoad L{&in, P.ev_loaded[in_q][j], P.starts[j], plane, &P.link_bytes};
        rc = solve_with(b, s, load_block, &L);
      }
      if (rc) return fail(c, rc, std::string("block solve: ") + b->err);
      CK(cudaMemcpyAsync(&P.flags[flag_i++], b->d_error, sizeof(int), cudaMemcpyDeviceToHost, s),
         "cudaMemcpyAsync(block error flag)");
      for (int q = 0; q < 3; ++q) {
        kind_ms[q] += b->kind_ms[q] * b->kind_count[q];
        kind_count[q] += b->kind_count[q];
      }
      launches += b->launches;
      // the store overwrites planes of copy out_q that the previous round's
      // loads of this block and its neighbours read
      if (r >= 2 || (cont && r >= 1))
        for (int m = lo; m <= hi; ++m)
          CK(cudaStreamWaitEvent(s, P.ev_loaded[out_q][m], 0), "cudaStreamWaitEvent(loaded)");
      const int z1 = j + 1 < nb ? P.owned[j + 1] : V.vz;
      // (REF_CPU never moves the flows: they stay the zeros of set 0)
      const int flow_set = cpu ? 0 : (kr & 1);
      if (int rc2 = store_block(c, P, out, b, P.starts[j], P.owned[j], z1, flow_set, plane, s)) return rc2;
      CK(cudaEventRecord(P.ev_stored[out_q][j], s), "cudaEventRecord(stored)");
    }
  }
  for (int i = 0; i < kBlockContexts; ++i) {
    CK(cudaEventRecord(P.ev_end[i], P.st[i]), "cudaEventRecord(done)");
    CK(cudaStreamWaitEvent(user, P.ev_end[i], 0), "cudaStreamWaitEvent(done)");
  }
  // inputs read from host memory cross the link once per block per round
  P.link_bytes += (long long)link_inputs * nb * (long long)T * plane * (long long)sizeof(float) * P.rounds;
  c->launches = launches;
  for (int q = 0; q < 3; ++q) {
    c->kind_count[q] = kind_count[q];
    c->kind_ms[q] = kind_count[q] ? kind_ms[q] / kind_count[q] : 0.0;
  }
  c->solved = true;
  c->continuable = true;
  return HMF_OK;
}

int paged_copy_out(hmf_ctx* c, bool labels, int node, float* out, int where, void* stream) {
  PagedState& P = *c->pg;
  if (!out) return fail(c, HMF_ERR_INVALID_ARGUMENT, "output pointer is NULL");
  if (where != HMF_HOST && where != HMF_DEVICE) return fail(c, HMF_ERR_INVALID_ARGUMENT, "bad `where`");
  if (where == HMF_DEVICE)
    if (int rc = check_device_pointer(c, out, "output")) return rc;
  const auto& V = c->vols[0];
  const size_t bytes = (size_t)V.vx * V.vy * V.vz * sizeof(float);
  const HostState& H = P.host[P.final_copy];
  const float* src = labels ? H.label[node] : H.sink[node];
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (where == HMF_DEVICE) {
    CK(cudaMemcpyAsync(out, src, bytes, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(paged output)");
    return HMF_OK;
  }
  CK(cudaStreamSynchronize(s), "cudaStreamSynchronize(paged output)");
  int flag = 0;
  for (int i = 0; i < P.n_flags; ++i) flag |= P.flags[i];
  if (int rc = decode_error_flag(c, flag)) return rc;
  std::memcpy(out, src, bytes);
  return HMF_OK;
}

}  // namespace hmfi

using namespace hmfi;

extern "C" {

int hmf_set_paged_plan(hmf_ctx* c, int block_planes, int round_iterations, int inputs) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (!c->pg) return fail(c, HMF_ERR_STATE, "hmf_set_paged_plan needs an out-of-core context (hmf_create_paged)");
  if (block_planes < 0 || round_iterations < 0)
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "block planes and iterations per round must be >= 0");
  if (inputs != HMF_PAGED_INPUTS_AUTO && inputs != HMF_PAGED_INPUTS_HOST && inputs != HMF_PAGED_INPUTS_DEVICE)
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "unknown input placement");
  c->pg->forced_planes = block_planes;
  c->pg->forced_iterations = round_iterations;
  c->pg->inputs_mode = inputs;
  return HMF_OK;
}

int hmf_get_paged_plan(const hmf_ctx* c, int* blocks, int* block_planes, int* round_iterations, int* rounds,
                       long long* link_bytes) {
  if (!c || !c->pg) return HMF_ERR_INVALID_ARGUMENT;
  const PagedState& P = *c->pg;
  if (blocks) *blocks = (int)P.starts.size();
  if (block_planes) *block_planes = P.block_planes;
  if (round_iterations) *round_iterations = P.round_iterations;
  if (rounds) *rounds = P.rounds;
  if (link_bytes) *link_bytes = P.link_bytes;
  return HMF_OK;
}

int hmf_paged_layout(int vz, int block_planes, int halo_planes, int* starts, int* owned, int capacity) {
  if (vz < 1 || block_planes < 1 || halo_planes < 0) return HMF_ERR_INVALID_ARGUMENT;
  const int T = std::min(block_planes, vz), H = halo_planes;
  int nb = 1;
  if (T < vz) {
    // every block but the first and last owns T - 2H planes at most, and
    // with T >= 4H a block's owned planes are read only by its neighbours
    if (T < 4 * H || T - 2 * H < 1) return HMF_ERR_INVALID_ARGUMENT;
    nb = 1 + (int)(((long long)vz - T + (T - 2 * H) - 1) / (T - 2 * H));
  }
  std::vector<int> b(nb), a(nb);
  for (int j = 0; j < nb; ++j) {
    b[j] = nb == 1 ? 0 : (int)((long long)j * (vz - T) / (nb - 1));
    a[j] = j == 0 ? 0 : b[j] + H;
  }
  for (int j = 1; j < nb; ++j) {
    // block j-1 is exact up to b[j-1] + T - H; block j+1 starts at or after
    // what block j owns
    if (a[j] > b[j - 1] + T - H || a[j] <= a[j - 1]) return HMF_ERR_INVALID_ARGUMENT;
    if (j + 1 < nb && b[j + 1] < a[j]) return HMF_ERR_INVALID_ARGUMENT;
  }
  for (int j = 0; j < nb && j < capacity; ++j) {
    if (starts) starts[j] = b[j];
    if (owned) owned[j] = a[j];
  }
  return nb;
}

}  // extern "C"
