// hmf_dag.cuh -- the per-voxel part of the directed-acyclic-graph max-flow
// solver (DAGMF) as vtkCudaDirectedAcyclicGraphMaxFlowSegmentation runs it.
//
// The reference expresses an iteration as a task graph
// (vtkCudaDirectedAcyclicGraphMaxFlowSegmentation.cxx:343-842) over the
// kernels of CUDA_hierarchicalmaxflow.cu; its scheduler breaks ties between
// ready tasks with rand() (vtkCudaMaxFlowSegmentationScheduler.cxx:232-236).
// This file runs that graph in one fixed topological order, per voxel, after
// the spatial flow step (flow_tma_kernel, whose "inc" map points at each
// node's own source buffer here):
//
//   (2) leaves: s = clamp(inc - div + u/CC, 0, D) (kern_FindLeafSinkPotential
//       :166, kern_ApplyCapacity :187), then u = sat(u + CC(inc - div - s))
//       (kern_UpdateLabel :211); branches: s = (1-k) s + k (inc - div + u/CC)
//       (kern_ResetSinkBuffer :610); the root: s = 1*s + shift (TranslateBuffer,
//       CUDA_commonKernels.cu:96);
//   not in the last iteration (those tasks run one time fewer):
//   (3) nodes deepest first, each in-edge in edge order: s_parent +=
//       w_up (s - inc + div - u/CC) (kern_PushUpSourceFlows :631); then a
//       branch's label update;
//   (4) every node: inc = 0 + sum over in-edges of w_down s_parent
//       (ZeroOutBuffer, SumScaledBuffers CUDA_commonKernels.cu:419).
//
// Entries are the nodes in the rooted DAG's forward-iterator order (level by
// level from the root; vtkRootedDirectedAcyclicGraphForwardIterator.cxx:95-120),
// the root at entry 0.
//
// dag_bulk_kernel (the default) streams the volume through shared memory:
// a persistent CTA walks chunks of VC voxels, brings every array the sweep
// reads (per non-root node sink, source, divergence, label; each leaf's data
// term; the root's source) into one of two stages with one cp.async.bulk per
// array, completed by an mbarrier, and each thread sweeps one voxel of the
// staged chunk in place while the next chunk is in flight.  dag_sweep_kernel
// is the same arithmetic reading global memory directly, each thread keeping
// the nodes' values in shared-memory columns [quantity][entry][thread]
// (HMF_DAG_KERNEL=simple).
#pragma once

#include "hmf_async.cuh"
#include "hmf_types.cuh"

namespace hmf {

constexpr int kDagThreads = 128;

__device__ __forceinline__ void dag_copy_table(DagTable& T, const DagTable* table) {
  for (int i = threadIdx.x; i < (int)(sizeof(DagTable) / 4); i += blockDim.x)
    reinterpret_cast<int*>(&T)[i] = reinterpret_cast<const int*>(table)[i];
}

// Initialisation (vtkCudaDirectedAcyclicGraphMaxFlowSegmentation.cxx:884-1045):
// source = min over leaves of D (kern_MinBuffers, leaves in forward order);
// every sink and source buffer = that minimum (kern_Copy2Buffers); leaf labels
// [s == D] / sum (kern_Lbl, SumBuffers, kern_DivideBuffers); branch labels,
// deepest first, 0 + sum over out-edges of w u_child (SumScaledBuffers).
__global__ void __launch_bounds__(kDagThreads) dag_init_kernel(const DagTable* __restrict__ table, long long n_vox) {
  __shared__ DagTable T;
  extern __shared__ float dag_st[];  // labels [entry][thread]
  dag_copy_table(T, table);
  __syncthreads();
  const int n = T.n, t = threadIdx.x;
  auto U = [&](int e) -> float& { return dag_st[e * kDagThreads + t]; };
  for (long long i = (long long)blockIdx.x * kDagThreads + t; i < n_vox; i += (long long)gridDim.x * kDagThreads) {
    float src = T.e[T.leaves[0]].data[i];
    for (int j = 1; j < T.n_leaves; ++j) {
      const float d = T.e[T.leaves[j]].data[i];
      src = (src < d) ? src : d;
    }
    T.e[0].sink[i] = src;
    for (int e = 1; e < n; ++e) {
      T.e[e].sink[i] = src;
      T.e[e].inc[i] = src;
    }
    float acc = 0.0f;
    for (int j = 0; j < T.n_leaves; ++j) {
      const int l = T.leaves[j];
      const float lbl = (src == T.e[l].data[i]) ? 1.0f : 0.0f;
      U(l) = lbl;
      acc = acc + lbl;
    }
    for (int j = 0; j < T.n_leaves; ++j) U(T.leaves[j]) = U(T.leaves[j]) / acc;
    for (int e = n - 1; e >= 1; --e) {
      const DagEntry& E = T.e[e];
      if (E.leaf) continue;
      float u = 0.0f;
      for (int j = E.first_out; j < E.first_out + E.n_out; ++j) u = u + T.out_w[j] * U(T.out_child[j]);
      U(e) = u;
    }
    for (int e = 1; e < n; ++e) T.e[e].label[i] = U(e);
  }
}

// The sink, source and label part of one iteration (see the file comment);
// `last` drops (3) and (4), which the reference runs one time fewer.
__global__ void __launch_bounds__(kDagThreads)
    dag_sweep_kernel(const DagTable* __restrict__ table, long long n_vox, int last) {
  __shared__ DagTable T;
  extern __shared__ float dag_st[];  // [sink, inc, div, label][entry][thread]
  dag_copy_table(T, table);
  __syncthreads();
  const int n = T.n, t = threadIdx.x;
  const float cc = T.cc, icc = T.icc;
  float* const Sa = dag_st;
  float* const Ca = dag_st + n * kDagThreads;
  float* const Da = dag_st + 2 * n * kDagThreads;
  float* const Ua = dag_st + 3 * n * kDagThreads;
  auto S = [&](int e) -> float& { return Sa[e * kDagThreads + t]; };
  auto C = [&](int e) -> float& { return Ca[e * kDagThreads + t]; };
  auto D = [&](int e) -> float& { return Da[e * kDagThreads + t]; };
  auto U = [&](int e) -> float& { return Ua[e * kDagThreads + t]; };
  for (long long i = (long long)blockIdx.x * kDagThreads + t; i < n_vox; i += (long long)gridDim.x * kDagThreads) {
    S(0) = T.e[0].sink[i];
    for (int e = 1; e < n; ++e) {
      const DagEntry& E = T.e[e];
      S(e) = E.sink[i];
      C(e) = E.inc[i];
      D(e) = E.div[i];
      U(e) = E.label[i];
    }
    // (2)
    S(0) = 1.0f * S(0) + T.shift;
    for (int e = 1; e < n; ++e) {
      const DagEntry& E = T.e[e];
      const float c = C(e), d = D(e), u = U(e);
      if (E.leaf) {
        float v = (c - d) + u * icc;
        const float cap = E.data[i];
        v = (v < 0.0f) ? 0.0f : v;
        v = (v > cap) ? cap : v;
        S(e) = v;
        U(e) = __saturatef(u + cc * ((c - d) - v));
      } else {
        S(e) = (1.0f - E.k) * S(e) + E.k * ((c - d) + u * icc);
      }
    }
    if (!last) {
      // (3) deepest first: every push into a node precedes its own
      for (int e = n - 1; e >= 1; --e) {
        const DagEntry& E = T.e[e];
        const float s = S(e), c = C(e), d = D(e), u = U(e);
        const float pot = ((s - c) + d) - u * icc;
        for (int j = E.first_in; j < E.first_in + E.n_in; ++j) {
          float& ps = S(T.in_parent[j]);
          ps = ps + T.in_wup[j] * pot;
        }
        if (!E.leaf) U(e) = __saturatef(u + cc * ((c - d) - s));
      }
      // (4)
      for (int e = 1; e < n; ++e) {
        const DagEntry& E = T.e[e];
        float c = 0.0f;
        for (int j = E.first_in; j < E.first_in + E.n_in; ++j) c = c + T.in_wdown[j] * S(T.in_parent[j]);
        C(e) = c;
      }
    }
    T.e[0].sink[i] = S(0);
    for (int e = 1; e < n; ++e) {
      const DagEntry& E = T.e[e];
      E.sink[i] = S(e);
      E.label[i] = U(e);
      if (!last) E.inc[i] = C(e);
    }
  }
}

// Staged arrays of dag_bulk_kernel: non-root entry e >= 1 -> sink 4(e-1),
// source 4(e-1)+1, divergence 4(e-1)+2, label 4(e-1)+3; leaf j's data term
// 4(n-1)+j; the root's source 4(n-1)+n_leaves.
__host__ __device__ inline int dag_bulk_arrays(int n, int n_leaves) { return 4 * (n - 1) + n_leaves + 1; }
constexpr int kDagBulkStages = 2;
constexpr int kDagBulkSmemBudget = 64 * 1024;  // both stages: three CTAs per SM

// Chunk length (voxels, one per thread): the largest power of two <= 256
// whose stages fit the budget (at least 32).
__host__ __device__ inline int dag_bulk_chunk(int arrays) {
  int vc = 256;
  while (vc > 32 && kDagBulkStages * arrays * vc * 4 > kDagBulkSmemBudget) vc /= 2;
  return vc;
}

__host__ __device__ inline int dag_bulk_smem_bytes(int arrays) {
  return 128 + kDagBulkStages * arrays * dag_bulk_chunk(arrays) * 4;
}

__global__ void dag_bulk_kernel(const DagTable* __restrict__ table, long long n_vox, int last,
                                int* __restrict__ error_flag) {
  __shared__ DagTable T;
  __shared__ int abort_cta, stall_cta, stop_cta;
  __shared__ int leaf_slot[kMaxVertices];  // entry -> staged data slot
  extern __shared__ __align__(128) unsigned char db_raw[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(db_raw);  // [kDagBulkStages]
  float* const stage0 = reinterpret_cast<float*>(db_raw + 128);
  dag_copy_table(T, table);
  __syncthreads();  // thread 0 reads the table below
  if (threadIdx.x == 0) {
    const int flag = error_flag ? *(volatile int*)error_flag : 0;
    abort_cta = flag & 2;
    stall_cta = take_stall_request(error_flag, flag);
    stop_cta = 0;
    if (smem_addr(db_raw) & 15) {
      abort_cta = 1;
      if (error_flag) atomicOr(error_flag, 4);
    }
    // one arrival per staged array (the copies are spread over the threads)
    for (int s = 0; s < kDagBulkStages; ++s) mbar_init(&bars[s], (unsigned)dag_bulk_arrays(T.n, T.n_leaves));
    mbar_init(&bars[kDagBulkStages], 1);  // completed by nothing: a requested stall waits on it
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (abort_cta) return;
  const int n = T.n, nl = T.n_leaves;
  for (int e = threadIdx.x; e < n; e += blockDim.x) leaf_slot[e] = -1;
  __syncthreads();
  for (int j = threadIdx.x; j < nl; j += blockDim.x) leaf_slot[T.leaves[j]] = 4 * (n - 1) + j;
  __syncthreads();
  const int A = dag_bulk_arrays(n, nl);
  const int VC = dag_bulk_chunk(A);
  const int root_slot = 4 * (n - 1) + nl;
  const long long nchunks = (n_vox + VC - 1) / VC;
  const float cc = T.cc, icc = T.icc;

  // Staged slot c of a chunk is copied by thread c (c, c + blockDim, ...),
  // each copy with its own expected bytes and mbarrier arrival: entry e's
  // sink, source, divergence and label (slots 4(e-1) .. 4(e-1)+3), leaf j's
  // data term (4(n-1) + j), the root sink (root_slot).
  auto slot_src = [&](int c) -> const float* {
    if (c < 4 * (n - 1)) {
      const DagEntry& E = T.e[c / 4 + 1];
      const int kind = c % 4;
      return kind == 0 ? E.sink : kind == 1 ? E.inc : kind == 2 ? E.div : E.label;
    }
    if (c < root_slot) return T.e[T.leaves[c - 4 * (n - 1)]].data;
    return T.e[0].sink;
  };
  auto issue = [&](long long chunk, int s) {
    const long long v0 = chunk * VC;
    const unsigned bytes = (unsigned)(min((long long)VC, n_vox - v0) * 4);
    float* dst = stage0 + (size_t)s * A * VC;
    for (int c = threadIdx.x; c < A; c += blockDim.x) {
      mbar_expect_tx(&bars[s], bytes);
      bulk_load(dst + (size_t)c * VC, slot_src(c) + v0, bytes, &bars[s]);
    }
  };

  bool timed_out = false;
  int nissued[kDagBulkStages] = {0, 0};  // kept by every thread (thread 0 always issues)
  long long chunk = blockIdx.x;
  if (chunk < nchunks) issue(chunk, 0), ++nissued[0];
  if (chunk + gridDim.x < nchunks) issue(chunk + gridDim.x, 1), ++nissued[1];
  // a requested stall: a wait that runs out, so the time-out path runs
  if (threadIdx.x == 0 && stall_cta && !mbar_wait_bounded(&bars[kDagBulkStages], 0, kTmaWaitLimitNs)) {
    timed_out = true;
    *(volatile int*)&stop_cta = 1;
  }
  for (int j = 0; chunk < nchunks; ++j, chunk += gridDim.x) {
    const int s = j & 1;
    if (!timed_out && !mbar_wait_bounded(&bars[s], (unsigned)((j >> 1) & 1), kTmaWaitLimitNs)) {
      timed_out = true;
      *(volatile int*)&stop_cta = 1;
    }
    const long long v0 = chunk * VC;
    const int len = (int)min((long long)VC, n_vox - v0);
    const int q = threadIdx.x;
    if (q < len) {
      float* st = stage0 + (size_t)s * A * VC + q;
      auto S = [&](int e) -> float& { return st[(e ? 4 * (e - 1) : root_slot) * VC]; };
      auto C = [&](int e) -> float& { return st[(4 * (e - 1) + 1) * VC]; };
      auto D = [&](int e) -> float& { return st[(4 * (e - 1) + 2) * VC]; };
      auto U = [&](int e) -> float& { return st[(4 * (e - 1) + 3) * VC]; };
      // (2)
      S(0) = 1.0f * S(0) + T.shift;
      for (int e = 1; e < n; ++e) {
        const float c = C(e), d = D(e), u = U(e);
        if (leaf_slot[e] >= 0) {
          float v = (c - d) + u * icc;
          const float cap = st[leaf_slot[e] * VC];
          v = (v < 0.0f) ? 0.0f : v;
          v = (v > cap) ? cap : v;
          S(e) = v;
          U(e) = __saturatef(u + cc * ((c - d) - v));
        } else {
          const float k = T.e[e].k;
          S(e) = (1.0f - k) * S(e) + k * ((c - d) + u * icc);
        }
      }
      if (!last) {
        // (3) deepest first: every push into a node precedes its own
        for (int e = n - 1; e >= 1; --e) {
          const DagEntry& E = T.e[e];
          const float sv = S(e), c = C(e), d = D(e), u = U(e);
          const float pot = ((sv - c) + d) - u * icc;
          for (int k = E.first_in; k < E.first_in + E.n_in; ++k) {
            float& ps = S(T.in_parent[k]);
            ps = ps + T.in_wup[k] * pot;
          }
          if (leaf_slot[e] < 0) U(e) = __saturatef(u + cc * ((c - d) - sv));
        }
        // (4)
        for (int e = 1; e < n; ++e) {
          const DagEntry& E = T.e[e];
          float c = 0.0f;
          for (int k = E.first_in; k < E.first_in + E.n_in; ++k) c = c + T.in_wdown[k] * S(T.in_parent[k]);
          C(e) = c;
        }
      }
      const long long i = v0 + q;
      T.e[0].sink[i] = S(0);
      for (int e = 1; e < n; ++e) {
        const DagEntry& E = T.e[e];
        E.sink[i] = S(e);
        E.label[i] = U(e);
        if (!last) E.inc[i] = C(e);
      }
    }
    // The sweep wrote into stage s with ordinary stores; order them before
    // the bulk copy that refills the stage (async proxy).
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (stop_cta) break;  // a copy wait ran out: no further copies
    if (chunk + 2LL * gridDim.x < nchunks) issue(chunk + 2LL * gridDim.x, s), ++nissued[s];
  }
  __syncthreads();
  // Copies into this CTA's shared memory must have landed before it exits:
  // after a time-out each issuing thread waits (bounded) for the last copy it
  // issued into each stage (nothing is issued after stop_cta).
  if (stop_cta) {
    if (threadIdx.x == 0 && error_flag) atomicOr(error_flag, 2);
    for (int s = 0; s < kDagBulkStages; ++s)
      if (nissued[s]) mbar_wait_bounded(&bars[s], (unsigned)((nissued[s] - 1) & 1), kTmaWaitLimitNs);
  }
}

// dag_bulk_kernel for graphs of N <= 8 entries without repeated edges: the
// graph in kernel parameters, staged slots at compile-time offsets (entry
// e >= 1: sink 4(e-1), source +1, divergence +2, label +3, data term
// 4(N-1) + e-1; the root's source 5(N-1)), so the per-voxel program reads no
// table.  Same arithmetic and order as dag_bulk_kernel.
constexpr int kDagNVc = 256;
__host__ __device__ constexpr int dag_bulk_n_arrays(int N) { return 5 * (N - 1) + 1; }
__host__ __device__ constexpr int dag_bulk_n_smem_bytes(int N) {
  return 128 + kDagBulkStages * dag_bulk_n_arrays(N) * kDagNVc * 4;
}

template <int N>
__global__ void __launch_bounds__(kDagNVc)
    dag_bulk_n_kernel(const __grid_constant__ DagRegParams P, long long n_vox, int last, int* __restrict__ error_flag) {
  constexpr int A = dag_bulk_n_arrays(N);
  constexpr int VC = kDagNVc;
  constexpr int ROOT = 5 * (N - 1);
  __shared__ int abort_cta, stall_cta, stop_cta;
  extern __shared__ __align__(128) unsigned char dn_raw[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(dn_raw);
  float* const stage0 = reinterpret_cast<float*>(dn_raw + 128);
  if (threadIdx.x == 0) {
    const int flag = error_flag ? *(volatile int*)error_flag : 0;
    abort_cta = flag & 2;
    stall_cta = take_stall_request(error_flag, flag);
    stop_cta = 0;
    if (smem_addr(dn_raw) & 15) {
      abort_cta = 1;
      if (error_flag) atomicOr(error_flag, 4);
    }
    // one arrival per copied array: 4 per non-root node, the data term of
    // each leaf, the root sink
    const unsigned narr = 4u * (N - 1) + 1u + (unsigned)__popc(P.leaf_mask & ((1u << N) - 2u));
    for (int s = 0; s < kDagBulkStages; ++s) mbar_init(&bars[s], narr);
    mbar_init(&bars[kDagBulkStages], 1);  // completed by nothing: a requested stall waits on it
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (abort_cta) return;
  const float cc = P.cc, icc = P.icc;
  const long long nchunks = (n_vox + VC - 1) / VC;
  auto slot_s = [](int e) { return e ? 4 * (e - 1) : ROOT; };

  // Staged slot a of a chunk is copied by thread a, with its own expected
  // bytes and mbarrier arrival: node e's sink, source, divergence and label
  // (slots 4(e-1) .. 4(e-1)+3), a leaf's data term (4(N-1) + e-1; absent for
  // branches: no copy, no arrival), the root sink (ROOT).
  const int ta = threadIdx.x;
  const float* asrc = nullptr;
  if (ta < 4 * (N - 1)) {
    const int e = ta / 4 + 1, kind = ta % 4;
    asrc = kind == 0 ? P.sink[e] : kind == 1 ? P.inc[e] : kind == 2 ? P.div[e] : P.label[e];
  } else if (ta < ROOT) {
    const int e = ta - 4 * (N - 1) + 1;
    if ((P.leaf_mask >> e) & 1u) asrc = P.data[e];
  } else if (ta == ROOT) {
    asrc = P.sink[0];
  }
  auto issue = [&](long long chunk, int s) {  // threads with a slot to fill
    const long long v0 = chunk * VC;
    const unsigned bytes = (unsigned)(min((long long)VC, n_vox - v0) * 4);
    mbar_expect_tx(&bars[s], bytes);
    bulk_load(stage0 + (size_t)s * A * VC + (size_t)ta * VC, asrc + v0, bytes, &bars[s]);
  };

  bool timed_out = false;
  int nissued[kDagBulkStages] = {0, 0};  // kept by every issuing thread
  long long chunk = blockIdx.x;
  if (asrc) {
    if (chunk < nchunks) issue(chunk, 0), ++nissued[0];
    if (chunk + gridDim.x < nchunks) issue(chunk + gridDim.x, 1), ++nissued[1];
  }
  // a requested stall: a wait that runs out, so the time-out path runs
  if (threadIdx.x == 0 && stall_cta && !mbar_wait_bounded(&bars[kDagBulkStages], 0, kTmaWaitLimitNs)) {
    timed_out = true;
    *(volatile int*)&stop_cta = 1;
  }
  for (int j = 0; chunk < nchunks; ++j, chunk += gridDim.x) {
    const int s = j & 1;
    if (!timed_out && !mbar_wait_bounded(&bars[s], (unsigned)((j >> 1) & 1), kTmaWaitLimitNs)) {
      timed_out = true;
      *(volatile int*)&stop_cta = 1;
    }
    const long long v0 = chunk * VC;
    const int len = (int)min((long long)VC, n_vox - v0);
    const int q = threadIdx.x;
    if (q < len) {
      float* st = stage0 + (size_t)s * A * VC + q;
      float S[N], C[N], D[N], U[N];
      S[0] = st[ROOT * VC];
#pragma unroll
      for (int e = 1; e < N; ++e) {
        S[e] = st[(4 * (e - 1)) * VC];
        C[e] = st[(4 * (e - 1) + 1) * VC];
        D[e] = st[(4 * (e - 1) + 2) * VC];
        U[e] = st[(4 * (e - 1) + 3) * VC];
      }
      // (2)
      S[0] = 1.0f * S[0] + P.shift;
#pragma unroll
      for (int e = 1; e < N; ++e) {
        const float c = C[e], d = D[e], u = U[e];
        if ((P.leaf_mask >> e) & 1u) {
          float v = (c - d) + u * icc;
          const float cap = st[(4 * (N - 1) + e - 1) * VC];
          v = (v < 0.0f) ? 0.0f : v;
          v = (v > cap) ? cap : v;
          S[e] = v;
          U[e] = __saturatef(u + cc * ((c - d) - v));
        } else {
          S[e] = (1.0f - P.k[e]) * S[e] + P.k[e] * ((c - d) + u * icc);
        }
      }
      if (!last) {
        // (3) deepest first; a node's parents precede it in forward order
#pragma unroll
        for (int e = N - 1; e >= 1; --e) {
          const float pot = ((S[e] - C[e]) + D[e]) - U[e] * icc;
#pragma unroll
          for (int p = 0; p < e; ++p)
            if ((P.pmask[e] >> p) & 1u) S[p] = S[p] + P.wup[e][p] * pot;
          if (!((P.leaf_mask >> e) & 1u)) U[e] = __saturatef(U[e] + cc * ((C[e] - D[e]) - S[e]));
        }
        // (4) parents in in-edge order
#pragma unroll
        for (int e = 1; e < N; ++e) {
          float c = 0.0f;
          for (int k = 0; k < P.n_in[e]; ++k) {
            const int p = P.parent_ord[e][k];
            float sp = S[0];
#pragma unroll
            for (int w = 1; w < e; ++w) sp = (w == p) ? S[w] : sp;
            c = c + P.wdown_ord[e][k] * sp;
          }
          C[e] = c;
        }
      }
      const long long i = v0 + q;
      P.sink[0][i] = S[0];
#pragma unroll
      for (int e = 1; e < N; ++e) {
        P.sink[e][i] = S[e];
        P.label[e][i] = U[e];
        if (!last) P.inc[e][i] = C[e];
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();  // stage s is free again
    if (stop_cta) break;  // a copy wait ran out: no further copies
    if (asrc && chunk + 2LL * gridDim.x < nchunks) issue(chunk + 2LL * gridDim.x, s), ++nissued[s];
  }
  __syncthreads();
  // Copies into this CTA's shared memory must have landed before it exits:
  // after a time-out each issuing thread waits (bounded) for the last copy it
  // issued into each stage (nothing is issued after stop_cta).
  if (stop_cta) {
    if (threadIdx.x == 0 && error_flag) atomicOr(error_flag, 2);
    for (int s = 0; s < kDagBulkStages; ++s)
      if (nissued[s]) mbar_wait_bounded(&bars[s], (unsigned)((nissued[s] - 1) & 1), kTmaWaitLimitNs);
  }
}

}  // namespace hmf
