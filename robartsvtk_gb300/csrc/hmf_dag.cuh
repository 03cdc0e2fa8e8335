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
// the root at entry 0.  Each thread owns one voxel and keeps the nodes' values
// in shared-memory columns [quantity][entry][thread].
#pragma once

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

}  // namespace hmf
