// hmf_adjoint_sweep.cuh -- reverse of the per-voxel sink / label sweep for
// trees of N <= 8 vertices with every per-vertex quantity in registers (the
// register form of adj_tree_kernel in hmf_adjoint.cuh; same FP32 operations
// in the same order).
//
// One thread per voxel of the pitched layout (padding columns included: their
// values are finite and never read back).  All inputs of the voxel are
// independent coalesced loads issued before any arithmetic: the sweep parts
// of the later state's sink and label adjoints, the later flow reverse's gb,
// the sinks and labels before the iteration, the sinks and divergences after
// it, the data terms and the leaves' accumulated data-term gradients (so the
// double-precision accumulation is not a dependent read-modify-write at the
// end).  Per-vertex arrays are indexed only by unrolled
// compile-time indices; a runtime vertex (a parent, a child, the pre-order
// position) is reached through predicated selects, which keeps them in
// registers.
#pragma once

#include "hmf_adjoint.cuh"

namespace hmf {

constexpr int kSwThreads = 128;
constexpr int kSwMaxN = 8;

template <int N>
__device__ __forceinline__ float sw_sel(const float (&a)[N], int v) {
  float r = a[0];
#pragma unroll
  for (int w = 1; w < N; ++w) r = (w == v) ? a[w] : r;
  return r;
}

// a[v] = a[v] + x (x already carries its sign: a - b == a + (-b) exactly)
template <int N>
__device__ __forceinline__ void sw_add(float (&a)[N], int v, float x) {
#pragma unroll
  for (int w = 0; w < N; ++w)
    if (w == v) a[w] = a[w] + x;
}

template <int N>
__device__ __forceinline__ void sw_addd(double (&a)[N], bool (&hit)[N], int v, float x) {
#pragma unroll
  for (int w = 0; w < N; ++w)
    if (w == v) {
      a[w] += (double)x;
      hit[w] = true;
    }
}

template <int N>
__global__ void __launch_bounds__(kSwThreads) adj_sweep_reg_kernel(const AdjTree* __restrict__ table, const Geometry G,
                                                                   const AdjSweep S) {
  __shared__ AdjTree T;
  for (int i = threadIdx.x; i < (int)(sizeof(AdjTree) / 4); i += blockDim.x)
    reinterpret_cast<int*>(&T)[i] = reinterpret_cast<const int*>(table)[i];
  __syncthreads();
  const int root = T.root;
  const float cc = T.cc, icc = T.icc, step = T.step, step_icc = T.step * T.icc;
  const long long arr = S.arr;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol;
       i += (long long)gridDim.x * blockDim.x) {
    float SBN[N], UB[N], GB[N], AS[N], AU[N], BS[N], BD[N], D[N];
    double DB[N];  // data-term gradients of the leaves, read with the inputs
    bool hit[N];
#pragma unroll
    for (int v = 0; v < N; ++v) {
      const long long b = T.sbase[v];
      SBN[v] = S.sbn[v * arr + i];
      BS[v] = S.stB[b * arr + i];
      AS[v] = T.n_kids[v] ? S.stA[b * arr + i] : 0.f;   // read by leaf children
      D[v] = T.n_kids[v] ? 0.f : T.data[v][i];
      DB[v] = T.n_kids[v] ? 0.0 : T.Db[v][i];
      hit[v] = false;
      const bool nr = v != root;
      UB[v] = nr ? S.ubn[v * arr + i] : 0.f;
      GB[v] = nr ? S.gbn[v * arr + i] : 0.f;
      AU[v] = nr ? S.stA[(b + kAdjLabel) * arr + i] : 0.f;
      BD[v] = nr ? S.stB[(b + kAdjDiv) * arr + i] : 0.f;
    }
    // full adjoints of the later state: sinks (sweep part, then the flow
    // part vertex by vertex in id order: own +step*gb, children's -step*gb)
    // and labels (sweep part - step*icc*gb)
#pragma unroll
    for (int w = 0; w < N; ++w) {
      float a = SBN[w];
#pragma unroll
      for (int v = 0; v < N; ++v) {
        if (v == root) continue;
        const float d = step * GB[v];
        if (v == w) a = a + d;
        else if (T.parent[v] == w) a = a - d;
      }
      SBN[w] = a;
      UB[w] = UB[w] - step_icc * GB[w];
    }
    float SBO[N], UBO[N], DBP[N];
#pragma unroll
    for (int v = 0; v < N; ++v) SBO[v] = UBO[v] = DBP[v] = 0.f;
    // labels: u' = sat(u + cc*((s'_parent - d') - s')), vertex id order
#pragma unroll
    for (int v = 0; v < N; ++v) {
      if (v == root) continue;
      const int p = T.parent[v];
      const float zv = AU[v] + cc * ((sw_sel(BS, p) - BD[v]) - BS[v]);
      const float zb = (zv > 0.0f && zv < 1.0f) ? UB[v] : 0.0f;
      UBO[v] = UBO[v] + zb;
      sw_add(SBN, p, cc * zb);
      DBP[v] = DBP[v] - cc * zb;
      SBN[v] = SBN[v] - cc * zb;
    }
    // sinks, parents before children (pre-order)
#pragma unroll
    for (int k = 0; k < N; ++k) {
      const int v = T.preorder[k];
      const float sbn = sw_sel(SBN, v);
      if (T.n_kids[v] == 0) {
        const int p = T.parent[v];
        const float yv = (sw_sel(AS, p) - sw_sel(BD, v)) + sw_sel(AU, v) * icc;
        if (yv < 0.0f) continue;
        if (yv > sw_sel(D, v)) {
          sw_addd(DB, hit, v, sbn);
          continue;
        }
        sw_add(SBO, p, sbn);
        sw_add(DBP, v, -sbn);
        sw_add(UBO, v, icc * sbn);
      } else {
        const float Wb = sbn * T.inv_kids[v];
        if (v != root) {
          sw_add(SBO, T.parent[v], Wb);
          sw_add(DBP, v, -Wb);
          sw_add(UBO, v, icc * Wb);
        }
        const float iW = icc * Wb;
#pragma unroll
        for (int w = 0; w < N; ++w)
          if (T.parent[w] == v) {
            SBN[w] = SBN[w] + Wb;
            DBP[w] = DBP[w] + Wb;
            UBO[w] = UBO[w] - iW;
          }
      }
    }
#pragma unroll
    for (int v = 0; v < N; ++v) {
      S.sbo[v * arr + i] = SBO[v];
      if (v != root) {
        S.ubo[v * arr + i] = UBO[v];
        S.dbp[v * arr + i] = DBP[v];
      }
      if (hit[v]) T.Db[v][i] = DB[v];
    }
  }
}

}  // namespace hmf
