// hmf_post.cuh -- what follows a solve: the label vote and the energy
// decomposition of a labelling.
//
//  vote_kernel    per voxel, the id of the input image with the largest
//                 value: semantics 0 follows vtkCudaImageVote (running
//                 maximum starting at input 0, each input in port order
//                 taking over when value >= maximum, CUDA_imagevote.cu:30-46
//                 launched per input :249-256: the last of a tie wins),
//                 semantics 1 follows vtkImageVote (first input, then any
//                 strictly greater one: vtkImageVote.cxx:285-306).  One pass:
//                 every input read once, one int written.  vote4_kernel is
//                 the same four voxels at a time for 16-byte aligned rows.
//  energy_kernel  f0 = sum of D_l * u_l over leaves and voxels; per non-root
//                 vertex f_v = sum of S_v * 0.5*sqrt(|grad u_v|^2) with the
//                 clamped central differences of kern_GHMFD_GradientBuffer
//                 (CUDA_hierarchicalmaxflowdecomp.cu:19-38; its `g += d*d`
//                 compiled to fused multiply-adds), a branch's labelling
//                 being the sum of its children's in child order
//                 (vtkCudaHierarchicalMaxFlowDecomposition.cxx:750-806).  One
//                 pass over all vertices per voxel (the reference makes one
//                 gradient, one multiply and one reduction pass per vertex);
//                 per-voxel terms in FP32 in the reference's operation order,
//                 sums in FP64 (the reference reduces in FP32).
//                 energy_reg_kernel<N> is the same for trees of N <= 8
//                 non-root vertices: the tree in kernel parameters (bit
//                 masks: no table reads per voxel), every per-vertex value
//                 in registers, one warp per row at a time.
// Arrays are pitched rows (`pitch` floats per row, dense when pitch == vx);
// outputs of the vote are dense.  The energy kernels walk rows, so no voxel
// index is divided; per-thread sums are float-float (FP32 pipes), merged in
// FP64 per warp.
#pragma once

#include "hmf_types.cuh"

namespace hmf {

constexpr int kPostThreads = 256;

struct VoteInputs {
  const float* in[kMaxVertices];
  int values[kMaxVertices];
  int n;
  int semantics;
};

__global__ void __launch_bounds__(kPostThreads) vote_kernel(const VoteInputs V, const Geometry G, int* __restrict__ out) {
  const long long dense = (long long)G.vx * G.vy * G.vz;
  for (long long d = (long long)blockIdx.x * blockDim.x + threadIdx.x; d < dense;
       d += (long long)gridDim.x * blockDim.x) {
    const long long r = d / G.vx;
    const long long i = r * G.pitch + (d - r * G.vx);
    int id;
    if (V.semantics == 0) {
      float mx = __ldg(V.in[0] + i);
      id = V.values[0];
      for (int k = 1; k < V.n; ++k) {
        const float v = __ldg(V.in[k] + i);
        if (v >= mx) {
          id = V.values[k];
          mx = v;
        }
      }
    } else {
      id = -1;
      float mx = 0.0f;
      for (int k = 0; k < V.n; ++k) {
        const float v = __ldg(V.in[k] + i);
        if (id == -1 || v > mx) {
          id = V.values[k];
          mx = v;
        }
      }
      if (id == -1) id = 0;
    }
    out[d] = id;
  }
}

// The vote over pitched rows four voxels at a time: requires pitch % 4 == 0
// and 16-byte aligned inputs (every solver array is).  Quad q covers pitched
// elements 4q..4q+3 of one row; outputs only where x < vx.
__global__ void __launch_bounds__(kPostThreads) vote4_kernel(const VoteInputs V, const Geometry G, int* __restrict__ out) {
  const long long rows = (long long)G.vy * G.vz;
  const int qpr = G.pitch >> 2;  // quads per row
  const long long nq = rows * qpr;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += (long long)gridDim.x * blockDim.x) {
    const long long r = q / qpr;
    const int x = (int)(q - r * qpr) * 4;
    const long long i = r * G.pitch + x;
    float4 mx = __ldg(reinterpret_cast<const float4*>(V.in[0] + i));
    int id0, id1, id2, id3;
    id0 = id1 = id2 = id3 = V.values[0];  // input 0 always takes the first turn
    if (V.semantics == 0) {
      for (int k = 1; k < V.n; ++k) {
        const float4 v = __ldg(reinterpret_cast<const float4*>(V.in[k] + i));
        const int val = V.values[k];
        if (v.x >= mx.x) id0 = val, mx.x = v.x;
        if (v.y >= mx.y) id1 = val, mx.y = v.y;
        if (v.z >= mx.z) id2 = val, mx.z = v.z;
        if (v.w >= mx.w) id3 = val, mx.w = v.w;
      }
    } else {
      // "no winner yet" stays true while the winning id is -1 (vtkImageVote's marker)
      bool none0 = id0 == -1, none1 = none0, none2 = none0, none3 = none0;
      for (int k = 1; k < V.n; ++k) {
        const float4 v = __ldg(reinterpret_cast<const float4*>(V.in[k] + i));
        const int val = V.values[k];
        if (none0 || v.x > mx.x) id0 = val, mx.x = v.x, none0 = val == -1;
        if (none1 || v.y > mx.y) id1 = val, mx.y = v.y, none1 = val == -1;
        if (none2 || v.z > mx.z) id2 = val, mx.z = v.z, none2 = val == -1;
        if (none3 || v.w > mx.w) id3 = val, mx.w = v.w, none3 = val == -1;
      }
      if (id0 == -1) id0 = 0;
      if (id1 == -1) id1 = 0;
      if (id2 == -1) id2 = 0;
      if (id3 == -1) id3 = 0;
    }
    int* o = out + r * G.vx + x;
    if (x < G.vx) o[0] = id0;
    if (x + 1 < G.vx) o[1] = id1;
    if (x + 2 < G.vx) o[2] = id2;
    if (x + 3 < G.vx) o[3] = id3;
  }
}

// Tree in post-order for the energy: entry e's children precede it.
struct EnergyTable {
  int n;  // entries (the root excluded)
  int n_kids_total;
  int first_kid[kMaxVertices];
  int n_kids[kMaxVertices];
  int kids[kMaxVertices];             // entry indices, child order
  int vertex[kMaxVertices];           // vertex id of each entry
  int parent_entry[kMaxVertices];     // entry index of the parent (-1: the root)
  const float* label[kMaxVertices];   // leaves: labelling
  const float* data[kMaxVertices];    // leaves: data term
  const float* smooth[kMaxVertices];  // smoothness image or null (S = 1)
};

// kern_GHMFD_GradientBuffer's term from the labelling at the voxel's six
// neighbours (+x, -x, +y, -y, +z, -z in u[1..6]), as compiled: g += d*d is
// one fused multiply-add per axis.
__device__ __forceinline__ float energy_grad_term(const float* u) {
  const float dx = u[1] - u[2], dy = u[3] - u[4], dz = u[5] - u[6];
  float g2 = __fmaf_rn(dx, dx, 0.0f);
  g2 = __fmaf_rn(dy, dy, g2);
  g2 = __fmaf_rn(dz, dz, g2);
  return 0.5f * sqrtf(g2);
}

// Neighbour offsets of voxel (x, y, z) in pitched memory; at the border the
// neighbour is the voxel itself.
__device__ __forceinline__ void energy_offsets(const Geometry& G, int x, int y, int z, long long (&o)[7]) {
  o[0] = 0;
  o[1] = x == G.vx - 1 ? 0 : 1;
  o[2] = x == 0 ? 0 : -1;
  o[3] = y == G.vy - 1 ? 0 : (long long)G.pitch;
  o[4] = y == 0 ? 0 : -(long long)G.pitch;
  o[5] = z == G.vz - 1 ? 0 : G.plane;
  o[6] = z == 0 ? 0 : -G.plane;
}

// Float-float running sum (hi + lo): each term is added with Knuth's
// TwoSum, its rounding error collected in lo.  FP32 instructions only (the
// FP64 rate of this part is a small fraction of FP32's); relative error about
// n * 2^-48 after n terms of one sign, against 2^-24 for a plain float sum.
struct FF {
  float hi, lo;
};

__device__ __forceinline__ void ff_add(FF& a, float t) {
  const float s = a.hi + t;
  const float bb = s - a.hi;
  const float err = (a.hi - (s - bb)) + (t - bb);
  a.hi = s;
  a.lo += err;
}

__device__ __forceinline__ FF ff_merge(FF a, FF b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float err = (a.hi - (s - bb)) + (b.hi - bb);
  return {s, (a.lo + b.lo) + err};
}

// Block sum of one quantity into *dst (float-float across the warp, double
// across warps, one atomic per block).  Every thread of the block calls it.
__device__ __forceinline__ void energy_reduce_to(FF v, double* dst, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int s = 16; s > 0; s >>= 1) {
    const FF o = {__shfl_down_sync(0xffffffffu, v.hi, s), __shfl_down_sync(0xffffffffu, v.lo, s)};
    v = ff_merge(v, o);
  }
  if (lane == 0) red[warp] = (double)v.hi + (double)v.lo;
  __syncthreads();
  if (warp == 0) {
    double t = lane < kPostThreads / 32 ? red[lane] : 0.0;
    for (int s = kPostThreads / 64; s > 0; s >>= 1) t += __shfl_down_sync(0xffffffffu, t, s);
    if (lane == 0 && t != 0.0) atomicAdd(dst, t);
  }
  __syncthreads();
}

// sums[0] = f0, sums[1 + vertex of entry e-1] = f of that vertex.
__device__ __forceinline__ void energy_reduce_one(const EnergyTable& T, FF v, int e, double* sums, double* red) {
  energy_reduce_to(v, &sums[e == 0 ? 0 : 1 + T.vertex[e - 1]], red);
}

__global__ void __launch_bounds__(kPostThreads) energy_kernel(const EnergyTable* __restrict__ table, const Geometry G,
                                                              double* __restrict__ sums /* [0] f0, [1+vertex] f */) {
  __shared__ EnergyTable T;
  __shared__ double red[kPostThreads / 32];
  for (int i = threadIdx.x; i < (int)(sizeof(EnergyTable) / 4); i += blockDim.x)
    reinterpret_cast<int*>(&T)[i] = reinterpret_cast<const int*>(table)[i];
  __syncthreads();
  const int n = T.n;
  FF acc[kMaxVertices + 1];  // [0] f0, [1+e] entry e
  for (int e = 0; e <= n; ++e) acc[e] = {0.0f, 0.0f};
  float u7[kMaxVertices][7];  // labelling at the voxel and its six neighbours
  const int rows = G.vy * G.vz;
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    const int z = r / G.vy, y = r - z * G.vy;
    for (int x = threadIdx.x; x < G.vx; x += blockDim.x) {
      const long long i = (long long)r * G.pitch + x;
      long long o[7];
      energy_offsets(G, x, y, z, o);
      for (int e = 0; e < n; ++e) {
        if (T.n_kids[e] == 0) {
          const float* L = T.label[e];
#pragma unroll
          for (int p = 0; p < 7; ++p) u7[e][p] = __ldg(L + i + o[p]);
          ff_add(acc[0], __ldg(T.data[e] + i) * u7[e][0]);
        } else {
#pragma unroll
          for (int p = 0; p < 7; ++p) u7[e][p] = 0.0f;
          for (int k = 0; k < T.n_kids[e]; ++k) {
            const int c = T.kids[T.first_kid[e] + k];
#pragma unroll
            for (int p = 0; p < 7; ++p) u7[e][p] = u7[e][p] + u7[c][p];
          }
        }
        float term = energy_grad_term(u7[e]);
        if (T.smooth[e]) term = __ldg(T.smooth[e] + i) * term;
        ff_add(acc[1 + e], term);
      }
    }
  }
  for (int e = 0; e <= n; ++e) energy_reduce_one(T, acc[e], e, sums, red);
}

// The tree of energy_reg_kernel: entries in post-order (a branch's children
// are earlier entries, in child order).
constexpr int kEnergyRegMax = 8;
struct EnergyRegParams {
  const float* label[kEnergyRegMax];   // leaves: labelling
  const float* data[kEnergyRegMax];    // leaves: data term
  const float* smooth[kEnergyRegMax];  // smoothness image or null (S = 1)
  unsigned kids[kEnergyRegMax];        // bit k: entry k is a child of entry e
  int sum_index[kEnergyRegMax + 1];    // quantity q (0: f0, 1+e: entry e) -> index into sums
  unsigned leaf_mask;                  // bit e: entry e is a leaf
};

// The energy for trees of N non-root vertices (N <= 8).  Each warp takes a
// row (y, z) at a time, lanes across x; the y and z neighbour offsets are set
// once per row (`plane` below 2^31 floats).
template <int N>
__global__ void __launch_bounds__(kPostThreads, 3) energy_reg_kernel(const __grid_constant__ EnergyRegParams P,
                                                                  const Geometry G, double* __restrict__ sums) {
  __shared__ double red[kPostThreads / 32];
  FF acc[N + 1];
#pragma unroll
  for (int q = 0; q <= N; ++q) acc[q] = {0.0f, 0.0f};
  const int lane = threadIdx.x & 31;
  const int n_warps = gridDim.x * (kPostThreads / 32);
  const int rows = G.vy * G.vz;
  for (int r = blockIdx.x * (kPostThreads / 32) + (threadIdx.x >> 5); r < rows; r += n_warps) {
    const int z = r / G.vy, y = r - z * G.vy;
    const long long row = (long long)r * G.pitch;
    const int dyp = y == G.vy - 1 ? 0 : G.pitch;
    const int dym = y == 0 ? 0 : -G.pitch;
    const int dzp = z == G.vz - 1 ? 0 : (int)G.plane;
    const int dzm = z == 0 ? 0 : -(int)G.plane;
    for (int x = lane; x < G.vx; x += 32) {
      const long long i = row + x;
      const int xp = x == G.vx - 1 ? 0 : 1;
      const int xm = x == 0 ? 0 : -1;
      float u7[N][7];
#pragma unroll
      for (int e = 0; e < N; ++e) {
        if (P.leaf_mask >> e & 1u) {
          const float* c = P.label[e] + i;
          u7[e][0] = __ldg(c);
          u7[e][1] = __ldg(c + xp);
          u7[e][2] = __ldg(c + xm);
          u7[e][3] = __ldg(c + dyp);
          u7[e][4] = __ldg(c + dym);
          u7[e][5] = __ldg(c + dzp);
          u7[e][6] = __ldg(c + dzm);
          ff_add(acc[0], __ldg(P.data[e] + i) * u7[e][0]);
        } else {
#pragma unroll
          for (int p = 0; p < 7; ++p) u7[e][p] = 0.0f;
#pragma unroll
          for (int k = 0; k < e; ++k)
            if (P.kids[e] >> k & 1u) {
#pragma unroll
              for (int p = 0; p < 7; ++p) u7[e][p] = u7[e][p] + u7[k][p];
            }
        }
        float term = energy_grad_term(u7[e]);
        if (P.smooth[e]) term = __ldg(P.smooth[e] + i) * term;
        ff_add(acc[1 + e], term);
      }
    }
  }
#pragma unroll
  for (int q = 0; q <= N; ++q) energy_reduce_to(acc[q], sums + P.sum_index[q], red);
}

}  // namespace hmf
