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
//                 every input read once, one int written.
//  energy_kernel  f0 = sum of D_l * u_l over leaves and voxels; per non-root
//                 vertex f_v = sum of S_v * 0.5*sqrt(|grad u_v|^2) with the
//                 clamped central differences of kern_GHMFD_GradientBuffer
//                 (CUDA_hierarchicalmaxflowdecomp.cu:19-38; its `g += d*d`
//                 compiled to fused multiply-adds), a branch's
//                 labelling being the sum of its children's in child order
//                 (vtkCudaHierarchicalMaxFlowDecomposition.cxx:750-806).  One
//                 pass over all vertices per voxel (the reference makes one
//                 gradient, one multiply and one reduction pass per vertex);
//                 per-voxel terms in FP32 in the reference's operation order,
//                 sums in FP64 (the reference reduces in FP32).
// Arrays are pitched rows (`pitch` floats per row, dense when pitch == vx);
// outputs of the vote are dense.
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

// Tree in post-order for the energy: entry e's children precede it.
struct EnergyTable {
  int n;  // entries (the root excluded)
  int n_kids_total;
  int first_kid[kMaxVertices];
  int n_kids[kMaxVertices];
  int kids[kMaxVertices];             // entry indices, child order
  int vertex[kMaxVertices];           // vertex id of each entry
  const float* label[kMaxVertices];   // leaves: labelling
  const float* data[kMaxVertices];    // leaves: data term
  const float* smooth[kMaxVertices];  // smoothness image or null (S = 1)
};

__global__ void __launch_bounds__(kPostThreads) energy_kernel(const EnergyTable* __restrict__ table, const Geometry G,
                                                              double* __restrict__ sums /* [0] f0, [1+vertex] f */) {
  __shared__ EnergyTable T;
  __shared__ double red[kPostThreads / 32];
  for (int i = threadIdx.x; i < (int)(sizeof(EnergyTable) / 4); i += blockDim.x)
    reinterpret_cast<int*>(&T)[i] = reinterpret_cast<const int*>(table)[i];
  __syncthreads();
  const int n = T.n;
  double acc[kMaxVertices + 1];  // [0] f0, [1+e] entry e
  for (int e = 0; e <= n; ++e) acc[e] = 0.0;
  float u7[kMaxVertices][7];  // labelling at the voxel and its six neighbours (clamped)
  const long long dense = (long long)G.vx * G.vy * G.vz;
  for (long long d = (long long)blockIdx.x * blockDim.x + threadIdx.x; d < dense;
       d += (long long)gridDim.x * blockDim.x) {
    const long long r = d / G.vx;
    const int x = (int)(d - r * G.vx);
    const int y = (int)(r % G.vy), z = (int)(r / G.vy);
    const long long i = r * G.pitch + x;
    // neighbour offsets: +x, -x, +y, -y, +z, -z; at the border the voxel itself
    const long long o[7] = {0,
                            x == G.vx - 1 ? 0 : 1,
                            x == 0 ? 0 : -1,
                            y == G.vy - 1 ? 0 : (long long)G.pitch,
                            y == 0 ? 0 : -(long long)G.pitch,
                            z == G.vz - 1 ? 0 : G.plane,
                            z == 0 ? 0 : -G.plane};
    for (int e = 0; e < n; ++e) {
      if (T.n_kids[e] == 0) {
        const float* L = T.label[e];
#pragma unroll
        for (int p = 0; p < 7; ++p) u7[e][p] = __ldg(L + i + o[p]);
        acc[0] += (double)(__ldg(T.data[e] + i) * u7[e][0]);
      } else {
#pragma unroll
        for (int p = 0; p < 7; ++p) u7[e][p] = 0.0f;
        for (int k = 0; k < T.n_kids[e]; ++k) {
          const int c = T.kids[T.first_kid[e] + k];
#pragma unroll
          for (int p = 0; p < 7; ++p) u7[e][p] = u7[e][p] + u7[c][p];
        }
      }
      // kern_GHMFD_GradientBuffer as compiled (multiply-add contraction):
      // g += d*d is one fused multiply-add per axis
      const float dx = u7[e][1] - u7[e][2], dy = u7[e][3] - u7[e][4], dz = u7[e][5] - u7[e][6];
      float g2 = __fmaf_rn(dx, dx, 0.0f);
      g2 = __fmaf_rn(dy, dy, g2);
      g2 = __fmaf_rn(dz, dz, g2);
      float term = 0.5f * sqrtf(g2);
      if (T.smooth[e]) term = __ldg(T.smooth[e] + i) * term;
      acc[1 + e] += (double)term;
    }
  }
  // block sums, one atomic per quantity per block
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int e = 0; e <= n; ++e) {
    double v = acc[e];
    for (int s = 16; s > 0; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
      double t = lane < kPostThreads / 32 ? red[lane] : 0.0;
      for (int s = 16; s > 0; s >>= 1) t += __shfl_down_sync(0xffffffffu, t, s);
      if (lane == 0 && t != 0.0) atomicAdd(&sums[e == 0 ? 0 : 1 + T.vertex[e - 1]], t);
    }
    __syncthreads();
  }
}

}  // namespace hmf
