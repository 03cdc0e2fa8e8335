// hmf_adjoint.cuh -- reverse-mode adjoint of the REF_CUDA iteration.
//
// No counterpart in the reference (it only runs the solver forward).  For the
// loss L = -(1/V) sum_i log(max(u_leaf(truth_i)(i), eps)) on the final leaf
// labels, one backward step turns the adjoints of the state after iteration t
// (flows P, sinks s', labels u') into the adjoints of the state before it and
// accumulates dL/dD (leaf data terms, per voxel) and dL/dalpha (smoothness
// weights).  The forward arithmetic being reversed is kern_CalcGradStep ..
// kern_Divergence and the sink / label updates of
// CUDA_hierarchicalmaxflow.cu:124-456 (restated in hmf_kernels.cuh).
//
// Conventions at the kinks: saturate passes the gradient strictly inside
// (0, 1); the leaf capacity clamp passes it to its input inside [0, D] and to
// D above D; the projection multiplier depends on |p| and alpha only where
// |p| > alpha*S; the initial sink min(D) sends its gradient to the leaf that
// kern_MinBuffers keeps (the last one of a tie).
//
// Every kernel is one thread per voxel over the pitched layout of a single
// volume and evaluates the same FP32 operations in the same order as the
// oracle's restatement, so that the per-voxel gradients agree exactly; only
// the alpha gradient (a sum over voxels, reduced in double) depends on the
// summation order.
//
// Forward states live in "state slots": A = 6(n-1)+1 arrays of `arr` floats
// each; non-root vertex j (in id order, root skipped) owns arrays 6j+0 sink,
// +1 label, +2 px, +3 py, +4 pz, +5 divergence of those flows; the root's sink
// (the source flow) is array 6(n-1).  The forward kernels write every
// iteration's state into its slot directly.
//
// The adjoint of a state's sinks and labels is the sum of a sweep part
// (adj_tree_kernel of the later iteration) and a flow part (-/+ step * gb of
// the later iteration's flow reverse, gb = adjoint of its gradient-step
// values); the sum is formed where it is consumed, in the order the oracle
// accumulates it (sweep part first, then vertex by vertex in id order).
#pragma once

#include "hmf_types.cuh"

namespace hmf {

enum { kAdjSink = 0, kAdjLabel = 1, kAdjPx = 2, kAdjPy = 3, kAdjPz = 4, kAdjDiv = 5, kAdjPerVertex = 6 };
constexpr int kAdjTreeThreads = 128;

__device__ __forceinline__ bool adj_coords(const Geometry& G, long long i, int& x, int& y, int& z) {
  z = (int)(i / G.plane);
  const long long r = i - (long long)z * G.plane;
  y = (int)(r / G.pitch);
  x = (int)(r - (long long)y * G.pitch);
  return x < G.vx;
}

// kern_Divergence of the flows at voxel i
__device__ __forceinline__ float adj_div(const float* px, const float* py, const float* pz, const Geometry& G,
                                         long long i, int x, int y, int z) {
  float d = px[i] + py[i] + pz[i];
  if (x != G.vx - 1) d -= px[i + 1];
  if (y != G.vy - 1) d -= py[i + G.pitch];
  if (z != G.vz - 1) d -= pz[i + G.plane];
  return d;
}

// ---------------------------------------------------------------------------
// Copies between the solver's state arrays and a state slot: blockIdx.y =
// array j; ctx[j] = the solver's array j (null: none -- zero-filled in the
// slot, skipped the other way); slot + j*arr = the slot's.
// ---------------------------------------------------------------------------
__global__ void adj_state_copy_kernel(const float* const* __restrict__ ctx, float* slot, long long arr, int to_slot) {
  const int j = blockIdx.y;
  float4* a = reinterpret_cast<float4*>(const_cast<float*>(ctx[j]));
  float4* b = reinterpret_cast<float4*>(slot + (long long)j * arr);
  const long long n4 = arr / 4;
  const long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x, di = (long long)gridDim.x * blockDim.x;
  if (!a) {
    if (to_slot)
      for (long long i = i0; i < n4; i += di) b[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  const float4* src = to_slot ? a : b;
  float4* dst = to_slot ? b : a;
  for (long long i = i0; i < n4; i += di) dst[i] = src[i];
}

// ---------------------------------------------------------------------------
// Loss on the final leaf labels and the adjoint it seeds.
// ---------------------------------------------------------------------------
struct AdjLoss {
  const float* u[kMaxVertices];  // final labels of the leaves, in leaf order
  float* ub[kMaxVertices];       // adjoint of those labels
  int n_leaves;
  int pad_;
  double n_voxels;
  double eps;
};

__global__ void adj_loss_kernel(const AdjLoss L, const int* __restrict__ truth, const Geometry G, double* loss,
                                int* error_flag) {
  double acc = 0.0;
  int bad = 0;
  const float eps = (float)L.eps;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol; i += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    if (!adj_coords(G, i, x, y, z)) continue;
    const long long dense = ((long long)z * G.vy + y) * G.vx + x;
    const int cls = truth[dense];
    for (int j = 0; j < L.n_leaves; ++j) L.ub[j][i] = 0.0f;
    if (cls < 0 || cls >= L.n_leaves) {
      bad = 1;
      continue;
    }
    const float uv = L.u[cls][i];
    const float ue = uv > eps ? uv : eps;
    acc -= log((double)ue) / L.n_voxels;
    if (uv > eps) L.ub[cls][i] = (float)(-1.0 / (L.n_voxels * (double)uv));
  }
  if (bad) atomicOr(error_flag, 8);
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) atomicAdd(loss, v);
  }
}

// ---------------------------------------------------------------------------
// Reverse of the per-voxel sink / label sweep (all vertices of a voxel in one
// thread).  Forward: sinks in post-order from the old parent sink, labels
// afterwards from the new sinks.  Reverse: labels (vertex id order), then
// sinks with parents before children (pre-order).
// ---------------------------------------------------------------------------
struct AdjTree {
  int n, root;
  float cc, icc;
  float step;  // StepSize (tau)
  int pad_;
  int parent[kMaxVertices];
  int first_kid[kMaxVertices];
  int n_kids[kMaxVertices];
  float inv_kids[kMaxVertices];
  int kids[kMaxVertices];
  int preorder[kMaxVertices];
  int sbase[kMaxVertices];  // state-slot array index of the vertex's sink
  // flow part of vertex w's sink adjoint: entries comb_first[w] ..
  // comb_first[w+1]-1, vertex id order; +1: += step*gb(v) (v == w), -1:
  // -= step*gb(v) (v a child of w)
  int comb_first[kMaxVertices + 1];
  int comb_v[2 * kMaxVertices];
  int comb_sign[2 * kMaxVertices];
  const float* data[kMaxVertices];
  double* Db[kMaxVertices];
};

// Adjoint of vertex w's sink in a state: sweep part plus flow part.
__device__ __forceinline__ float adj_sink_adjoint(const AdjTree& T, int w, const float* sweep, const float* gb,
                                                  long long arr, long long i) {
  float acc = sweep[w * arr + i];
  for (int q = T.comb_first[w]; q < T.comb_first[w + 1]; ++q) {
    const float d = T.step * gb[T.comb_v[q] * arr + i];
    acc = T.comb_sign[q] > 0 ? acc + d : acc - d;
  }
  return acc;
}

struct AdjSweep {
  const float* stA;  // state slot before the iteration
  const float* stB;  // state slot after it
  long long arr;     // floats per array
  const float* sbn;  // [v*arr] sweep part of the new sinks' adjoint
  const float* ubn;  // [v*arr] sweep part of the new labels' adjoint
  const float* gbn;  // [v*arr] gb of the later iteration's flow reverse (zero for the last)
  float* sbo;        // [v*arr] out: sweep part of the old sinks' adjoint
  float* ubo;        // [v*arr] out: sweep part of the old labels' adjoint
  float* dbp;        // [v*arr] out: adjoint of the new divergence
};

__global__ void __launch_bounds__(kAdjTreeThreads) adj_tree_kernel(const AdjTree* __restrict__ table, const Geometry G,
                                                                   const AdjSweep S) {
  __shared__ AdjTree T;
  extern __shared__ float av[];
  for (int i = threadIdx.x; i < (int)(sizeof(AdjTree) / 4); i += blockDim.x)
    reinterpret_cast<int*>(&T)[i] = reinterpret_cast<const int*>(table)[i];
  __syncthreads();
  const int n = T.n, nb = blockDim.x, t = threadIdx.x, root = T.root;
  float* SBN = av;
  float* DN = av + n * nb;
  float* SBO = av + 2 * n * nb;
  float* UBO = av + 3 * n * nb;
  float* DBP = av + 4 * n * nb;
  const float cc = T.cc, icc = T.icc, step_icc = T.step * T.icc;
  const long long arr = S.arr;
  const bool small = G.vol < (1LL << 31);  // 32-bit voxel coordinates
  for (long long i = (long long)blockIdx.x * nb + t; i < G.vol; i += (long long)gridDim.x * nb) {
    if (small) {
      const unsigned iu = (unsigned)i, r = iu % (unsigned)G.plane;
      if (r % (unsigned)G.pitch >= (unsigned)G.vx) continue;  // a padding column
    } else {
      int x, y, z;
      if (!adj_coords(G, i, x, y, z)) continue;
    }
#pragma unroll 4
    for (int v = 0; v < n; ++v) {
      SBN[v * nb + t] = adj_sink_adjoint(T, v, S.sbn, S.gbn, arr, i);
      SBO[v * nb + t] = 0.0f;
      UBO[v * nb + t] = 0.0f;
      DBP[v * nb + t] = 0.0f;
      if (v != root) DN[v * nb + t] = S.stB[((long long)T.sbase[v] + kAdjDiv) * arr + i];
    }
    // labels: u' = sat(u + cc*((s'_parent - d') - s'))
#pragma unroll 4
    for (int v = 0; v < n; ++v) {
      if (v == root) continue;
      const int p = T.parent[v];
      const float uo = S.stA[((long long)T.sbase[v] + kAdjLabel) * arr + i];
      const float sp = S.stB[(long long)T.sbase[p] * arr + i];
      const float sv = S.stB[(long long)T.sbase[v] * arr + i];
      const float zv = uo + cc * ((sp - DN[v * nb + t]) - sv);
      const float ub = S.ubn[v * arr + i] - step_icc * S.gbn[v * arr + i];
      const float zb = (zv > 0.0f && zv < 1.0f) ? ub : 0.0f;
      UBO[v * nb + t] += zb;
      SBN[p * nb + t] += cc * zb;
      DBP[v * nb + t] -= cc * zb;
      SBN[v * nb + t] -= cc * zb;
    }
    // sinks, parents before children
    for (int k = 0; k < n; ++k) {
      const int v = T.preorder[k];
      const int nk = T.n_kids[v];
      if (nk == 0) {
        const int p = T.parent[v];
        const float spo = S.stA[(long long)T.sbase[p] * arr + i];
        const float uo = S.stA[((long long)T.sbase[v] + kAdjLabel) * arr + i];
        const float yv = (spo - DN[v * nb + t]) + uo * icc;
        const float cap = T.data[v][i];
        if (yv < 0.0f) continue;
        if (yv > cap) {
          T.Db[v][i] += (double)SBN[v * nb + t];
          continue;
        }
        const float yb = SBN[v * nb + t];
        SBO[p * nb + t] += yb;
        DBP[v * nb + t] -= yb;
        UBO[v * nb + t] += icc * yb;
      } else {
        const float Wb = SBN[v * nb + t] * T.inv_kids[v];
        if (v != root) {
          SBO[T.parent[v] * nb + t] += Wb;
          DBP[v * nb + t] -= Wb;
          UBO[v * nb + t] += icc * Wb;
        }
        for (int q = 0; q < nk; ++q) {
          const int c = T.kids[T.first_kid[v] + q];
          SBN[c * nb + t] += Wb;
          DBP[c * nb + t] += Wb;
          UBO[c * nb + t] -= icc * Wb;
        }
      }
    }
    for (int v = 0; v < n; ++v) {
      S.sbo[v * arr + i] = SBO[v * nb + t];
      if (v != root) {
        S.ubo[v * arr + i] = UBO[v * nb + t];
        S.dbp[v * arr + i] = DBP[v * nb + t];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Reverse of the flow step of one vertex (kern_CalcGradStep, kern_Descent-
// SpatialFlow, kern_ComputeFlowMag*, kern_Project, kern_Divergence).
// ---------------------------------------------------------------------------
struct AdjVertex {
  // forward state before the iteration
  const float* px;
  const float* py;
  const float* pz;
  const float* s;    // own sink
  const float* c;    // parent's sink
  const float* u;
  const float* smooth;  // nullptr: S = 1
  float alpha;
  int pad_;
  // recomputed intermediates
  float* g;
  float* ppx;
  float* ppy;
  float* ppz;
  float* m;
  float* Fm;
  // adjoints
  float* Pbx;  // of the new flows on entry, of the old flows on exit
  float* Pby;
  float* Pbz;
  const float* dbp;  // of the new divergence (sweep reverse)
  float* F2b;        // of the squared flow magnitude
  float* qx;         // of the descended flows p'
  float* qy;
  float* qz;
  float* dbo;        // of the old divergence
  float* gb;         // out: of the gradient-step values g
  double* alpha_grad;
};

struct AdjParams {
  Geometry G;
  float step, icc;
};

// g = step * (((s + d) - c) - u * icc) of the old state
__global__ void adj_grad_kernel(const AdjVertex V, const AdjParams P) {
  const Geometry& G = P.G;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol; i += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    if (!adj_coords(G, i, x, y, z)) continue;
    const float d = adj_div(V.px, V.py, V.pz, G, i, x, y, z);
    V.g[i] = P.step * (((V.s[i] + d) - V.c[i]) - V.u[i] * P.icc);
  }
}

// p' and the projection multiplier
__global__ void adj_flow_kernel(const AdjVertex V, const AdjParams P) {
  const Geometry& G = P.G;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol; i += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    if (!adj_coords(G, i, x, y, z)) continue;
    const float gi = V.g[i];
    const bool hx = x != G.vx - 1, hy = y != G.vy - 1, hz = z != G.vz - 1;
    const float ax = x ? V.px[i] - (gi - V.g[i - 1]) : 0.f;
    const float ay = y ? V.py[i] - (gi - V.g[i - G.pitch]) : 0.f;
    const float az = z ? V.pz[i] - (gi - V.g[i - G.plane]) : 0.f;
    const float bx = hx ? V.px[i + 1] - (V.g[i + 1] - gi) : 0.f;
    const float by = hy ? V.py[i + G.pitch] - (V.g[i + G.pitch] - gi) : 0.f;
    const float bz = hz ? V.pz[i + G.plane] - (V.g[i + G.plane] - gi) : 0.f;
    float up = ax * ax;
    float dn = hx ? bx * bx : 0.f;
    float F = up + dn;
    up = ay * ay;
    dn = hy ? by * by : 0.f;
    F += up + dn;
    up = az * az;
    dn = hz ? bz * bz : 0.f;
    F += up + dn;
    const float Fm = sqrtf(0.5f * F);
    const float lim = V.smooth ? V.alpha * V.smooth[i] : V.alpha;
    V.ppx[i] = ax;
    V.ppy[i] = ay;
    V.ppz[i] = az;
    V.Fm[i] = Fm;
    V.m[i] = (Fm > lim) ? lim / Fm : 1.0f;
  }
}

// total adjoint of the new flow component at j: incoming plus through the
// new divergence (d'(j) has +P(j); d'(j-stride) has -P(j))
__device__ __forceinline__ float adj_ptot(const float* Pb, const float* dbp, long long j, long long stride, bool low) {
  return Pb[j] + dbp[j] - (low ? dbp[j - stride] : 0.f);
}

// adjoint of the multiplier -> of |p|^2 and of alpha
__global__ void adj_mult_kernel(const AdjVertex V, const AdjParams P) {
  const Geometry& G = P.G;
  double asum = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol; i += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    if (!adj_coords(G, i, x, y, z)) continue;
    float mb = 0.f;
    if (x) mb += adj_ptot(V.Pbx, V.dbp, i, 1, true) * 0.5f * V.ppx[i];
    if (x != G.vx - 1) mb += adj_ptot(V.Pbx, V.dbp, i + 1, 1, true) * 0.5f * V.ppx[i + 1];
    if (y) mb += adj_ptot(V.Pby, V.dbp, i, G.pitch, true) * 0.5f * V.ppy[i];
    if (y != G.vy - 1) mb += adj_ptot(V.Pby, V.dbp, i + G.pitch, G.pitch, true) * 0.5f * V.ppy[i + G.pitch];
    if (z) mb += adj_ptot(V.Pbz, V.dbp, i, G.plane, true) * 0.5f * V.ppz[i];
    if (z != G.vz - 1) mb += adj_ptot(V.Pbz, V.dbp, i + G.plane, G.plane, true) * 0.5f * V.ppz[i + G.plane];
    const float Fm = V.Fm[i];
    const float S = V.smooth ? V.smooth[i] : 1.0f;
    const float lim = V.smooth ? V.alpha * S : V.alpha;
    float f2b = 0.f;
    if (Fm > lim) {
      f2b = -mb * lim / (4.0f * Fm * Fm * Fm);
      asum += (double)(mb / Fm * S);
    }
    V.F2b[i] = f2b;
  }
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) asum += __shfl_down_sync(0xffffffffu, asum, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = asum;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0 && v != 0.0) atomicAdd(V.alpha_grad, v);
  }
}

// adjoint of p' (through the projection and through |p|^2)
__global__ void adj_descent_kernel(const AdjVertex V, const AdjParams P) {
  const Geometry& G = P.G;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol; i += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    if (!adj_coords(G, i, x, y, z)) continue;
    const float mi = V.m[i], fi = V.F2b[i];
    V.qx[i] = x ? adj_ptot(V.Pbx, V.dbp, i, 1, true) * 0.5f * (mi + V.m[i - 1]) + 2.0f * V.ppx[i] * (fi + V.F2b[i - 1])
                : 0.f;
    V.qy[i] = y ? adj_ptot(V.Pby, V.dbp, i, G.pitch, true) * 0.5f * (mi + V.m[i - G.pitch]) +
                      2.0f * V.ppy[i] * (fi + V.F2b[i - G.pitch])
                : 0.f;
    V.qz[i] = z ? adj_ptot(V.Pbz, V.dbp, i, G.plane, true) * 0.5f * (mi + V.m[i - G.plane]) +
                      2.0f * V.ppz[i] * (fi + V.F2b[i - G.plane])
                : 0.f;
  }
}

// adjoint of g (it reaches the own and parent's old sinks and the old label
// through adj_sink_adjoint / the label adjoint of the next sweep reverse) and
// of the old divergence
__global__ void adj_gsum_kernel(const AdjVertex V, const AdjParams P) {
  const Geometry& G = P.G;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol; i += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    if (!adj_coords(G, i, x, y, z)) continue;
    float gb = -(V.qx[i] + V.qy[i] + V.qz[i]);
    if (x != G.vx - 1) gb += V.qx[i + 1];
    if (y != G.vy - 1) gb += V.qy[i + G.pitch];
    if (z != G.vz - 1) gb += V.qz[i + G.plane];
    V.gb[i] = gb;
    V.dbo[i] = P.step * gb;
  }
}

// adjoint of the old flows
__global__ void adj_oldflow_kernel(const AdjVertex V, const AdjParams P) {
  const Geometry& G = P.G;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol; i += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    if (!adj_coords(G, i, x, y, z)) continue;
    const float d = V.dbo[i];
    V.Pbx[i] = V.qx[i] + d - (x ? V.dbo[i - 1] : 0.f);
    V.Pby[i] = V.qy[i] + d - (y ? V.dbo[i - G.pitch] : 0.f);
    V.Pbz[i] = V.qz[i] + d - (z ? V.dbo[i - G.plane] : 0.f);
  }
}

// ---------------------------------------------------------------------------
// Initial sinks: every sink starts at min over the leaves of D
// (kern_MinBuffers keeps the last of a tie); their adjoints go to that leaf.
// ---------------------------------------------------------------------------
struct AdjInit {
  const float* data[kMaxVertices];  // leaves, in leaf order
  double* Db[kMaxVertices];         // leaves, in leaf order
  const float* sb;                  // [v*arr] sweep part of the initial sinks' adjoint
  const float* gb;                  // [v*arr] gb of iteration 0's flow reverse
  long long arr;
  int n_leaves;
  int n;
};

__global__ void adj_init_kernel(const AdjTree* __restrict__ table, const AdjInit A, const Geometry G) {
  __shared__ AdjTree T;
  for (int i = threadIdx.x; i < (int)(sizeof(AdjTree) / 4); i += blockDim.x)
    reinterpret_cast<int*>(&T)[i] = reinterpret_cast<const int*>(table)[i];
  __syncthreads();
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol; i += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    if (!adj_coords(G, i, x, y, z)) continue;
    int arg = 0;
    float mv = A.data[0][i];
    for (int k = 1; k < A.n_leaves; ++k) {
      const float d = A.data[k][i];
      if (!(mv < d)) {
        mv = d;
        arg = k;
      }
    }
    double tot = 0.0;
    for (int v = 0; v < A.n; ++v) tot += (double)adj_sink_adjoint(T, v, A.sb, A.gb, A.arr, i);
    A.Db[arg][i] += tot;
  }
}

}  // namespace hmf
