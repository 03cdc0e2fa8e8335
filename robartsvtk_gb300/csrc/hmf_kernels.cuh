// hmf_kernels.cuh -- sm_103a kernels of the hierarchical max-flow (HMF) solver.
//
// One primal-dual iteration of the reference
// (vtkCudaHierarchicalMaxFlowSegmentation.cxx:106-476 issuing the kernels of
// CUDA_hierarchicalmaxflow.cu:124-456, 2 + 9*leaves + 10*branches full-volume
// passes) is done here in two launches:
//
//  flow_kernel   every non-root vertex, independently: gradient step,
//                descent of the spatial flows, |p| <= alpha*S projection
//                multiplier, projection and the new divergence.  A CTA owns an
//                xy tile of one vertex and marches along z, keeping the
//                intermediate planes in shared-memory rings, so each flow
//                component is read once and written once per iteration.  The
//                divergence of the previous iteration is recomputed from the
//                flows instead of being stored.
//  tree_kernel   per voxel, all vertices: sink and source flows in post-order,
//                then every label (CUDA_hierarchicalmaxflow.cu:124-220 fused).
//
// Arithmetic follows the reference kernels operation by operation (the file
// is compiled with -fmad=false, IEEE sqrt and division), so results match the
// FP32 CPU restatement of those kernels exactly.
#pragma once

#include "hmf_types.cuh"

namespace hmf {

// ---------------------------------------------------------------------------
// flow_kernel
// ---------------------------------------------------------------------------
// Shared-memory planes cover the tile plus a halo: local x in [-2, TX+2],
// local y in [-2, TY+2].  Per z plane k the CTA computes
//   G(k)  gradient-step values g on  x,y in [-2, T+1]   (kern_CalcGradStep)
//   P'(k) descended flows        on  x,y in [-1, T+1]   (kern_DescentSpatialFlow)
//   M(k)  projection multipliers on  x,y in [-1, T]     (kern_ComputeFlowMag*)
//   Out(k) projected flows and divergence on the tile   (kern_Project, kern_Divergence)
// with the schedule  load(f+1), G(f), P'(f), M(f-1), Out(f-2).  Rings:
// raw flows 2 planes, g 2, P' 3, M 3.
template <int TX, int TY>
struct FlowTile {
  static constexpr int SW = TX + 5;
  static constexpr int SH = TY + 5;
  static constexpr int PL = SW * SH;
  static constexpr int NT = TX * TY;
  static constexpr int PLANES = 6 + 2 + 9 + 3;
  static constexpr int SMEM_BYTES = PLANES * PL * (int)sizeof(float);
  __device__ static int at(int lx, int ly) { return (ly + 2) * SW + (lx + 2); }
};

template <int TX, int TY>
__global__ void __launch_bounds__(TX * TY)
flow_kernel(const FlowVertex* __restrict__ vertices, const Geometry G, const FlowParams fp) {
  using T = FlowTile<TX, TY>;
  constexpr int SW = T::SW, PL = T::PL, NT = T::NT;
  extern __shared__ float sm[];
  float* raw = sm;              // [2][3][PL]
  float* gs = raw + 6 * PL;     // [2][PL]
  float* pp = gs + 2 * PL;      // [3][3][PL]
  float* ms = pp + 9 * PL;      // [3][PL]

  const FlowVertex V = vertices[blockIdx.z];
  const int x0 = (int)(blockIdx.x % fp.tiles_x) * TX;
  const int y0 = (int)(blockIdx.x / fp.tiles_x) * TY;
  const int zs = (int)blockIdx.y * fp.zchunk;
  const int ze = min(zs + fp.zchunk, G.vz);
  const int tid = threadIdx.x + threadIdx.y * TX;
  const float step = fp.step, icc = fp.icc;

  auto load_raw = [&](int k) {
    float* dst = raw + (k & 1) * 3 * PL;
    const long long zoff = (long long)k * G.plane;
    for (int i = tid; i < PL; i += NT) {
      const int lx = i % SW - 2, ly = i / SW - 2;
      const int gx = x0 + lx, gy = y0 + ly;
      float a = 0.f, b = 0.f, c = 0.f;
      if (gx >= 0 && gx < G.vx && gy >= 0 && gy < G.vy) {
        const long long o = zoff + (long long)gy * G.pitch + gx;
        a = V.px_in[o];
        b = V.py_in[o];
        c = V.pz_in[o];
      }
      dst[i] = a;
      dst[PL + i] = b;
      dst[2 * PL + i] = c;
    }
  };

  // G(k): g = step * (((sink + div) - inc) - label * icc), div recomputed from
  // the stored flows exactly as kern_Divergence formed it.
  auto comp_g = [&](int k) {
    const float* r = raw + (k & 1) * 3 * PL;
    const float* rn = raw + ((k + 1) & 1) * 3 * PL;
    float* g = gs + (k & 1) * PL;
    const bool ztop = (k == G.vz - 1);
    const long long zoff = (long long)k * G.plane;
    constexpr int W4 = TX + 4, N4 = (TX + 4) * (TY + 4);
    for (int i = tid; i < N4; i += NT) {
      const int lx = i % W4 - 2, ly = i / W4 - 2;
      const int gx = x0 + lx, gy = y0 + ly;
      const int s = T::at(lx, ly);
      float val = 0.f;
      if (gx >= 0 && gx < G.vx && gy >= 0 && gy < G.vy) {
        float d = (r[s] + r[PL + s]) + r[2 * PL + s];
        if (gx != G.vx - 1) d = d - r[s + 1];
        if (gy != G.vy - 1) d = d - r[PL + s + SW];
        if (!ztop) d = d - rn[2 * PL + s];
        const long long o = zoff + (long long)gy * G.pitch + gx;
        const float sk = V.sink[o], c = V.inc[o], u = V.label[o];
        val = step * (((sk + d) - c) - u * icc);
      }
      g[s] = val;
    }
  };

  // P'(k): flow -= g(i) - g(i - e_a); zero on the low face of axis a.
  auto comp_pp = [&](int k) {
    const float* r = raw + (k & 1) * 3 * PL;
    const float* g = gs + (k & 1) * PL;
    const float* gm = gs + ((k + 1) & 1) * PL;  // plane k-1
    float* p = pp + (k % 3) * 3 * PL;
    constexpr int W3 = TX + 3, N3 = (TX + 3) * (TY + 3);
    for (int i = tid; i < N3; i += NT) {
      const int lx = i % W3 - 1, ly = i / W3 - 1;
      const int gx = x0 + lx, gy = y0 + ly;
      const int s = T::at(lx, ly);
      float a = 0.f, b = 0.f, c = 0.f;
      if (gx >= 0 && gx < G.vx && gy >= 0 && gy < G.vy) {
        const float cur = g[s];
        a = gx ? r[s] - (cur - g[s - 1]) : 0.f;
        b = gy ? r[PL + s] - (cur - g[s - SW]) : 0.f;
        c = k ? r[2 * PL + s] - (cur - gm[s]) : 0.f;
      }
      p[s] = a;
      p[PL + s] = b;
      p[2 * PL + s] = c;
    }
  };

  // M(k): multiplier = |p| > alpha*S ? alpha*S / |p| : 1 with
  // |p| = sqrt(0.5 * sum over the six faces of the squared flows).
  auto comp_m = [&](int k) {
    const float* p = pp + (k % 3) * 3 * PL;
    const float* pn = pp + ((k + 1) % 3) * 3 * PL;
    float* m = ms + (k % 3) * PL;
    const bool ztop = (k == G.vz - 1);
    const long long zoff = (long long)k * G.plane;
    constexpr int W2 = TX + 2, N2 = (TX + 2) * (TY + 2);
    for (int i = tid; i < N2; i += NT) {
      const int lx = i % W2 - 1, ly = i / W2 - 1;
      const int gx = x0 + lx, gy = y0 + ly;
      const int s = T::at(lx, ly);
      float val = 1.f;
      if (gx >= 0 && gx < G.vx && gy >= 0 && gy < G.vy) {
        float up = p[s] * p[s];
        float dn = (gx != G.vx - 1) ? p[s + 1] * p[s + 1] : 0.f;
        float F = up + dn;
        up = p[PL + s] * p[PL + s];
        dn = (gy != G.vy - 1) ? p[PL + s + SW] * p[PL + s + SW] : 0.f;
        F = F + (up + dn);
        up = p[2 * PL + s] * p[2 * PL + s];
        dn = !ztop ? pn[2 * PL + s] * pn[2 * PL + s] : 0.f;
        F = F + (up + dn);
        F = sqrtf(0.5f * F);
        const long long o = zoff + (long long)gy * G.pitch + gx;
        const float lim = V.smooth ? V.alpha * V.smooth[o] : V.alpha;
        val = (F > lim) ? lim / F : 1.0f;
      }
      m[s] = val;
    }
  };

  // Out(k): projected flows of the tile and their divergence.
  auto comp_out = [&](int k) {
    const float* p = pp + (k % 3) * 3 * PL;
    const float* pn = pp + ((k + 1) % 3) * 3 * PL;
    const float* m0 = ms + (k % 3) * PL;
    const float* mm = ms + ((k + 2) % 3) * PL;  // plane k-1
    const float* mp = ms + ((k + 1) % 3) * PL;  // plane k+1
    const int lx = threadIdx.x, ly = threadIdx.y;
    const int gx = x0 + lx, gy = y0 + ly;
    if (gx < G.vx && gy < G.vy) {
      const int s = T::at(lx, ly);
      const float Px = gx ? (p[s] * 0.5f) * (m0[s] + m0[s - 1]) : 0.f;
      const float Py = gy ? (p[PL + s] * 0.5f) * (m0[s] + m0[s - SW]) : 0.f;
      const float Pz = k ? (p[2 * PL + s] * 0.5f) * (m0[s] + mm[s]) : 0.f;
      float d = (Px + Py) + Pz;
      if (gx != G.vx - 1) d = d - (p[s + 1] * 0.5f) * (m0[s + 1] + m0[s]);
      if (gy != G.vy - 1) d = d - (p[PL + s + SW] * 0.5f) * (m0[s + SW] + m0[s]);
      if (k != G.vz - 1) d = d - (pn[2 * PL + s] * 0.5f) * (mp[s] + m0[s]);
      const long long o = (long long)k * G.plane + (long long)gy * G.pitch + gx;
      V.px_out[o] = Px;
      V.py_out[o] = Py;
      V.pz_out[o] = Pz;
      V.div[o] = d;
    }
  };

  if (zs - 2 >= 0) load_raw(zs - 2);
  for (int f = zs - 2; f <= ze + 1; ++f) {
    if (f + 1 >= 0 && f + 1 < G.vz) load_raw(f + 1);
    __syncthreads();
    if (f >= 0 && f < G.vz) comp_g(f);
    __syncthreads();
    if (f >= 0 && f >= zs - 1 && f < G.vz) comp_pp(f);
    __syncthreads();
    const int km = f - 1;
    if (km >= 0 && km >= zs - 1 && km < G.vz && km <= ze) comp_m(km);
    __syncthreads();
    const int ko = f - 2;
    if (ko >= zs && ko < ze) comp_out(ko);
  }
}

// ---------------------------------------------------------------------------
// tree_kernel: per voxel, post-order sink/source update then labels.
//  leaf   sink = clamp((inc - div) + u*icc, 0, D)          (kern_FindLeafSinkPotential, kern_ApplyCapacity)
//  branch W = sum over kids ((W + s_c) + d_c) - u_c*icc,    (kern_FindSourcePotentialAndStore)
//         W = ((W + inc) - div) + u*icc,                     (kern_FindSinkPotentialAndStore)
//         sink = W * (1/(kids+1))                            (MultiplyAndStoreBuffer)
//  root   W from 1/CC over its kids, source = W * (1/kids)
//  labels u = sat(u + cc*((inc_new - div) - sink))         (kern_UpdateLabel)
// Per-thread values of every vertex live in shared memory [n][blockDim].
// ---------------------------------------------------------------------------
__global__ void tree_kernel(const TreeTable* __restrict__ table, const Geometry G) {
  __shared__ TreeTable T;
  extern __shared__ float vals[];
  for (int i = threadIdx.x; i < (int)(sizeof(TreeTable) / 4); i += blockDim.x)
    reinterpret_cast<int*>(&T)[i] = reinterpret_cast<const int*>(table)[i];
  __syncthreads();
  const int n = T.n, nb = blockDim.x, t = threadIdx.x;
  float* S = vals;            // [n][nb]
  float* D = vals + n * nb;   // [n][nb]
  float* U = vals + 2 * n * nb;
  const float icc = T.icc, cc = T.cc;
  const int root = n - 1;
  for (long long i = (long long)blockIdx.x * nb + t; i < G.vol; i += (long long)gridDim.x * nb) {
    for (int e = 0; e < root; ++e) {
      D[e * nb + t] = T.e[e].div[i];
      U[e * nb + t] = T.e[e].label[i];
      if (T.e[e].n_kids) S[e * nb + t] = T.e[e].sink[i];
    }
    S[root * nb + t] = T.e[root].sink[i];
    for (int e = 0; e < n; ++e) {
      const TreeEntry& E = T.e[e];
      if (E.n_kids == 0) {
        float v = (S[E.parent * nb + t] - D[e * nb + t]) + U[e * nb + t] * icc;
        const float cap = E.data[i];
        v = (v < 0.0f) ? 0.0f : v;
        v = (v > cap) ? cap : v;
        S[e * nb + t] = v;
      } else {
        float W = (e == root) ? T.root_init : 0.0f;
        for (int j = 0; j < E.n_kids; ++j) {
          const int c = T.kids[E.first_kid + j];
          W = ((W + S[c * nb + t]) + D[c * nb + t]) - U[c * nb + t] * icc;
        }
        if (e != root) W = ((W + S[E.parent * nb + t]) - D[e * nb + t]) + U[e * nb + t] * icc;
        S[e * nb + t] = W * E.inv_kids;
      }
    }
    for (int e = 0; e < root; ++e) {
      const TreeEntry& E = T.e[e];
      const float u = U[e * nb + t] + cc * ((S[E.parent * nb + t] - D[e * nb + t]) - S[e * nb + t]);
      E.label_out[i] = __saturatef(u);
      E.sink_out[i] = S[e * nb + t];
    }
    T.e[root].sink_out[i] = S[root * nb + t];
  }
}

// ---------------------------------------------------------------------------
// tree4_kernel: tree_kernel on four consecutive voxels per thread (float4
// loads and stores; rows are padded to a multiple of 4 floats, so every array
// length is a multiple of 4).  Every load of a voxel quad is issued before the
// sweep, and the per-vertex values (sink, divergence, label, capacity) live
// in shared memory [n][blockDim] as float4.  Same arithmetic as tree_kernel,
// component by component.
// ---------------------------------------------------------------------------
constexpr int kTree4Threads = 128;
constexpr int kTree4MaxVertices = 24;

__device__ __forceinline__ float4 ld4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }

__global__ void __launch_bounds__(kTree4Threads) tree4_kernel(const TreeTable* __restrict__ table, const Geometry G) {
  __shared__ TreeTable T;
  extern __shared__ float4 v4[];
  for (int i = threadIdx.x; i < (int)(sizeof(TreeTable) / 4); i += blockDim.x)
    reinterpret_cast<int*>(&T)[i] = reinterpret_cast<const int*>(table)[i];
  __syncthreads();
  const int n = T.n, nb = blockDim.x, t = threadIdx.x;
  float4* S = v4;             // [n][nb]
  float4* D = v4 + n * nb;    // [n][nb]
  float4* U = v4 + 2 * n * nb;
  float4* C = v4 + 3 * n * nb;  // capacities of leaves
  const float icc = T.icc, cc = T.cc;
  const int root = n - 1;
  const long long nq = G.vol / 4;
  for (long long q = (long long)blockIdx.x * nb + t; q < nq; q += (long long)gridDim.x * nb) {
    const long long i = q * 4;
#pragma unroll 4
    for (int e = 0; e < root; ++e) {
      const TreeEntry& E = T.e[e];
      D[e * nb + t] = ld4(E.div + i);
      U[e * nb + t] = ld4(E.label + i);
      if (E.n_kids) S[e * nb + t] = ld4(E.sink + i);
      else C[e * nb + t] = ld4(E.data + i);
    }
    S[root * nb + t] = ld4(T.e[root].sink + i);
    for (int e = 0; e < n; ++e) {
      const TreeEntry& E = T.e[e];
      float4 r;
      if (E.n_kids == 0) {
        const float4 inc = S[E.parent * nb + t], d = D[e * nb + t], u = U[e * nb + t], cap = C[e * nb + t];
        float v;
#define HMF_LEAF(c)                          \
  v = (inc.c - d.c) + u.c * icc;             \
  v = (v < 0.0f) ? 0.0f : v;                 \
  v = (v > cap.c) ? cap.c : v;               \
  r.c = v;
        HMF_LEAF(x) HMF_LEAF(y) HMF_LEAF(z) HMF_LEAF(w)
#undef HMF_LEAF
      } else {
        const float w0 = (e == root) ? T.root_init : 0.0f;
        float4 W = make_float4(w0, w0, w0, w0);
        for (int j = 0; j < E.n_kids; ++j) {
          const int c = T.kids[E.first_kid + j];
          const float4 sc = S[c * nb + t], dc = D[c * nb + t], uc = U[c * nb + t];
          W.x = ((W.x + sc.x) + dc.x) - uc.x * icc;
          W.y = ((W.y + sc.y) + dc.y) - uc.y * icc;
          W.z = ((W.z + sc.z) + dc.z) - uc.z * icc;
          W.w = ((W.w + sc.w) + dc.w) - uc.w * icc;
        }
        if (e != root) {
          const float4 inc = S[E.parent * nb + t], d = D[e * nb + t], u = U[e * nb + t];
          W.x = ((W.x + inc.x) - d.x) + u.x * icc;
          W.y = ((W.y + inc.y) - d.y) + u.y * icc;
          W.z = ((W.z + inc.z) - d.z) + u.z * icc;
          W.w = ((W.w + inc.w) - d.w) + u.w * icc;
        }
        r = make_float4(W.x * E.inv_kids, W.y * E.inv_kids, W.z * E.inv_kids, W.w * E.inv_kids);
      }
      S[e * nb + t] = r;
    }
    for (int e = 0; e < root; ++e) {
      const TreeEntry& E = T.e[e];
      const float4 inc = S[E.parent * nb + t], d = D[e * nb + t], s = S[e * nb + t], u = U[e * nb + t];
      float4 o;
      o.x = __saturatef(u.x + cc * ((inc.x - d.x) - s.x));
      o.y = __saturatef(u.y + cc * ((inc.y - d.y) - s.y));
      o.z = __saturatef(u.z + cc * ((inc.z - d.z) - s.z));
      o.w = __saturatef(u.w + cc * ((inc.w - d.w) - s.w));
      st4(E.label_out + i, o);
      st4(E.sink_out + i, s);
    }
    st4(T.e[root].sink_out + i, S[root * nb + t]);
  }
}

// ---------------------------------------------------------------------------
// init_kernel (vtkCudaHierarchicalMaxFlowSegmentation.cxx:547-658 and
// PropogateLabels :63-104): sinks and source = min over leaves of D; leaf
// labels = [D == min] / count; branch labels = sums of their kids.  Also
// flags negative data terms or smoothness values (the reference rejects
// them, vtkHierarchicalMaxFlowSegmentation.cxx:434-438, :470-474).
// ---------------------------------------------------------------------------
__global__ void init_kernel(const TreeTable* __restrict__ table, const Geometry G,
                            const float* const* __restrict__ smooth_list, int n_smooth,
                            int cpu_min, int* __restrict__ error_flag) {
  __shared__ TreeTable T;
  extern __shared__ float vals[];
  for (int i = threadIdx.x; i < (int)(sizeof(TreeTable) / 4); i += blockDim.x)
    reinterpret_cast<int*>(&T)[i] = reinterpret_cast<const int*>(table)[i];
  __syncthreads();
  const int n = T.n, nb = blockDim.x, t = threadIdx.x;
  float* U = vals;  // [n][nb]
  const int root = n - 1;
  int bad = 0;
  for (long long i = (long long)blockIdx.x * nb + t; i < G.vol; i += (long long)gridDim.x * nb) {
    // pitch 0: several volumes of different pitches back to back, whose
    // padding columns are zero (never written), so every element is checked
    const long long row = G.pitch ? i / G.pitch : 0;
    const bool inside = G.pitch == 0 || (i - row * G.pitch) < G.vx;
    float m = T.e[T.leaves[0]].data[i];
    for (int j = 1; j < T.n_leaves; ++j) {
      const float d = T.e[T.leaves[j]].data[i];
      // kern_MinBuffers (CUDA_hierarchicalmaxflow.cu:489-499) or, for REF_CPU,
      // minBuffer (vtkMaxFlowSegmentationUtilities.cxx:77-83); they differ
      // only for NaN and signed zeros.
      m = cpu_min ? ((m > d) ? d : m) : ((m < d) ? m : d);
    }
    float cnt = 0.0f;
    for (int j = 0; j < T.n_leaves; ++j) {
      const int e = T.leaves[j];
      const float d = T.e[e].data[i];
      if (inside && d < 0.0f) bad = 1;
      const float lab = (m == d) ? 1.0f : 0.0f;
      U[e * nb + t] = lab;
      cnt = cnt + lab;
    }
    for (int j = 0; j < T.n_leaves; ++j) {
      const int e = T.leaves[j];
      U[e * nb + t] = U[e * nb + t] / cnt;
    }
    for (int e = 0; e < root; ++e) {
      const TreeEntry& E = T.e[e];
      if (E.n_kids) {
        float acc = 0.0f;
        for (int j = 0; j < E.n_kids; ++j) acc = acc + U[T.kids[E.first_kid + j] * nb + t];
        U[e * nb + t] = acc;
      }
      E.label[i] = U[e * nb + t];
      E.sink[i] = m;
    }
    T.e[root].sink[i] = m;
    for (int j = 0; j < n_smooth; ++j)
      if (inside && smooth_list[j][i] < 0.0f) bad = 1;
  }
  if (bad) atomicOr(error_flag, 1);
}

// ---------------------------------------------------------------------------
// refcpu_kernel: REF_CPU semantics (vtkHierarchicalMaxFlowSegmentation.cxx:1083-1259
// over vtkMaxFlowSegmentationUtilities.cxx).  There the spatial flows start at
// zero and are only ever multiplied (ghmf_applyStep :261-273, ghmf_projectOntoSet
// :309-321), so they and every divergence stay zero; divAndStoreBuffer is called
// with (working, sink) (:1186, :1196), so branch sinks and the source keep their
// initial value, the minimum data term m.  What remains is, per leaf and voxel,
//   sink = (m - 0) + u / CC;  sink = sink > D ? D : sink;  u += CC*((m - 0) - sink)
// with no saturation, and branch labels that never change.  Every iteration of
// a voxel is independent of its neighbours, so all iterations run in registers.
// Called after init_kernel.
// ---------------------------------------------------------------------------
__global__ void refcpu_kernel(const TreeTable* __restrict__ table, const Geometry G, int iterations) {
  __shared__ TreeTable T;
  for (int i = threadIdx.x; i < (int)(sizeof(TreeTable) / 4); i += blockDim.x)
    reinterpret_cast<int*>(&T)[i] = reinterpret_cast<const int*>(table)[i];
  __syncthreads();
  const float cc = T.cc;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol;
       i += (long long)gridDim.x * blockDim.x) {
    for (int j = 0; j < T.n_leaves; ++j) {
      const TreeEntry& E = T.e[T.leaves[j]];
      const float m = T.e[E.parent].sink[i];
      const float cap = E.data[i];
      float u = E.label[i];
      float s = E.sink[i];
      for (int it = 0; it < iterations; ++it) {
        s = (m - 0.0f) + u / cc;
        s = (s > cap) ? cap : s;
        u = u + cc * ((m - 0.0f) - s);
      }
      E.label[i] = u;
      E.sink[i] = s;
    }
  }
}

}  // namespace hmf
