// hmf_fp64.cu -- the REF_CUDA iteration of hmf_solve evaluated in FP64 on
// the GPU, and the measurements taken against it (include/hmf.h,
// "Reference precision").
//
// The FP32 solver reproduces the reference kernels' FP32 arithmetic bit for
// bit; this solver runs the same operations, in the same order, in double, so
// that the FP32 result's distance from the exact solution of the iteration
// can be stated for every run at full size.  Its results equal the oracle's
// FP64 restatement (CudaOracle<double>) bit for bit.  Reference operations:
//
//   init      vtkCudaHierarchicalMaxFlowSegmentation.cxx:547-658, PropogateLabels :63-104
//   grad      kern_CalcGradStep           CUDA_hierarchicalmaxflow.cu:233-241
//   descent   kern_DescentSpatialFlow     :254-285
//   magnitude kern_ComputeFlowMag{Vari,Const}Smooth :299-380
//   project   kern_Project                :401-420
//   div       kern_Divergence             :434-456
//   sweep     kern_FindLeafSinkPotential, kern_ApplyCapacity, kern_FindSinkPotentialAndStore,
//             kern_FindSourcePotentialAndStore, MultiplyAndStoreBuffer, kern_UpdateLabel
//             (:124-220, CUDA_commonKernels.cu:499) in the order of
//             vtkCudaHierarchicalMaxFlowSegmentation.cxx:106-476
//
// It is a checking instrument, not a fast path: one simple per-voxel pass per
// reference kernel group (five flow passes over every non-root vertex, one
// sweep), state in double, dense pitched arrays with the FP32 solver's
// geometry.  The host parameters are those of the FP64 oracle: step and CC
// are the FP32 values widened, 1/CC and 1/(children+1) are formed in double,
// alpha is the FP32-stored scalar widened (the reference keeps it as float).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/hmf.h"
#include "hmf_ctx.hpp"

namespace hmf {

struct F64Entry {  // post-order entries, the root last
  double* sink;    // the root: source flow
  double* u;       // null for the root
  double* div;     // null for the root (holds g, then m, then the divergence)
  double* fx;
  double* fy;
  double* fz;
  const double* inc;    // parent's sink (the root's: the source flow)
  const float* data;    // leaves
  const float* smooth;  // non-root vertices with a smoothness image
  double alpha;
  int parent;  // entry index, -1 for the root
  int first_kid, n_kids;
  int pad_;
};

struct F64Table {
  int n, n_leaves;
  int n_flow;  // non-root entries (flow passes run over entries 0 .. n_flow-1 in flow_entry order)
  int probe_entry;           // entry whose data term is overridden at one voxel (-1: none)
  long long probe_index;     // pitched element index of that voxel
  double probe_value;        // the data term there (double)
  double step, cc, icc, root_work;
  int kids[kMaxVertices];
  int leaves[kMaxVertices];      // entry indices of the leaves in DFS pre-order
  int flow_entry[kMaxVertices];  // entry index of each non-root vertex
  F64Entry e[kMaxVertices];
};

namespace {

__device__ __forceinline__ bool f64_coords(const Geometry& G, long long i, int& x, int& y, int& z) {
  const long long row = i / G.pitch;
  x = (int)(i - row * G.pitch);
  if (x >= G.vx) return false;  // padding column
  y = (int)(row % G.vy);
  z = (int)(row / G.vy);
  return true;
}

__device__ __forceinline__ double f64_data(const F64Table& T, int e, long long i) {
  return (e == T.probe_entry && i == T.probe_index) ? T.probe_value : (double)T.e[e].data[i];
}

__device__ __forceinline__ double f64_sat(double x) {  // __saturatef widened: NaN -> 0
  if (x != x) return 0.0;
  return x < 0.0 ? 0.0 : (x > 1.0 ? 1.0 : x);
}

// Initialisation: every sink and the source = min over leaves of D; leaf
// labels = [D == min] / ties; branch labels = sums of their children; flows
// and divergences 0.
__global__ void f64_init_kernel(const F64Table* __restrict__ tp, const Geometry G) {
  const F64Table& T = *tp;
  const int root = T.n - 1;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol;
       i += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    if (!f64_coords(G, i, x, y, z)) continue;
    double m = f64_data(T, T.leaves[0], i);
    for (int j = 1; j < T.n_leaves; ++j) {
      const double d = f64_data(T, T.leaves[j], i);
      m = (m < d) ? m : d;
    }
    double cnt = 0.0;
    for (int j = 0; j < T.n_leaves; ++j) {
      const int e = T.leaves[j];
      const double lab = (m == f64_data(T, e, i)) ? 1.0 : 0.0;
      T.e[e].u[i] = lab;
      cnt = cnt + lab;
    }
    for (int j = 0; j < T.n_leaves; ++j) {
      const int e = T.leaves[j];
      T.e[e].u[i] = T.e[e].u[i] / cnt;
    }
    for (int e = 0; e < root; ++e) {  // post-order: children before their parent
      const F64Entry& E = T.e[e];
      if (E.n_kids) {
        double acc = 0.0;
        for (int k = 0; k < E.n_kids; ++k) acc = acc + T.e[T.kids[E.first_kid + k]].u[i];
        E.u[i] = acc;
      }
      E.sink[i] = m;
      E.div[i] = 0.0;
      E.fx[i] = 0.0;
      E.fy[i] = 0.0;
      E.fz[i] = 0.0;
    }
    T.e[root].sink[i] = m;
  }
}

// The five flow passes; blockIdx.y selects the non-root vertex.
__global__ void f64_grad_kernel(const F64Table* __restrict__ tp, const Geometry G) {
  const F64Entry& E = tp->e[tp->flow_entry[blockIdx.y]];
  const double step = tp->step, icc = tp->icc;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol;
       i += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    if (!f64_coords(G, i, x, y, z)) continue;
    E.div[i] = step * (((E.sink[i] + E.div[i]) - E.inc[i]) - E.u[i] * icc);
  }
}

__global__ void f64_descent_kernel(const F64Table* __restrict__ tp, const Geometry G) {
  const F64Entry& E = tp->e[tp->flow_entry[blockIdx.y]];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol;
       i += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    if (!f64_coords(G, i, x, y, z)) continue;
    const double cur = E.div[i];
    E.fx[i] = x ? E.fx[i] - (cur - E.div[i - 1]) : 0.0;
    E.fy[i] = y ? E.fy[i] - (cur - E.div[i - G.pitch]) : 0.0;
    E.fz[i] = z ? E.fz[i] - (cur - E.div[i - G.plane]) : 0.0;
  }
}

// m = |p| > lim ? lim/|p| : 1 with |p| = sqrt(0.5 F).  For lim in
// (1e-150, 1e150) the test h < RN(RN(lim*lim) * (1 - 2^-49)) implies
// h < lim^2 exactly (two roundings of relative error <= 2^-53 cannot undo
// the factor), so sqrt(h) < lim, RN(sqrt(h)) <= lim and m is exactly 1
// without the square root and the division.
__global__ void f64_magnitude_kernel(const F64Table* __restrict__ tp, const Geometry G) {
  const F64Entry& E = tp->e[tp->flow_entry[blockIdx.y]];
  const double a = E.alpha;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol;
       i += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    if (!f64_coords(G, i, x, y, z)) continue;
    double up = E.fx[i] * E.fx[i];
    double dn = (x != G.vx - 1) ? E.fx[i + 1] * E.fx[i + 1] : 0.0;
    double F = up + dn;
    up = E.fy[i] * E.fy[i];
    dn = (y != G.vy - 1) ? E.fy[i + G.pitch] * E.fy[i + G.pitch] : 0.0;
    F = F + (up + dn);
    up = E.fz[i] * E.fz[i];
    dn = (z != G.vz - 1) ? E.fz[i + G.plane] * E.fz[i + G.plane] : 0.0;
    F = F + (up + dn);
    const double h = 0.5 * F;
    const double lim = E.smooth ? a * (double)E.smooth[i] : a;
    double m = 1.0;
    if (!(lim > 1e-150 && lim < 1e150 && h < (lim * lim) * (1.0 - 0x1p-49))) {
      const double Fs = sqrt(h);
      m = (Fs > lim) ? lim / Fs : 1.0;
    }
    E.div[i] = m;
  }
}

__global__ void f64_project_kernel(const F64Table* __restrict__ tp, const Geometry G) {
  const F64Entry& E = tp->e[tp->flow_entry[blockIdx.y]];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol;
       i += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    if (!f64_coords(G, i, x, y, z)) continue;
    const double cur = E.div[i];
    E.fx[i] = x ? (E.fx[i] * 0.5) * (cur + E.div[i - 1]) : 0.0;
    E.fy[i] = y ? (E.fy[i] * 0.5) * (cur + E.div[i - G.pitch]) : 0.0;
    E.fz[i] = z ? (E.fz[i] * 0.5) * (cur + E.div[i - G.plane]) : 0.0;
  }
}

__global__ void f64_divergence_kernel(const F64Table* __restrict__ tp, const Geometry G) {
  const F64Entry& E = tp->e[tp->flow_entry[blockIdx.y]];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol;
       i += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    if (!f64_coords(G, i, x, y, z)) continue;
    double dv = (E.fx[i] + E.fy[i]) + E.fz[i];
    if (x != G.vx - 1) dv = dv - E.fx[i + 1];
    if (y != G.vy - 1) dv = dv - E.fy[i + G.pitch];
    if (z != G.vz - 1) dv = dv - E.fz[i + G.plane];
    E.div[i] = dv;
  }
}

// Per voxel, all vertices: sinks in post-order from the old parent sinks,
// the source, then every label from the new sinks.
__global__ void f64_sweep_kernel(const F64Table* __restrict__ tp, const Geometry G) {
  const F64Table& T = *tp;
  const int n = T.n, root = n - 1;
  const double icc = T.icc, cc = T.cc;
  double S[kMaxVertices], W[kMaxVertices];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol;
       i += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    if (!f64_coords(G, i, x, y, z)) continue;
    for (int e = 0; e < n; ++e) S[e] = T.e[e].sink[i];
    for (int e = 0; e < n; ++e) {
      const F64Entry& E = T.e[e];
      if (E.n_kids == 0) {
        double v = (S[E.parent] - E.div[i]) + E.u[i] * icc;
        const double cap = f64_data(T, e, i);
        v = (v < 0.0) ? 0.0 : v;
        v = (v > cap) ? cap : v;
        W[e] = v;
      } else {
        double w = (e == root) ? T.root_work : 0.0;
        for (int k = 0; k < E.n_kids; ++k) {
          const int c = T.kids[E.first_kid + k];
          w = ((w + W[c]) + T.e[c].div[i]) - T.e[c].u[i] * icc;
        }
        if (e != root) {
          w = ((w + S[E.parent]) - E.div[i]) + E.u[i] * icc;
          W[e] = w * (1.0 / (double)(E.n_kids + 1));
        } else {
          W[e] = w * (1.0 / (double)E.n_kids);
        }
      }
    }
    for (int e = 0; e < root; ++e) {
      const F64Entry& E = T.e[e];
      E.u[i] = f64_sat(E.u[i] + cc * ((W[E.parent] - E.div[i]) - W[e]));
      E.sink[i] = W[e];
    }
    T.e[root].sink[i] = W[root];
  }
}

// Distance of FP32 leaf labels from the FP64 ones: max |u32 - u64| and the
// number of voxels whose argmax leaf (first maximum) agrees.
struct F64Compare {
  const float* u32[kMaxVertices];   // leaves in DFS pre-order
  const double* u64[kMaxVertices];
  int n_leaves;
};

__global__ void f64_compare_kernel(const F64Compare C, const Geometry G, unsigned long long* max_bits,
                                   unsigned long long* agree) {
  double mx = 0.0;
  unsigned long long same = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol;
       i += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    if (!f64_coords(G, i, x, y, z)) continue;
    int a32 = 0, a64 = 0;
    float b32 = C.u32[0][i];
    double b64 = C.u64[0][i];
    for (int j = 0; j < C.n_leaves; ++j) {
      const float f = C.u32[j][i];
      const double d = C.u64[j][i];
      const double diff = fabs((double)f - d);
      mx = (diff > mx || diff != diff) ? diff : mx;
      if (f > b32) b32 = f, a32 = j;
      if (d > b64) b64 = d, a64 = j;
    }
    same += (a32 == a64);
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double m2 = __shfl_down_sync(0xffffffffu, mx, o);
    mx = (m2 > mx || m2 != m2) ? m2 : mx;
    same += __shfl_down_sync(0xffffffffu, same, o);
  }
  if ((threadIdx.x & 31) == 0) {
    // a non-negative double orders like its bit pattern (NaN above infinity)
    atomicMax(max_bits, (unsigned long long)__double_as_longlong(mx != mx ? __longlong_as_double(0x7ff8000000000000ll) : mx));
    atomicAdd(agree, same);
  }
}

// L = -(1/V) sum_i log(max(u_{leaf(truth_i)}(i), eps)) on the FP64 labels,
// summed in a fixed order (per block, then over the blocks on the host), so
// that two solves that differ in a few voxels give losses whose difference
// comes from those voxels only -- what a finite difference needs.
constexpr int kF64LossThreads = 256;
__global__ void __launch_bounds__(kF64LossThreads)
f64_loss_kernel(const F64Compare C, const int* __restrict__ truth, const Geometry G, double eps, double n_voxels,
                double* partial, int* bad_flag) {
  double acc = 0.0;
  int bad = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < G.vol;
       i += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    if (!f64_coords(G, i, x, y, z)) continue;
    const int cls = truth[((long long)z * G.vy + y) * G.vx + x];
    if (cls < 0 || cls >= C.n_leaves) {
      bad = 1;
      continue;
    }
    const double u = C.u64[cls][i];
    acc -= log(u > eps ? u : eps) / n_voxels;
  }
  if (bad) atomicOr(bad_flag, 1);
  __shared__ double warp_sum[kF64LossThreads / 32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.0;
    for (int w = 0; w < kF64LossThreads / 32; ++w) b += warp_sum[w];
    partial[blockIdx.x] = b;
  }
}

}  // namespace
}  // namespace hmf

// FP64 state of a context, created by the first hmf_solve_fp64.
struct Fp64State {
  char* arena = nullptr;
  size_t bytes = 0;
  hmf::F64Table* d_table = nullptr;
  unsigned long long* d_red = nullptr;  // [0] max bits, [1] agreeing voxels, [2] loss (double), [3] flag
  int* d_truth = nullptr;               // hmf_fp64_loss's copy of a host class map
  double* d_partial = nullptr;          // hmf_fp64_loss's per-block sums
  std::vector<double*> sink, u;         // per vertex id
  hmf::F64Table h_table{};
  bool solved = false;
  // measurement overrides (hmf_set_fp64_probe)
  int probe_vertex = -1;
  long long probe_voxel = -1;
  double probe_value = 0.0;
  std::vector<double> alpha_override;  // NaN: none
};

namespace hmfi {

void fp64_free(hmf_ctx* c) {
  if (!c->f64) return;
  if (c->f64->arena) cudaFree(c->f64->arena);
  if (c->f64->d_table) cudaFree(c->f64->d_table);
  if (c->f64->d_red) cudaFree(c->f64->d_red);
  if (c->f64->d_truth) cudaFree(c->f64->d_truth);
  if (c->f64->d_partial) cudaFree(c->f64->d_partial);
  delete c->f64;
  c->f64 = nullptr;
}

size_t fp64_bytes(const hmf_ctx* c) { return c->f64 ? c->f64->bytes : 0; }

}  // namespace hmfi

using namespace hmfi;

namespace {

constexpr int kF64Threads = 256;

int fp64_usable(hmf_ctx* c) {
  if (!c) return HMF_ERR_INVALID_ARGUMENT;
  if (int rc = refuse_paged(c, "the FP64 solve")) return rc;
  if (c->dag) return fail(c, HMF_ERR_INVALID_ARGUMENT, "the FP64 solve is for label trees (hmf_create)");
  if (c->vols.size() != 1) return fail(c, HMF_ERR_INVALID_ARGUMENT, "the FP64 solve is for single-volume contexts");
  if (c->semantics != HMF_SEMANTICS_REF_CUDA)
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "the FP64 solve evaluates REF_CUDA semantics");
  return HMF_OK;
}

Fp64State* fp64_state(hmf_ctx* c) {
  if (!c->f64) {
    c->f64 = new Fp64State();
    c->f64->alpha_override.assign(c->n, std::nan(""));
  }
  return c->f64;
}

int fp64_allocate(hmf_ctx* c) {
  Fp64State* F = fp64_state(c);
  if (F->arena) return HMF_OK;
  const size_t arr = round_up((size_t)c->total * sizeof(double), 256);
  const int nonroot = c->n - 1;
  const size_t bytes = arr * ((size_t)nonroot * 6 + 1);  // per non-root: sink, u, div, 3 flows; the source
  cudaError_t e = cudaMalloc(&F->arena, bytes);
  if (e != cudaSuccess) {
    F->arena = nullptr;
    cudaGetLastError();
    return fail(c, HMF_ERR_OUT_OF_MEMORY, "cudaMalloc(FP64 state) failed: " + std::string(cudaGetErrorString(e)));
  }
  F->bytes = bytes;
  CK(cudaMalloc(&F->d_table, sizeof(hmf::F64Table)), "cudaMalloc(FP64 table)");
  CK(cudaMalloc(&F->d_red, 4 * sizeof(unsigned long long)), "cudaMalloc(FP64 sums)");
  F->sink.assign(c->n, nullptr);
  F->u.assign(c->n, nullptr);
  char* p = F->arena;
  auto take = [&]() {
    double* r = reinterpret_cast<double*>(p);
    p += arr;
    return r;
  };
  std::vector<int> entry(c->n, -1);
  for (int i = 0; i < c->n; ++i) entry[c->postorder[i]] = i;
  hmf::F64Table& T = F->h_table;
  std::memset(&T, 0, sizeof(T));
  for (int i = 0; i < c->n; ++i) {
    const int v = c->postorder[i];
    hmf::F64Entry& E = T.e[i];
    E.sink = F->sink[v] = take();
    if (v != c->root) {
      E.u = F->u[v] = take();
      E.div = take();
      E.fx = take();
      E.fy = take();
      E.fz = take();
    }
  }
  return HMF_OK;
}

// Table of one FP64 solve: pointers, inputs, parameters, probe.
void fp64_fill_table(hmf_ctx* c, const Staged& in) {
  Fp64State* F = c->f64;
  hmf::F64Table& T = F->h_table;
  std::vector<int> entry(c->n, -1);
  for (int i = 0; i < c->n; ++i) entry[c->postorder[i]] = i;
  T.n = c->n;
  T.n_leaves = (int)c->leaves.size();
  T.step = (double)c->step;
  T.cc = (double)c->cc;
  T.icc = 1.0 / (double)c->cc;
  T.root_work = 1.0 / (double)c->cc;
  int kpos = 0, nf = 0;
  for (int i = 0; i < c->n; ++i) {
    const int v = c->postorder[i];
    hmf::F64Entry& E = T.e[i];
    E.parent = v == c->root ? -1 : entry[c->parent[v]];
    E.inc = v == c->root ? nullptr : F->sink[c->parent[v]];
    E.first_kid = kpos;
    E.n_kids = (int)c->kids[v].size();
    for (int k : c->kids[v]) T.kids[kpos++] = entry[k];
    E.data = in.data[v];
    E.smooth = v == c->root ? nullptr : in.smooth[v];
    const double ov = F->alpha_override[v];
    E.alpha = ov == ov ? ov : (double)(float)c->alpha[v];  // stored as float, as the reference does
  }
  for (int v : c->preorder)
    if (v != c->root) T.flow_entry[nf++] = entry[v];
  T.n_flow = nf;
  for (size_t j = 0; j < c->leaves.size(); ++j) T.leaves[j] = entry[c->leaves[j]];
  T.probe_entry = -1;
  T.probe_index = -1;
  T.probe_value = 0.0;
  if (F->probe_vertex >= 0) {
    const auto& V = c->vols[0];
    const long long vox = F->probe_voxel;
    const long long x = vox % V.vx, y = (vox / V.vx) % V.vy, z = vox / ((long long)V.vx * V.vy);
    T.probe_entry = entry[F->probe_vertex];
    T.probe_index = z * V.plane + y * V.pitch + x;
    T.probe_value = F->probe_value;
  }
}

int fp64_grid(hmf_ctx* c) {
  const long long blocks = (c->total + kF64Threads - 1) / kF64Threads;
  return (int)std::max(1LL, std::min(blocks, (long long)c->sm_count * 8));
}

int fp64_flow_grid(hmf_ctx* c) {
  const long long blocks = (c->total + kF64Threads - 1) / kF64Threads;
  return (int)std::max(1LL, std::min(blocks, (long long)c->sm_count * 8 / std::max(1, c->n - 1) + 1));
}

hmf::F64Compare fp64_compare_table(hmf_ctx* c) {
  hmf::F64Compare C;
  std::memset(&C, 0, sizeof(C));
  C.n_leaves = (int)c->leaves.size();
  for (int j = 0; j < C.n_leaves; ++j) {
    C.u32[j] = c->label[c->leaves[j]];
    C.u64[j] = c->f64->u[c->leaves[j]];
  }
  return C;
}

// Order c->stream after the caller's queued work.
int join_user(hmf_ctx* c, cudaStream_t user) {
  CK(cudaEventRecord(c->ev_join, user), "cudaEventRecord(join)");
  CK(cudaStreamWaitEvent(c->stream, c->ev_join, 0), "cudaStreamWaitEvent(join)");
  return HMF_OK;
}

int hand_back(hmf_ctx* c, cudaStream_t user) {
  CK(cudaEventRecord(c->ev_join, c->stream), "cudaEventRecord(done)");
  CK(cudaStreamWaitEvent(user, c->ev_join, 0), "cudaStreamWaitEvent(done)");
  return HMF_OK;
}

}  // namespace

extern "C" {

int hmf_solve_fp64(hmf_ctx* c, void* stream) {
  if (int rc = fp64_usable(c)) return rc;
  for (int l : c->leaves)
    if (!c->data[0][l].ptr) return fail(c, HMF_ERR_MISSING_INPUT, "Missing data prior for leaf node.");
  DeviceGuard dg(c->device);
  cudaStream_t user = reinterpret_cast<cudaStream_t>(stream);
  cudaStream_t s = c->stream;
  if (int rc = fp64_allocate(c)) return rc;
  Fp64State* F = c->f64;
  F->solved = false;
  if (int rc = join_user(c, user)) return rc;
  Staged staged;
  if (int rc = stage_inputs(c, s, staged)) return rc;
  fp64_fill_table(c, staged);
  CK(cudaMemcpyAsync(F->d_table, &F->h_table, sizeof(hmf::F64Table), cudaMemcpyHostToDevice, s),
     "cudaMemcpyAsync(FP64 table)");
  const hmf::Geometry G = c->geo;
  const int grid = fp64_grid(c);
  const dim3 fgrid(fp64_flow_grid(c), c->n - 1);
  hmf::f64_init_kernel<<<grid, kF64Threads, 0, s>>>(F->d_table, G);
  CK(cudaGetLastError(), "f64_init_kernel launch");
  for (int it = 0; it < c->iterations; ++it) {
    hmf::f64_grad_kernel<<<fgrid, kF64Threads, 0, s>>>(F->d_table, G);
    hmf::f64_descent_kernel<<<fgrid, kF64Threads, 0, s>>>(F->d_table, G);
    hmf::f64_magnitude_kernel<<<fgrid, kF64Threads, 0, s>>>(F->d_table, G);
    hmf::f64_project_kernel<<<fgrid, kF64Threads, 0, s>>>(F->d_table, G);
    hmf::f64_divergence_kernel<<<fgrid, kF64Threads, 0, s>>>(F->d_table, G);
    hmf::f64_sweep_kernel<<<grid, kF64Threads, 0, s>>>(F->d_table, G);
    CK(cudaGetLastError(), "FP64 iteration launch");
  }
  if (int rc = hand_back(c, user)) return rc;
  F->solved = true;
  return HMF_OK;
}

int hmf_get_labels_fp64(hmf_ctx* c, int node, double* out, int where, void* stream) {
  if (int rc = fp64_usable(c)) return rc;
  if (!valid_vertex(c, node) || node == c->root)
    return fail(c, HMF_ERR_INVALID_ARGUMENT, "node must be a non-root vertex");
  if (!c->f64 || !c->f64->solved) return fail(c, HMF_ERR_STATE, "hmf_solve_fp64 has not run");
  if (!out) return fail(c, HMF_ERR_INVALID_ARGUMENT, "output pointer is NULL");
  if (where != HMF_HOST && where != HMF_DEVICE) return fail(c, HMF_ERR_INVALID_ARGUMENT, "bad `where`");
  DeviceGuard dg(c->device);
  if (where == HMF_DEVICE)
    if (int rc = check_device_pointer(c, out, "output")) return rc;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const auto& V = c->vols[0];
  CK(cudaMemcpy2DAsync(out, (size_t)V.vx * sizeof(double), c->f64->u[node], (size_t)V.pitch * sizeof(double),
                       (size_t)V.vx * sizeof(double), (size_t)V.vy * V.vz,
                       where == HMF_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s),
     "cudaMemcpy2DAsync(FP64 labels)");
  if (where == HMF_HOST) CK(cudaStreamSynchronize(s), "cudaStreamSynchronize(FP64 labels)");
  return HMF_OK;
}

int hmf_fp64_error(hmf_ctx* c, double* max_abs_err, double* argmax_agreement, void* stream) {
  if (int rc = fp64_usable(c)) return rc;
  if (!c->solved) return fail(c, HMF_ERR_STATE, "hmf_solve has not run");
  if (!c->f64 || !c->f64->solved) return fail(c, HMF_ERR_STATE, "hmf_solve_fp64 has not run");
  DeviceGuard dg(c->device);
  cudaStream_t user = reinterpret_cast<cudaStream_t>(stream);
  cudaStream_t s = c->stream;
  Fp64State* F = c->f64;
  if (int rc = join_user(c, user)) return rc;
  CK(cudaMemsetAsync(F->d_red, 0, 2 * sizeof(unsigned long long), s), "cudaMemsetAsync(FP64 sums)");
  hmf::f64_compare_kernel<<<fp64_grid(c), kF64Threads, 0, s>>>(fp64_compare_table(c), c->geo, F->d_red,
                                                                F->d_red + 1);
  CK(cudaGetLastError(), "f64_compare_kernel launch");
  unsigned long long h[2] = {0, 0};
  CK(cudaMemcpyAsync(h, F->d_red, sizeof(h), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync(FP64 sums)");
  CK(cudaStreamSynchronize(s), "cudaStreamSynchronize(FP64 sums)");
  double mx;
  std::memcpy(&mx, &h[0], sizeof(mx));
  const auto& V = c->vols[0];
  if (max_abs_err) *max_abs_err = mx;
  if (argmax_agreement) *argmax_agreement = (double)h[1] / ((double)V.vx * V.vy * V.vz);
  return hand_back(c, user);
}

int hmf_fp64_loss(hmf_ctx* c, const int* truth, int where, double eps, double* loss, void* stream) {
  if (int rc = fp64_usable(c)) return rc;
  if (!c->f64 || !c->f64->solved) return fail(c, HMF_ERR_STATE, "hmf_solve_fp64 has not run");
  if (!truth || !loss) return fail(c, HMF_ERR_INVALID_ARGUMENT, "truth and loss must not be NULL");
  if (!(eps > 0.0) || !(eps < 1.0)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "eps must lie in (0, 1)");
  if (where != HMF_HOST && where != HMF_DEVICE) return fail(c, HMF_ERR_INVALID_ARGUMENT, "bad `where`");
  DeviceGuard dg(c->device);
  if (where == HMF_DEVICE)
    if (int rc = check_device_pointer(c, truth, "truth")) return rc;
  cudaStream_t user = reinterpret_cast<cudaStream_t>(stream);
  cudaStream_t s = c->stream;
  Fp64State* F = c->f64;
  const auto& V = c->vols[0];
  const long long nvox = (long long)V.vx * V.vy * V.vz;
  if (int rc = join_user(c, user)) return rc;
  const int* d_truth = truth;
  if (where == HMF_HOST) {
    if (!F->d_truth) CK(cudaMalloc(&F->d_truth, (size_t)nvox * sizeof(int)), "cudaMalloc(truth)");
    CK(cudaMemcpyAsync(F->d_truth, truth, (size_t)nvox * sizeof(int), cudaMemcpyHostToDevice, s),
       "cudaMemcpyAsync(truth)");
    d_truth = F->d_truth;
  }
  const int grid = fp64_grid(c);
  if (!F->d_partial) CK(cudaMalloc(&F->d_partial, (size_t)c->sm_count * 8 * sizeof(double)), "cudaMalloc(FP64 sums)");
  CK(cudaMemsetAsync(F->d_red + 3, 0, sizeof(unsigned long long), s), "cudaMemsetAsync(FP64 flag)");
  hmf::f64_loss_kernel<<<grid, hmf::kF64LossThreads, 0, s>>>(fp64_compare_table(c), d_truth, c->geo, eps,
                                                              (double)nvox, F->d_partial,
                                                              reinterpret_cast<int*>(F->d_red + 3));
  CK(cudaGetLastError(), "f64_loss_kernel launch");
  std::vector<double> part(grid);
  unsigned long long flag = 0;
  CK(cudaMemcpyAsync(part.data(), F->d_partial, sizeof(double) * grid, cudaMemcpyDeviceToHost, s),
     "cudaMemcpyAsync(FP64 loss)");
  CK(cudaMemcpyAsync(&flag, F->d_red + 3, sizeof(flag), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync(FP64 flag)");
  CK(cudaStreamSynchronize(s), "cudaStreamSynchronize(FP64 loss)");
  if (flag & 1u) return fail(c, HMF_ERR_INVALID_ARGUMENT, "a ground-truth class index is not a leaf index");
  double sum = 0.0;
  for (double v : part) sum += v;
  *loss = sum;
  return hand_back(c, user);
}

int hmf_set_fp64_probe(hmf_ctx* c, int kind, int node, long long voxel, double value) {
  if (int rc = fp64_usable(c)) return rc;
  Fp64State* F = fp64_state(c);
  const auto& V = c->vols[0];
  if (kind == HMF_FP64_PROBE_NONE) {
    F->probe_vertex = -1;
    F->probe_voxel = -1;
    std::fill(F->alpha_override.begin(), F->alpha_override.end(), std::nan(""));
    return HMF_OK;
  }
  if (kind == HMF_FP64_PROBE_DATA) {
    if (!valid_vertex(c, node) || node == c->root || !c->kids[node].empty())
      return fail(c, HMF_ERR_INVALID_ARGUMENT, "a data probe needs a leaf vertex");
    if (voxel < 0 || voxel >= (long long)V.vx * V.vy * V.vz)
      return fail(c, HMF_ERR_INVALID_ARGUMENT, "probe voxel out of range");
    if (!(value >= 0.0)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "a data term must be non-negative");
    F->probe_vertex = node;
    F->probe_voxel = voxel;
    F->probe_value = value;
    return HMF_OK;
  }
  if (kind == HMF_FP64_PROBE_ALPHA) {
    if (!valid_vertex(c, node) || node == c->root)
      return fail(c, HMF_ERR_INVALID_ARGUMENT, "an alpha probe needs a non-root vertex");
    if (!(value >= 0.0)) return fail(c, HMF_ERR_INVALID_ARGUMENT, "alpha must be non-negative");
    F->alpha_override[node] = value;
    return HMF_OK;
  }
  return fail(c, HMF_ERR_INVALID_ARGUMENT, "unknown probe kind");
}

}  // extern "C"
