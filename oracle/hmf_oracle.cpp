// hmf_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the oracle).
//
// CPU restatement of the RobartsVTK hierarchical max-flow (HMF) solver, used
// solely as the checker for the CUDA implementation in robartsvtk_gb300/.
// Nothing in the product links, loads or calls this file: only tests/,
// __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm do.
//
// Two semantics are restated, because the reference's CPU and CUDA classes
// compute different things (see the per-function citations):
//
//  * REF_CUDA  -- what vtkCudaHierarchicalMaxFlowSegmentation runs on the GPU:
//      kernels  ImageProcessing/vtkCudaImageAnalytics/CUDA_hierarchicalmaxflow.cu:124-456
//      launches ImageProcessing/vtkCudaImageAnalytics/vtkCudaHierarchicalMaxFlowSegmentation.cxx:106-476
//      init     ImageProcessing/vtkCudaImageAnalytics/vtkCudaHierarchicalMaxFlowSegmentation.cxx:547-658
//    Restated kernel by kernel (one full-volume pass each, same launch order,
//    same FP32 operation order), templated on float / double so the same
//    code is also the FP64 oracle.  Build with -ffp-contract=off.
//
//  * REF_CPU   -- what vtkHierarchicalMaxFlowSegmentation runs on the host:
//      driver   Common/vtkRobartsCommon/vtkHierarchicalMaxFlowSegmentation.cxx:973-1259
//      kernels  Common/vtkRobartsCommon/vtkMaxFlowSegmentationUtilities.cxx:29-339
//    The driver below is a restatement of the recursion; the per-voxel loops
//    come from a "Utils" policy.  PortUtils restates the reference utility
//    loops (OpenMP over voxels, bit-identical per element).  When built with
//    -DHMF_ORACLE_WITH_REFERENCE the same driver is linked against the
//    reference's own compiled vtkMaxFlowSegmentationUtilities.cxx (recipe in
//    oracle/build_oracle.py, output in oracle/_ref/), which pins the port.
//
// Tree convention shared with the product: vertices 0..n-1, parent[v] == -1
// for the single root, children of a vertex in increasing id order (the order
// vtkTree::AddChild assigns).  Leaves and branches are numbered in DFS
// pre-order exactly as CheckInputConsistancy does
// (vtkHierarchicalMaxFlowSegmentation.cxx:383-398).

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef HMF_ORACLE_WITH_REFERENCE
// The reference's own utility loops, compiled from its source file.
void zeroOutBuffer(float* buffer, int size);
void setBufferToValue(float* buffer, float value, int size);
void sumBuffer(float* bufferOut, float* bufferIn, int size);
void copyBuffer(float* bufferOut, float* bufferIn, int size);
void minBuffer(float* bufferOut, float* bufferIn, int size);
void divBuffer(float* bufferOut, float* bufferIn, int size);
void divAndStoreBuffer(float* bufferOut, float* bufferIn, float value, int size);
void lblBuffer(float* label, float* sink, float* cap, int size);
void constrainBuffer(float* sink, float* cap, int size);
void updateLeafSinkFlow(float* sink, float* inc, float* div, float* label, float CC, int size);
void updateLabel(float* sink, float* inc, float* div, float* label, float CC, int size);
void storeSinkFlowInBuffer(float* working, float* inc, float* div, float* label, float CC, int size);
void storeSourceFlowInBuffer(float* working, float* sink, float* div, float* label, float CC, int size);
void ghmf_flowGradientStep(float* sink, float* inc, float* div, float* label, float StepSize, float CC, int size);
void ghmf_applyStep(float* div, float* flowX, float* flowY, float* flowZ, int VX, int VY, int VZ, int size);
void ghmf_computeFlowMag(float* div, float* flowX, float* flowY, float* flowZ, float* smooth, float alpha, int VX, int VY, int VZ, int size);
void ghmf_projectOntoSet(float* div, float* flowX, float* flowY, float* flowZ, int VX, int VY, int VZ, int size);
#endif

namespace {

thread_local std::string g_err;

// ---------------------------------------------------------------------------
// Tree bookkeeping (vtkHierarchicalMaxFlowSegmentation.cxx:363-505, :872-905)
// ---------------------------------------------------------------------------
struct Tree {
  int n = 0;
  int root = -1;
  std::vector<int> parent;
  std::vector<std::vector<int>> kids;
  std::vector<int> preorder;    // DFS discovery order from the root
  std::vector<int> leaf_index;  // vertex -> LeafMap value or -1
  std::vector<int> branch_index;  // vertex -> BranchMap value or -1
  int n_leaves = 0, n_branches = 0;

  bool build(int n_nodes, const int* par) {
    n = n_nodes;
    if (n < 2) { g_err = "tree needs a root and at least one leaf"; return false; }
    parent.assign(par, par + n);
    kids.assign(n, {});
    for (int v = 0; v < n; ++v) {
      if (parent[v] < 0) {
        if (root >= 0) { g_err = "tree has more than one root"; return false; }
        root = v;
      } else if (parent[v] >= n || parent[v] == v) {
        g_err = "tree parent id out of range"; return false;
      } else {
        kids[parent[v]].push_back(v);  // increasing id order
      }
    }
    if (root < 0) { g_err = "tree has no root"; return false; }
    std::vector<int> stack{root};
    std::vector<char> seen(n, 0);
    while (!stack.empty()) {
      int v = stack.back(); stack.pop_back();
      if (seen[v]) { g_err = "tree has a cycle"; return false; }
      seen[v] = 1;
      preorder.push_back(v);
      for (int k = (int)kids[v].size() - 1; k >= 0; --k) stack.push_back(kids[v][k]);
    }
    if ((int)preorder.size() != n) { g_err = "tree is not connected"; return false; }
    if (kids[root].empty()) { g_err = "root has no children"; return false; }
    leaf_index.assign(n, -1);
    branch_index.assign(n, -1);
    for (int v : preorder) {
      if (kids[v].empty()) leaf_index[v] = n_leaves++;
      else if (v != root) branch_index[v] = n_branches++;
    }
    return true;
  }
  bool leaf(int v) const { return kids[v].empty(); }
};

template <class T> inline T sat01(T x) {
  // __saturatef: clamp to [0,1], NaN -> 0 (CUDA_hierarchicalmaxflow.cu:215)
  if (x != x) return T(0);
  return x < T(0) ? T(0) : (x > T(1) ? T(1) : x);
}

// ---------------------------------------------------------------------------
// REF_CUDA restatement
// ---------------------------------------------------------------------------
template <class T>
struct CudaOracle {
  int VX, VY, VZ;
  long V;
  const Tree& t;
  // per vertex state (root uses sink = source flow, work = source working)
  std::vector<std::vector<T>> fx, fy, fz, div, sink, u, work;
  std::vector<const float*> data, smooth;
  std::vector<T> alpha;
  T step, cc, icc, root_work;

  CudaOracle(const Tree& tr, int vx, int vy, int vz) : VX(vx), VY(vy), VZ(vz), t(tr) {
    V = (long)vx * vy * vz;
  }

  void alloc() {
    int n = t.n;
    fx.assign(n, {}); fy.assign(n, {}); fz.assign(n, {}); div.assign(n, {});
    sink.assign(n, {}); u.assign(n, {}); work.assign(n, {});
    for (int v = 0; v < n; ++v) {
      sink[v].assign(V, T(0));
      if (v != t.root) {
        fx[v].assign(V, T(0)); fy[v].assign(V, T(0)); fz[v].assign(V, T(0));
        div[v].assign(V, T(0)); u[v].assign(V, T(0));
      }
      if (!t.leaf(v)) work[v].assign(V, T(0));
    }
  }

  // vtkCudaHierarchicalMaxFlowSegmentation.cxx:547-658 and :63-104
  void init() {
    std::vector<int> leaves;
    for (int v : t.preorder) if (t.leaf(v)) leaves.push_back(v);
    const long n = V;
    // leafSink[i] = D[i]  (CopyBuffers)
    for (int l : leaves) {
      T* s = sink[l].data(); const float* d = data[l];
#pragma omp parallel for schedule(static)
      for (long i = 0; i < n; ++i) s[i] = T(d[i]);
    }
    // leafSink[0] = min over leaves  (kern_MinBuffers, CUDA_hierarchicalmaxflow.cu:489-499)
    T* s0 = sink[leaves[0]].data();
    for (size_t k = 1; k < leaves.size(); ++k) {
      const T* sk = sink[leaves[k]].data();
#pragma omp parallel for schedule(static)
      for (long i = 0; i < n; ++i) { T a = s0[i], b = sk[i]; s0[i] = (a < b) ? a : b; }
    }
    // labels: [sink == D] / count  (kern_Lbl :519-529, SumBuffers, kern_DivideBuffers :584-594)
    std::vector<T>& cnt = work[t.root];
    std::fill(cnt.begin(), cnt.end(), T(0));
    for (size_t k = 0; k < leaves.size(); ++k) {
      int l = leaves[k];
      T* sl = sink[l].data(); T* ul = u[l].data(); const float* d = data[l]; T* c = cnt.data();
#pragma omp parallel for schedule(static)
      for (long i = 0; i < n; ++i) {
        if (k > 0) sl[i] = s0[i];
        ul[i] = (sl[i] == T(d[i])) ? T(1) : T(0);
        c[i] = c[i] + ul[i];
      }
    }
    for (int l : leaves) {
      T* ul = u[l].data(); const T* c = cnt.data();
#pragma omp parallel for schedule(static)
      for (long i = 0; i < n; ++i) ul[i] = ul[i] / c[i];
    }
    // branch sinks and the source flow = min
    for (int v = 0; v < t.n; ++v) if (!t.leaf(v)) {
      T* s = sink[v].data();
#pragma omp parallel for schedule(static)
      for (long i = 0; i < n; ++i) s[i] = s0[i];
    }
    propagate(t.root);
  }

  void propagate(int v) {  // PropogateLabels, vtkCudaHierarchicalMaxFlowSegmentation.cxx:63-104
    if (!t.leaf(v) && v != t.root) std::fill(u[v].begin(), u[v].end(), T(0));
    for (int k : t.kids[v]) propagate(k);
    if (v == t.root) return;
    int p = t.parent[v];
    if (p == t.root) return;
    T* up = u[p].data(); const T* uv = u[v].data();
    const long n = V;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) up[i] = up[i] + uv[i];
  }

  // kern_CalcGradStep (CUDA_hierarchicalmaxflow.cu:233-241)
  void grad_step(int v) {
    const T* s = sink[v].data(); const T* c = sink[t.parent[v]].data();
    const T* uu = u[v].data(); T* d = div[v].data();
    const long n = V;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) d[i] = step * (((s[i] + d[i]) - c[i]) - uu[i] * icc);
  }

  // kern_DescentSpatialFlow (:254-285)
  void descent(int v) {
    const T* g = div[v].data(); T* px = fx[v].data(); T* py = fy[v].data(); T* pz = fz[v].data();
    const long n = V, sxy = (long)VX * VY;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
      const int x = (int)(i % VX), y = (int)((i / VX) % VY), z = (int)(i / sxy);
      T cur = g[i];
      px[i] = x ? px[i] - (cur - g[i - 1]) : T(0);
      py[i] = y ? py[i] - (cur - g[i - VX]) : T(0);
      pz[i] = z ? pz[i] - (cur - g[i - sxy]) : T(0);
    }
  }

  // kern_ComputeFlowMagVariSmooth / ConstSmooth (:299-380)
  void flow_mag(int v) {
    T* m = div[v].data(); const T* px = fx[v].data(); const T* py = fy[v].data(); const T* pz = fz[v].data();
    const float* S = smooth[v]; const T a = alpha[v];
    const long n = V, sxy = (long)VX * VY;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
      const int x = (int)(i % VX), y = (int)((i / VX) % VY);
      T up = px[i] * px[i];
      T dn = (x != VX - 1) ? px[i + 1] * px[i + 1] : T(0);
      T F = up + dn;
      up = py[i] * py[i];
      dn = (y != VY - 1) ? py[i + VX] * py[i + VX] : T(0);
      F += up + dn;
      up = pz[i] * pz[i];
      dn = (i + sxy < n) ? pz[i + sxy] * pz[i + sxy] : T(0);
      F += up + dn;
      F = std::sqrt(T(0.5) * F);
      T sm = S ? a * T(S[i]) : a;
      m[i] = (F > sm) ? sm / F : T(1);
    }
  }

  // kern_Project + kern_Divergence (:401-456)
  void project_div(int v) {
    T* d = div[v].data(); T* px = fx[v].data(); T* py = fy[v].data(); T* pz = fz[v].data();
    const long n = V, sxy = (long)VX * VY;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
      const int x = (int)(i % VX), y = (int)((i / VX) % VY), z = (int)(i / sxy);
      T cur = d[i];
      px[i] = x ? px[i] * T(0.5) * (cur + d[i - 1]) : T(0);
      py[i] = y ? py[i] * T(0.5) * (cur + d[i - VX]) : T(0);
      pz[i] = z ? pz[i] * T(0.5) * (cur + d[i - sxy]) : T(0);
    }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
      const int x = (int)(i % VX), y = (int)((i / VX) % VY);
      T dv = px[i] + py[i] + pz[i];
      if (x != VX - 1) dv -= px[i + 1];
      if (y != VY - 1) dv -= py[i + VX];
      if (i < n - sxy) dv -= pz[i + sxy];
      d[i] = dv;
    }
  }

  // SolveMaxFlow / UpdateLabel, vtkCudaHierarchicalMaxFlowSegmentation.cxx:106-476
  void solve(int v) {
    const bool is_root = (v == t.root), is_leaf = t.leaf(v), is_branch = !is_root && !is_leaf;
    const long n = V;
    const int nk = (int)t.kids[v].size();
    if (!is_leaf) {
      T init = is_branch ? T(0) : root_work;
      std::fill(work[v].begin(), work[v].end(), init);
    }
    if (!is_root) { grad_step(v); descent(v); flow_mag(v); project_div(v); }
    for (int k : t.kids[v]) solve(k);
    if (is_branch) {
      // kern_FindSinkPotentialAndStore (:124-132), MultiplyAndStoreBuffer (CUDA_commonKernels.cu:499)
      T* w = work[v].data(); const T* c = sink[t.parent[v]].data(); const T* d = div[v].data();
      const T* uu = u[v].data(); T* s = sink[v].data();
      const T inv = T(1) / T(nk + 1);
#pragma omp parallel for schedule(static)
      for (long i = 0; i < n; ++i) {
        w[i] = ((w[i] + c[i]) - d[i]) + uu[i] * icc;
        s[i] = w[i] * inv;
      }
    }
    if (is_root) {
      T* w = work[v].data(); T* s = sink[v].data();
      const T inv = T(1) / T(nk);
#pragma omp parallel for schedule(static)
      for (long i = 0; i < n; ++i) s[i] = w[i] * inv;
    }
    if (is_leaf) {
      // kern_FindLeafSinkPotential (:166-174) + kern_ApplyCapacity (:187-198)
      T* s = sink[v].data(); const T* c = sink[t.parent[v]].data(); const T* d = div[v].data();
      const T* uu = u[v].data(); const float* D = data[v];
#pragma omp parallel for schedule(static)
      for (long i = 0; i < n; ++i) {
        T val = (c[i] - d[i]) + uu[i] * icc;
        T cap = T(D[i]);
        val = (val < T(0)) ? T(0) : val;
        val = (val > cap) ? cap : val;
        s[i] = val;
      }
    }
    for (int k = nk - 1; k >= 0; --k) {
      // kern_UpdateLabel (:211-220)
      int kid = t.kids[v][k];
      const T* s = sink[kid].data(); const T* c = sink[v].data(); const T* d = div[kid].data();
      T* uu = u[kid].data();
#pragma omp parallel for schedule(static)
      for (long i = 0; i < n; ++i) uu[i] = sat01(uu[i] + cc * ((c[i] - d[i]) - s[i]));
    }
    if (!is_root) {
      // kern_FindSourcePotentialAndStore (:145-153)
      T* w = work[t.parent[v]].data(); const T* s = sink[v].data(); const T* d = div[v].data();
      const T* uu = u[v].data();
#pragma omp parallel for schedule(static)
      for (long i = 0; i < n; ++i) w[i] = ((w[i] + s[i]) + d[i]) - uu[i] * icc;
    }
  }
};

// ---------------------------------------------------------------------------
// REF_CPU: per-voxel loops of vtkMaxFlowSegmentationUtilities.cxx restated.
// The reference reads a few floats outside some buffers (its neighbour tests
// are inverted); here those reads are guarded and give 0, the value the
// oracle's padded buffers hold there.  With the flows identically zero (the
// reference multiplies them, :261-273) those terms never reach a result.
// ---------------------------------------------------------------------------
struct PortUtils {
  static void zeroOut(float* b, int n) {
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) b[x] = 0.0f;
  }
  static void setValue(float* b, float v, int n) {
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) b[x] = v;
  }
  static void sum(float* o, float* i, int n) {  // :53-59
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) o[x] += i[x];
  }
  static void copy(float* o, float* i, int n) {  // :69-75
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) o[x] = i[x];
  }
  static void min(float* o, float* i, int n) {  // :77-83
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) o[x] = (o[x] > i[x]) ? i[x] : o[x];
  }
  static void div(float* o, float* i, int n) {  // :85-91
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) o[x] /= i[x];
  }
  static void divAndStore(float* o, float* i, float v, int n) {  // :93-99
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) o[x] = i[x] / v;
  }
  static void lbl(float* l, float* s, float* c, int n) {  // :101-107
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) l[x] = (s[x] == c[x]) ? 1.0f : 0.0f;
  }
  static void constrain(float* s, float* c, int n) {  // :109-115
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) s[x] = (s[x] > c[x]) ? c[x] : s[x];
  }
  static void leafSink(float* s, float* inc, float* d, float* l, float CC, int n) {  // :117-123
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) s[x] = inc[x] - d[x] + l[x] / CC;
  }
  static void label(float* s, float* inc, float* d, float* l, float CC, int n) {  // :125-131
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) l[x] += CC * (inc[x] - d[x] - s[x]);
  }
  static void storeSink(float* w, float* inc, float* d, float* l, float CC, int n) {  // :141-147
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) w[x] = inc[x] - d[x] + l[x] / CC;
  }
  static void storeSource(float* w, float* s, float* d, float* l, float CC, int n) {  // :156-162
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) w[x] += s[x] + d[x] - l[x] / CC;
  }
  static void gradStep(float* s, float* inc, float* d, float* l, float step, float CC, int n) {  // :253-259
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) d[x] = step * (s[x] + d[x] - inc[x] - l[x] / CC);
  }
  static void applyStep(float* d, float* fx, float* fy, float* fz, int VX, int VY, int VZ, int n) {  // :261-273
    (void)VZ;
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) {
      float cur = d[x];
      float xa = (x % VX) ? d[x - 1] : 0.0f;
      fx[x] *= 0.5f * (cur - xa);
      float ya = (x / VX % VY) ? d[x - VX] : 0.0f;
      fy[x] *= 0.5f * (cur - ya);
      float za = (x >= VX * VY) ? d[x - VX * VY] : 0.0f;
      fz[x] *= 0.5f * (cur - za);
    }
  }
  static void flowMag(float* d, float* fx, float* fy, float* fz, float* sm, float alpha,
                      int VX, int VY, int VZ, int n) {  // :275-307
    (void)fy; (void)fz; (void)VZ;
    auto at = [&](long k) -> float { return (k >= 0 && k < n) ? fx[k] : 0.0f; };
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) d[x] = fx[x] * fx[x] + fy[x] * fy[x] + fz[x] * fz[x];
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) d[x] += ((x + 1) % VX) ? 0.0f : at(x + 1) * at(x + 1);
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) d[x] += (((x + VX) / VX) % VY) ? 0.0f : at((long)x + VX) * at((long)x + VX);
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n - VX * VY; ++x) d[x] += fx[x + VX * VY] * fx[x + VX * VY];
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) d[x] = sqrtf(d[x]);
    if (sm) {
#pragma omp parallel for schedule(static)
      for (int x = 0; x < n; ++x) d[x] = (d[x] > alpha * sm[x]) ? alpha * sm[x] / d[x] : 1.0f;
    } else {
#pragma omp parallel for schedule(static)
      for (int x = 0; x < n; ++x) d[x] = (d[x] > alpha) ? alpha / d[x] : 1.0f;
    }
  }
  static void project(float* d, float* fx, float* fy, float* fz, int VX, int VY, int VZ, int n) {  // :309-339
    auto atz = [&](long k) -> float { return (k >= 0 && k < n) ? fz[k] : 0.0f; };
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) {
      float cur = d[x];
      float xa = (x % VX) ? d[x - 1] : -cur;
      fx[x] *= 0.5f * (cur + xa);
      float ya = (x / VX % VY) ? d[x - VX] : -cur;
      fy[x] *= 0.5f * (cur + ya);
      float za = (x >= VX * VY) ? d[x - VX * VY] : -cur;
      fz[x] *= 0.5f * (cur + za);
    }
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) d[x] = fx[x] + fy[x] + fz[x];
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) d[x] -= (x % VX) ? fx[x - 1] : 0.0f;
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) d[x] -= (x / VX % VY) ? fy[x - VX] : 0.0f;
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; ++x) d[x] -= (x >= VX * VY) ? atz((long)x - (long)VX * VZ) : 0.0f;
  }
};

#ifdef HMF_ORACLE_WITH_REFERENCE
struct RefUtils {
  static void zeroOut(float* b, int n) { zeroOutBuffer(b, n); }
  static void setValue(float* b, float v, int n) { setBufferToValue(b, v, n); }
  static void sum(float* o, float* i, int n) { sumBuffer(o, i, n); }
  static void copy(float* o, float* i, int n) { copyBuffer(o, i, n); }
  static void min(float* o, float* i, int n) { minBuffer(o, i, n); }
  static void div(float* o, float* i, int n) { divBuffer(o, i, n); }
  static void divAndStore(float* o, float* i, float v, int n) { divAndStoreBuffer(o, i, v, n); }
  static void lbl(float* l, float* s, float* c, int n) { lblBuffer(l, s, c, n); }
  static void constrain(float* s, float* c, int n) { constrainBuffer(s, c, n); }
  static void leafSink(float* s, float* inc, float* d, float* l, float CC, int n) { updateLeafSinkFlow(s, inc, d, l, CC, n); }
  static void label(float* s, float* inc, float* d, float* l, float CC, int n) { updateLabel(s, inc, d, l, CC, n); }
  static void storeSink(float* w, float* inc, float* d, float* l, float CC, int n) { storeSinkFlowInBuffer(w, inc, d, l, CC, n); }
  static void storeSource(float* w, float* s, float* d, float* l, float CC, int n) { storeSourceFlowInBuffer(w, s, d, l, CC, n); }
  static void gradStep(float* s, float* inc, float* d, float* l, float st, float CC, int n) { ghmf_flowGradientStep(s, inc, d, l, st, CC, n); }
  static void applyStep(float* d, float* fx, float* fy, float* fz, int VX, int VY, int VZ, int n) { ghmf_applyStep(d, fx, fy, fz, VX, VY, VZ, n); }
  static void flowMag(float* d, float* fx, float* fy, float* fz, float* sm, float a, int VX, int VY, int VZ, int n) { ghmf_computeFlowMag(d, fx, fy, fz, sm, a, VX, VY, VZ, n); }
  static void project(float* d, float* fx, float* fy, float* fz, int VX, int VY, int VZ, int n) { ghmf_projectOntoSet(d, fx, fy, fz, VX, VY, VZ, n); }
};
#endif

// Restatement of vtkHierarchicalMaxFlowSegmentation.cxx:973-1259 over a Utils policy.
// Every buffer carries `pad` zero floats on both sides so that the reference's
// loops, which index a little outside their buffers, stay inside memory here.
template <class U>
struct CpuDriver {
  const Tree& t;
  int VX, VY, VZ, V;
  long pad;
  std::vector<std::vector<float>> store;
  std::vector<float*> fx, fy, fz, div, sink, inc, lab, work;
  std::vector<float*> data, smooth;
  std::vector<float> alpha;
  float step, cc;

  CpuDriver(const Tree& tr, int vx, int vy, int vz) : t(tr), VX(vx), VY(vy), VZ(vz) {
    V = vx * vy * vz;
    pad = (long)vx * (vy + vz + 2) + 16;
  }
  float* buffer() {
    store.emplace_back((size_t)(V + 2 * pad), 0.0f);
    return store.back().data() + pad;
  }
  void alloc() {
    int n = t.n;
    fx.assign(n, nullptr); fy = fx; fz = fx; div = fx; sink = fx; inc = fx; lab = fx; work = fx;
    store.reserve(8 * n + 4);
    for (int v = 0; v < n; ++v) {
      sink[v] = buffer();
      if (!t.leaf(v)) work[v] = buffer();
      if (v != t.root) { fx[v] = buffer(); fy[v] = buffer(); fz[v] = buffer(); div[v] = buffer(); lab[v] = buffer(); }
    }
    for (int v = 0; v < n; ++v) if (v != t.root) inc[v] = sink[t.parent[v]];  // :872-905
  }
  void init() {  // :973-1031
    std::vector<int> leaves;
    for (int v : t.preorder) if (t.leaf(v)) leaves.push_back(v);
    for (int v = 0; v < t.n; ++v) if (v != t.root && !t.leaf(v)) {
      U::zeroOut(fx[v], V); U::zeroOut(fy[v], V); U::zeroOut(fz[v], V); U::zeroOut(div[v], V);
    }
    for (int l : leaves) { U::zeroOut(fx[l], V); U::zeroOut(fy[l], V); U::zeroOut(fz[l], V); U::zeroOut(div[l], V); }
    for (int l : leaves) U::copy(sink[l], data[l], V);
    for (size_t k = 1; k < leaves.size(); ++k) U::min(sink[leaves[0]], sink[leaves[k]], V);
    float* src_work = work[t.root];
    U::zeroOut(src_work, V);
    U::lbl(lab[leaves[0]], sink[leaves[0]], data[leaves[0]], V);
    U::sum(src_work, lab[leaves[0]], V);
    for (size_t k = 1; k < leaves.size(); ++k) {
      U::copy(sink[leaves[k]], sink[leaves[0]], V);
      U::lbl(lab[leaves[k]], sink[leaves[k]], data[leaves[k]], V);
      U::sum(src_work, lab[leaves[k]], V);
    }
    for (int l : leaves) U::div(lab[l], src_work, V);
    for (int v : t.preorder) if (v != t.root && !t.leaf(v)) U::copy(sink[v], sink[leaves[0]], V);
    U::copy(sink[t.root], sink[leaves[0]], V);
    propagate(t.root);
  }
  void propagate(int v) {  // :1047-1081
    if (!t.leaf(v)) { if (v != t.root) U::zeroOut(lab[v], V); }
    for (int k : t.kids[v]) propagate(k);
    if (v == t.root) return;
    int p = t.parent[v];
    if (p == t.root) return;
    U::sum(lab[p], lab[v], V);
  }
  void solve(int v) {  // :1083-1240
    const bool is_root = (v == t.root), is_leaf = t.leaf(v), is_branch = !is_root && !is_leaf;
    const int nk = (int)t.kids[v].size();
    if (!is_leaf) {
      if (is_branch) U::zeroOut(work[v], V);
      else U::setValue(work[v], 1.0f / cc, V);
    }
    if (!is_root) {
      U::gradStep(sink[v], inc[v], div[v], lab[v], step, cc, V);
      U::applyStep(div[v], fx[v], fy[v], fz[v], VX, VY, VZ, V);
      U::flowMag(div[v], fx[v], fy[v], fz[v], smooth[v], alpha[v], VX, VY, VZ, V);
      U::project(div[v], fx[v], fy[v], fz[v], VX, VY, VZ, V);
    }
    for (int k : t.kids[v]) solve(k);
    if (is_branch) {
      U::storeSink(work[v], inc[v], div[v], lab[v], cc, V);
      // The reference passes (working, sink): the branch sink is the input and
      // the working buffer the output (:1186-1187).
      U::divAndStore(work[v], sink[v], (float)(nk + 1), V);
    }
    if (is_root) U::divAndStore(work[v], sink[v], (float)nk, V);  // same order, :1196
    if (is_leaf) {
      U::leafSink(sink[v], inc[v], div[v], lab[v], cc, V);
      U::constrain(sink[v], data[v], V);
    }
    for (int k = nk - 1; k >= 0; --k) {
      int kid = t.kids[v][k];
      U::label(sink[kid], inc[kid], div[kid], lab[kid], cc, V);
    }
    if (!is_root) U::storeSource(work[t.parent[v]], sink[v], div[v], lab[v], cc, V);
  }
};

struct Problem {
  int vx, vy, vz, n_nodes;
  const int* parent;
  const float* const* data;
  const float* const* smooth;
  const double* alpha;
  int iterations;
  float step, cc;
};

template <class T>
int run_cuda_semantics(const Problem& P, const Tree& t, double* u_out, double* sink_out, double* div_out) {
  CudaOracle<T> o(t, P.vx, P.vy, P.vz);
  o.alloc();
  o.data.assign(t.n, nullptr); o.smooth.assign(t.n, nullptr); o.alpha.assign(t.n, T(1));
  for (int v = 0; v < t.n; ++v) {
    o.data[v] = P.data ? P.data[v] : nullptr;
    o.smooth[v] = P.smooth ? P.smooth[v] : nullptr;
    // the reference stores the scalar as float (leafSmoothnessConstants, :692)
    o.alpha[v] = P.alpha ? T((float)P.alpha[v]) : T(1);
  }
  for (int v = 0; v < t.n; ++v) if (t.leaf(v) && !o.data[v]) { g_err = "missing data term for a leaf"; return -3; }
  if (sizeof(T) == sizeof(float)) {
    o.step = T(P.step); o.cc = T(P.cc);
    o.icc = T(1.0f / P.cc);       // host-side 1.0f/CC (CUDA_hierarchicalmaxflow.cu:138)
    o.root_work = T(1.0f / P.cc);  // CUDA_SetBufferToValue(…, 1.0f/CC) (.cxx:139)
  } else {
    o.step = T(P.step); o.cc = T(P.cc);
    o.icc = T(1) / T(P.cc);
    o.root_work = T(1) / T(P.cc);
  }
  o.init();
  for (int it = 0; it < P.iterations; ++it) o.solve(t.root);
  const long V = o.V;
  for (int v = 0; v < t.n; ++v) {
    for (long i = 0; i < V; ++i) {
      if (u_out) u_out[(long)v * V + i] = (v == t.root) ? 0.0 : (double)o.u[v][i];
      if (sink_out) sink_out[(long)v * V + i] = (double)o.sink[v][i];
      if (div_out) div_out[(long)v * V + i] = (v == t.root) ? 0.0 : (double)o.div[v][i];
    }
  }
  return 0;
}

template <class U>
int run_cpu_semantics(const Problem& P, const Tree& t, double* u_out, double* sink_out, double* div_out) {
  CpuDriver<U> d(t, P.vx, P.vy, P.vz);
  d.alloc();
  d.data.assign(t.n, nullptr); d.smooth.assign(t.n, nullptr); d.alpha.assign(t.n, 1.0f);
  std::vector<std::vector<float>> copies;
  copies.reserve(2 * t.n);
  for (int v = 0; v < t.n; ++v) {
    if (P.data && P.data[v]) {
      copies.emplace_back(P.data[v], P.data[v] + d.V);
      d.data[v] = copies.back().data();
    }
    if (P.smooth && P.smooth[v]) {
      copies.emplace_back(P.smooth[v], P.smooth[v] + d.V);
      d.smooth[v] = copies.back().data();
    }
    d.alpha[v] = P.alpha ? (float)P.alpha[v] : 1.0f;
  }
  for (int v = 0; v < t.n; ++v) if (t.leaf(v) && !d.data[v]) { g_err = "missing data term for a leaf"; return -3; }
  d.step = P.step; d.cc = P.cc;
  d.init();
  for (int it = 0; it < P.iterations; ++it) d.solve(t.root);
  const long V = d.V;
  for (int v = 0; v < t.n; ++v) {
    for (long i = 0; i < V; ++i) {
      if (u_out) u_out[(long)v * V + i] = (v == t.root) ? 0.0 : (double)d.lab[v][i];
      if (sink_out) sink_out[(long)v * V + i] = (double)d.sink[v][i];
      if (div_out) div_out[(long)v * V + i] = (v == t.root) ? 0.0 : (double)d.div[v][i];
    }
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Adjoint of the REF_CUDA iteration (reverse mode), restated on the CPU.
//
// Loss: L = -(1/V) sum_i log(max(u_{leaf(truth(i))}(i), eps)) over the final
// leaf labels.  Gradients: dL/dD for every leaf data term (per voxel) and
// dL/dalpha for every non-root vertex.  Conventions at the kinks: saturate
// passes the gradient only strictly inside (0, 1); the leaf capacity clamp
// passes it to the sink input strictly inside (0, D) and to D when the input
// exceeds D; the multiplier depends on |p| and alpha only when |p| > alpha*S;
// the initial sink min(D) sends its gradient to the leaf kern_MinBuffers keeps
// (the last one of a tie).  Forward states of every iteration are stored
// (small problems only).
// ---------------------------------------------------------------------------
template <class T>
struct AdjointRun {
  const Tree& t;
  CudaOracle<T>& o;
  int VX, VY, VZ;
  long V, sxy;
  struct State {
    std::vector<std::vector<T>> px, py, pz, s, u;
  };
  std::vector<State> states;

  AdjointRun(const Tree& tr, CudaOracle<T>& ora) : t(tr), o(ora), VX(ora.VX), VY(ora.VY), VZ(ora.VZ) {
    V = o.V;
    sxy = (long)VX * VY;
  }
  State snap() const {
    State st;
    st.px = o.fx;
    st.py = o.fy;
    st.pz = o.fz;
    st.s = o.sink;
    st.u = o.u;
    return st;
  }
  int xo(long i) const { return (int)(i % VX); }
  int yo(long i) const { return (int)((i / VX) % VY); }
  int zo(long i) const { return (int)(i / sxy); }
  // kern_Divergence of flows (px, py, pz)
  void divergence(const std::vector<T>& px, const std::vector<T>& py, const std::vector<T>& pz, std::vector<T>& d) const {
    d.assign(V, T(0));
    for (long i = 0; i < V; ++i) {
      T dv = px[i] + py[i] + pz[i];
      if (xo(i) != VX - 1) dv -= px[i + 1];
      if (yo(i) != VY - 1) dv -= py[i + VX];
      if (i < V - sxy) dv -= pz[i + sxy];
      d[i] = dv;
    }
  }

  // Backward through iteration t: (Pb, sbn, ubn) are the adjoints of state
  // t+1 on entry and of state t on exit; Db, ab accumulate.
  void backward_step(int it, std::vector<std::vector<T>>& Pbx, std::vector<std::vector<T>>& Pby,
                     std::vector<std::vector<T>>& Pbz, std::vector<std::vector<T>>& sbn,
                     std::vector<std::vector<T>>& ubn, std::vector<std::vector<double>>& Db, std::vector<double>& ab) {
    const State& A = states[it];
    const State& B = states[it + 1];
    const int n = t.n, root = t.root;
    const T icc = o.icc, cc = o.cc, tau = o.step;
    std::vector<std::vector<T>> dnew(n), dbp(n, std::vector<T>(V, T(0)));
    std::vector<std::vector<T>> sbo(n, std::vector<T>(V, T(0))), ubo(n, std::vector<T>(V, T(0)));
    for (int v = 0; v < n; ++v)
      if (v != root) divergence(B.px[v], B.py[v], B.pz[v], dnew[v]);
    // --- phase 2 reverse: labels, then sinks in reverse post-order
    std::vector<std::vector<T>> sbN = sbn;  // adjoint of the new sinks
    for (int v = 0; v < n; ++v) {
      if (v == root) continue;
      const int p = t.parent[v];
      for (long i = 0; i < V; ++i) {
        const T z = A.u[v][i] + cc * ((B.s[p][i] - dnew[v][i]) - B.s[v][i]);
        const T zb = (z > T(0) && z < T(1)) ? ubn[v][i] : T(0);
        ubo[v][i] += zb;
        sbN[p][i] += cc * zb;
        dbp[v][i] -= cc * zb;
        sbN[v][i] -= cc * zb;
      }
    }
    std::vector<int> rev(t.preorder.begin(), t.preorder.end());  // parents before children
    for (int v : rev) {
      const auto& kids = t.kids[v];
      if (kids.empty()) {
        const int p = t.parent[v];
        for (long i = 0; i < V; ++i) {
          const T y = (A.s[p][i] - dnew[v][i]) + A.u[v][i] * icc;
          const T cap = T(o.data[v][i]);
          if (y < T(0)) continue;
          if (y > cap) {
            Db[v][i] += (double)sbN[v][i];
            continue;
          }
          const T yb = sbN[v][i];
          sbo[p][i] += yb;
          dbp[v][i] -= yb;
          ubo[v][i] += icc * yb;
        }
      } else {
        const T inv = (v == root) ? T(1) / T((int)kids.size()) : T(1) / T((int)kids.size() + 1);
        for (long i = 0; i < V; ++i) {
          const T Wb = sbN[v][i] * inv;
          if (v != root) {
            sbo[t.parent[v]][i] += Wb;
            dbp[v][i] -= Wb;
            ubo[v][i] += icc * Wb;
          }
          for (int k : kids) {
            sbN[k][i] += Wb;
            dbp[k][i] += Wb;
            ubo[k][i] -= icc * Wb;
          }
        }
      }
    }
    // --- phase 1 reverse, vertex by vertex
    for (int v = 0; v < n; ++v) {
      if (v == root) continue;
      const int p = t.parent[v];
      std::vector<T> dold, g(V), ppx(V), ppy(V), ppz(V), Fm(V), lim(V), m(V);
      divergence(A.px[v], A.py[v], A.pz[v], dold);
      for (long i = 0; i < V; ++i) g[i] = tau * (((A.s[v][i] + dold[i]) - A.s[p][i]) - A.u[v][i] * icc);
      for (long i = 0; i < V; ++i) {
        ppx[i] = xo(i) ? A.px[v][i] - (g[i] - g[i - 1]) : T(0);
        ppy[i] = yo(i) ? A.py[v][i] - (g[i] - g[i - VX]) : T(0);
        ppz[i] = zo(i) ? A.pz[v][i] - (g[i] - g[i - sxy]) : T(0);
      }
      for (long i = 0; i < V; ++i) {
        T up = ppx[i] * ppx[i];
        T dn = (xo(i) != VX - 1) ? ppx[i + 1] * ppx[i + 1] : T(0);
        T F = up + dn;
        up = ppy[i] * ppy[i];
        dn = (yo(i) != VY - 1) ? ppy[i + VX] * ppy[i + VX] : T(0);
        F += up + dn;
        up = ppz[i] * ppz[i];
        dn = (i + sxy < V) ? ppz[i + sxy] * ppz[i + sxy] : T(0);
        F += up + dn;
        Fm[i] = std::sqrt(T(0.5) * F);
        lim[i] = o.smooth[v] ? o.alpha[v] * T(o.smooth[v][i]) : o.alpha[v];
        m[i] = (Fm[i] > lim[i]) ? lim[i] / Fm[i] : T(1);
      }
      // total adjoint of the new flows P: incoming plus through div'
      std::vector<T> tx(V), ty(V), tz(V);
      for (long i = 0; i < V; ++i) {
        tx[i] = Pbx[v][i] + dbp[v][i] - (xo(i) ? dbp[v][i - 1] : T(0));
        ty[i] = Pby[v][i] + dbp[v][i] - (yo(i) ? dbp[v][i - VX] : T(0));
        tz[i] = Pbz[v][i] + dbp[v][i] - (zo(i) ? dbp[v][i - sxy] : T(0));
      }
      std::vector<T> F2b(V, T(0));
      double asum = 0.0;
      for (long i = 0; i < V; ++i) {
        T mb = T(0);
        if (xo(i)) mb += tx[i] * T(0.5) * ppx[i];
        if (xo(i) != VX - 1) mb += tx[i + 1] * T(0.5) * ppx[i + 1];
        if (yo(i)) mb += ty[i] * T(0.5) * ppy[i];
        if (yo(i) != VY - 1) mb += ty[i + VX] * T(0.5) * ppy[i + VX];
        if (zo(i)) mb += tz[i] * T(0.5) * ppz[i];
        if (i + sxy < V) mb += tz[i + sxy] * T(0.5) * ppz[i + sxy];
        if (Fm[i] > lim[i]) {
          F2b[i] = -mb * lim[i] / (T(4) * Fm[i] * Fm[i] * Fm[i]);
          asum += (double)(mb / Fm[i] * (o.smooth[v] ? T(o.smooth[v][i]) : T(1)));
        }
      }
      ab[v] += asum;
      std::vector<T> qx(V), qy(V), qz(V);  // adjoint of p'
      for (long i = 0; i < V; ++i) {
        qx[i] = xo(i) ? tx[i] * T(0.5) * (m[i] + m[i - 1]) + T(2) * ppx[i] * (F2b[i] + F2b[i - 1]) : T(0);
        qy[i] = yo(i) ? ty[i] * T(0.5) * (m[i] + m[i - VX]) + T(2) * ppy[i] * (F2b[i] + F2b[i - VX]) : T(0);
        qz[i] = zo(i) ? tz[i] * T(0.5) * (m[i] + m[i - sxy]) + T(2) * ppz[i] * (F2b[i] + F2b[i - sxy]) : T(0);
      }
      std::vector<T> dbo(V);
      for (long i = 0; i < V; ++i) {
        T gb = -(qx[i] + qy[i] + qz[i]);
        if (xo(i) != VX - 1) gb += qx[i + 1];
        if (yo(i) != VY - 1) gb += qy[i + VX];
        if (i + sxy < V) gb += qz[i + sxy];
        sbo[v][i] += tau * gb;
        ubo[v][i] -= tau * icc * gb;
        sbo[p][i] -= tau * gb;
        dbo[i] = tau * gb;
      }
      for (long i = 0; i < V; ++i) {
        Pbx[v][i] = qx[i] + dbo[i] - (xo(i) ? dbo[i - 1] : T(0));
        Pby[v][i] = qy[i] + dbo[i] - (yo(i) ? dbo[i - VX] : T(0));
        Pbz[v][i] = qz[i] + dbo[i] - (zo(i) ? dbo[i - sxy] : T(0));
      }
    }
    sbn = sbo;
    ubn = ubo;
  }
};

template <class T>
int run_adjoint(const Problem& P, const Tree& t, const int* truth, double eps, double* loss_out,
                double* dD_out /* [n][V] */, double* dalpha_out /* [n] */, double* u_out) {
  CudaOracle<T> o(t, P.vx, P.vy, P.vz);
  o.alloc();
  o.data.assign(t.n, nullptr);
  o.smooth.assign(t.n, nullptr);
  o.alpha.assign(t.n, T(1));
  for (int v = 0; v < t.n; ++v) {
    o.data[v] = P.data ? P.data[v] : nullptr;
    o.smooth[v] = P.smooth ? P.smooth[v] : nullptr;
    o.alpha[v] = P.alpha ? T((float)P.alpha[v]) : T(1);
  }
  for (int v = 0; v < t.n; ++v) if (t.leaf(v) && !o.data[v]) { g_err = "missing data term for a leaf"; return -3; }
  if (sizeof(T) == sizeof(float)) {
    o.step = T(P.step); o.cc = T(P.cc); o.icc = T(1.0f / P.cc); o.root_work = T(1.0f / P.cc);
  } else {
    o.step = T(P.step); o.cc = T(P.cc); o.icc = T(1) / T(P.cc); o.root_work = T(1) / T(P.cc);
  }
  o.init();
  AdjointRun<T> A(t, o);
  A.states.push_back(A.snap());
  for (int it = 0; it < P.iterations; ++it) {
    o.solve(t.root);
    A.states.push_back(A.snap());
  }
  const long V = o.V;
  std::vector<int> leaves;
  for (int v : t.preorder) if (t.leaf(v)) leaves.push_back(v);
  // loss and its gradient on the final leaf labels
  const int n = t.n;
  std::vector<std::vector<T>> Pbx(n, std::vector<T>(V, T(0))), Pby = Pbx, Pbz = Pbx, sbn = Pbx, ubn = Pbx;
  double loss = 0.0;
  const auto& U = A.states.back().u;
  for (long i = 0; i < V; ++i) {
    const int cls = truth[i];
    if (cls < 0 || cls >= (int)leaves.size()) { g_err = "truth class out of range"; return -1; }
    const int l = leaves[cls];
    const T uv = U[l][i];
    const T ue = uv > T(eps) ? uv : T(eps);
    loss -= std::log((double)ue) / (double)V;
    if (uv > T(eps)) ubn[l][i] = T(-1.0 / ((double)V * (double)uv));
  }
  std::vector<std::vector<double>> Db(n, std::vector<double>(V, 0.0));
  std::vector<double> ab(n, 0.0);
  for (int it = P.iterations - 1; it >= 0; --it) A.backward_step(it, Pbx, Pby, Pbz, sbn, ubn, Db, ab);
  // initial sinks = min over leaves (kern_MinBuffers keeps the last of a tie)
  for (long i = 0; i < V; ++i) {
    int arg = leaves[0];
    float mv = o.data[leaves[0]][i];
    for (size_t k = 1; k < leaves.size(); ++k) {
      const float d = o.data[leaves[k]][i];
      if (!(mv < d)) { mv = d; arg = leaves[k]; }
    }
    double tot = 0.0;
    for (int v = 0; v < n; ++v) tot += (double)sbn[v][i];
    Db[arg][i] += tot;
  }
  if (loss_out) *loss_out = loss;
  for (int v = 0; v < n; ++v) {
    if (dalpha_out) dalpha_out[v] = ab[v];
    for (long i = 0; i < V; ++i) {
      if (dD_out) dD_out[(long)v * V + i] = Db[v][i];
      if (u_out) u_out[(long)v * V + i] = (v == t.root) ? 0.0 : (double)U[v][i];
    }
  }
  return 0;
}

}  // namespace

extern "C" {

// semantics: 0 = REF_CUDA, 1 = REF_CPU.  precision: 32 or 64 (REF_CUDA only).
// Outputs (each [n_nodes * V] doubles, row v = vertex v, may be NULL):
//   u_out labels (root row 0), sink_out sinks (root row = source flow),
//   div_out divergence buffers (root row 0).
// Returns 0 on success, a negative code on error (oracle_last_error()).
#ifdef HMF_ORACLE_WITH_REFERENCE
#define ORACLE_ENTRY oracle_ref_hmf_solve
#else
#define ORACLE_ENTRY oracle_hmf_solve
#endif
int ORACLE_ENTRY(int semantics, int precision, int threads, int vx, int vy, int vz,
                 int n_nodes, const int* parent, const float* const* data,
                 const float* const* smooth, const double* alpha, int iterations,
                 float step, float cc, double* u_out, double* sink_out, double* div_out) {
  g_err.clear();
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  if (vx <= 0 || vy <= 0 || vz <= 0) { g_err = "bad dimensions"; return -1; }
  if ((long)vx * vy * vz > 0x7fffffffL) { g_err = "volume too large for the oracle"; return -1; }
  Tree t;
  if (!t.build(n_nodes, parent)) return -2;
  Problem P{vx, vy, vz, n_nodes, parent, data, smooth, alpha, iterations, step, cc};
#ifdef HMF_ORACLE_WITH_REFERENCE
  if (semantics != 1) { g_err = "the reference build only restates REF_CPU"; return -4; }
  (void)precision;
  return run_cpu_semantics<RefUtils>(P, t, u_out, sink_out, div_out);
#else
  if (semantics == 1) return run_cpu_semantics<PortUtils>(P, t, u_out, sink_out, div_out);
  if (semantics != 0) { g_err = "unknown semantics"; return -4; }
  if (precision == 64) return run_cuda_semantics<double>(P, t, u_out, sink_out, div_out);
  return run_cuda_semantics<float>(P, t, u_out, sink_out, div_out);
#endif
}

#ifndef HMF_ORACLE_WITH_REFERENCE
// REF_CUDA in FP32 from a given state: `iterations` iterations of the
// restatement above (after its initialisation from the data terms when init
// != 0) on the per-vertex state arrays [n_nodes * V] -- flows, divergence and
// labels of the non-root vertices, the sinks of all (root: source flow) --
// read and updated in place.  The building block of the slab simulation of a
// sharded solve (each rank iterates its slab plus halo planes).
int oracle_hmf_iterate(int threads, int vx, int vy, int vz, int n_nodes, const int* parent,
                       const float* const* data, const float* const* smooth, const double* alpha, int init,
                       int iterations, float step, float cc, float* fx, float* fy, float* fz, float* div,
                       float* u, float* sink) {
  g_err.clear();
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  if (vx <= 0 || vy <= 0 || vz <= 0) { g_err = "bad dimensions"; return -1; }
  if ((long)vx * vy * vz > 0x7fffffffL) { g_err = "volume too large for the oracle"; return -1; }
  Tree t;
  if (!t.build(n_nodes, parent)) return -2;
  CudaOracle<float> o(t, vx, vy, vz);
  o.alloc();
  o.data.assign(t.n, nullptr);
  o.smooth.assign(t.n, nullptr);
  o.alpha.assign(t.n, 1.0f);
  for (int v = 0; v < t.n; ++v) {
    o.data[v] = data ? data[v] : nullptr;
    o.smooth[v] = smooth ? smooth[v] : nullptr;
    o.alpha[v] = alpha ? (float)alpha[v] : 1.0f;
  }
  for (int v = 0; v < t.n; ++v) if (t.leaf(v) && !o.data[v]) { g_err = "missing data term for a leaf"; return -3; }
  o.step = step;
  o.cc = cc;
  o.icc = 1.0f / cc;
  o.root_work = 1.0f / cc;
  const long V = o.V;
  if (init) {
    o.init();
  } else {
    for (int v = 0; v < t.n; ++v) {
      std::copy(sink + (long)v * V, sink + (long)(v + 1) * V, o.sink[v].begin());
      if (v == t.root) continue;
      std::copy(fx + (long)v * V, fx + (long)(v + 1) * V, o.fx[v].begin());
      std::copy(fy + (long)v * V, fy + (long)(v + 1) * V, o.fy[v].begin());
      std::copy(fz + (long)v * V, fz + (long)(v + 1) * V, o.fz[v].begin());
      std::copy(div + (long)v * V, div + (long)(v + 1) * V, o.div[v].begin());
      std::copy(u + (long)v * V, u + (long)(v + 1) * V, o.u[v].begin());
    }
  }
  for (int it = 0; it < iterations; ++it) o.solve(t.root);
  for (int v = 0; v < t.n; ++v) {
    std::copy(o.sink[v].begin(), o.sink[v].end(), sink + (long)v * V);
    if (v == t.root) continue;
    std::copy(o.fx[v].begin(), o.fx[v].end(), fx + (long)v * V);
    std::copy(o.fy[v].begin(), o.fy[v].end(), fy + (long)v * V);
    std::copy(o.fz[v].begin(), o.fz[v].end(), fz + (long)v * V);
    std::copy(o.div[v].begin(), o.div[v].end(), div + (long)v * V);
    std::copy(o.u[v].begin(), o.u[v].end(), u + (long)v * V);
  }
  return 0;
}

// Label vote over n_inputs float images of n voxels (the step after the
// solve that turns label probabilities into one label per voxel).
// semantics 0 = vtkCudaImageVote: the running maximum starts at input 0 and
// each input k in port order replaces it when value >= maximum
// (CUDA_imagevote.cu:30-46, launched per input :249-256), so the last of a
// tie wins.  semantics 1 = vtkImageVote (CPU, vtkImageVote.cxx:285-306): the
// first input, then any strictly greater one, wins; no input -> 0.
int oracle_vote(int semantics, int n_inputs, const float* const* inputs, const int* values, long long n, int* out) {
  g_err.clear();
  if (n_inputs < 1) { g_err = "the vote needs at least one input"; return -1; }
  for (long long i = 0; i < n; ++i) {
    if (semantics == 0) {
      float mx = inputs[0][i];
      int id = values[0];
      for (int k = 0; k < n_inputs; ++k) {
        const float v = inputs[k][i];
        if (v >= mx) { id = values[k]; mx = v; }
      }
      out[i] = id;
    } else {
      int id = -1;
      float mx = 0.0f;
      for (int k = 0; k < n_inputs; ++k)
        if (id == -1 || inputs[k][i] > mx) { id = values[k]; mx = inputs[k][i]; }
      out[i] = id == -1 ? 0 : id;
    }
  }
  return 0;
}

// Energy decomposition of a labelling (vtkCudaHierarchicalMaxFlowDecomposition,
// .cxx:640-806, kernels CUDA_hierarchicalmaxflowdecomp.cu:19-279).
//   f0   = sum over leaves and voxels of D_l * u_l            (:670, :40-86)
//   f[v] = sum over voxels of S_v * g_v for every non-root vertex, where
//          g = 0.5f * sqrtf(fma(dZ, dZ, fma(dY, dY, fma(dX, dX, 0)))) (the
//          reference kernel as nvcc contracts it) with central
//          differences clamped at the volume border (:19-38) and S_v = 1
//          without a smoothness image; a branch's labelling is the sum of its
//          children's, added in child order (:750-806).
// Per-voxel terms in FP32 as the reference kernels form them; the sums over
// voxels in FP64 (the reference reduces in FP32).  terms_out (optional,
// [n][V]): the per-voxel terms S_v*g_v.
int oracle_energy(int vx, int vy, int vz, int n_nodes, const int* parent, const float* const* data,
                  const float* const* labels, const float* const* smooth, double* f0_out, double* f_out,
                  float* terms_out) {
  g_err.clear();
  if (vx <= 0 || vy <= 0 || vz <= 0) { g_err = "bad dimensions"; return -1; }
  Tree t;
  if (!t.build(n_nodes, parent)) return -2;
  const long V = (long)vx * vy * vz;
  for (int v = 0; v < n_nodes; ++v)
    if (t.leaf(v) && (!data || !data[v] || !labels || !labels[v])) { g_err = "missing leaf data or label"; return -3; }
  // labellings of every non-root vertex: leaves as given, branches summed
  std::vector<std::vector<float>> u(n_nodes);
  std::vector<int> post;
  {
    std::vector<std::pair<int, int>> st{{t.root, 0}};
    while (!st.empty()) {
      auto& top = st.back();
      if (top.second < (int)t.kids[top.first].size()) {
        const int k = t.kids[top.first][top.second++];
        st.push_back({k, 0});
      } else {
        post.push_back(top.first);
        st.pop_back();
      }
    }
  }
  for (int v : post) {
    if (v == t.root) continue;
    if (t.leaf(v)) {
      u[v].assign(labels[v], labels[v] + V);
    } else {
      u[v].assign(V, 0.0f);
      for (int k : t.kids[v])
        for (long i = 0; i < V; ++i) u[v][i] = u[v][i] + u[k][i];
    }
  }
  double f0 = 0.0;
  for (int v : t.preorder)
    if (t.leaf(v))
      for (long i = 0; i < V; ++i) f0 += (double)(data[v][i] * u[v][i]);
  const long sxy = (long)vx * vy;
  for (int v = 0; v < n_nodes; ++v) {
    double fv = 0.0;
    if (v != t.root) {
      const std::vector<float>& b = u[v];
      for (long i = 0; i < V; ++i) {
        const int x = (int)(i % vx), y = (int)((i / vx) % vy), z = (int)(i / sxy);
        const float cur = b[i];
        // the reference kernel is compiled with multiply-add contraction:
        // each `g += d*d` is one fused multiply-add
        float g2 = 0.0f;
        const float xh = x == vx - 1 ? cur : b[i + 1], xl = x == 0 ? cur : b[i - 1];
        g2 = std::fma(xh - xl, xh - xl, g2);
        const float yh = y == vy - 1 ? cur : b[i + vx], yl = y == 0 ? cur : b[i - vx];
        g2 = std::fma(yh - yl, yh - yl, g2);
        const float zh = z == vz - 1 ? cur : b[i + sxy], zl = z == 0 ? cur : b[i - sxy];
        g2 = std::fma(zh - zl, zh - zl, g2);
        float term = 0.5f * std::sqrt(g2);
        if (smooth && smooth[v]) term = smooth[v][i] * term;
        if (terms_out) terms_out[(long)v * V + i] = term;
        fv += (double)term;
      }
    }
    if (f_out) f_out[v] = fv;
  }
  if (f0_out) *f0_out = f0;
  return 0;
}

// Loss and gradients of the REF_CUDA solve (see AdjointRun).  truth: class
// per voxel = index into the DFS pre-order leaf list.  dD_out [n_nodes * V]
// (leaf rows filled), dalpha_out [n_nodes], u_out [n_nodes * V] final labels.
int oracle_hmf_adjoint(int precision, int threads, int vx, int vy, int vz, int n_nodes, const int* parent,
                       const float* const* data, const float* const* smooth, const double* alpha,
                       int iterations, float step, float cc, const int* truth, double eps,
                       double* loss_out, double* dD_out, double* dalpha_out, double* u_out) {
  g_err.clear();
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  if (vx <= 0 || vy <= 0 || vz <= 0) { g_err = "bad dimensions"; return -1; }
  Tree t;
  if (!t.build(n_nodes, parent)) return -2;
  Problem P{vx, vy, vz, n_nodes, parent, data, smooth, alpha, iterations, step, cc};
  if (precision == 64) return run_adjoint<double>(P, t, truth, eps, loss_out, dD_out, dalpha_out, u_out);
  return run_adjoint<float>(P, t, truth, eps, loss_out, dD_out, dalpha_out, u_out);
}
#endif

const char* oracle_last_error(void) { return g_err.c_str(); }

}  // extern "C"
