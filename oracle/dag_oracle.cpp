// dag_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the oracle).
//
// CPU restatement of the RobartsVTK directed-acyclic-graph max-flow solver
// (DAGMF) as vtkCudaDirectedAcyclicGraphMaxFlowSegmentation runs it, used
// solely as the checker for the CUDA implementation in robartsvtk_gb300/.
// Nothing in the product links, loads or calls this file.
//
// The reference class expresses one iteration as a task graph
// (ImageProcessing/vtkCudaImageAnalytics/vtkCudaDirectedAcyclicGraphMaxFlowSegmentation.cxx:343-842)
// whose tasks run the kernels of CUDA_hierarchicalmaxflow.cu and
// CUDA_commonKernels.cu (vtkCudaMaxFlowSegmentationTask.cxx:309-492).  Its
// scheduler picks among ready tasks of equal cost with rand()
// (vtkCudaMaxFlowSegmentationScheduler.cxx:232-236), so the reference fixes
// neither the order of the weighted accumulations into a sink or a source
// buffer nor whether a branch pushes its potential up before or after its
// own label update.  This restatement runs the task graph in one fixed
// topological order, the one the product implements:
//
//   per iteration t = 1..T
//   (1) every non-root n: the spatial flow step of CUDA_hierarchicalmaxflow.cu
//       :233-456 with inc = n's own source buffer;
//   (2) leaves: s = clamp(inc - div + u/CC, 0, D) (kern_FindLeafSinkPotential
//       :166, kern_ApplyCapacity :187), then u = sat(u + CC(inc - div - s))
//       (kern_UpdateLabel :211); branches: s = (1-k) s + k (inc - div + u/CC),
//       k = 1/(weighted children + 1) (kern_ResetSinkBuffer :610); the root:
//       s = 1*s + 1/(CC * weighted children) (TranslateBuffer,
//       CUDA_commonKernels.cu:96);
//   and for t < T only:
//   (3) nodes in backward-iterator order (deepest level first), each in-edge
//       (parent p) in edge order: s_p += w (s - inc + div - u/CC)
//       (kern_PushUpSourceFlows :631), w = edge weight (else 1/#parents)
//       divided by the parent's weighted children (+1 for a branch); then a
//       branch's label update (kern_UpdateLabel);
//   (4) every non-root c: inc = 0, then per in-edge in edge order
//       inc = inc + w s_p (SumScaledBuffers, CUDA_commonKernels.cu:419), w =
//       edge weight (else 1/#parents).
//   Initialisation (vtkCudaDirectedAcyclicGraphMaxFlowSegmentation.cxx:844-1045):
//   flows and divergences 0; source = min over leaves of D (kern_MinBuffers,
//   leaves in forward order); every sink and source buffer = that minimum
//   (kern_Copy2Buffers); leaf labels [s == D] / sum (kern_Lbl, SumBuffers,
//   kern_DivideBuffers); branch labels, deepest first, 0 + sum over out-edges
//   of w u_child (SumScaledBuffers, w as in (4)).
//   Weighted children of v: sum over out-edges of (w / #parents(child))^2 with
//   #parents the sum of in-edge weights (vtkDirectedAcyclicGraphMaxFlowSegmentation.cxx:928-995).
//   A vertex without AddSmoothnessScalar gets alpha 0: the class reads its
//   scalar map with operator[] (vtkCudaDirectedAcyclicGraphMaxFlowSegmentation.cxx:365).
//
// Templated on float / double (the FP32 oracle and the FP64 error statement);
// build with -ffp-contract=off.  The CPU class's own DAG loops are not
// restated: its dagmf_computeFlowMag reads VX floats past the end of the x
// flow on every call (vtkMaxFlowSegmentationUtilities.cxx:197-200), so its
// output depends on the host heap.
//
// Graph convention shared with the product: vertices 0..n-1; edges given as
// (parent, child, weight) in edge order; the children of a vertex are its
// out-edges in edge order, its parents its in-edges in edge order.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local std::string g_dag_err;

// vtkRootedDirectedAcyclicGraph (vtkRootedDirectedAcyclicGraph.cxx:145-243) and
// its forward iterator (vtkRootedDirectedAcyclicGraphForwardIterator.cxx:95-120).
struct Dag {
  int n = 0, root = -1;
  std::vector<int> ep, ec;
  std::vector<float> ew;
  bool weighted = false;
  std::vector<std::vector<int>> in_e, out_e;
  std::vector<int> level, forward;
  std::vector<float> n_parents, wkids;  // #parents (weighted), weighted children

  bool build(int n_nodes, int n_edges, const int* p, const int* c, const float* w) {
    n = n_nodes;
    if (n < 2 || n_edges < 1 || !p || !c) { g_dag_err = "the graph needs a root, a leaf and an edge"; return false; }
    ep.assign(p, p + n_edges);
    ec.assign(c, c + n_edges);
    weighted = w != nullptr;
    ew.assign(n_edges, 1.0f);
    if (w) ew.assign(w, w + n_edges);
    in_e.assign(n, {});
    out_e.assign(n, {});
    for (int e = 0; e < n_edges; ++e) {
      if (ep[e] < 0 || ep[e] >= n || ec[e] < 0 || ec[e] >= n || ep[e] == ec[e]) {
        g_dag_err = "edge vertex out of range";
        return false;
      }
      if (weighted && !(ew[e] > 0.0f)) { g_dag_err = "edge weights must be positive"; return false; }
      out_e[ep[e]].push_back(e);
      in_e[ec[e]].push_back(e);
    }
    for (int v = 0; v < n; ++v)
      if (in_e[v].empty()) {
        if (root >= 0) { g_dag_err = "the graph has more than one root"; return false; }
        root = v;
      }
    if (root < 0) { g_dag_err = "the graph has no root"; return false; }
    // longest path from the root (UpLevel) by Kahn's order
    std::vector<int> indeg(n), topo;
    for (int v = 0; v < n; ++v) indeg[v] = (int)in_e[v].size();
    level.assign(n, 0);
    topo.push_back(root);
    for (size_t i = 0; i < topo.size(); ++i) {
      const int v = topo[i];
      for (int e : out_e[v]) {
        const int k = ec[e];
        level[k] = std::max(level[k], level[v] + 1);
        if (--indeg[k] == 0) topo.push_back(k);
      }
    }
    if ((int)topo.size() != n) { g_dag_err = "the graph has a cycle or an unreachable vertex"; return false; }
    // forward iterator: breadth first, a child entered from a parent one level up
    std::vector<char> seen(n, 0);
    forward.clear();
    forward.push_back(root);
    seen[root] = 1;
    for (size_t i = 0; i < forward.size(); ++i) {
      const int v = forward[i];
      for (int e : out_e[v]) {
        const int k = ec[e];
        if (level[k] != level[v] + 1 || seen[k]) continue;
        seen[k] = 1;
        forward.push_back(k);
      }
    }
    n_parents.assign(n, 0.0f);
    for (int v = 0; v < n; ++v)
      for (int e : in_e[v]) n_parents[v] += weighted ? ew[e] : 1.0f;
    wkids.assign(n, 0.0f);
    for (int v = 0; v < n; ++v)
      for (int e : out_e[v]) {
        const float t = (float)((weighted ? (double)ew[e] : 1.0) / n_parents[ec[e]]);
        wkids[v] += t * t;
      }
    return true;
  }
  bool leaf(int v) const { return out_e[v].empty(); }
  // push-down / label weight of edge e (constant1 of the PushDownSinkFlows and
  // AccumulateLabelsWeighted tasks)
  float wdown(int e) const { return weighted ? ew[e] : (float)(1.0 / (double)in_e[ec[e]].size()); }
  // push-up weight (constant1 of the PushUpSourceFlows tasks)
  float wup(int e) const {
    float W = weighted ? ew[e] : (float)(1.0 / (double)in_e[ec[e]].size());
    return ep[e] == root ? W / wkids[root] : W / (wkids[ep[e]] + 1.0f);
  }
};

template <class T> inline T sat01(T x) {
  if (x != x) return T(0);
  return x < T(0) ? T(0) : (x > T(1) ? T(1) : x);
}

template <class T>
struct DagCuda {
  int VX, VY, VZ;
  long V;
  const Dag& g;
  std::vector<std::vector<T>> fx, fy, fz, div, sink, inc, u;
  std::vector<const float*> data, smooth;
  std::vector<T> alpha;
  T step, cc, icc;

  DagCuda(const Dag& d, int vx, int vy, int vz) : VX(vx), VY(vy), VZ(vz), g(d) { V = (long)vx * vy * vz; }

  void alloc() {
    const int n = g.n;
    fx.assign(n, {}); fy.assign(n, {}); fz.assign(n, {}); div.assign(n, {});
    sink.assign(n, {}); inc.assign(n, {}); u.assign(n, {});
    for (int v = 0; v < n; ++v) {
      sink[v].assign(V, T(0));
      if (v == g.root) continue;
      fx[v].assign(V, T(0)); fy[v].assign(V, T(0)); fz[v].assign(V, T(0));
      div[v].assign(V, T(0)); inc[v].assign(V, T(0)); u[v].assign(V, T(0));
    }
  }

  void init() {
    std::vector<int> leaves;
    for (int v : g.forward) if (g.leaf(v)) leaves.push_back(v);
    const long n = V;
    std::vector<T>& src = sink[g.root];
    {
      const float* d0 = data[leaves[0]];
      for (long i = 0; i < n; ++i) src[i] = T(d0[i]);
    }
    for (size_t k = 1; k < leaves.size(); ++k) {
      const float* dk = data[leaves[k]];
#pragma omp parallel for schedule(static)
      for (long i = 0; i < n; ++i) { T a = src[i], b = T(dk[i]); src[i] = (a < b) ? a : b; }
    }
    for (int v = 0; v < g.n; ++v) {
      if (v == g.root) continue;
      for (long i = 0; i < n; ++i) sink[v][i] = inc[v][i] = src[i];
    }
    std::vector<T> acc(n, T(0));
    for (int l : leaves) {
      const float* d = data[l];
      T* ul = u[l].data();
#pragma omp parallel for schedule(static)
      for (long i = 0; i < n; ++i) {
        ul[i] = (sink[l][i] == T(d[i])) ? T(1) : T(0);
        acc[i] = acc[i] + ul[i];
      }
    }
    for (int l : leaves) {
      T* ul = u[l].data();
#pragma omp parallel for schedule(static)
      for (long i = 0; i < n; ++i) ul[i] = ul[i] / acc[i];
    }
    for (int j = g.n - 1; j >= 0; --j) {
      const int b = g.forward[j];
      if (b == g.root || g.leaf(b)) continue;
      T* ub = u[b].data();
      std::fill(u[b].begin(), u[b].end(), T(0));
      for (int e : g.out_e[b]) {
        const T w = T(g.wdown(e));
        const T* uc = u[g.ec[e]].data();
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n; ++i) ub[i] = ub[i] + w * uc[i];
      }
    }
  }

  // the spatial flow step of CUDA_hierarchicalmaxflow.cu:233-456 (kern_CalcGradStep,
  // kern_DescentSpatialFlow, kern_ComputeFlowMag*, kern_Project, kern_Divergence)
  void flows(int v) {
    const long n = V, sxy = (long)VX * VY;
    T* d = div[v].data(); T* px = fx[v].data(); T* py = fy[v].data(); T* pz = fz[v].data();
    const T* s = sink[v].data(); const T* c = inc[v].data(); const T* uu = u[v].data();
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) d[i] = step * (((s[i] + d[i]) - c[i]) - uu[i] * icc);
    std::vector<T> gcopy(d, d + n);
    const T* gg = gcopy.data();
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
      const int x = (int)(i % VX), y = (int)((i / VX) % VY), z = (int)(i / sxy);
      T cur = gg[i];
      px[i] = x ? px[i] - (cur - gg[i - 1]) : T(0);
      py[i] = y ? py[i] - (cur - gg[i - VX]) : T(0);
      pz[i] = z ? pz[i] - (cur - gg[i - sxy]) : T(0);
    }
    const float* S = smooth[v];
    const T a = alpha[v];
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
      d[i] = (F > sm) ? sm / F : T(1);
    }
    std::vector<T> mcopy(d, d + n);
    const T* m = mcopy.data();
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
      const int x = (int)(i % VX), y = (int)((i / VX) % VY), z = (int)(i / sxy);
      T cur = m[i];
      px[i] = x ? px[i] * T(0.5) * (cur + m[i - 1]) : T(0);
      py[i] = y ? py[i] * T(0.5) * (cur + m[i - VX]) : T(0);
      pz[i] = z ? pz[i] * T(0.5) * (cur + m[i - sxy]) : T(0);
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

  void iterate(bool last) {
    const long n = V;
    for (int v : g.forward) if (v != g.root) flows(v);
    // (2)
    const T shift = T((float)(1.0 / (double)(cc_f * g.wkids[g.root])));
    for (int v = 0; v < g.n; ++v) {
      T* s = sink[v].data();
      if (v == g.root) {
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n; ++i) s[i] = T(1) * s[i] + shift;
        continue;
      }
      const T* c = inc[v].data(); const T* d = div[v].data(); T* uu = u[v].data();
      if (g.leaf(v)) {
        const float* D = data[v];
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n; ++i) {
          T val = (c[i] - d[i]) + uu[i] * icc;
          const T cap = T(D[i]);
          val = (val < T(0)) ? T(0) : val;
          val = (val > cap) ? cap : val;
          s[i] = val;
          uu[i] = sat01(uu[i] + cc * ((c[i] - d[i]) - s[i]));
        }
      } else {
        const T k = T((float)(1.0 / ((double)g.wkids[v] + 1.0)));
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n; ++i) s[i] = (T(1) - k) * s[i] + k * ((c[i] - d[i]) + uu[i] * icc);
      }
    }
    if (last) return;
    // (3)
    for (int j = g.n - 1; j >= 0; --j) {
      const int v = g.forward[j];
      if (v == g.root) continue;
      const T* s = sink[v].data(); const T* c = inc[v].data(); const T* d = div[v].data(); T* uu = u[v].data();
      for (int e : g.in_e[v]) {
        T* ps = sink[g.ep[e]].data();
        const T w = T(g.wup(e));
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n; ++i) ps[i] = ps[i] + w * (((s[i] - c[i]) + d[i]) - uu[i] * icc);
      }
      if (!g.leaf(v)) {
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n; ++i) uu[i] = sat01(uu[i] + cc * ((c[i] - d[i]) - s[i]));
      }
    }
    // (4)
    for (int v = 0; v < g.n; ++v) {
      if (v == g.root) continue;
      T* c = inc[v].data();
      std::fill(inc[v].begin(), inc[v].end(), T(0));
      for (int e : g.in_e[v]) {
        const T w = T(g.wdown(e));
        const T* ps = sink[g.ep[e]].data();
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n; ++i) c[i] = c[i] + w * ps[i];
      }
    }
  }

  float cc_f = 0.25f;
};

template <class T>
int run_dag(const Dag& g, int vx, int vy, int vz, const float* const* data, const float* const* smooth,
            const double* alpha, int iterations, float step, float cc, double* u_out, double* sink_out,
            double* inc_out) {
  DagCuda<T> o(g, vx, vy, vz);
  o.data.assign(data, data + g.n);
  o.smooth.assign(g.n, nullptr);
  if (smooth) o.smooth.assign(smooth, smooth + g.n);
  o.alpha.assign(g.n, T(0));
  for (int v = 0; v < g.n; ++v) o.alpha[v] = (alpha && !std::isnan(alpha[v])) ? T((float)alpha[v]) : T(0);
  o.step = T(step);
  o.cc = T(cc);
  o.cc_f = cc;
  o.icc = T(1.0f / cc);
  for (int v = 0; v < g.n; ++v)
    if (g.leaf(v) && !o.data[v]) { g_dag_err = "missing data term for a leaf"; return -1; }
  o.alloc();
  o.init();
  for (int t = 0; t < iterations; ++t) o.iterate(t == iterations - 1);
  const long V = o.V;
  for (int v = 0; v < g.n; ++v) {
    for (long i = 0; i < V; ++i) {
      if (sink_out) sink_out[(size_t)v * V + i] = (double)o.sink[v][i];
      if (v == g.root) continue;
      if (u_out) u_out[(size_t)v * V + i] = (double)o.u[v][i];
      if (inc_out) inc_out[(size_t)v * V + i] = (double)o.inc[v][i];
    }
  }
  return 0;
}

}  // namespace

extern "C" {

// REF_CUDA DAGMF in the order above.  precision 32 or 64; alpha[v] NaN = not
// set (alpha 0).  u_out / sink_out / inc_out: n_nodes x V doubles (may be null).
int oracle_dag_solve(int precision, int threads, int vx, int vy, int vz, int n_nodes, int n_edges,
                     const int* edge_parent, const int* edge_child, const float* edge_weight,
                     const float* const* data, const float* const* smooth, const double* alpha, int iterations,
                     float step, float cc, double* u_out, double* sink_out, double* inc_out) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  Dag g;
  if (!g.build(n_nodes, n_edges, edge_parent, edge_child, edge_weight)) return -1;
  if (vx < 1 || vy < 1 || vz < 1) { g_dag_err = "bad volume size"; return -1; }
  if (precision == 64)
    return run_dag<double>(g, vx, vy, vz, data, smooth, alpha, iterations, step, cc, u_out, sink_out, inc_out);
  return run_dag<float>(g, vx, vy, vz, data, smooth, alpha, iterations, step, cc, u_out, sink_out, inc_out);
}

// The forward-iterator order of the graph (leaves in it are the output order).
int oracle_dag_forward(int n_nodes, int n_edges, const int* edge_parent, const int* edge_child,
                       const float* edge_weight, int* out) {
  Dag g;
  if (!g.build(n_nodes, n_edges, edge_parent, edge_child, edge_weight)) return -1;
  for (int i = 0; i < g.n; ++i) out[i] = g.forward[i];
  return 0;
}

const char* oracle_dag_last_error(void) { return g_dag_err.c_str(); }

}  // extern "C"
