// hmf_ctx.hpp -- the solver context behind the opaque hmf_ctx handle of
// include/hmf.h, and the forward-solve helpers that the translation units of
// the library share (hmf_capi.cu defines them; hmf_adjoint.cu reuses them).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/hmf.h"
#include "hmf_types.cuh"

struct hmf_ctx {
  int device = 0;
  int semantics = HMF_SEMANTICS_REF_CUDA;
  int sm_count = 0;

  // volumes, back to back in every per-vertex array
  struct Volume {
    int vx, vy, vz, pitch;
    long long plane, vol, off;  // elements: plane, whole block, offset of the block
  };
  std::vector<Volume> vols;
  long long total = 0;
  hmf::Geometry geo{};  // per-voxel view of the concatenation (pitch 0 for batches)

  // tree
  int n = 0, root = -1;
  std::vector<int> parent;
  std::vector<std::vector<int>> kids;
  std::vector<int> preorder, postorder, leaves;  // leaves in DFS pre-order

  // directed acyclic graph (hmf_create_dag): edges in edge order; kids, leaves
  // and preorder above then hold out-edge children, leaves and nodes in the
  // rooted DAG's forward-iterator order, parent the first parent
  bool dag = false;
  std::vector<int> e_parent, e_child;
  std::vector<float> e_weight;
  bool e_weighted = false;
  std::vector<std::vector<int>> in_e, out_e;
  std::vector<float> n_parents, wkids;  // weighted parent count, weighted children

  // parameters (vtkHierarchicalMaxFlowSegmentation.cxx:57-59)
  int iterations = 100;
  float step = 0.1f;
  float cc = 0.25f;
  std::vector<double> alpha;

  struct Input {
    const float* ptr = nullptr;
    int where = HMF_HOST;
  };
  std::vector<std::vector<Input>> data, smooth;  // [volume][vertex]

  // device state
  char* arena = nullptr;
  size_t arena_bytes = 0;
  std::vector<float*> sink, label, div;
  std::vector<float*> fx[2], fy[2], fz[2];
  std::vector<float*> inc;  // DAG: each non-root node's own source buffer
  // input staging
  char* staging = nullptr;
  size_t staging_bytes = 0;
  hmf::FlowVertex* d_flow[2] = {nullptr, nullptr};  // shared-memory ring flow kernel (one volume)
  hmf::FlowVertexTMA* d_tma = nullptr;              // TMA flow kernel, [volume][non-root vertex]
  hmf::FlowVolume* d_fvol = nullptr;
  hmf::FlowItem* d_items = nullptr;
  int n_items = 0;
  int zchunk = 0;  // planes per window column (0: not planned yet)
  int flow_warps = 8;  // flow_tma_kernel<W>: windows of 32 x 4W (hmf_set_flow_window)
  int flow_units = 1;  // flow_tma_kernel: (window, vertex) units marched by one CTA (hmf_set_flow_units)
  hmf::TreeTable* d_tree = nullptr;
  hmf::DagTable* d_dag = nullptr;
  bool dag_last = false;  // the next sweep is the last iteration's
  bool dag_simple = false;   // dag_sweep_kernel (HMF_DAG_KERNEL=simple)
  bool dag_generic = false;  // dag_bulk_kernel even for small graphs (HMF_DAG_KERNEL=generic)
  bool use_tma = true;  // flow_tma_kernel (else the shared-memory ring flow_kernel)
  int tree_kind = 0;    // 0 tree_bulk_kernel, 1 tree4_kernel, 2 tree_kernel
  const float** d_smooth_list = nullptr;
  int* d_error = nullptr;
  int* h_error = nullptr;  // pinned copy of *d_error read with host outputs (allocated at first use)
  int n_smooth_list = 0;

  cudaStream_t stream = nullptr;
  cudaEvent_t ev_join = nullptr;
  cudaEvent_t ev_t0 = nullptr, ev_t1 = nullptr;
  cudaGraphExec_t graph_pair = nullptr;  // two iterations (both flow parities)
  cudaGraphExec_t graph_one = nullptr;   // one iteration, parity 0
  cudaGraphExec_t graph_many = nullptr;  // pipelined solves: several iterations per replay

  // z-slab pipeline of the replayed iterations (hmf_set_pipeline)
  bool pipeline = true;
  int n_slabs = 0;         // segments: z slabs of a single volume, or groups of a batch's volumes
  int seg_neighbours = 1;  // slabs wait for the neighbouring slabs (1), volume groups for none (0)
  std::vector<int> seg_first_item, seg_items;  // flow work items of each segment
  std::vector<long long> seg_base;             // first element of each segment
  std::vector<hmf::Geometry> slab_geo;         // each segment's elements (vol = their count)
  std::vector<hmf::TreeTable> h_tree_slabs;
  hmf::TreeTable* d_tree_slabs = nullptr;
  std::vector<cudaStream_t> slab_streams;
  std::vector<cudaEvent_t> slab_ev_flow, slab_ev_sweep;

  // failure-path controls (hmf_set_wait_limit, hmf_inject_wait_stall)
  unsigned long long wait_limit_ns = hmf::kTmaWaitLimitNs;
  int stall_kind = -1;  // HMF_STALL_* of the next launch of that kind that is to stall (-1: none)

  // convergence log (hmf_set_convergence_log): per iteration max and sum of |u_new - u_old|
  bool gap_on = false;
  char* d_gap = nullptr;  // counter[2], max bits[gap_cap], sums[gap_cap]
  int gap_cap = 0;
  int gap_logged = 0;     // iterations logged by the last solve
  int gap_t = 0;          // iteration (within the graph being captured) of the sweep launched next

  bool timing = false;
  long long launches = 0;
  double kind_ms[3] = {0, 0, 0};
  long long kind_count[3] = {0, 0, 0};
  bool solved = false;
  int flow_parity = 0;       // the flow set holding the current flows (after the last solve or continuation)
  bool continuable = false;  // the arrays hold the state the last solve ended in

  // host copies of the device tables (kept per context: pageable-memory
  // cudaMemcpyAsync stages them before returning)
  std::vector<hmf::FlowVertex> h_flow;
  std::vector<hmf::FlowVertexTMA> h_tma;
  std::vector<hmf::FlowVolume> h_fvol;
  std::vector<hmf::FlowItem> h_items;
  hmf::TreeTable h_tree{};
  hmf::DagTable h_dag{};
  hmf::DagRegParams h_dagreg{};
  bool dag_reg_ok = false;  // h_dagreg describes the graph (<= 8 nodes, no repeated edge)
  std::vector<const float*> h_smooth_list;

  // the staged inputs of the last solve (per vertex; for hmf_get_energy)
  std::vector<const float*> st_data, st_smooth;
  char* d_post = nullptr;  // hmf_get_energy's table and sums (hmf_post.cu), made on first use

  // reverse-mode state of hmf_solve_adjoint (hmf_adjoint.cu), created on demand
  struct AdjointState* adj = nullptr;
  // FP64 evaluation of the same iteration (hmf_fp64.cu), created on demand
  struct Fp64State* f64 = nullptr;
  // out-of-core solve (hmf_create_paged, hmf_paged.cu): the state lives in
  // pinned host memory and blocks of planes are iterated on the device; such
  // a context holds no device state of its own (arena == nullptr)
  struct PagedState* pg = nullptr;

  long long adj_max_bytes = 0;  // hmf_set_adjoint_memory (0: 85% of the free device memory)
  int adj_max_slots = 0;        // (0: no cap)

  std::string err;
};

namespace hmfi {

int fail(hmf_ctx* c, int code, const std::string& msg);
int cuda_fail(hmf_ctx* c, cudaError_t e, const char* what);

// A buffer passed as HMF_DEVICE is read or written by kernels and device
// copies, so it must be device memory of the current device or managed
// memory.  device_pointer_problem returns "" when `p` (non-null) qualifies,
// else the reason; check_device_pointer turns that into an error status, so
// that a host buffer labelled as device memory is refused before any kernel
// dereferences it.
std::string device_pointer_problem(const void* p);
int check_device_pointer(hmf_ctx* c, const void* p, const char* what);

#define CK(call, what)                                  \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, what); \
  } while (0)

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int d) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != d) cudaSetDevice(d);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

inline size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Inputs as device arrays over the concatenation of the volumes.
struct Staged {
  std::vector<const float*> data;      // [vertex], leaves only
  std::vector<const float*> smooth;    // [vertex], base of its smoothness group (or null)
  std::vector<const float*> distinct;  // bases of the smoothness groups
};

// Device arrays of the inputs over the concatenation of the volumes (host
// inputs and unaligned or pitched device inputs copied into staging arrays),
// queued on `s`.
int stage_inputs(hmf_ctx* c, cudaStream_t s, Staged& out);
// Joins the caller's stream, stages the inputs, writes the kernel tables,
// zeroes the parity-0 flows and runs the initialisation kernel on c->stream.
int begin_solve(hmf_ctx* c, cudaStream_t user, Staged& staged);
// Hands c->stream's work back to the caller's stream.
int end_solve(hmf_ctx* c, cudaStream_t user);
// One flow launch (reads flow set `parity`, writes the other) and one sweep.
int launch_flow(hmf_ctx* c, int parity, cudaStream_t s);
int launch_tree(hmf_ctx* c, cudaStream_t s);
// The TMA flow kernel and the bulk sweep over caller-built tables.
int launch_flow_tma_with(hmf_ctx* c, const hmf::FlowVertexTMA* table, int parity, cudaStream_t s);
int launch_flow_tma_items(hmf_ctx* c, const hmf::FlowVertexTMA* table, int parity, int first_item, int n_items,
                          cudaStream_t s);
int launch_tree_bulk_with(hmf_ctx* c, const hmf::TreeTable* table, cudaStream_t s, bool gap_log = false,
                          int gap_t = 0);
// Tensor map of one pitched volume block; box = kTmaBoxX columns x `rows`
// rows (0: the rows of the context's flow window).
int encode_plane_map(hmf_ctx* c, CUtensorMap* m, const float* base, const hmf_ctx::Volume& V, int rows = 0);
bool valid_vertex(const hmf_ctx* c, int v);
bool valid_volume(const hmf_ctx* c, int b);
// When c->stall_kind == kind: queue on `s` the request that makes the next
// copy-pipeline kernel stall once (its bounded wait runs out), and clear it.
int maybe_request_stall(hmf_ctx* c, int kind, cudaStream_t s);
// Error flag set by the kernels (bit 0 negative input, 1 wait time-out,
// 2 misaligned staging, 3 label index out of range), as a status.
int check_error_flag(hmf_ctx* c);
int decode_error_flag(hmf_ctx* c, int flag);

// hmf_solve's body: stage the inputs, write the tables, then either
// initialise (load == nullptr) or call load(c, c->stream, arg), which must
// fill every array the iterations read (sinks, labels, divergences and the
// parity-0 flows), and run c->iterations iterations.
using StateLoader = int (*)(hmf_ctx* c, cudaStream_t s, void* arg);
int solve_with(hmf_ctx* c, cudaStream_t user, StateLoader load, void* arg);
// Calls that need the device state of an in-core context refuse
// out-of-core contexts.
inline int refuse_paged(hmf_ctx* c, const char* what) {
  if (!c || !c->pg) return HMF_OK;
  return fail(c, HMF_ERR_STATE, std::string(what) + " is not available on an out-of-core context (hmf_create_paged)");
}

// hmf_paged.cu
int paged_setup(hmf_ctx* c, double max_gpu_usage);
int paged_solve(hmf_ctx* c, cudaStream_t user, bool cont = false);
int paged_copy_out(hmf_ctx* c, bool labels, int node, float* out, int where, void* stream);
void paged_free(hmf_ctx* c);
size_t paged_bytes(const hmf_ctx* c);

// hmf_adjoint.cu
void adjoint_free(hmf_ctx* c);
size_t adjoint_bytes(const hmf_ctx* c);
// hmf_fp64.cu
void fp64_free(hmf_ctx* c);
size_t fp64_bytes(const hmf_ctx* c);

}  // namespace hmfi
