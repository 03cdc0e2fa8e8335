/* hmf.h -- C ABI of the GB300 (sm_103a) hierarchical max-flow segmentation
 * library, libhmf_gb300.so.
 *
 * This is the drop-in boundary for the RobartsVTK HMF path.  The reference
 * reaches its GPU through free C functions on raw device buffers
 * (ImageProcessing/vtkCudaImageAnalytics/CUDA_hierarchicalmaxflow.h:17-50),
 * driven one full-volume pass at a time by
 * vtkCudaHierarchicalMaxFlowSegmentation::InitializeAlgorithm/RunAlgorithm
 * (vtkCudaHierarchicalMaxFlowSegmentation.cxx:478-716).  Here the whole solve
 * (initialisation plus every primal-dual iteration) is one call on an opaque
 * context, so that the iteration can be fused on the device.
 *
 * Conventions
 *  - Volumes are float32, x fastest, [VZ][VY][VX] (VTK scalar layout).
 *  - The label tree is a parent array: vertices 0..n-1, parent[v] == -1 for
 *    the single root; the children of a vertex are taken in increasing id
 *    order (the order vtkTree::AddChild assigns).  Leaves are the disjoint
 *    labels; every leaf needs a data term (cost), all values >= 0.
 *  - `where` says whether a pointer is host memory (HMF_HOST) or device
 *    memory of the context's GPU (HMF_DEVICE).  Input pointers are borrowed,
 *    as VTK borrows its input images: they must stay valid until the next
 *    hmf_solve() returns.  Host inputs are copied to the device inside
 *    hmf_solve(); device inputs are read in place.  A pointer passed as
 *    HMF_DEVICE that is not device memory of the GPU the call runs on (or
 *    managed memory) is refused with HMF_ERR_INVALID_ARGUMENT before any
 *    kernel or copy touches it.
 *  - `stream` is a cudaStream_t (NULL = the legacy default stream).  All work
 *    is ordered after the work already queued on it; calls return once the
 *    work is queued (hmf_get_labels to host memory returns after the copy).
 *  - Every call returns HMF_OK (0) or a negative HMF_ERR_* code; the message
 *    is available from hmf_last_error().  No call resets the device.
 *  - A context is not thread-safe; distinct contexts are independent.
 */
#ifndef HMF_GB300_H
#define HMF_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HMF_OK 0
#define HMF_ERR_INVALID_ARGUMENT -1
#define HMF_ERR_TREE -2
#define HMF_ERR_MISSING_INPUT -3
#define HMF_ERR_CUDA -4
#define HMF_ERR_OUT_OF_MEMORY -5
#define HMF_ERR_STATE -6

#define HMF_HOST 0
#define HMF_DEVICE 1

/* Which reference behaviour hmf_solve reproduces.
 *  REF_CUDA: vtkCudaHierarchicalMaxFlowSegmentation (the regularised
 *            primal-dual solver the reference runs on the GPU,
 *            CUDA_hierarchicalmaxflow.cu:124-456).
 *  REF_CPU:  vtkHierarchicalMaxFlowSegmentation's host code as written
 *            (vtkMaxFlowSegmentationUtilities.cxx:29-339): its spatial flows
 *            stay zero and branch sinks keep their initial value, so the
 *            solve reduces to a per-voxel leaf iteration. */
#define HMF_SEMANTICS_REF_CUDA 0
#define HMF_SEMANTICS_REF_CPU 1

typedef struct hmf_ctx hmf_ctx;

/* Create a solver for one volume size and one label tree on CUDA device
 * `device`.  Replaces the buffer planning of
 * vtkHierarchicalMaxFlowSegmentation::RequestData (.cxx:555-905) and the GPU
 * buffer acquisition of vtkCudaHierarchicalMaxFlowSegmentation::InitializeAlgorithm
 * (.cxx:513-538, CUDA_GetGPUBuffers CUDA_hierarchicalmaxflow.cu:33-60).
 * Device memory for the whole solver state is allocated here, once. */
int hmf_create(hmf_ctx** out, int vx, int vy, int vz, const int* parent, int n_nodes,
               int semantics, int device);

/* Create a solver for a directed acyclic graph of labels: the problem of
 * vtkCudaDirectedAcyclicGraphMaxFlowSegmentation (its InitializeAlgorithm /
 * RunAlgorithm, vtkCudaDirectedAcyclicGraphMaxFlowSegmentation.cxx:150-286,
 * over a vtkRootedDirectedAcyclicGraph).  Edge e runs from edge_parent[e] to
 * edge_child[e]; edge order is the graph's edge order (a vertex's children are
 * its out-edges in that order).  edge_weight: one positive weight per edge
 * (the graph's "Weights" edge array) or NULL for none.  The single vertex
 * without parents is the root; every vertex must be reachable from it and
 * the graph acyclic (<= 64 vertices, <= 256 edges).  semantics must be
 * HMF_SEMANTICS_REF_CUDA.  The reference's scheduler orders ready tasks at
 * random; this library runs its task graph in one fixed order (the order of
 * its weighted accumulations and, for a branch, its potential pushed up
 * before its label update).  A vertex without hmf_set_smoothness_scalar has
 * alpha 0, as the reference class reads its scalar map with operator[].
 * Leaves are numbered in the graph's forward-iterator order (hmf_leaf_order).
 * Every other call taking a context works on it, except the batch, adjoint
 * and energy calls. */
int hmf_create_dag(hmf_ctx** out, int vx, int vy, int vz, int n_nodes, int n_edges, const int* edge_parent,
                   const int* edge_child, const float* edge_weight, int semantics, int device);
int hmf_destroy(hmf_ctx* ctx);

/* Data term (cost) of a leaf.  Replaces SetDataInputDataObject(idx, image)
 * (vtkHierarchicalMaxFlowSegmentation.h:84-87). */
int hmf_set_data(hmf_ctx* ctx, int node, const float* data, int where);

/* Optional per-voxel smoothness image of a non-root vertex (NULL removes it;
 * without an image S(x) = 1).  Replaces SetSmoothnessInputDataObject
 * (vtkHierarchicalMaxFlowSegmentation.h:94-97).  Vertices may share one
 * image pointer; it is then read once per voxel. */
int hmf_set_smoothness(hmf_ctx* ctx, int node, const float* smooth, int where);

/* Smoothness weight alpha >= 0 of a non-root vertex (default 1).  Replaces
 * AddSmoothnessScalar(node, alpha) (vtkHierarchicalMaxFlowSegmentation.cxx:93-104);
 * unlike the reference's std::map::insert, a later call replaces the value. */
int hmf_set_smoothness_scalar(hmf_ctx* ctx, int node, double alpha);

/* NumberOfIterations (clamped to [0, INT_MAX]), StepSize and CC (each clamped
 * to [0, 1]) as vtkSetClampMacro does (vtkHierarchicalMaxFlowSegmentation.h:64-77).
 * Defaults 100, 0.1, 0.25 (.cxx:57-59). */
int hmf_set_params(hmf_ctx* ctx, int iterations, float step_size, float cc);

/* Initialise and run all iterations.  Replaces
 * vtkCudaHierarchicalMaxFlowSegmentation::InitializeAlgorithm + RunAlgorithm
 * (.cxx:478-716). */
int hmf_solve(hmf_ctx* ctx, void* stream);

/* Run NumberOfIterations more iterations from the state the last hmf_solve
 * or hmf_solve_continue ended in, without the initialisation: a solve of
 * k1 iterations continued by k2 gives bit-identically the solve of k1 + k2
 * (same inputs and parameters).  No counterpart in the reference, which
 * always starts from the initialisation (.cxx:478-716); with the convergence
 * log it lets a caller iterate in rounds and stop when the label change is
 * small.  Label-tree contexts (batches and out-of-core contexts included),
 * both semantics; refused with HMF_ERR_INVALID_ARGUMENT for graphs
 * (hmf_create_dag), and with HMF_ERR_STATE when the last call that wrote
 * the state was not a solve (hmf_solve_adjoint, hmf_autotune) or failed.  The inputs
 * are staged again, so data terms and smoothness may change between calls;
 * the FP64 evaluation and the adjoint always start from the initialisation. */
int hmf_solve_continue(hmf_ctx* ctx, void* stream);

/* Copy the labelling of a non-root vertex (the leaves are the reference's
 * outputs, GetOutputDataObject(idx), vtkHierarchicalMaxFlowSegmentation.cxx:337-346;
 * branch labellings are also available) to `out` (VX*VY*VZ floats). */
int hmf_get_labels(hmf_ctx* ctx, int node, float* out, int where, void* stream);

/* Same for the sink flow of a vertex (the root's is the source flow). */
int hmf_get_sink(hmf_ctx* ctx, int node, float* out, int where, void* stream);

/* Leaf order used by the reference for its output ports (DFS pre-order,
 * vtkHierarchicalMaxFlowSegmentation.cxx:383-398): writes up to `cap` vertex
 * ids, returns the number of leaves (or a negative error). */
int hmf_leaf_order(const hmf_ctx* ctx, int* out, int cap);

/* Bytes of device memory the context holds. */
size_t hmf_device_bytes(const hmf_ctx* ctx);

/* Launch-level statistics of the last hmf_solve: kernels launched, and the
 * average device time (ms) of each kernel kind measured with CUDA events on
 * the launching stream when `timed` solves were requested through
 * hmf_set_timing(ctx, 1).  kinds: 0 = flow (stencil), 1 = tree (per-voxel
 * sink/label sweep), 2 = init. */
int hmf_set_timing(hmf_ctx* ctx, int enabled);
int hmf_get_stats(const hmf_ctx* ctx, long long* launches, double* avg_ms_by_kind, int n_kinds);

/* ---- Out-of-core solve (GPU memory budget) ---------------------------------
 * Replaces the GPU buffer pager of vtkCudaHierarchicalMaxFlowSegmentation:
 * MaxGPUUsage (vtkCudaHierarchicalMaxFlowSegmentation.h:52, a fraction of the
 * device's memory, default 0.75), the buffer acquisition of
 * CUDA_GetGPUBuffers (CUDA_hierarchicalmaxflow.cu:33-60) and the next-use
 * paging of GetGPUBuffersV2 / SimulateIterationForBufferOrdering
 * (vtkCudaHierarchicalMaxFlowSegmentation.cxx:884-1294), which move whole
 * buffers across the host link before every pass once the state does not
 * fit.
 *
 * hmf_create_paged makes a context whose solver state lives in pinned host
 * memory (two copies of 5 x (n_nodes - 1) + 1 arrays of VX*VY*VZ floats;
 * one copy when one round suffices) and whose device memory stays within
 * max_gpu_usage x the device's memory (clamped to [0, 1]).  hmf_solve covers
 * the volume with blocks of T z-planes (T from the budget: three block
 * contexts of T planes fit) and iterates in rounds of k <= 12 iterations: each
 * block is loaded, iterated k times with the in-core kernels, and stores back
 * the planes at least 2k + 1 planes from its inner faces, which equal the
 * in-core solve's.  Labels and sinks are therefore identical to hmf_create +
 * hmf_solve's.  Volumes of 2^31 elements or more are allowed (each block is
 * below that).  Works with hmf_set_data / hmf_set_smoothness (host inputs
 * are copied once per solve into pinned memory unless already pinned; device
 * inputs are read in place), hmf_set_smoothness_scalar, hmf_set_params,
 * hmf_solve, hmf_solve_continue (from the host copy the last solve ended
 * in), hmf_get_labels, hmf_get_sink, hmf_leaf_order, hmf_device_bytes,
 * hmf_set_timing / hmf_get_stats; every other call taking a context returns
 * HMF_ERR_STATE.  Label trees, single volumes, both semantics (REF_CPU
 * iterates per voxel: one round, no halo).
 *  - hmf_set_paged_plan: block planes T and iterations per round k for later
 *    solves (0: from the budget, k = min(12, (T - 4) / 8)); T >= 4 x (2k + 1)
 *    unless one block covers the volume (then k > 0 splits the solve into
 *    rounds of k iterations on that block); and where host inputs are read
 *    from: HMF_PAGED_INPUTS_AUTO (on the device for the whole solve when
 *    they take at most a quarter of the budget, else from host memory every
 *    round), HMF_PAGED_INPUTS_HOST, HMF_PAGED_INPUTS_DEVICE.  Three block
 *    contexts of T planes are in flight (one loading, one iterating, one
 *    storing), and the host state is double-buffered between rounds.
 *  - hmf_get_paged_plan: blocks, T, k and rounds of the last solve, and the
 *    bytes it moved between host and device.
 *  - hmf_paged_layout: host only (no device work): the blocks covering vz
 *    planes with blocks of block_planes planes and halo_planes planes of
 *    halo; writes up to `capacity` first planes (starts) and first owned
 *    planes (owned: block j owns owned[j] .. owned[j+1]-1, the last block up
 *    to vz-1) and returns the number of blocks, or HMF_ERR_INVALID_ARGUMENT
 *    when the blocks are thinner than four halos. */
int hmf_create_paged(hmf_ctx** out, int vx, int vy, int vz, const int* parent, int n_nodes, int semantics,
                     int device, double max_gpu_usage);
#define HMF_PAGED_INPUTS_AUTO 0
#define HMF_PAGED_INPUTS_HOST 1
#define HMF_PAGED_INPUTS_DEVICE 2
int hmf_set_paged_plan(hmf_ctx* ctx, int block_planes, int round_iterations, int inputs);
int hmf_get_paged_plan(const hmf_ctx* ctx, int* blocks, int* block_planes, int* round_iterations, int* rounds,
                       long long* link_bytes);
int hmf_paged_layout(int vz, int block_planes, int halo_planes, int* starts, int* owned, int capacity);

/* ---- Batches --------------------------------------------------------------
 * No counterpart in the reference, which solves one volume per filter
 * update: many volumes of different sizes that share one label tree, one set
 * of smoothness weights and one set of parameters are solved together, every
 * iteration in the same two kernel launches (captured in a CUDA graph), so
 * small volumes do not leave the GPU idle.  dims holds n_volumes triples
 * (VX, VY, VZ).  The single-volume calls above act on volume 0. */
int hmf_create_batch(hmf_ctx** out, int n_volumes, const int* dims, const int* parent, int n_nodes,
                     int semantics, int device);
int hmf_num_volumes(const hmf_ctx* ctx);
int hmf_batch_set_data(hmf_ctx* ctx, int volume, int node, const float* data, int where);
int hmf_batch_set_smoothness(hmf_ctx* ctx, int volume, int node, const float* smooth, int where);
int hmf_batch_get_labels(hmf_ctx* ctx, int volume, int node, float* out, int where, void* stream);
int hmf_batch_get_sink(hmf_ctx* ctx, int volume, int node, float* out, int where, void* stream);

/* Autotuner (no counterpart in the reference): times a few iterations of the
 * flow kernel for each window shape (hmf_set_flow_window) and candidate
 * z-chunk length (planes per CTA column), then the best of those with 2 and
 * 4 units per CTA (hmf_set_flow_units), on the context's current inputs,
 * keeps the fastest for this context and caches it for contexts of the same
 * shape created later (key: SM count, semantics, tree shape, volume sizes
 * rounded up to multiples of 16).  The cache lives for the process; with the
 * environment variable HMF_AUTOTUNE_CACHE naming a file it is also read from
 * and appended to that file.  Inputs must be set; the labels are not kept. */
int hmf_autotune(hmf_ctx* ctx, void* stream);
/* The flow kernel's z-chunk length (planes each CTA marches): set it (z >= 1;
 * 0 restores the default plan) or read the current one. */
int hmf_set_zchunk(hmf_ctx* ctx, int z);
int hmf_get_zchunk(const hmf_ctx* ctx);
/* The flow kernel's window: 32 columns x `rows` rows per CTA, rows 32 (two
 * CTAs of 8 warps per SM) or 64 (one CTA of 16 warps per SM, fewer halo rows
 * per output); 0 restores the default.  hmf_autotune times both shapes.  The
 * z chunk returns to its default plan for the shape. */
int hmf_set_flow_window(hmf_ctx* ctx, int rows);
int hmf_get_flow_window(const hmf_ctx* ctx);
/* Units of flow-kernel work per CTA: a unit is one vertex's z-march over one
 * window and z chunk; a CTA marches `units` of them one after another (the
 * vertices of a window first, so that their shared parent sinks and
 * smoothness planes come from L2), in 1..64 (0 restores 1).  Fewer, longer
 * CTAs save per-CTA set-up on small volumes and batches; hmf_autotune times
 * 1, 2 and 4 with its best window and chunk.  Results do not depend on it. */
int hmf_set_flow_units(hmf_ctx* ctx, int units);
int hmf_get_flow_units(const hmf_ctx* ctx);
/* Slab pipeline of the replayed iterations (single volumes of label trees,
 * REF_CUDA, convergence log off): each iteration's flow and sweep launches
 * are cut at the flow plan's z chunks into per-slab graph nodes that wait
 * only for the slabs their stencil touches, so sweeps overlap flows and
 * consecutive iterations overlap.  Same arithmetic, bit-identical results.
 * On by default; hmf_get_pipeline returns 1 when the next solve runs
 * pipelined. */
int hmf_set_pipeline(hmf_ctx* ctx, int enabled);
int hmf_get_pipeline(const hmf_ctx* ctx);

/* ---- Convergence log --------------------------------------------------------
 * No counterpart in the reference, which runs a fixed number of iterations
 * and computes no convergence measure (its header gives the cost as the
 * reason, vtkHierarchicalMaxFlowSegmentation.h:61-63).  With the log on,
 * the label sweep of every iteration also reduces, over all non-root
 * vertices and voxels, max |u_new - u_old| and the sum of |u_new - u_old|
 * (warp shuffles and a few atomics per CTA inside the same kernel; no extra
 * pass over memory).  hmf_get_convergence writes, for the iterations of the
 * last hmf_solve (up to `capacity`), the maximum and the mean (the sum over
 * (n_nodes - 1) x voxels) and returns the number of iterations logged.
 * REF_CUDA tree contexts; a batch's volumes are pooled (each volume's VX a
 * multiple of 4).  Toggling re-captures the iteration graphs. */
int hmf_set_convergence_log(hmf_ctx* ctx, int enabled);
int hmf_get_convergence(hmf_ctx* ctx, double* max_change, double* mean_change, int capacity);

/* ---- Bounded copy waits ----------------------------------------------------
 * No counterpart in the reference, whose kernels have no waits.  The
 * kernels that stream their inputs through shared memory (TMA / bulk copies
 * completed on mbarriers) bound every wait: a wait that runs out makes the
 * kernel stop issuing copies, wait (0.5 s at most) for the copies still in
 * flight into its shared memory, and leave; the call then returns
 * HMF_ERR_CUDA ("... timed out ...") and the context stays usable.
 *  - hmf_set_wait_limit: the bound (ns) of the flow kernels' waits, forward
 *    and reverse (0: the default 0.5 s).  The sweep kernels keep 0.5 s.
 *  - hmf_inject_wait_stall: makes one CTA of the next launch of `kernel`
 *    wait on a barrier that no copy completes, so that its bounded wait runs
 *    out on healthy hardware: the failure path on demand, for tests (-1
 *    cancels).  A solve with a pending request runs its launches one by one
 *    instead of replaying its CUDA graph. */
#define HMF_STALL_FLOW 0
#define HMF_STALL_SWEEP 1
#define HMF_STALL_REVERSE_FLOW 2
#define HMF_STALL_REVERSE_SWEEP 3
int hmf_set_wait_limit(hmf_ctx* ctx, long long limit_ns);
int hmf_inject_wait_stall(hmf_ctx* ctx, int kernel);

/* ---- Adjoint (reverse mode) -----------------------------------------------
 * No counterpart in the reference, which only solves forward.  Solves like
 * hmf_solve (REF_CUDA semantics, single-volume contexts) and differentiates
 * the loss
 *     L = -(1/V) * sum_i log(max(u_{leaf(truth_i)}(i), eps))
 * of the final leaf labels through every iteration: truth holds one class per
 * voxel (int32, x fastest, dense VX*VY*VZ) indexing the leaves in the order
 * of hmf_leaf_order.  Afterwards hmf_get_data_gradient returns dL/dD for each
 * leaf data term (per voxel, double) and hmf_get_alpha_gradient dL/dalpha for
 * every vertex's smoothness weight; labels and sinks read as after hmf_solve.
 * Forward states are kept in HBM every checkpoint_every iterations and the
 * states in between recomputed segment by segment (ceil(T/k) + k state
 * slots).  checkpoint_every = 0 is automatic: every state is kept when T + 1
 * state slots fit in the memory budget (85% of the free device memory, or
 * hmf_set_adjoint_memory's), else the budget's slots are scheduled for the
 * fewest forward iterations (a revolve-style binomial schedule: states kept
 * and recomputed recursively; fails with HMF_ERR_OUT_OF_MEMORY when too few
 * slots fit for T iterations).  One state slot holds 6(n_nodes-1)+1 arrays
 * of the padded volume.  The call returns after the backward pass
 * (it synchronises c's stream to read the loss).  Kinks follow the forward
 * code: saturate and the leaf capacity clamp pass gradients strictly inside
 * their linear ranges, the projection multiplier only where |p| > alpha*S. */
int hmf_solve_adjoint(hmf_ctx* ctx, const int* truth, int where, int checkpoint_every, double eps,
                      double* loss, void* stream);
int hmf_get_data_gradient(hmf_ctx* ctx, int leaf, double* out, int where, void* stream);
/* Writes min(n, n_nodes) values (vertex id order; root and vertices without a
 * smoothness term read 0 and their alpha respectively); returns n_nodes. */
int hmf_get_alpha_gradient(hmf_ctx* ctx, double* out, int n);
/* The checkpoint interval the last hmf_solve_adjoint used and how many of its
 * segments were recomputed. */
int hmf_get_adjoint_plan(const hmf_ctx* ctx, int* checkpoint_every, int* recomputed_segments);
/* Memory budget of later hmf_solve_adjoint calls with checkpoint_every = 0:
 * at most max_bytes of device memory for the adjoint's arrays (0: 85% of the
 * free device memory) and at most max_state_slots state slots (0: no cap).
 * The analogue of the reference's MaxGPUUsage
 * (vtkCudaHierarchicalMaxFlowSegmentation2.h:74-82), for the adjoint. */
int hmf_set_adjoint_memory(hmf_ctx* ctx, long long max_bytes, int max_state_slots);
/* The schedule the last hmf_solve_adjoint ran: state slots, forward
 * iterations (first pass included; T when every state is kept) and backward
 * steps (T). */
int hmf_get_adjoint_schedule(const hmf_ctx* ctx, int* state_slots, long long* forward_iterations,
                             long long* backward_steps);
/* The schedule itself, host only (no device work): checkpoint_every > 0 gives
 * the fixed-interval schedule, 0 the fewest-forward-iterations schedule over
 * state_slots slots.  Writes up to `capacity` actions of four ints (kind: 0
 * forward iteration t from slot a to slot b, 1 loss on x_T in slot a, 2
 * backward step of iteration t with x_t in slot a and x_{t+1} in slot b;
 * t; a; b; x_0 starts in slot 0) and returns the number of actions, or
 * HMF_ERR_OUT_OF_MEMORY when no schedule exists with that many slots. */
long long hmf_adjoint_schedule(int iterations, int state_slots, int checkpoint_every, int* actions,
                               long long capacity);

/* ---- Reference precision (FP64) -------------------------------------------
 * No counterpart in the reference, which computes in FP32 only.  The error
 * of an FP32 solve against the exact solution of the same iteration is
 * measured by running the REF_CUDA iteration of hmf_solve
 * (CUDA_hierarchicalmaxflow.cu:124-456 in the launch order of
 * vtkCudaHierarchicalMaxFlowSegmentation.cxx:106-476, initialisation
 * :547-658) in FP64 on the GPU: every operation in the reference's order, in
 * double; step and CC are the FP32 parameters widened, 1/CC and
 * 1/(children+1) are formed in double, alpha is the FP32-stored scalar
 * widened.  Single-volume REF_CUDA tree contexts only.  The FP64 state (six
 * doubles per non-root vertex and voxel) is allocated by the first call and
 * kept with the context.
 *  - hmf_solve_fp64: initialise and iterate in FP64 on the context's current
 *    inputs and parameters (queued on `stream`).
 *  - hmf_get_labels_fp64: the FP64 labelling of a non-root vertex
 *    (VX*VY*VZ doubles).
 *  - hmf_fp64_error: max over leaves and voxels of |u_fp32 - u_fp64| between
 *    the last hmf_solve and the last hmf_solve_fp64, and the fraction of
 *    voxels whose argmax leaf (first maximum) agrees.  Synchronous.
 *  - hmf_fp64_loss: the adjoint's loss -(1/V) sum_i log(max(u_{truth_i}, eps))
 *    on the FP64 labels (truth as for hmf_solve_adjoint).  Synchronous.
 *  - hmf_set_fp64_probe: inputs of later FP64 solves that differ from the
 *    FP32 inputs, for finite differences: HMF_FP64_PROBE_DATA sets the data
 *    term of leaf `node` at dense voxel index `voxel` (x fastest) to `value`
 *    (double); HMF_FP64_PROBE_ALPHA sets the smoothness weight of vertex
 *    `node` to `value` (double, not rounded to float); HMF_FP64_PROBE_NONE
 *    clears both.  One data probe at a time. */
#define HMF_FP64_PROBE_NONE 0
#define HMF_FP64_PROBE_DATA 1
#define HMF_FP64_PROBE_ALPHA 2
int hmf_solve_fp64(hmf_ctx* ctx, void* stream);
int hmf_get_labels_fp64(hmf_ctx* ctx, int node, double* out, int where, void* stream);
int hmf_fp64_error(hmf_ctx* ctx, double* max_abs_err, double* argmax_agreement, void* stream);
int hmf_fp64_loss(hmf_ctx* ctx, const int* truth, int where, double eps, double* loss, void* stream);
int hmf_set_fp64_probe(hmf_ctx* ctx, int kind, int node, long long voxel, double value);

/* ---- Vote and energy (the steps after a solve) ----------------------------
 * hmf_vote replaces CUDA_CIV_COMPUTE (CUDA_imagevote.h, the vtkCudaImageVote
 * filter) for float inputs and int labels: out[i] = values[k] of the input k
 * with the largest value at voxel i (values NULL: k).  semantics
 * HMF_SEMANTICS_REF_CUDA follows vtkCudaImageVote (running maximum from
 * input 0, an input takes over when value >= maximum: the last of a tie
 * wins, CUDA_imagevote.cu:30-46), HMF_SEMANTICS_REF_CPU follows vtkImageVote
 * (the first maximum wins, vtkImageVote.cxx:285-306).  `where` applies to
 * the inputs and the output alike; errors read with hmf_last_error(NULL).
 * hmf_get_vote / hmf_batch_get_vote vote over a context's final leaf labels
 * (leaves in hmf_leaf_order, ids = vertex ids; the context's semantics picks
 * the tie rule); the output is dense VX*VY*VZ. */
int hmf_vote(int n_inputs, const float* const* inputs, const int* values, long long n_voxels, int semantics,
             int* out, int where, void* stream);
int hmf_get_vote(hmf_ctx* ctx, int* out, int where, void* stream);
int hmf_batch_get_vote(hmf_ctx* ctx, int volume, int* out, int where, void* stream);

/* Energy decomposition of a labelling; replaces the CUDA_GHMFD_* launchers
 * (CUDA_hierarchicalmaxflowdecomp.h) behind
 * vtkCudaHierarchicalMaxFlowDecomposition::GetF0 / GetF
 * (vtkCudaHierarchicalMaxFlowDecomposition.h).  f0 = sum over leaves and
 * voxels of D*u; f[v] (per vertex id, root 0) = sum over voxels of
 * S_v * 0.5*sqrt(|grad u_v|^2) with clamped central differences, S_v = 1
 * without a smoothness image, a branch's labelling being the sum of its
 * children's.  Per-voxel terms in FP32 as the reference forms them, sums in
 * FP64.  data, labels: per vertex id (leaves needed); smooth may be NULL.
 * Synchronous.  hmf_get_energy / hmf_batch_get_energy evaluate a context's
 * final labels with its own inputs (which must still be valid); they return
 * n_nodes. */
int hmf_decomposition_energy(int vx, int vy, int vz, const int* parent, int n_nodes, const float* const* data,
                             const float* const* labels, const float* const* smooth, int where, double* f0,
                             double* f, void* stream);
int hmf_get_energy(hmf_ctx* ctx, double* f0, double* f, int n);
int hmf_batch_get_energy(hmf_ctx* ctx, int volume, double* f0, double* f, int n);

/* Data term of vtkImageDataTerm (Common/vtkRobartsCommon/vtkImageDataTerm.cxx:62-470),
 * per voxel of float32 images in1 (and optionally in2, same size):
 *   HMF_DATA_TERM_CONSTANT  C1                       (entropy: -log C1)
 *   HMF_DATA_TERM_LOGISTIC  1/(1+e^-(K1(x1-C1))) [x 1/(1+e^-(K2(x2-C2)))]   (entropy: -log of it)
 *   HMF_DATA_TERM_GAUSSIAN  e^-(((x1-C1)/K1)^2/2 [+ ((x2-C2)/K2)^2/2])        (entropy: the exponent)
 *   HMF_DATA_TERM_SPIKE     x1 == K1 ? C1 : C2, one image only
 * in the reference's double arithmetic and its constant handling (one
 * image: the spike's second value is C1 unless entropy takes logarithms;
 * two images: no normalisation).  normalize rescales one-image results by
 * in1's range as the reference does.  The numeric codes are the reference's
 * VTK_CONSTANT .. VTK_SPIKE; note that its SetOperationToGaussian selects
 * VTK_SPIKE and SetOperationToSpike VTK_GAUSSIAN (vtkImageDataTerm.h).
 * Synchronous for host buffers.  Returns a status. */
#define HMF_DATA_TERM_CONSTANT 0
#define HMF_DATA_TERM_LOGISTIC 1
#define HMF_DATA_TERM_GAUSSIAN 2
#define HMF_DATA_TERM_SPIKE 3
int hmf_data_term(int op, int entropy, int normalize, double k1, double c1, double k2, double c2, const float* in1,
                  const float* in2, long long n_voxels, float* out, int where, void* stream);

/* Maximum-likelihood data term of vtkImageLogLikelihood
 * (Common/vtkRobartsCommon/vtkImageLogLikelihood.cxx:140-250): voxels where
 * at least required_agreement of the non-NULL int32 label maps equal
 * label_id are the seeds; a histogram of the float32 image (1 or 2
 * interleaved components) over the seeds with bins of `resolution`; per voxel
 * -log(bin frequency + 1e-10), -log(1e-10) outside the histogram, divided by
 * -log(1e-10) if normalize; 1 everywhere without seeds.  The bin count is the
 * reference's (int)(max - min/resolution) + 1; inputs whose seeds would fall
 * past it (where the reference writes out of bounds) are rejected.
 * Synchronous.  Returns a status. */
#define HMF_MAX_LABEL_MAPS 32
int hmf_log_likelihood(const float* image, int components, const int* const* label_maps, int n_label_maps,
                       long long n_voxels, int label_id, float resolution, double required_agreement, int normalize,
                       float* out, int where, void* stream);

/* Message of the last failed call on ctx (or, when ctx is NULL, of the last
 * failed hmf_create or hmf_solve_noalloc on this thread). */
const char* hmf_last_error(const hmf_ctx* ctx);

/* Allocation-free solve.  No counterpart in the reference: it exists for
 * callers that must not allocate device memory while they run, such as a
 * plugin inside an image-guidance or streaming application that reserves all
 * GPU memory at start-up and forbids later allocations (cudaMalloc and
 * cudaFree can synchronise the device and stall the application's other
 * streams), or code that works inside a memory pool it does not own.
 *
 * It runs the same initialisation and iterations as hmf_create + hmf_solve +
 * hmf_get_labels on the current device, but keeps all solver state in one
 * statically sized device array of this library, HMF_NOALLOC_SCRATCH_BYTES
 * (64 MiB), which every GPU that loads the library holds until the process
 * exits.  It calls no cudaMalloc, cudaFree or other allocating routine.
 *
 *  - Inputs and outputs are the caller's device buffers of VX*VY*VZ floats,
 *    indexed by tree vertex: data[v] for every leaf, smooth[v] (or a NULL
 *    array / NULL entry for S = 1), alpha[v] (NULL: all 1), labels[v] for
 *    each non-root vertex whose labelling is wanted (NULL entries skipped).
 *  - The scratch needed is 4 bytes x VX' x VY x VZ x (9 x (n_nodes - 1) + 1
 *    + leaves + distinct smoothness images) plus about 24 KiB of tables, with
 *    VX' = VX rounded up to a multiple of 4; a larger problem is rejected with
 *    HMF_ERR_INVALID_ARGUMENT before anything is queued.
 *  - Every call looks up the array's device address in the current context
 *    and sets the kernels' attributes (neither allocates).  The call cannot
 *    be recorded into a graph: inside a stream capture it returns
 *    HMF_ERR_INVALID_ARGUMENT before anything is queued.
 *  - Work is queued on `stream`; the call returns after it has finished
 *    (it synchronises `stream` to report negative inputs).
 *  - Every call shares the one array: calls whose work overlaps on the GPU
 *    (other threads, other streams) race and corrupt each other.  Each call
 *    clears the part of the array it uses before using it. */
#define HMF_NOALLOC_SCRATCH_BYTES (64u << 20)
int hmf_solve_noalloc(int vx, int vy, int vz, const int* parent, int n_nodes, int semantics,
                      const float* const* data, const float* const* smooth, const double* alpha,
                      int iterations, float step_size, float cc, float* const* labels, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* HMF_GB300_H */
