// hmf_tree_bulk.cuh -- the per-voxel sink / source / label sweep of one
// iteration (CUDA_hierarchicalmaxflow.cu:124-220 and MultiplyAndStoreBuffer,
// launched in the order of vtkCudaHierarchicalMaxFlowSegmentation.cxx:268-426),
// streamed through shared memory with bulk copies.
//
// A persistent CTA walks chunks of Vc consecutive voxels.  For every chunk it
// brings in, with one cp.async.bulk per array, the 3(n-1)+1 arrays the sweep
// reads -- per non-root entry its divergence, its label and either its sink
// (branch) or its data term (leaf), plus the source flow -- into one of two
// shared-memory stages completed by an mbarrier, so one chunk is in flight
// while the other is swept.  Each thread sweeps four voxels (float4); new
// sinks overwrite the staged sink / data slots in post-order (a parent's old
// sink is read by its children before the parent replaces it), labels and
// sinks go straight to global memory (sink_out / label_out: in place in a
// solve, the next state slot in the adjoint's forward pass).  Same arithmetic
// as tree_kernel.
#pragma once

#include "hmf_async.cuh"
#include "hmf_kernels.cuh"

namespace hmf {

constexpr int kTreeBulkStages = 2;

// Convergence log of a solve: per iteration, max and sum over non-root
// vertices and voxels of |u_new - u_old|, reduced inside the label sweep
// (warp shuffles, one pair of atomics per warp).  A sweep launch logs into
// entry *base + t: `base` is the first iteration of the replayed graph it
// belongs to (advanced by the graph's last node), `t` its iteration within
// that graph -- so the sweeps of one iteration cut into slabs, and sweeps of
// consecutive iterations running side by side, log where they belong.
// Padding columns (x >= vx of each row of `pitch` elements; pitch 0: none)
// are left out.
struct GapLog {
  unsigned int* max_bits;  // [capacity] float bits (non-negative floats order as unsigned ints)
  double* sum;             // [capacity]
  const unsigned int* base;
  int t;
  int capacity;
  int vx, pitch;
};

// The graph's last node with the log on: the next replay's first iteration.
__global__ void gap_advance_kernel(unsigned int* base, int n_iter) { *base += (unsigned)n_iter; }

// Shared memory of one sweep CTA's two stages.  96 KB (512-voxel chunks for a
// 7-vertex tree, ~78 KB) lets a sweep CTA sit beside one flow CTA on an SM,
// so the sweep of one z slab overlaps the flow steps of its neighbours: on a
// GB300 at 256^3 (two-level, 4-leaf tree) an iteration took 1.153 ms against
// 1.164 ms with 200 KB (1024-voxel chunks), though the sweep launched alone
// is 3 % slower (0.347 against 0.336 ms); 64 KB measured 1.160 ms.
constexpr int kTreeBulkSmemBudget = 96 * 1024;

// Chunk length (voxels) for a tree of n entries: the largest power of two
// <= 1024 whose two stages fit the shared-memory budget.
__host__ __device__ constexpr int tree_bulk_chunk(int n) {
  const int arrays = 3 * (n - 1) + 1;
  int vc = 1024;
  while (vc > 32 && kTreeBulkStages * arrays * vc * 4 > kTreeBulkSmemBudget) vc /= 2;
  return vc;
}

__host__ __device__ constexpr int tree_bulk_smem_bytes(int n) {
  return 128 + kTreeBulkStages * (3 * (n - 1) + 1) * tree_bulk_chunk(n) * 4;
}

// End of a sweep launch with the convergence log on (every thread):
// warp-shuffle max and sum, one pair of atomics per warp into the entry of
// this launch's iteration.
__device__ __forceinline__ void gap_log_commit(const GapLog& gap, float gmax, float gsum) {
  const unsigned it = *gap.base + (unsigned)gap.t;
  for (int o = 16; o > 0; o >>= 1) {
    gmax = fmaxf(gmax, __shfl_down_sync(0xffffffffu, gmax, o));
    gsum += __shfl_down_sync(0xffffffffu, gsum, o);
  }
  if ((threadIdx.x & 31) == 0 && it < (unsigned)gap.capacity) {
    atomicMax(&gap.max_bits[it], __float_as_uint(gmax));
    atomicAdd(&gap.sum[it], (double)gsum);
  }
}

__global__ void tree_bulk_kernel(const TreeTable* __restrict__ table, const Geometry G, int* __restrict__ error_flag,
                                 const GapLog gap = GapLog{}) {
  __shared__ TreeTable T;
  __shared__ int abort_cta, stall_cta, stop_cta;
  extern __shared__ __align__(128) unsigned char tb_raw[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(tb_raw);  // [2], then the stall barrier
  float* stage0 = reinterpret_cast<float*>(tb_raw + 128);

  for (int i = threadIdx.x; i < (int)(sizeof(TreeTable) / 4); i += blockDim.x)
    reinterpret_cast<int*>(&T)[i] = reinterpret_cast<const int*>(table)[i];
  __syncthreads();  // thread 0 reads the table below
  if (threadIdx.x == 0) {
    const int flag = error_flag ? *(volatile int*)error_flag : 0;
    abort_cta = flag & 2;
    stall_cta = take_stall_request(error_flag, flag);
    stop_cta = 0;
    // bulk-copy destinations must be 16-byte aligned: refuse to run otherwise.
    if (smem_addr(tb_raw) & 15) {
      abort_cta = 1;
      if (error_flag) atomicOr(error_flag, 4);
    }
    // one arrival per staged array (the copies are spread over the threads)
    for (int s = 0; s < kTreeBulkStages; ++s) mbar_init(&bars[s], (unsigned)(3 * (T.n - 1) + 1));
    mbar_init(&bars[kTreeBulkStages], 1);  // completed by nothing: a requested stall waits on it
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (abort_cta) return;

  const int n = T.n, root = n - 1;
  const int arrays = 3 * (n - 1) + 1;
  const int vc = tree_bulk_chunk(n);
  const long long nchunks = (G.vol + vc - 1) / vc;
  const float icc = T.icc, cc = T.cc;
  auto stage = [&](int s) { return stage0 + (size_t)s * arrays * vc; };
  // staged array slot of each quantity: entry e < root -> div 3e, label 3e+1,
  // sink (branch) / data (leaf) 3e+2; the root's source flow -> 3(n-1)
  auto sink_slot = [&](int e) { return e == root ? 3 * root : 3 * e + 2; };

  // Staged array c of a chunk is copied by thread c (c, c + blockDim, ...),
  // each copy with its own expected bytes and mbarrier arrival.
  auto array_src = [&](int c) -> const float* {
    if (c == 3 * root) return T.e[root].sink;
    const TreeEntry& E = T.e[c / 3];
    return c % 3 == 0 ? E.div : c % 3 == 1 ? E.label : (E.n_kids ? E.sink : E.data);
  };
  auto issue = [&](long long chunk, int s) {
    const long long v0 = chunk * vc;
    const unsigned bytes = (unsigned)(min((long long)vc, G.vol - v0) * 4);
    uint64_t* bar = &bars[s];
    float* dst = stage(s);
    for (int c = threadIdx.x; c < arrays; c += blockDim.x) {
      mbar_expect_tx(bar, bytes);
      bulk_load(dst + (size_t)c * vc, array_src(c) + v0, bytes, bar);
    }
  };

  // A wait that runs out raises stop_cta; after the CTA barrier that ends the
  // chunk every thread sees it and the loop ends before another copy is
  // issued, so the copies in flight are exactly the last one of each stage.
  bool timed_out = false;
  auto wait_stage = [&](uint64_t* bar, unsigned parity) {
    if (timed_out) return;
    if (!mbar_wait_bounded(bar, parity, kTmaWaitLimitNs)) {
      timed_out = true;
      *(volatile int*)&stop_cta = 1;
    }
  };
  float gmax = 0.0f, gsum = 0.0f;  // convergence log: this thread's max and sum of |u_new - u_old|
  int nissued[kTreeBulkStages] = {0, 0};  // kept by every thread (thread 0 always issues)
  long long chunk = blockIdx.x;
  if (chunk < nchunks) issue(chunk, 0), ++nissued[0];
  if (chunk + gridDim.x < nchunks) issue(chunk + gridDim.x, 1), ++nissued[1];
  if (threadIdx.x == 0 && stall_cta) wait_stage(&bars[kTreeBulkStages], 0);
  for (int j = 0; chunk < nchunks; ++j, chunk += gridDim.x) {
    const int s = j & 1;
    wait_stage(&bars[s], (unsigned)((j >> 1) & 1));
    float* st = stage(s);
    const long long v0 = chunk * vc;
    const int len = (int)min((long long)vc, G.vol - v0);
    const int q = threadIdx.x * 4;
    if (q < len) {
      auto at = [&](int slot) -> float4& { return *reinterpret_cast<float4*>(st + (size_t)slot * vc + q); };
      for (int e = 0; e < n; ++e) {
        const TreeEntry& E = T.e[e];
        if (E.n_kids == 0) {
          const float4 inc = at(sink_slot(E.parent)), d = at(3 * e), u = at(3 * e + 1), cap = at(3 * e + 2);
          float4 r;
          float v;
#define HMF_LEAF(c)              \
  v = (inc.c - d.c) + u.c * icc; \
  v = (v < 0.0f) ? 0.0f : v;     \
  v = (v > cap.c) ? cap.c : v;   \
  r.c = v;
          HMF_LEAF(x) HMF_LEAF(y) HMF_LEAF(z) HMF_LEAF(w)
#undef HMF_LEAF
          at(3 * e + 2) = r;
        } else {
          const float w0 = (e == root) ? T.root_init : 0.0f;
          float4 W = make_float4(w0, w0, w0, w0);
          for (int k = 0; k < E.n_kids; ++k) {
            const int c = T.kids[E.first_kid + k];
            const float4 sc = at(sink_slot(c)), dc = at(3 * c), uc = at(3 * c + 1);
            W.x = ((W.x + sc.x) + dc.x) - uc.x * icc;
            W.y = ((W.y + sc.y) + dc.y) - uc.y * icc;
            W.z = ((W.z + sc.z) + dc.z) - uc.z * icc;
            W.w = ((W.w + sc.w) + dc.w) - uc.w * icc;
          }
          if (e != root) {
            const float4 inc = at(sink_slot(E.parent)), d = at(3 * e), u = at(3 * e + 1);
            W.x = ((W.x + inc.x) - d.x) + u.x * icc;
            W.y = ((W.y + inc.y) - d.y) + u.y * icc;
            W.z = ((W.z + inc.z) - d.z) + u.z * icc;
            W.w = ((W.w + inc.w) - d.w) + u.w * icc;
          }
          at(sink_slot(e)) = make_float4(W.x * E.inv_kids, W.y * E.inv_kids, W.z * E.inv_kids, W.w * E.inv_kids);
        }
      }
      const long long i = v0 + q;
      const int nvalid = gap.pitch ? min(4, max(0, gap.vx - (int)(i % gap.pitch))) : 4;
      for (int e = 0; e < root; ++e) {
        const TreeEntry& E = T.e[e];
        const float4 inc = at(sink_slot(E.parent)), d = at(3 * e), sk = at(3 * e + 2), u = at(3 * e + 1);
        float4 o;
        o.x = __saturatef(u.x + cc * ((inc.x - d.x) - sk.x));
        o.y = __saturatef(u.y + cc * ((inc.y - d.y) - sk.y));
        o.z = __saturatef(u.z + cc * ((inc.z - d.z) - sk.z));
        o.w = __saturatef(u.w + cc * ((inc.w - d.w) - sk.w));
        if (gap.max_bits) {
          const float a0 = nvalid > 0 ? fabsf(o.x - u.x) : 0.0f, a1 = nvalid > 1 ? fabsf(o.y - u.y) : 0.0f;
          const float a2 = nvalid > 2 ? fabsf(o.z - u.z) : 0.0f, a3 = nvalid > 3 ? fabsf(o.w - u.w) : 0.0f;
          gmax = fmaxf(gmax, fmaxf(fmaxf(a0, a1), fmaxf(a2, a3)));
          gsum += (a0 + a1) + (a2 + a3);
        }
        *reinterpret_cast<float4*>(E.label_out + i) = o;
        *reinterpret_cast<float4*>(E.sink_out + i) = sk;
      }
      *reinterpret_cast<float4*>(T.e[root].sink_out + i) = at(3 * root);
    }
    // The sweep wrote sinks into stage s with ordinary stores; order them
    // before the bulk copy that will refill the stage (async proxy).
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();  // stage s is free again
    if (stop_cta) break;
    if (chunk + 2LL * gridDim.x < nchunks) issue(chunk + 2LL * gridDim.x, s), ++nissued[s];
  }
  __syncthreads();
  if (stop_cta && threadIdx.x == 0) {
    if (error_flag) atomicOr(error_flag, 2);
    // Copies into this CTA's shared memory must have landed before it exits:
    // wait (bounded) for the last one issued into each stage.
    for (int s = 0; s < kTreeBulkStages; ++s)
      if (nissued[s]) mbar_wait_bounded(&bars[s], (unsigned)((nissued[s] - 1) & 1), kTmaWaitLimitNs);
  }
  if (gap.max_bits) gap_log_commit(gap, gmax, gsum);
}

// The same sweep for trees of N <= 16 entries (the root last, entries in
// post-order).  The tree's shape is read once per CTA into registers -- per
// entry the staged offset of its parent's sink, a bit mask of its children,
// 1/(kids+1) and the output pointers -- and the chunk length is a
// compile-time constant, so every staged array is an immediate offset from
// one shared-memory base and the per-voxel code reads no table.
template <int N, bool GAP = false>
__global__ void __launch_bounds__(tree_bulk_chunk(N) / 4)
    tree_bulk_n_kernel(const TreeTable* __restrict__ table, const Geometry G, int* __restrict__ error_flag,
                       const GapLog gap = GapLog{}) {
  constexpr int R = N - 1;  // the root entry
  constexpr int A = 3 * R + 1;
  constexpr int VC = tree_bulk_chunk(N);
  constexpr int Q = VC / 4;  // float4 per staged array
  __shared__ TreeTable T;
  __shared__ int abort_cta, stall_cta, stop_cta;
  extern __shared__ __align__(128) unsigned char tb_raw[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(tb_raw);  // [2], then the stall barrier
  float4* stage0 = reinterpret_cast<float4*>(tb_raw + 128);

  for (int i = threadIdx.x; i < (int)(sizeof(TreeTable) / 4); i += blockDim.x)
    reinterpret_cast<int*>(&T)[i] = reinterpret_cast<const int*>(table)[i];
  if (threadIdx.x == 0) {
    const int flag = error_flag ? *(volatile int*)error_flag : 0;
    abort_cta = flag & 2;
    stall_cta = take_stall_request(error_flag, flag);
    stop_cta = 0;
    if (smem_addr(tb_raw) & 15) {
      abort_cta = 1;
      if (error_flag) atomicOr(error_flag, 4);
    }
    for (int s = 0; s < kTreeBulkStages; ++s) mbar_init(&bars[s], A);  // one arrival per staged array
    mbar_init(&bars[kTreeBulkStages], 1);  // completed by nothing: a requested stall waits on it
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (abort_cta) return;

  // staged slot of entry e's sink (root: the source flow) / divergence / label
  auto ss = [](int e) { return e == R ? 3 * R : 3 * e + 2; };
  unsigned leaf_mask = 0, kmask[N];
  int poff[N];
  float inv[N];
  float* lout[N];
  float* sout[N];
#pragma unroll
  for (int e = 0; e < N; ++e) {
    const TreeEntry& E = T.e[e];
    if (e != R && E.n_kids == 0) leaf_mask |= 1u << e;
    poff[e] = e == R ? 0 : (E.parent == R ? 3 * R : 3 * E.parent + 2) * Q;
    inv[e] = E.inv_kids;
    lout[e] = E.label_out;
    sout[e] = E.sink_out;
    kmask[e] = 0;
#pragma unroll
    for (int k = 0; k < R; ++k)
      if (T.e[k].parent == e) kmask[e] |= 1u << k;
  }
  const float icc = T.icc, cc = T.cc, w0r = T.root_init;
  const long long nchunks = (G.vol + VC - 1) / VC;

  // Staged array a of a chunk is copied by thread a (a < A), each copy with
  // its own expected bytes and mbarrier arrival: per entry e < R its
  // divergence (3e), label (3e+1) and sink or data term (3e+2); the source
  // flow (3R).
  const int ta = threadIdx.x;
  const float* asrc = nullptr;
  if (ta < 3 * R) {
    const TreeEntry& E = T.e[ta / 3];
    asrc = ta % 3 == 0 ? E.div : ta % 3 == 1 ? E.label : (E.n_kids ? E.sink : E.data);
  } else if (ta == 3 * R) {
    asrc = T.e[R].sink;
  }
  auto issue = [&](long long chunk, int s) {  // threads 0 .. A-1
    const long long v0 = chunk * VC;
    const unsigned bytes = (unsigned)(min((long long)VC, G.vol - v0) * 4);
    uint64_t* bar = &bars[s];
    mbar_expect_tx(bar, bytes);
    bulk_load(reinterpret_cast<float*>(stage0 + s * A * Q) + ta * VC, asrc + v0, bytes, bar);
  };

  // A wait that runs out raises stop_cta; after the CTA barrier that ends the
  // chunk every thread sees it and the loop ends before another copy is
  // issued, so the copies in flight are exactly the last one of each stage.
  bool timed_out = false;
  auto wait_stage = [&](uint64_t* bar, unsigned parity) {
    if (timed_out) return;
    if (!mbar_wait_bounded(bar, parity, kTmaWaitLimitNs)) {
      timed_out = true;
      *(volatile int*)&stop_cta = 1;
    }
  };
  float gmax = 0.0f, gsum = 0.0f;  // convergence log: this thread's max and sum of |u_new - u_old|
  int nissued[kTreeBulkStages] = {0, 0};  // kept by every issuing thread
  long long chunk = blockIdx.x;
  if (ta < A) {
    if (chunk < nchunks) issue(chunk, 0), ++nissued[0];
    if (chunk + gridDim.x < nchunks) issue(chunk + gridDim.x, 1), ++nissued[1];
  }
  if (threadIdx.x == 0 && stall_cta) wait_stage(&bars[kTreeBulkStages], 0);
  for (int j = 0; chunk < nchunks; ++j, chunk += gridDim.x) {
    const int s = j & 1;
    wait_stage(&bars[s], (unsigned)((j >> 1) & 1));
    const long long v0 = chunk * VC;
    const int len = (int)min((long long)VC, G.vol - v0);
    if ((int)threadIdx.x * 4 < len) {
      float4* b = stage0 + s * A * Q + threadIdx.x;  // this thread's four voxels of staged array 0
      // ---- sinks in post-order (a parent's old sink is read before it is replaced)
#pragma unroll
      for (int e = 0; e < N; ++e) {
        if (e != R && (leaf_mask >> e & 1u)) {
          const float4 inc = b[poff[e]], d = b[(3 * e) * Q], u = b[(3 * e + 1) * Q], cap = b[(3 * e + 2) * Q];
          float4 r;
          float v;
#define HMF_LEAF(c)              \
  v = (inc.c - d.c) + u.c * icc; \
  v = (v < 0.0f) ? 0.0f : v;     \
  v = (v > cap.c) ? cap.c : v;   \
  r.c = v;
          HMF_LEAF(x) HMF_LEAF(y) HMF_LEAF(z) HMF_LEAF(w)
#undef HMF_LEAF
          b[(3 * e + 2) * Q] = r;
        } else {
          const float w0 = e == R ? w0r : 0.0f;
          float4 W = make_float4(w0, w0, w0, w0);
          auto add_child = [&](int k) {
            const float4 sc = b[ss(k) * Q], dc = b[(3 * k) * Q], uc = b[(3 * k + 1) * Q];
            W.x = ((W.x + sc.x) + dc.x) - uc.x * icc;
            W.y = ((W.y + sc.y) + dc.y) - uc.y * icc;
            W.z = ((W.z + sc.z) + dc.z) - uc.z * icc;
            W.w = ((W.w + sc.w) + dc.w) - uc.w * icc;
          };
          if constexpr (N <= 8) {
#pragma unroll
            for (int k = 0; k < e; ++k)
              if (kmask[e] >> k & 1u) add_child(k);
          } else {
            // children in increasing entry order, as a loop over the mask's
            // set bits: unrolling all N^2 (entry, child) pairs overflows the
            // instruction cache for large trees
#pragma unroll 1
            for (unsigned m = kmask[e]; m; m &= m - 1u) add_child(__ffs(m) - 1);
          }
          if (e != R) {
            const float4 inc = b[poff[e]], d = b[(3 * e) * Q], u = b[(3 * e + 1) * Q];
            W.x = ((W.x + inc.x) - d.x) + u.x * icc;
            W.y = ((W.y + inc.y) - d.y) + u.y * icc;
            W.z = ((W.z + inc.z) - d.z) + u.z * icc;
            W.w = ((W.w + inc.w) - d.w) + u.w * icc;
          }
          b[ss(e) * Q] = make_float4(W.x * inv[e], W.y * inv[e], W.z * inv[e], W.w * inv[e]);
        }
      }
      // ---- labels, then every new sink and label to global memory
      const long long i = v0 + threadIdx.x * 4;
      int nvalid = 4;  // voxels of the quad inside the volume (rows are padded to 4 floats)
      if constexpr (GAP) {
        if (gap.pitch) nvalid = min(4, max(0, gap.vx - (int)(i % gap.pitch)));
      }
#pragma unroll
      for (int e = 0; e < R; ++e) {
        const float4 inc = b[poff[e]], d = b[(3 * e) * Q], sk = b[(3 * e + 2) * Q], u = b[(3 * e + 1) * Q];
        float4 o;
        o.x = __saturatef(u.x + cc * ((inc.x - d.x) - sk.x));
        o.y = __saturatef(u.y + cc * ((inc.y - d.y) - sk.y));
        o.z = __saturatef(u.z + cc * ((inc.z - d.z) - sk.z));
        o.w = __saturatef(u.w + cc * ((inc.w - d.w) - sk.w));
        if constexpr (GAP) {
          const float a0 = fabsf(o.x - u.x), a1 = nvalid > 1 ? fabsf(o.y - u.y) : 0.0f;
          const float a2 = nvalid > 2 ? fabsf(o.z - u.z) : 0.0f, a3 = nvalid > 3 ? fabsf(o.w - u.w) : 0.0f;
          const float q0 = nvalid > 0 ? a0 : 0.0f;
          gmax = fmaxf(gmax, fmaxf(fmaxf(q0, a1), fmaxf(a2, a3)));
          gsum += (q0 + a1) + (a2 + a3);
        }
        *reinterpret_cast<float4*>(lout[e] + i) = o;
        *reinterpret_cast<float4*>(sout[e] + i) = sk;
      }
      *reinterpret_cast<float4*>(sout[R] + i) = b[(3 * R) * Q];
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();  // stage s is free again
    if (stop_cta) break;
    if (ta < A && chunk + 2LL * gridDim.x < nchunks) issue(chunk + 2LL * gridDim.x, s), ++nissued[s];
  }
  __syncthreads();
  // Copies into this CTA's shared memory must have landed before it exits:
  // after a time-out every issuing thread waits (bounded) for the last copy
  // it issued into each stage.
  if (stop_cta && ta < A) {
    if (threadIdx.x == 0 && error_flag) atomicOr(error_flag, 2);
    for (int s = 0; s < kTreeBulkStages; ++s)
      if (nissued[s]) mbar_wait_bounded(&bars[s], (unsigned)((nissued[s] - 1) & 1), kTmaWaitLimitNs);
  }
  if constexpr (GAP) gap_log_commit(gap, gmax, gsum);
}

}  // namespace hmf
