// hmf_adjoint_sweep.cuh -- reverse of the per-voxel sink / label sweep for
// trees of N <= 8 vertices (the staged, register-resident form of
// adj_tree_kernel in hmf_adjoint.cuh; same FP32 operations in the same
// order).
//
// A persistent CTA walks chunks of 256 consecutive voxels of the pitched
// layout (padding columns included: their values are finite and never read
// back).  For every chunk lane v of warp 0 issues vertex v's cp.async.bulk
// copies, one per input array -- per vertex the sweep parts of the later state's sink and label
// adjoints, the later flow reverse's gb, the sink and label before the
// iteration, the sink and divergence after it, the data term and the
// accumulated data-term gradient (double) -- into one of two shared-memory
// stages; a stage is refilled as soon as its chunk has been read into
// registers, so two chunks stream in while one is reversed.  Stage
// slots sit at fixed [quantity][vertex] positions (absent quantities are not
// copied and not read), so every shared-memory offset is a compile-time
// constant; one thread reverses one voxel with all per-vertex values in
// registers.  When the vertex ids are in pre-order (PRE), the sink pass runs
// in compile-time vertex order; otherwise runtime vertices (parents,
// children, pre-order positions) are reached through predicated selects.
// FLAT trees (root 0, every other vertex a leaf under it) also have their
// parents at compile time, so no select or parent test is left; the
// operations and their order are the same.
#pragma once

#include "hmf_adjoint.cuh"
#include "hmf_async.cuh"

namespace hmf {

constexpr int kSwVc = 256;     // voxels per chunk = threads per CTA
constexpr int kSwMaxN = 8;
constexpr int kSwKinds = 10;   // float slots per vertex: 8 quantities + one double (2 floats)

enum { kSwSBN = 0, kSwUB, kSwGB, kSwAS, kSwAU, kSwBS, kSwBD, kSwD, kSwDB };  // kSwDB: double, 2 slots

__host__ __device__ constexpr int adj_sweep_smem_bytes(int N) { return 128 + 2 * kSwKinds * N * kSwVc * 4; }

template <int N>
__device__ __forceinline__ float sw_sel(const float (&a)[N], int v) {
  float r = a[0];
#pragma unroll
  for (int w = 1; w < N; ++w) r = (w == v) ? a[w] : r;
  return r;
}

// a[v] = a[v] + x (x already carries its sign: a - b == a + (-b) exactly)
template <int N>
__device__ __forceinline__ void sw_add(float (&a)[N], int v, float x) {
#pragma unroll
  for (int w = 0; w < N; ++w)
    if (w == v) a[w] = a[w] + x;
}

template <int N, bool PRE, bool FLAT>
__global__ void __launch_bounds__(kSwVc) adj_sweep_kernel(const AdjTree* __restrict__ table, const Geometry G,
                                                          const AdjSweep S, int* __restrict__ error_flag) {
  __shared__ AdjTree T;
  __shared__ int abort_cta, stall_cta, stop_cta;
  extern __shared__ __align__(128) unsigned char sw_raw[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(sw_raw);  // [2], then the stall barrier
  float* stage0 = reinterpret_cast<float*>(sw_raw + 128);
  constexpr int kStage = kSwKinds * N * kSwVc;  // floats per stage

  for (int i = threadIdx.x; i < (int)(sizeof(AdjTree) / 4); i += blockDim.x)
    reinterpret_cast<int*>(&T)[i] = reinterpret_cast<const int*>(table)[i];
  if (threadIdx.x == 0) {
    const int flag = error_flag ? *(volatile int*)error_flag : 0;
    abort_cta = flag & 2;
    stall_cta = take_stall_request(error_flag, flag);
    stop_cta = 0;
    if (smem_addr(sw_raw) & 15) {  // bulk-copy destinations must be 16-byte aligned
      abort_cta = 1;
      if (error_flag) atomicOr(error_flag, 4);
    }
    for (int s = 0; s < 2; ++s) mbar_init(&bars[s], N);  // one arrival per vertex lane
    mbar_init(&bars[2], 1);  // completed by nothing: a requested stall waits on it
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (abort_cta) return;

  static_assert(!FLAT || PRE, "a flat tree with root 0 has its ids in pre-order");
  const int root = FLAT ? 0 : T.root;
  auto par = [&](int v) { return FLAT ? (v == 0 ? -1 : 0) : T.parent[v]; };
  auto is_leaf = [&](int v) { return FLAT ? v != 0 : T.n_kids[v] == 0; };
  const float cc = T.cc, icc = T.icc, step = T.step, step_icc = T.step * T.icc;
  const long long arr = S.arr;
  const long long nchunks = (G.vol + kSwVc - 1) / kSwVc;

  // Vertex v's arrays of a chunk, issued by lane v of warp 0 (each lane its
  // own expected bytes, before its copies complete against them).
  auto issue = [&](long long chunk, int s, int v) {
    const long long v0 = chunk * kSwVc;
    const unsigned len = (unsigned)min((long long)kSwVc, G.vol - v0);
    uint64_t* bar = &bars[s];
    float* dst = stage0 + (size_t)s * kStage;
    {
      const bool nr = v != root, leaf = is_leaf(v);
      mbar_expect_tx(bar, len * 4 * (3 + (nr ? 4 : 0)) + (leaf ? len * 8 : 0));
    }
    auto ld = [&](int kind, int v, const float* src) {
      bulk_load(dst + (size_t)(kind * N + v) * kSwVc, src + v0, len * 4, bar);
    };
    {
      const long long b = T.sbase[v];
      const bool nr = v != root, leaf = is_leaf(v);
      ld(kSwSBN, v, S.sbn + v * arr);
      ld(kSwBS, v, S.stB + b * arr);
      if (leaf) ld(kSwD, v, T.data[v]);
      else ld(kSwAS, v, S.stA + b * arr);
      if (nr) {
        ld(kSwUB, v, S.ubn + v * arr);
        ld(kSwGB, v, S.gbn + v * arr);
        ld(kSwAU, v, S.stA + (b + kAdjLabel) * arr);
        ld(kSwBD, v, S.stB + (b + kAdjDiv) * arr);
      }
      if (leaf) bulk_load(dst + (size_t)(kSwDB * N + 2 * v) * kSwVc, T.Db[v] + v0, len * 8, bar);
    }
  };

  bool timed_out = false;
  int nissued[2] = {0, 0};
  long long chunk = blockIdx.x;
  if (threadIdx.x < N) {
    if (chunk < nchunks) issue(chunk, 0, threadIdx.x), ++nissued[0];
    if (chunk + gridDim.x < nchunks) issue(chunk + gridDim.x, 1, threadIdx.x), ++nissued[1];
  }
  // a requested stall: a wait that runs out, so the time-out path runs
  if (threadIdx.x == 0 && stall_cta && !mbar_wait_bounded(&bars[2], 0, kTmaWaitLimitNs)) {
    timed_out = true;
    *(volatile int*)&stop_cta = 1;
  }
  for (int j = 0; chunk < nchunks; ++j, chunk += gridDim.x) {
    const int s = j & 1;
    if (!timed_out && !mbar_wait_bounded(&bars[s], (unsigned)((j >> 1) & 1), kTmaWaitLimitNs)) {
      timed_out = true;
      *(volatile int*)&stop_cta = 1;
    }
    const float* st = stage0 + (size_t)s * kStage;
    const long long v0 = chunk * kSwVc;
    const int len = (int)min((long long)kSwVc, G.vol - v0);
    const int q = threadIdx.x;
    float SBN[N], UB[N], GB[N], AS[N], AU[N], BS[N], BD[N], D[N];
    double DB[N];
    bool hit[N];
    if (q < len) {
      auto at = [&](int kind, int v) { return st[(kind * N + v) * kSwVc + q]; };
#pragma unroll
      for (int v = 0; v < N; ++v) {
        const bool nr = v != root, leaf = is_leaf(v);
        SBN[v] = at(kSwSBN, v);
        BS[v] = at(kSwBS, v);
        AS[v] = leaf ? 0.f : at(kSwAS, v);
        D[v] = leaf ? at(kSwD, v) : 0.f;
        DB[v] = leaf ? reinterpret_cast<const double*>(st + (kSwDB * N + 2 * v) * kSwVc)[q] : 0.0;
        UB[v] = nr ? at(kSwUB, v) : 0.f;
        GB[v] = nr ? at(kSwGB, v) : 0.f;
        AU[v] = nr ? at(kSwAU, v) : 0.f;
        BD[v] = nr ? at(kSwBD, v) : 0.f;
        hit[v] = false;
      }
    }
    // Every value of the chunk is in registers now: stage s is free.  Order
    // these generic reads before the bulk copies that refill it (async
    // proxy), then issue the chunk after next, so that two chunks stream in
    // while this one is reversed.
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (stop_cta) break;  // a copy wait ran out: no further copies
    if (threadIdx.x < N && chunk + 2LL * gridDim.x < nchunks)
      issue(chunk + 2LL * gridDim.x, s, threadIdx.x), ++nissued[s];
    if (q < len) {
      // full adjoints of the later state: sinks (sweep part, then the flow
      // part vertex by vertex in id order: own +step*gb, children's -step*gb)
      // and labels (sweep part - step*icc*gb)
#pragma unroll
      for (int w = 0; w < N; ++w) {
        float a = SBN[w];
#pragma unroll
        for (int v = 0; v < N; ++v) {
          if (v == root) continue;
          const float d = step * GB[v];
          if (v == w) a = a + d;
          else if (par(v) == w) a = a - d;
        }
        SBN[w] = a;
        UB[w] = UB[w] - step_icc * GB[w];
      }
      float SBO[N], UBO[N], DBP[N];
#pragma unroll
      for (int v = 0; v < N; ++v) SBO[v] = UBO[v] = DBP[v] = 0.f;
      // labels: u' = sat(u + cc*((s'_parent - d') - s')), vertex id order
#pragma unroll
      for (int v = 0; v < N; ++v) {
        if (v == root) continue;
        const int p = par(v);
        const float zv = AU[v] + cc * ((sw_sel(BS, p) - BD[v]) - BS[v]);
        const float zb = (zv > 0.0f && zv < 1.0f) ? UB[v] : 0.0f;
        UBO[v] = UBO[v] + zb;
        sw_add(SBN, p, cc * zb);
        DBP[v] = DBP[v] - cc * zb;
        SBN[v] = SBN[v] - cc * zb;
      }
      // sinks, parents before children (pre-order)
#pragma unroll
      for (int k = 0; k < N; ++k) {
        if (PRE) {
          const int v = k;  // ids are in pre-order
          if (is_leaf(v)) {
            const int p = par(v);
            const float yv = (sw_sel(AS, p) - BD[v]) + AU[v] * icc;
            if (yv < 0.0f) continue;
            if (yv > D[v]) {
              DB[v] += (double)SBN[v];
              hit[v] = true;
              continue;
            }
            const float yb = SBN[v];
            sw_add(SBO, p, yb);
            DBP[v] = DBP[v] - yb;
            UBO[v] = UBO[v] + icc * yb;
          } else {
            const float Wb = SBN[v] * T.inv_kids[v];
            if (v != root) {
              sw_add(SBO, par(v), Wb);
              DBP[v] = DBP[v] - Wb;
              UBO[v] = UBO[v] + icc * Wb;
            }
            const float iW = icc * Wb;
#pragma unroll
            for (int w = v + 1; w < N; ++w)  // children follow their parent in pre-order
              if (par(w) == v) {
                SBN[w] = SBN[w] + Wb;
                DBP[w] = DBP[w] + Wb;
                UBO[w] = UBO[w] - iW;
              }
          }
        } else {
          const int v = T.preorder[k];
          const float sbn = sw_sel(SBN, v);
          if (T.n_kids[v] == 0) {
            const int p = T.parent[v];
            const float yv = (sw_sel(AS, p) - sw_sel(BD, v)) + sw_sel(AU, v) * icc;
            if (yv < 0.0f) continue;
            if (yv > sw_sel(D, v)) {
#pragma unroll
              for (int w = 0; w < N; ++w)
                if (w == v) {
                  DB[w] += (double)sbn;
                  hit[w] = true;
                }
              continue;
            }
            sw_add(SBO, p, sbn);
            sw_add(DBP, v, -sbn);
            sw_add(UBO, v, icc * sbn);
          } else {
            const float Wb = sbn * T.inv_kids[v];
            if (v != root) {
              sw_add(SBO, T.parent[v], Wb);
              sw_add(DBP, v, -Wb);
              sw_add(UBO, v, icc * Wb);
            }
            const float iW = icc * Wb;
#pragma unroll
            for (int w = 0; w < N; ++w)
              if (T.parent[w] == v) {
                SBN[w] = SBN[w] + Wb;
                DBP[w] = DBP[w] + Wb;
                UBO[w] = UBO[w] - iW;
              }
          }
        }
      }
      const long long i = v0 + q;
#pragma unroll
      for (int v = 0; v < N; ++v) {
        S.sbo[v * arr + i] = SBO[v];
        if (v != root) {
          S.ubo[v * arr + i] = UBO[v];
          S.dbp[v * arr + i] = DBP[v];
        }
        if (hit[v]) T.Db[v][i] = DB[v];
      }
    }
  }
  __syncthreads();
  // Copies into this CTA's shared memory must have landed before it exits:
  // after a time-out each issuing thread waits (bounded) for the last copy it
  // issued into each stage (nothing is issued after stop_cta).
  if (stop_cta) {
    if (threadIdx.x == 0 && error_flag) atomicOr(error_flag, 2);
    for (int s = 0; s < 2; ++s)
      if (nissued[s]) mbar_wait_bounded(&bars[s], (unsigned)((nissued[s] - 1) & 1), kTmaWaitLimitNs);
  }
}

}  // namespace hmf
