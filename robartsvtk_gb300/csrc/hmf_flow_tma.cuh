// hmf_flow_tma.cuh -- the flow step of every non-root vertex (gradient step,
// flow descent, |p| <= alpha*S projection, divergence), TMA-fed.
//
// Same arithmetic as flow_kernel in hmf_kernels.cuh (kern_CalcGradStep,
// kern_DescentSpatialFlow, kern_ComputeFlowMag*, kern_Project and
// kern_Divergence of CUDA_hierarchicalmaxflow.cu:233-456, operation by
// operation), organised for sm_103a:
//
//  * A CTA owns a 32 x 4W (x, y) window of one vertex (W = 8 or 16 warps)
//    and marches along z.
//    Lane l of every warp is column x0-2+l, so x neighbours move by warp
//    shuffles; warp w holds rows 4w..4w+3 of the window in registers, so y
//    neighbours inside a warp are registers and only the rows on a warp
//    boundary go through shared memory.  z neighbours are carried in
//    registers from plane to plane.
//  * The six or seven input planes a step needs (three flow components, sink,
//    label, parent sink, smoothness) arrive by cp.async.bulk.tensor into
//    shared-memory rings completed by mbarriers, issued two steps before
//    their first use (kTmaMainLead, kTmaPzLead).  Every mbarrier wait is bounded: on time-out the kernel
//    sets an error flag instead of hanging.
//  * The stencil chain needs two halo columns/rows on the low side and up to
//    two (columns) / three (rows) on the high side, so a window yields up to
//    28 x (4W - 5) outputs: 28 x 27 or 28 x 59.
#pragma once

#include <cuda.h>

#include "hmf_async.cuh"
#include "hmf_kernels.cuh"

namespace hmf {

// Projection multiplier of kern_ComputeFlowMag*: m = |p| > lim ? lim/|p| : 1
// with |p| = sqrtf(h).  For lim > 1e-18 (so that lim*lim is a normal float),
// RN(RN(lim*lim) * (1 - 2^-20)) < lim^2 (1 - 2^-21); when h is below it,
// sqrt(h) < lim, hence RN(sqrt(h)) <= lim and the result is exactly 1 without
// evaluating the square root or the division.  Everything else (tiny lim,
// NaN, infinities) takes the exact path.
__device__ __forceinline__ bool projection_is_one(float h, float lim) {
  return lim > 1.0e-18f && h < (lim * lim) * (1.0f - 0x1p-20f);
}

__device__ __forceinline__ float projection_multiplier(float h, float lim) {
  if (lim > 1.0e-18f && h < (lim * lim) * (1.0f - 0x1p-20f)) return 1.0f;
  const float F = sqrtf(h);
  return (F > lim) ? lim / F : 1.0f;
}

// One unit of work: the z-march of one vertex over one work item (a window
// and z chunk of a volume); false when the CTA must stop (an earlier launch
// or this march timed out, or the shared window is misaligned).
// W warps per CTA: the window is 32 columns x 4W rows (FlowTmaShape<W>).
template <int W, bool MULTI>
__device__ __forceinline__ bool flow_tma_unit(const FlowVertexTMA* __restrict__ vertices, const FlowTmaParams& fp,
                                              const int unit_arg, const bool reinit) {
  const int unit = MULTI ? unit_arg : (int)blockIdx.x;
  constexpr int kPlane = FlowTmaShape<W>::kPlane;  // floats per staged array plane
  constexpr int kRows = FlowTmaShape<W>::kRows;
  // Pointers into the shared window are formed by pointer arithmetic only,
  // so the compiler keeps them in the shared address space (32-bit LDS/STS).
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  float* mslots = reinterpret_cast<float*>(smem_raw);            // [3][6][32][36]
  float* zslots = mslots + kTmaMainSlots * kTmaMainArrays * kPlane;  // [4][rows][36]
  float* xg = zslots + kTmaPzSlots * kPlane;                      // [W][32]  g(k), row 3 of each warp
  float* xpy = xg + W * 32;                                       // [W][32]  p'_y(k-1), row 0
  float* xm = xpy + W * 32;                                       // [W][32]  m(k-1), row 3
  float* xP = xm + W * 32;                                        // [2][W][32] P_y(k-2), row 0
  uint64_t* mbars = reinterpret_cast<uint64_t*>(xP + 2 * W * 32);  // [3]
  uint64_t* zbars = mbars + kTmaMainSlots;                        // [4]
  uint64_t* stall_bar = zbars + kTmaPzSlots;                      // [1] never completed (a requested stall)
  __shared__ int abort_cta;
  __shared__ int stop_cta;  // a copy wait ran out: the CTA stops issuing, drains its copies and leaves

  // unit = vertex + n_vertices * item: the vertices of one window run side
  // by side (or one after another in a CTA), so a parent sink and a shared
  // smoothness image read by several of them come from L2.
  const int nv = fp.n_vertices;
  const FlowItem item = fp.items[unit / nv];
  const FlowVolume FV = fp.vols[item.vol];
  const Geometry G = FV.G;
  const FlowVertexTMA* V = vertices + (size_t)item.vol * nv + (unit % nv);
  const int tile = item.tile;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned FULL = 0xffffffffu;
  const int tiles_x = FV.tiles_x;
  const int ocols = FV.out_x, orows = FV.out_y;
  const int x0 = (tile % tiles_x) * ocols;
  const int y0 = (tile / tiles_x) * orows;
  const int xs = ((x0 + 2) / 4) * 4 - 4;  // x0 - 2 rounded down to a multiple of 4 (x0 >= 0)
  const int off = (x0 - 2) - xs;           // 0..3
  const int x = x0 - 2 + lane;
  const int zs = item.zc * FV.zchunk;
  const int ze = min(zs + FV.zchunk, G.vz);
  const int kstart = max(zs - 2, 0);
  const int kend = ze + 1;
  const int kmain_end = min(ze + 1, G.vz - 1);  // last plane whose g is computed
  const int kpz_end = min(ze + 2, G.vz - 1);    // its divergence reads pz of the next plane
  const int par = fp.parity;
  const float step = fp.step, icc = fp.icc;
  // per-vertex values read once (the stores below could otherwise alias them)
  const bool has_s = V->has_smooth != 0;
  const int narr = has_s ? 6 : 5;  // main-ring arrays
  const float alpha = V->alpha;
  float* const out_x = V->flow_out[par][0];
  float* const out_y = V->flow_out[par][1];
  float* const out_z = V->flow_out[par][2];
  float* const out_d = V->div;
  const bool xin = x >= 0 && x < G.vx;
  const bool xpos = x > 0;
  const bool xnl = x != G.vx - 1;
  const bool xout = lane >= 2 && lane < 2 + ocols && x < G.vx;
  // per-row constants of this thread (rows warp*4 + r of the window)
  bool rin[4], ypos[4], ynl[4], rout[4];
  int rowoff[4];  // element offsets within a plane (a volume holds fewer than 2^31 elements)
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int row = warp * 4 + r;
    const int y = y0 - 2 + row;
    rin[r] = xin && y >= 0 && y < G.vy;
    ypos[r] = y > 0;
    ynl[r] = y != G.vy - 1;
    rout[r] = xout && row >= 2 && row < 2 + orows && y < G.vy;
    rowoff[r] = y * G.pitch + x;
  }

  // If a previous launch already timed out waiting for its copies, the whole
  // CTA returns (one read, shared by all threads), so that a broken
  // configuration fails fast instead of slowly.
  __shared__ int stall_cta;
  if (threadIdx.x == 0) {
    const int flag = fp.error_flag ? *(volatile int*)fp.error_flag : 0;
    abort_cta = flag & 2;
    stall_cta = take_stall_request(fp.error_flag, flag);
    // TMA destinations must be 128-byte aligned: refuse to run otherwise.
    if (smem_addr(smem_raw) & 127) {
      abort_cta = 1;
      if (fp.error_flag) atomicOr(fp.error_flag, 4);
    }
    // a later unit of the CTA: the previous march's barriers (every phase
    // complete, every copy landed) are invalidated before they are set up
    // again
    if (MULTI && reinit) {
      for (int s = 0; s < kTmaMainSlots; ++s) mbar_inval(&mbars[s]);
      for (int s = 0; s < kTmaPzSlots; ++s) mbar_inval(&zbars[s]);
      mbar_inval(stall_bar);
    }
    // one arrival per main-ring array: each array's copy is issued (with its
    // own expect_tx) by the lane 0 of its own warp
    for (int s = 0; s < kTmaMainSlots; ++s) mbar_init(&mbars[s], (unsigned)narr);
    for (int s = 0; s < kTmaPzSlots; ++s) mbar_init(&zbars[s], 1);
    mbar_init(stall_bar, 1);
    stop_cta = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (abort_cta) return false;

  auto mslot = [&](int p) { return mslots + ((p - kstart) % kTmaMainSlots) * (kTmaMainArrays * kPlane); };
  auto zslot = [&](int p) { return zslots + ((p - kstart) % kTmaPzSlots) * kPlane; };
  // Array a of plane p into the main ring (a: 0, 1 flows x, y; 2 sink;
  // 3 label; 4 parent sink; 5 smoothness -- the order of FlowVertexTMA's
  // maps).  One thread per array.
  auto main_map = [&](int a) -> const CUtensorMap* { return a < 2 ? &V->flow_in[par][a] : &V->sink + (a - 2); };
  auto issue_main_array = [&](int p, int a, const CUtensorMap* map) {
    uint64_t* bar = &mbars[(p - kstart) % kTmaMainSlots];
    mbar_expect_tx(bar, (unsigned)(kPlane * 4));
    tma_load_plane(mslot(p) + a * kPlane, map, xs, y0 - 2, p, bar);
  };
  const CUtensorMap* const warp_map = main_map(warp < narr ? warp : 0);  // this warp's array in the loop
  auto issue_pz = [&](int p) {  // one thread
    uint64_t* bar = &zbars[(p - kstart) % kTmaPzSlots];
    mbar_expect_tx(bar, (unsigned)(kPlane * 4));
    tma_load_plane(zslot(p), &V->flow_in[par][2], xs, y0 - 2, p, bar);
  };
  // A wait that runs out raises stop_cta before the CTA barrier that follows
  // every step's waits; after that barrier all threads see it, nobody issues
  // another copy, and the march ends.
  bool timed_out = false;
  int k_stop = -1;  // the step at which the march stopped (-1: it ran to the end)
  auto wait_on = [&](uint64_t* bar, unsigned parity) {
    if (timed_out) return;  // results are void already; do not wait again
    if (!mbar_wait_bounded(bar, parity, fp.wait_limit_ns)) {
      timed_out = true;
      *(volatile int*)&stop_cta = 1;
    }
  };

  // Lane 0 of warp a issues every copy of main-ring array a, lane 0 of the
  // last warp every z-flow copy; each first acquires the one map it uses
  // (the acquires run side by side in their warps).
  if (lane == 0) {
    if (warp < narr) {
      tensormap_acquire(warp_map);
      for (int p = kstart; p <= min(kstart + kTmaMainLead - 1, kmain_end); ++p) issue_main_array(p, warp, warp_map);
    }
    if (warp == W - 1) {
      tensormap_acquire(&V->flow_in[par][2]);
      for (int p = kstart; p <= min(kstart + kTmaPzLead, kpz_end); ++p) issue_pz(p);
    }
  }
  // the failure path on demand: a wait on a barrier that no copy completes
  if (threadIdx.x == 0 && stall_cta) wait_on(stall_bar, 0);

  // A window whose 32 x 32 columns/rows all lie strictly inside the volume
  // (not on its first or last column/row) needs none of the x / y boundary
  // masks; it runs a copy of the march with those tests folded away.
  const bool interior = x0 - 2 >= 1 && x0 + 29 <= G.vx - 2 && y0 - 2 >= 1 && y0 + kRows - 3 <= G.vy - 2;

  // The z-march.  Steps k in [zs + 2, min(ze + 1, vz - 2)] are steady: every
  // stage runs and no z boundary is near, so the step is compiled a second
  // time (ST) with those tests folded away; the few steps before and after
  // run the general form.
  auto march = [&](auto tag) {
    constexpr bool INT = decltype(tag)::value;
    // carries, one per row of this thread
    float gprev[4], ppx[4], ppy[4], ppz[4], mprev[4], Px[4], Py[4], Pz[4], Sprev[4], pzn_c[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      gprev[r] = ppx[r] = ppy[r] = ppz[r] = mprev[r] = Px[r] = Py[r] = Pz[r] = Sprev[r] = pzn_c[r] = 0.f;
    }
    bool have_pz = false;  // pzn_c holds pz of plane k (loaded in step k-1)
    // Ring positions of plane k, advanced step by step: slot and phase
    // parity in the main ring (3 slots) and the pz ring (4 slots).
    int rmi = 0, rzi = 0;
    unsigned phm = 0, phz = 0;

    // returns false when the march stops (a copy wait ran out)
    auto zstep = [&](const int k, auto stag) -> bool {
      constexpr bool ST = decltype(stag)::value;
      const bool doA = ST || k <= kmain_end;                                   // g(k), p'(k)
      const int kc = k - 1;
      const bool doC = ST || (kc >= max(zs - 1, 0) && kc <= min(ze, G.vz - 1));  // m(k-1), P(k-1)
      const int ko = k - 2;
      const bool doE = ST || (ko >= zs && ko < ze);                              // div(k-2), output

      // ---- stage A: g(k) from the staged inputs (kern_CalcGradStep on the
      // divergence kern_Divergence left, recomputed from the stored flows)
      float g[4], rx[4], ry_[4], rz[4], Scur[4];
      const int rz1 = rzi == kTmaPzSlots - 1 ? 0 : rzi + 1;  // pz slot of plane k + 1
      if (doA) {
        wait_on(&mbars[rmi], phm);
        const bool has_next = ST || k + 1 < G.vz;
        const bool pz_held = ST || have_pz;
        if (!pz_held) wait_on(&zbars[rzi], phz);
        if (has_next) wait_on(&zbars[rz1], rz1 == 0 ? phz ^ 1u : phz);
        const float* cur = mslots + rmi * (kTmaMainArrays * kPlane);
        const float* zc = zslots + rzi * kPlane;
        const float* zn = has_next ? zslots + rz1 * kPlane : zc;
        float pyv[5];
#pragma unroll
        for (int r = 0; r < 4; ++r) pyv[r] = cur[kPlane + (warp * 4 + r) * kTmaBoxX + off + lane];
        pyv[4] = warp < W - 1 ? cur[kPlane + (warp * 4 + 4) * kTmaBoxX + off + lane] : 0.f;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int i = (warp * 4 + r) * kTmaBoxX + off + lane;
          const float px = cur[i], py = pyv[r];
          const float pz = pz_held ? pzn_c[r] : zc[i];
          const float pxr = cur[i + 1];
          const float pyd = pyv[r + 1];
          const float pzn = zn[i];
          const float sk = cur[2 * kPlane + i], u = cur[3 * kPlane + i], c = cur[4 * kPlane + i];
          Scur[r] = has_s ? cur[5 * kPlane + i] : 0.f;
          float d = (px + py) + pz;
          if (INT || xnl) d = d - pxr;
          if (INT || ynl[r]) d = d - pyd;
          if (has_next) d = d - pzn;
          const float gv = step * (((sk + d) - c) - u * icc);
          g[r] = (INT || rin[r]) ? gv : 0.f;
          rx[r] = px;
          ry_[r] = py;
          rz[r] = pz;
          pzn_c[r] = pzn;
        }
        have_pz = has_next;
      } else {
#pragma unroll
        for (int r = 0; r < 4; ++r) g[r] = rx[r] = ry_[r] = rz[r] = Scur[r] = 0.f;
      }
      xg[warp * 32 + lane] = g[3];
      xpy[warp * 32 + lane] = ppy[0];
      xP[((k & 1) * W + warp) * 32 + lane] = Py[0];
      __syncthreads();  // (1)
      if (stop_cta) {
        k_stop = k;
        return false;
      }
      // the copies ahead, spread over the warps' first lanes: plane
      // k + kTmaMainLead into the main slot that plane k + kTmaMainLead -
      // kTmaMainSlots left (read in stage A at the latest), pz of plane
      // k + 1 + kTmaPzLead into the pz slot of plane k + 1 + kTmaPzLead -
      // kTmaPzSlots (read as zn in an earlier step, or as zc in this one)
      if (lane == 0) {
        if (warp < narr && k + kTmaMainLead <= kmain_end) {
          const int sl = (rmi + kTmaMainLead) % kTmaMainSlots;
          mbar_expect_tx(&mbars[sl], (unsigned)(kPlane * 4));
          tma_load_plane(mslots + sl * (kTmaMainArrays * kPlane) + warp * kPlane, warp_map, xs, y0 - 2,
                         k + kTmaMainLead, &mbars[sl]);
        }
        if (warp == W - 1 && k + 1 + kTmaPzLead <= kpz_end) {
          const int sl = (rzi + 1 + kTmaPzLead) % kTmaPzSlots;
          mbar_expect_tx(&zbars[sl], (unsigned)(kPlane * 4));
          tma_load_plane(zslots + sl * kPlane, &V->flow_in[par][2], xs, y0 - 2, k + 1 + kTmaPzLead, &zbars[sl]);
        }
      }

      // ---- stage B: p'(k) (kern_DescentSpatialFlow)
      float npx[4], npy[4], npz[4];
      const float gup = warp ? xg[(warp - 1) * 32 + lane] : 0.f;
      const bool zpos = ST || k > 0;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const float gxm = __shfl_up_sync(FULL, g[r], 1);
        const float gym = r ? g[r > 0 ? r - 1 : 0] : gup;
        const bool in = doA && (INT || rin[r]);
        npx[r] = (in && (INT || xpos)) ? rx[r] - (g[r] - gxm) : 0.f;
        npy[r] = (in && (INT || ypos[r])) ? ry_[r] - (g[r] - gym) : 0.f;
        npz[r] = (in && zpos) ? rz[r] - (g[r] - gprev[r]) : 0.f;
        gprev[r] = g[r];
      }

      // ---- stage C: m(k-1) (kern_ComputeFlowMag*).  |p|^2 of the four rows
      // is computed without branches so that their chains interleave; the
      // exact square root and division run only where a row's |p| is near or
      // above its bound (projection_multiplier's test), behind one warp vote.
      float m[4], h[4], lim[4];
      bool slow[4];
      const float pdown = warp < W - 1 ? xpy[(warp + 1) * 32 + lane] : 0.f;
      const bool znl = ST || kc != G.vz - 1;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const float pxr = __shfl_down_sync(FULL, ppx[r], 1);
        const float pyd = r < 3 ? ppy[r < 3 ? r + 1 : 3] : pdown;
        float up = ppx[r] * ppx[r];
        float dn = (INT || xnl) ? pxr * pxr : 0.f;
        float F = up + dn;
        up = ppy[r] * ppy[r];
        dn = (INT || ynl[r]) ? pyd * pyd : 0.f;
        F = F + (up + dn);
        up = ppz[r] * ppz[r];
        dn = znl ? npz[r] * npz[r] : 0.f;
        F = F + (up + dn);
        h[r] = 0.5f * F;
        lim[r] = has_s ? alpha * Sprev[r] : alpha;
        slow[r] = doC && (INT || rin[r]) && !projection_is_one(h[r], lim[r]);
        m[r] = 1.0f;
        Sprev[r] = Scur[r];
      }
      if (__any_sync(FULL, slow[0] || slow[1] || slow[2] || slow[3])) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          if (slow[r]) {
            const float Fs = sqrtf(h[r]);
            if (Fs > lim[r]) m[r] = lim[r] / Fs;
          }
        }
      }
      xm[warp * 32 + lane] = m[3];
      __syncthreads();  // (2)

      // ---- stage D: P(k-1) (kern_Project)
      float nPx[4], nPy[4], nPz[4];
      const float mup = warp ? xm[(warp - 1) * 32 + lane] : 0.f;
      const bool kcpos = ST || kc > 0;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const float mxm = __shfl_up_sync(FULL, m[r], 1);
        const float mym = r ? m[r > 0 ? r - 1 : 0] : mup;
        const bool in = doC && (INT || rin[r]);
        nPx[r] = (in && (INT || xpos)) ? (ppx[r] * 0.5f) * (m[r] + mxm) : 0.f;
        nPy[r] = (in && (INT || ypos[r])) ? (ppy[r] * 0.5f) * (m[r] + mym) : 0.f;
        nPz[r] = (in && kcpos) ? (ppz[r] * 0.5f) * (m[r] + mprev[r]) : 0.f;
        if (doC) mprev[r] = m[r];
      }

      // ---- stage E: divergence of P(k-2) (kern_Divergence), store P(k-2) and div(k-2)
      const float Pdown = warp < W - 1 ? xP[((k & 1) * W + warp + 1) * 32 + lane] : 0.f;
      const bool zonl = ST || ko != G.vz - 1;
      const int zoff = ko * (int)G.plane;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const float Pxr = __shfl_down_sync(FULL, Px[r], 1);
        const float Pyd = r < 3 ? Py[r < 3 ? r + 1 : 3] : Pdown;
        float dv = (Px[r] + Py[r]) + Pz[r];
        if (INT || xnl) dv = dv - Pxr;
        if (INT || ynl[r]) dv = dv - Pyd;
        if (zonl) dv = dv - nPz[r];
        if (doE && rout[r]) {
          const int o = zoff + rowoff[r];
          out_x[o] = Px[r];
          out_y[o] = Py[r];
          out_z[o] = Pz[r];
          out_d[o] = dv;
        }
      }

      // ---- rotate carries
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        ppx[r] = npx[r];
        ppy[r] = npy[r];
        ppz[r] = npz[r];
        Px[r] = nPx[r];
        Py[r] = nPy[r];
        Pz[r] = nPz[r];
      }
      if (++rmi == kTmaMainSlots) rmi = 0, phm ^= 1u;
      rzi = rz1;
      if (rzi == 0) phz ^= 1u;
      return true;
    };

    const int k_lo = zs + 2, k_hi = min(ze + 1, G.vz - 2);
    int k = kstart;
    bool go_on = true;
    for (; go_on && k <= kend && k < k_lo; ++k) go_on = zstep(k, BoolTag<false>{});
    for (; go_on && k <= k_hi; ++k) go_on = zstep(k, BoolTag<true>{});
    for (; go_on && k <= kend; ++k) go_on = zstep(k, BoolTag<false>{});
  };
  if (interior) march(BoolTag<true>{});
  else march(BoolTag<false>{});
  if (k_stop >= 0 && threadIdx.x == 0) {
    if (fp.error_flag) atomicOr(fp.error_flag, 2);
    // Copies still in flight into this CTA's shared memory must land before
    // it exits.  Steps before k_stop filled the main ring to plane
    // k_stop - 1 + kTmaMainLead and the pz ring to k_stop + kTmaPzLead (the
    // initial issue: kstart - 1 + kTmaMainLead, kstart + kTmaPzLead), each
    // slot holding at most one pending phase: wait for the last plane issued
    // into each slot, with the default bound.
    const int l_main = min(max(k_stop, kstart) - 1 + kTmaMainLead, kmain_end);
    const int l_pz = min(max(k_stop, kstart) + kTmaPzLead, kpz_end);
    for (int p = max(kstart, l_main - kTmaMainSlots + 1); p <= l_main; ++p)
      mbar_wait_bounded(&mbars[(p - kstart) % kTmaMainSlots],
                        (unsigned)(((p - kstart) / kTmaMainSlots) & 1), kTmaWaitLimitNs);
    for (int p = max(kstart, l_pz - kTmaPzSlots + 1); p <= l_pz; ++p)
      mbar_wait_bounded(&zbars[(p - kstart) % kTmaPzSlots], (unsigned)(((p - kstart) / kTmaPzSlots) & 1),
                        kTmaWaitLimitNs);
  }
  return k_stop < 0;
}

// One unit per CTA (MULTI false, the default plan), or fp.units_per_cta
// consecutive units (the vertices of one window first), one march after
// another: every copy of a march is waited for before it ends, so after a
// CTA barrier the next unit re-initialises the rings' mbarriers and reuses
// the shared memory.  Two instantiations, so that the loop's live values
// cost the single-unit kernel no registers.
template <int W, bool MULTI>
__global__ void __launch_bounds__(FlowTmaShape<W>::kThreads, FlowTmaShape<W>::kCtasPerSm)
flow_tma_kernel(const FlowVertexTMA* __restrict__ vertices, const __grid_constant__ FlowTmaParams fp) {
  // (a grid constant: the march's lambdas refer to fp in place, no local copy)
  if (!MULTI) {
    flow_tma_unit<W, false>(vertices, fp, 0, false);
    return;
  }
  const int total = fp.n_items * fp.n_vertices;
  const int u0 = blockIdx.x * fp.units_per_cta;
  const int u1 = min(u0 + fp.units_per_cta, total);
  for (int unit = u0; unit < u1; ++unit) {
    if (unit > u0) {
      // the rings' generic reads of the last march before the next march's
      // copies (async proxy) write the same shared memory
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
    }
    if (!flow_tma_unit<W, true>(vertices, fp, unit, unit > u0)) break;
  }
}

}  // namespace hmf
