// hmf_flow_tma.cuh -- the flow step of every non-root vertex (gradient step,
// flow descent, |p| <= alpha*S projection, divergence), TMA-fed.
//
// Same arithmetic as flow_kernel in hmf_kernels.cuh (kern_CalcGradStep,
// kern_DescentSpatialFlow, kern_ComputeFlowMag*, kern_Project and
// kern_Divergence of CUDA_hierarchicalmaxflow.cu:233-456, operation by
// operation), organised for sm_103a:
//
//  * A CTA owns a 32 x 32 (x, y) window of one vertex and marches along z.
//    Lane l of every warp is column x0-2+l, so x neighbours move by warp
//    shuffles; warp w holds rows 4w..4w+3 of the window in registers, so y
//    neighbours inside a warp are registers and only the rows on a warp
//    boundary go through shared memory.  z neighbours are carried in
//    registers from plane to plane.
//  * The six or seven input planes a step needs (three flow components, sink,
//    label, parent sink, smoothness) arrive by cp.async.bulk.tensor into a
//    three-slot shared-memory ring completed by mbarriers; plane k+2 is in
//    flight while plane k is computed.  Every mbarrier wait is bounded: on
//    time-out the kernel sets an error flag instead of hanging.
//  * The stencil chain needs two halo columns/rows on the low side and up to
//    two on the high side, so a window yields up to 28 x 27 outputs.
#pragma once

#include <cuda.h>

#include "hmf_async.cuh"
#include "hmf_kernels.cuh"

namespace hmf {

constexpr int kTmaBoxX = 36;   // box width: 16-byte aligned start plus 32 lanes plus 1
constexpr int kTmaRows = 32;   // window rows
constexpr int kTmaPlane = kTmaBoxX * kTmaRows;        // floats per staged array plane
constexpr int kTmaArrays = 7;                          // px, py, pz, sink, label, inc, smooth
constexpr int kTmaSlots = 3;
constexpr int kTmaMaxOutX = 28;
constexpr int kTmaMaxOutY = 27;
constexpr int kTmaThreads = 256;
constexpr int kTmaSmemBytes =
    1024 /* alignment slack */ + kTmaSlots * kTmaArrays * kTmaPlane * 4 + (3 * 256 + 2 * 256) * 4 + 64;

struct FlowVertexTMA {  // 64-byte aligned through its CUtensorMap members
  CUtensorMap flow_in[2][3];  // [parity][axis]: flows read in iterations of that parity
  CUtensorMap sink, label, inc, smooth;
  float* flow_out[2][3];      // [parity][axis]: flows written in iterations of that parity
  float* div;
  float alpha;
  int has_smooth;
};

struct FlowTmaParams {
  float step;
  float icc;
  int zchunk;
  int tiles_x;
  int out_x;  // output columns per window (<= 28)
  int out_y;  // output rows per window (<= 27)
  int parity;
  int pad_;
  int* error_flag;
};

constexpr uint64_t kTmaWaitLimitNs = 500000000ull;  // 0.5 s: far beyond any healthy copy

// Projection multiplier of kern_ComputeFlowMag*: m = |p| > lim ? lim/|p| : 1
// with |p| = sqrtf(h).  For lim > 1e-18 (so that lim*lim is a normal float),
// RN(RN(lim*lim) * (1 - 2^-20)) < lim^2 (1 - 2^-21); when h is below it,
// sqrt(h) < lim, hence RN(sqrt(h)) <= lim and the result is exactly 1 without
// evaluating the square root or the division.  Everything else (tiny lim,
// NaN, infinities) takes the exact path.
__device__ __forceinline__ float projection_multiplier(float h, float lim) {
  if (lim > 1.0e-18f && h < (lim * lim) * (1.0f - 0x1p-20f)) return 1.0f;
  const float F = sqrtf(h);
  return (F > lim) ? lim / F : 1.0f;
}

__global__ void __launch_bounds__(kTmaThreads, 2)
flow_tma_kernel(const FlowVertexTMA* __restrict__ vertices, const Geometry G, const FlowTmaParams fp) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  float* slots = reinterpret_cast<float*>(smem);                 // [3][7][32][36]
  float* xg = slots + kTmaSlots * kTmaArrays * kTmaPlane;        // [8][32]  g(k), row 3 of each warp
  float* xpy = xg + 256;                                          // [8][32]  p'_y(k-1), row 0
  float* xm = xpy + 256;                                          // [8][32]  m(k-1), row 3
  float* xP = xm + 256;                                           // [2][8][32] P_y(k-2), row 0
  uint64_t* bars = reinterpret_cast<uint64_t*>(xP + 512);        // [3]
  __shared__ int abort_cta;

  const FlowVertexTMA* V = vertices + blockIdx.z;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned FULL = 0xffffffffu;
  const int tiles_x = fp.tiles_x;
  const int x0 = (int)(blockIdx.x % tiles_x) * fp.out_x;
  const int y0 = (int)(blockIdx.x / tiles_x) * fp.out_y;
  const int xs = ((x0 + 2) / 4) * 4 - 4;  // x0 - 2 rounded down to a multiple of 4 (x0 >= 0)
  const int off = (x0 - 2) - xs;           // 0..3
  const int x = x0 - 2 + lane;
  const int zs = (int)blockIdx.y * fp.zchunk;
  const int ze = min(zs + fp.zchunk, G.vz);
  const int kstart = max(zs - 2, 0);
  const int kend = ze + 1;
  const int kload_end = min(ze + 2, G.vz - 1);
  const int par = fp.parity;
  const float step = fp.step, icc = fp.icc;
  // per-vertex values read once (the stores below could otherwise alias them)
  const bool has_s = V->has_smooth != 0;
  const int narr = has_s ? 7 : 6;
  const float alpha = V->alpha;
  float* const out_x = V->flow_out[par][0];
  float* const out_y = V->flow_out[par][1];
  float* const out_z = V->flow_out[par][2];
  float* const out_d = V->div;
  const bool xin = x >= 0 && x < G.vx;
  const bool xpos = x > 0;
  const bool xnl = x != G.vx - 1;
  const bool xout = lane >= 2 && lane < 2 + fp.out_x && x < G.vx;
  // per-row constants of this thread (rows warp*4 + r of the window)
  bool rin[4], ypos[4], ynl[4], rout[4];
  long long rowoff[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int row = warp * 4 + r;
    const int y = y0 - 2 + row;
    rin[r] = xin && y >= 0 && y < G.vy;
    ypos[r] = y > 0;
    ynl[r] = y != G.vy - 1;
    rout[r] = xout && row >= 2 && row < 2 + fp.out_y && y < G.vy;
    rowoff[r] = (long long)y * G.pitch + x;
  }

  // If a previous launch already timed out waiting for its copies, the whole
  // CTA returns (one read, shared by all threads), so that a broken
  // configuration fails fast instead of slowly.
  if (threadIdx.x == 0) {
    abort_cta = fp.error_flag ? (*(volatile int*)fp.error_flag & 2) : 0;
    for (int s = 0; s < kTmaSlots; ++s) mbar_init(&bars[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (abort_cta) return;

  auto slot_of = [&](int p) { return slots + ((p - kstart) % kTmaSlots) * (kTmaArrays * kTmaPlane); };
  auto issue = [&](int p) {  // thread 0 only
    uint64_t* bar = &bars[(p - kstart) % kTmaSlots];
    float* dst = slot_of(p);
    mbar_expect_tx(bar, (unsigned)(narr * kTmaPlane * 4));
    tma_load_plane(dst + 0 * kTmaPlane, &V->flow_in[par][0], xs, y0 - 2, p, bar);
    tma_load_plane(dst + 1 * kTmaPlane, &V->flow_in[par][1], xs, y0 - 2, p, bar);
    tma_load_plane(dst + 2 * kTmaPlane, &V->flow_in[par][2], xs, y0 - 2, p, bar);
    tma_load_plane(dst + 3 * kTmaPlane, &V->sink, xs, y0 - 2, p, bar);
    tma_load_plane(dst + 4 * kTmaPlane, &V->label, xs, y0 - 2, p, bar);
    tma_load_plane(dst + 5 * kTmaPlane, &V->inc, xs, y0 - 2, p, bar);
    if (has_s) tma_load_plane(dst + 6 * kTmaPlane, &V->smooth, xs, y0 - 2, p, bar);
  };
  bool timed_out = false;
  auto wait_plane = [&](int p) {
    if (timed_out) return;  // results are void already; do not wait again
    const unsigned parity = (unsigned)(((p - kstart) / kTmaSlots) & 1);
    if (!mbar_wait_bounded(&bars[(p - kstart) % kTmaSlots], parity, kTmaWaitLimitNs)) timed_out = true;
  };

  if (threadIdx.x == 0) {
    if (kstart <= kload_end) issue(kstart);
    if (kstart + 1 <= kload_end) issue(kstart + 1);
  }

  // carries, one per row of this thread
  float gprev[4], ppx[4], ppy[4], ppz[4], mprev[4], Px[4], Py[4], Pz[4], Sprev[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    gprev[r] = ppx[r] = ppy[r] = ppz[r] = mprev[r] = Px[r] = Py[r] = Pz[r] = Sprev[r] = 0.f;
  }

  for (int k = kstart; k <= kend; ++k) {
    const bool doA = k <= min(ze + 1, G.vz - 1);                     // g(k), p'(k)
    const int kc = k - 1;
    const bool doC = kc >= max(zs - 1, 0) && kc <= min(ze, G.vz - 1);  // m(k-1), P(k-1)
    const int ko = k - 2;
    const bool doE = ko >= zs && ko < ze;                              // div(k-2), output

    // ---- stage A: g(k) from the staged inputs (kern_CalcGradStep on the
    // divergence kern_Divergence left, recomputed from the stored flows)
    float g[4], rx[4], ry_[4], rz[4], Scur[4];
    if (doA) {
      wait_plane(k);
      const bool has_next = k + 1 < G.vz;
      if (has_next) wait_plane(k + 1);
      const float* cur = slot_of(k);
      const float* nxt = has_next ? slot_of(k + 1) : cur;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int row = warp * 4 + r;
        const int i = row * kTmaBoxX + off + lane;
        const float px = cur[i], py = cur[kTmaPlane + i], pz = cur[2 * kTmaPlane + i];
        const float pxr = cur[i + 1];
        const float pyd = row < kTmaRows - 1 ? cur[kTmaPlane + i + kTmaBoxX] : 0.f;
        const float pzn = nxt[2 * kTmaPlane + i];
        const float sk = cur[3 * kTmaPlane + i], u = cur[4 * kTmaPlane + i], c = cur[5 * kTmaPlane + i];
        Scur[r] = has_s ? cur[6 * kTmaPlane + i] : 0.f;
        float d = (px + py) + pz;
        if (xnl) d = d - pxr;
        if (ynl[r]) d = d - pyd;
        if (has_next) d = d - pzn;
        g[r] = rin[r] ? step * (((sk + d) - c) - u * icc) : 0.f;
        rx[r] = px;
        ry_[r] = py;
        rz[r] = pz;
      }
    } else {
#pragma unroll
      for (int r = 0; r < 4; ++r) g[r] = rx[r] = ry_[r] = rz[r] = Scur[r] = 0.f;
    }
    xg[warp * 32 + lane] = g[3];
    xpy[warp * 32 + lane] = ppy[0];
    xP[((k & 1) * 8 + warp) * 32 + lane] = Py[0];
    __syncthreads();  // (1)
    if (threadIdx.x == 0 && k + 2 <= kload_end) issue(k + 2);

    // ---- stage B: p'(k) (kern_DescentSpatialFlow)
    float npx[4], npy[4], npz[4];
    const float gup = warp ? xg[(warp - 1) * 32 + lane] : 0.f;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const float gxm = __shfl_up_sync(FULL, g[r], 1);
      const float gym = r ? g[r > 0 ? r - 1 : 0] : gup;
      const bool in = doA && rin[r];
      npx[r] = (in && xpos) ? rx[r] - (g[r] - gxm) : 0.f;
      npy[r] = (in && ypos[r]) ? ry_[r] - (g[r] - gym) : 0.f;
      npz[r] = (in && k > 0) ? rz[r] - (g[r] - gprev[r]) : 0.f;
      gprev[r] = g[r];
    }

    // ---- stage C: m(k-1) (kern_ComputeFlowMag*)
    float m[4];
    const float pdown = warp < 7 ? xpy[(warp + 1) * 32 + lane] : 0.f;
    const bool znl = kc != G.vz - 1;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const float pxr = __shfl_down_sync(FULL, ppx[r], 1);
      const float pyd = r < 3 ? ppy[r < 3 ? r + 1 : 3] : pdown;
      float mv = 1.0f;
      if (doC && rin[r]) {
        float up = ppx[r] * ppx[r];
        float dn = xnl ? pxr * pxr : 0.f;
        float F = up + dn;
        up = ppy[r] * ppy[r];
        dn = ynl[r] ? pyd * pyd : 0.f;
        F = F + (up + dn);
        up = ppz[r] * ppz[r];
        dn = znl ? npz[r] * npz[r] : 0.f;
        F = F + (up + dn);
        mv = projection_multiplier(0.5f * F, has_s ? alpha * Sprev[r] : alpha);
      }
      m[r] = mv;
      Sprev[r] = Scur[r];
    }
    xm[warp * 32 + lane] = m[3];
    __syncthreads();  // (2)

    // ---- stage D: P(k-1) (kern_Project)
    float nPx[4], nPy[4], nPz[4];
    const float mup = warp ? xm[(warp - 1) * 32 + lane] : 0.f;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const float mxm = __shfl_up_sync(FULL, m[r], 1);
      const float mym = r ? m[r > 0 ? r - 1 : 0] : mup;
      const bool in = doC && rin[r];
      nPx[r] = (in && xpos) ? (ppx[r] * 0.5f) * (m[r] + mxm) : 0.f;
      nPy[r] = (in && ypos[r]) ? (ppy[r] * 0.5f) * (m[r] + mym) : 0.f;
      nPz[r] = (in && kc > 0) ? (ppz[r] * 0.5f) * (m[r] + mprev[r]) : 0.f;
      if (doC) mprev[r] = m[r];
    }

    // ---- stage E: divergence of P(k-2) (kern_Divergence), store P(k-2) and div(k-2)
    const float Pdown = warp < 7 ? xP[((k & 1) * 8 + warp + 1) * 32 + lane] : 0.f;
    const bool zonl = ko != G.vz - 1;
    const long long zoff = (long long)ko * G.plane;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const float Pxr = __shfl_down_sync(FULL, Px[r], 1);
      const float Pyd = r < 3 ? Py[r < 3 ? r + 1 : 3] : Pdown;
      if (doE && rout[r]) {
        float dv = (Px[r] + Py[r]) + Pz[r];
        if (xnl) dv = dv - Pxr;
        if (ynl[r]) dv = dv - Pyd;
        if (zonl) dv = dv - nPz[r];
        const long long o = zoff + rowoff[r];
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
  }
  if (timed_out) {
    if (fp.error_flag) atomicOr(fp.error_flag, 2);
    // Let copies still in flight into this CTA's shared memory land (bounded)
    // before the CTA exits: the last plane issued into each slot.
    for (int p = max(kstart, kload_end - kTmaSlots + 1); p <= kload_end; ++p)
      mbar_wait_bounded(&bars[(p - kstart) % kTmaSlots], (unsigned)(((p - kstart) / kTmaSlots) & 1),
                        kTmaWaitLimitNs);
  }
}

}  // namespace hmf
