// hmf_adjoint_flow.cuh -- reverse of the flow step of every non-root vertex
// in one launch, TMA-fed (the fused form of adj_grad .. adj_oldflow in
// hmf_adjoint.cuh, same FP32 operations in the same order).
//
// Per voxel and vertex the reverse needs the state before the iteration
// (three flows, sink, parent sink, label, smoothness) and the adjoints of the
// new flows and of the new divergence, and produces the adjoints of the old
// flows and of the gradient-step values g.  Its stencil chain
//   g -> p' -> (|p|, m, adjoint of m -> F2b) -> q -> gb -> old-flow adjoint
// reaches three voxels to the low side and two to the high side, so a CTA
// owns a 32 x 32 (x, y) window with up to 27 x 27 outputs and marches along
// z: lane = column x0-3+lane, warp w holds rows 2w and 2w+1 (y0-3+row) in
// registers; x neighbours move by warp shuffles, y neighbours across a warp
// boundary through small exchange rows in shared memory, z neighbours stay
// in registers.  Per plane k the CTA computes g,
// p' and the total new-flow adjoint t on plane k, m / F2b and q on k-1, gb on
// k-2 and the old-flow adjoints on k-3 (two __syncthreads per plane).  Input
// planes arrive by cp.async.bulk.tensor into mbarrier rings two planes ahead;
// one thread waits for them, before a barrier; every wait is bounded and a
// time-out sets the error flag.  The plane copies are spread over the
// warps' first lanes (one array each, one mbarrier arrival per array), and
// the steady planes of the march -- every stage active, no z boundary near --
// run a copy of the step compiled without those tests.
#pragma once

#include <cuda.h>

#include "hmf_async.cuh"
#include "hmf_types.cuh"

namespace hmf {

constexpr int kAfBoxX = 36;                 // TMA box width (16-byte aligned start, 33 columns used)
constexpr int kAfBoxY = 33;                 // TMA box height (32 rows + the row below for div)
constexpr int kAfPlane = 1216;              // floats per staged plane (36 x 33 padded to 128 bytes)
constexpr int kAfMainArrays = 10;           // px, py, s, c, u, Pbx, Pby, Pbz, dbp, S
constexpr int kAfMainSlots = 3;
constexpr int kAfPzSlots = 4;
// Plane k + kAfMainLead (main ring) and pz of plane k + 1 + kAfPzLead are
// issued in step k after its first CTA barrier; the leads may rise to
// kAfMainSlots and kAfPzSlots - 1.
constexpr int kAfMainLead = 2;
constexpr int kAfPzLead = 2;
constexpr int kAfR = 2;                     // rows per thread
constexpr int kAfWarps = 32 / kAfR;
constexpr int kAfThreads = 32 * kAfWarps;   // 512
constexpr int kAfX = (kAfWarps + 2) * 32;   // exchange row per warp, plus zero rows for warps -1 and 16
constexpr int kAfXPlanes = 11;              // g, p'y[2], ty[2], m, F2b, qy[2], dbo[2]
constexpr int kAfMaxOut = 27;
constexpr int kAfSmemBytes =
    (kAfMainSlots * kAfMainArrays + kAfPzSlots) * kAfPlane * 4 + kAfXPlanes * kAfX * 4 + 64;

struct AdjFlowVertex {  // 64-byte aligned through its CUtensorMap members
  CUtensorMap px, py, pz, s, c, u, smooth;  // state before the iteration
  CUtensorMap pb[2][3];                     // [parity][axis] adjoint of the new flows
  CUtensorMap dbp;                          // adjoint of the new divergence
  float* pb_out[2][3];                      // [parity][axis] adjoint of the old flows
  float* gb;                                // adjoint of g
  double* alpha_grad;
  float alpha;
  int has_smooth;
};

struct AdjFlowParams {
  float step, icc;
  int parity;      // which Pb set is read (the other is written)
  int n_vertices;  // grid.x = n_vertices * items
  const FlowVolume* vols;
  const FlowItem* items;
  int* error_flag;
  unsigned long long wait_limit_ns;  // bound of every copy wait (kTmaWaitLimitNs unless a caller sets it)
};

__global__ void __launch_bounds__(kAfThreads, 1)
adj_flow_tma_kernel(const AdjFlowVertex* __restrict__ vertices, const AdjFlowParams fp) {
  extern __shared__ __align__(1024) unsigned char af_raw[];
  float* mslots = reinterpret_cast<float*>(af_raw);                      // [3][10][1216]
  float* zslots = mslots + kAfMainSlots * kAfMainArrays * kAfPlane;      // [4][1216]
  float* xp = zslots + kAfPzSlots * kAfPlane;                            // [11][18][32]
  uint64_t* mbars = reinterpret_cast<uint64_t*>(xp + kAfXPlanes * kAfX); // [3]
  uint64_t* zbars = mbars + kAfMainSlots;                                // [4]
  uint64_t* stall_bar = zbars + kAfPzSlots;                              // [1] never completed (a requested stall)
  // exchange rows: *_L = the last row of each warp (read by the next warp as
  // its y-1 neighbour), *_F = the first row (read by the previous warp as y+1)
  float* XG_L = xp;
  float* XPPY_F = xp + 1 * kAfX;  // [2] by plane parity
  float* XTY_F = xp + 3 * kAfX;   // [2]
  float* XM_L = xp + 5 * kAfX;
  float* XF_L = xp + 6 * kAfX;
  float* XQY_F = xp + 7 * kAfX;   // [2]
  float* XD_L = xp + 9 * kAfX;    // [2]
  __shared__ int abort_cta, stall_cta;
  __shared__ int stop;
  __shared__ double red[kAfWarps];

  const int nv = fp.n_vertices;
  const FlowItem item = fp.items[blockIdx.x / nv];
  const FlowVolume FV = fp.vols[item.vol];
  const Geometry G = FV.G;
  const AdjFlowVertex* V = vertices + (size_t)item.vol * nv + (blockIdx.x % nv);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned FULL = 0xffffffffu;
  const int ocols = FV.out_x, orows = FV.out_y;
  const int x0 = (item.tile % FV.tiles_x) * ocols;
  const int y0 = (item.tile / FV.tiles_x) * orows;
  const int xs = ((x0 + 1) / 4) * 4 - 4;  // x0 - 3 rounded down to a multiple of 4 (x0 >= 0)
  const int off = (x0 - 3) - xs;           // 0..3
  const int x = x0 - 3 + lane;
  const int zs = item.zc * FV.zchunk;
  const int ze = min(zs + FV.zchunk, G.vz);
  const int kstart = max(zs - 3, 0);
  const int kend = ze + 2;
  const int kA_end = min(ze + 1, G.vz - 1);   // last plane whose g is computed
  const int kpz_end = min(ze + 2, G.vz - 1);  // its divergence reads pz of the next plane
  const int par = fp.parity;
  const float step = fp.step, icc = fp.icc;
  const bool has_s = V->has_smooth != 0;
  const int narr = has_s ? 10 : 9;
  const float alpha = V->alpha;
  float* const ox = V->pb_out[par][0];
  float* const oy = V->pb_out[par][1];
  float* const oz = V->pb_out[par][2];
  float* const ogb = V->gb;
  const bool xin = x >= 0 && x < G.vx, xpos = x > 0, xnl = x != G.vx - 1;
  const bool xown = xin && lane >= 3 && lane < 3 + ocols;
  bool rin[kAfR], ypos[kAfR], ynl[kAfR], rown[kAfR];
  long long rowoff[kAfR];
  int si[kAfR];
#pragma unroll
  for (int j = 0; j < kAfR; ++j) {
    const int row = warp * kAfR + j;
    const int y = y0 - 3 + row;
    rin[j] = xin && y >= 0 && y < G.vy;
    ypos[j] = y > 0;
    ynl[j] = y != G.vy - 1;
    rown[j] = rin[j] && xown && row >= 3 && row < 3 + orows;
    rowoff[j] = (long long)y * G.pitch + x;
    si[j] = row * kAfBoxX + off + lane;  // element in a staged plane
  }
  const int xw = (warp + 1) * 32 + lane;  // this warp's entry in an exchange row

  if (threadIdx.x == 0) {
    const int flag = fp.error_flag ? *(volatile int*)fp.error_flag : 0;
    abort_cta = flag & 2;
    stall_cta = take_stall_request(fp.error_flag, flag);
    if (smem_addr(af_raw) & 127) {  // TMA destinations must be 128-byte aligned
      abort_cta = 1;
      if (fp.error_flag) atomicOr(fp.error_flag, 4);
    }
    for (int s = 0; s < kAfMainSlots; ++s) mbar_init(&mbars[s], (unsigned)narr);
    for (int s = 0; s < kAfPzSlots; ++s) mbar_init(&zbars[s], 1);
    mbar_init(stall_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    stop = 0;
  }
  // exchange rows of warps -1 and 16 are read as zeros (never written)
  for (int i = threadIdx.x; i < kAfXPlanes * kAfX; i += kAfThreads) xp[i] = 0.f;
  __syncthreads();
  if (abort_cta) return;

  auto mslot = [&](int p) { return mslots + ((p - kstart) % kAfMainSlots) * (kAfMainArrays * kAfPlane); };
  auto zslot = [&](int p) { return zslots + ((p - kstart) % kAfPzSlots) * kAfPlane; };
  // Array a of plane p into the main ring (px, py, s, c, u, Pb x/y/z, dbp, S):
  // one thread per array, each with its own expect_tx.
  auto main_map = [&](int a) -> const CUtensorMap* {
    return a < 5 ? &V->px + (a < 2 ? a : a + 1) : a < 8 ? &V->pb[par][a - 5] : a == 8 ? &V->dbp : &V->smooth;
  };
  auto issue_main_array = [&](int p, int a, const CUtensorMap* map) {
    uint64_t* bar = &mbars[(p - kstart) % kAfMainSlots];
    mbar_expect_tx(bar, (unsigned)(kAfBoxX * kAfBoxY * 4));
    tma_load_plane(mslot(p) + a * kAfPlane, map, xs, y0 - 3, p, bar);
  };
  const CUtensorMap* const warp_map = main_map(warp < narr ? warp : 0);
  auto issue_pz = [&](int p) {  // one thread
    uint64_t* bar = &zbars[(p - kstart) % kAfPzSlots];
    mbar_expect_tx(bar, (unsigned)(kAfBoxX * kAfBoxY * 4));
    tma_load_plane(zslot(p), &V->pz, xs, y0 - 3, p, bar);
  };
  // Thread 0 alone waits for the planes a step reads, just before a CTA
  // barrier that precedes the reads (the barrier extends its acquire to every
  // thread).  A wait that runs out raises `stop`, read by all after the
  // barrier: the CTA leaves the march, drains its copies and reports.
  auto wait0 = [&](uint64_t* bar, unsigned parity) {  // thread 0 only
    if (stop) return;
    if (!mbar_wait_bounded(bar, parity, fp.wait_limit_ns)) stop = 1;
  };
  int k_stop = -1;  // the step at which the march stopped (-1: it ran to the end)
  auto wait_main0 = [&](int p) {
    wait0(&mbars[(p - kstart) % kAfMainSlots], (unsigned)(((p - kstart) / kAfMainSlots) & 1));
  };
  auto wait_pz0 = [&](int p) {
    wait0(&zbars[(p - kstart) % kAfPzSlots], (unsigned)(((p - kstart) / kAfPzSlots) & 1));
  };
  // Lane 0 of warp a issues every copy of main-ring array a, lane 0 of the
  // last warp every z-flow copy; each first acquires the one map it uses.
  if (lane == 0) {
    if (warp < narr) {
      tensormap_acquire(warp_map);
      for (int p = kstart; p <= min(kstart + kAfMainLead - 1, kA_end); ++p) issue_main_array(p, warp, warp_map);
    }
    if (warp == kAfWarps - 1) {
      tensormap_acquire(&V->pz);
      for (int p = kstart; p <= min(kstart + kAfPzLead, kpz_end); ++p) issue_pz(p);
    }
  }
  if (threadIdx.x == 0) {
    wait_main0(kstart);
    wait_pz0(kstart);
    if (kstart + 1 < G.vz) wait_pz0(kstart + 1);
    // the failure path on demand: a wait on a barrier that no copy completes
    if (stall_cta) wait0(stall_bar, 0);
  }
  __syncthreads();

  // A window whose 32 x 32 columns / rows lie strictly inside the volume (not
  // on its first or last column / row) needs none of the x / y boundary
  // masks; it runs a copy of the march with them folded away.
  const bool interior = x0 - 3 >= 1 && x0 + 28 <= G.vx - 2 && y0 - 3 >= 1 && y0 + 28 <= G.vy - 2;
  double asum = 0.0;

  auto march = [&](auto tag) {
    constexpr bool INT = decltype(tag)::value;
    const bool vxpos = INT || xpos, vxnl = INT || xnl;
    // carries, one per row of this thread
    float gprev[kAfR], dbp_prev[kAfR];                                        // plane k-1
    float ppx_c[kAfR], ppy_c[kAfR], ppz_c[kAfR], tx_c[kAfR], ty_c[kAfR], tz_c[kAfR], S_c[kAfR];  // k-1
    float m_prev[kAfR], f_prev[kAfR];                                         // plane k-2
    float qx_e[kAfR], qy_e[kAfR], qz_e[kAfR];                                 // q of plane k-2
    float qx_f[kAfR], qy_f[kAfR], qz_f[kAfR];                                 // q of plane k-3
    float dbo_f[kAfR], dbo_ff[kAfR];                                          // dbo of planes k-3, k-4
    float pzn_c[kAfR];
#pragma unroll
    for (int j = 0; j < kAfR; ++j) {
      gprev[j] = dbp_prev[j] = ppx_c[j] = ppy_c[j] = ppz_c[j] = tx_c[j] = ty_c[j] = tz_c[j] = S_c[j] = 0.f;
      m_prev[j] = 1.f;
      f_prev[j] = qx_e[j] = qy_e[j] = qz_e[j] = qx_f[j] = qy_f[j] = qz_f[j] = dbo_f[j] = dbo_ff[j] = pzn_c[j] = 0.f;
    }
    bool have_pz = false;
    const float* cur = mslot(kstart);
    const float* zc = zslot(kstart);
    int msi = 0, zsi = 0;                           // ring positions of plane k
    long long go = (long long)(kstart - 2) * G.plane;  // plane offset of gb outputs (plane k-2)
    long long fo = (long long)(kstart - 3) * G.plane;  // ... of old-flow outputs (plane k-3)

    // returns false when the march stops (a copy wait ran out)
    auto zstep = [&](const int k, auto stag) -> bool {
      constexpr bool ST = decltype(stag)::value;  // a steady plane: every stage, no z boundary near
      const bool doA = ST || k <= kA_end;
      const int kc = k - 1;
      const bool doC = ST || (kc >= kstart && kc <= min(ze, G.vz - 1));
      const int ko = k - 2;
      const bool doE = ST || (ko >= kstart && ko <= ze - 1);
      const int kf = k - 3;
      const bool doF = ST || (kf >= zs && kf < ze);
      const int kb = k & 1;  // exchange-row parity of plane k

      // ---- stage A: g(k) (kern_CalcGradStep on the recomputed divergence)
      float g[kAfR], px[kAfR], py[kAfR], pz[kAfR], Pbx[kAfR], Pby[kAfR], Pbz[kAfR], dbp[kAfR], dbpl[kAfR],
          dbpu[kAfR], Sk[kAfR];
#pragma unroll
      for (int j = 0; j < kAfR; ++j)
        g[j] = px[j] = py[j] = pz[j] = Pbx[j] = Pby[j] = Pbz[j] = dbp[j] = dbpl[j] = dbpu[j] = Sk[j] = 0.f;
      if (doA) {
        const bool has_next = ST || k + 1 < G.vz;
        const int znext = zsi + 1 == kAfPzSlots ? 0 : zsi + 1;
        const float* zn = zslots + znext * kAfPlane;
#pragma unroll
        for (int j = 0; j < kAfR; ++j) {
          const int e = si[j];
          px[j] = cur[e];
          py[j] = cur[kAfPlane + e];
          pz[j] = (ST || have_pz) ? pzn_c[j] : zc[e];
          const float pxr = cur[e + 1];
          const float pyd = cur[kAfPlane + e + kAfBoxX];
          const float pzn = has_next ? zn[e] : 0.f;
          const float sk = cur[2 * kAfPlane + e], c = cur[3 * kAfPlane + e], u = cur[4 * kAfPlane + e];
          Pbx[j] = cur[5 * kAfPlane + e];
          Pby[j] = cur[6 * kAfPlane + e];
          Pbz[j] = cur[7 * kAfPlane + e];
          dbp[j] = cur[8 * kAfPlane + e];
          dbpl[j] = (off + lane) > 0 ? cur[8 * kAfPlane + e - 1] : 0.f;
          dbpu[j] = (warp * kAfR + j) > 0 ? cur[8 * kAfPlane + e - kAfBoxX] : 0.f;
          Sk[j] = has_s ? cur[9 * kAfPlane + e] : 0.f;
          float d = (px[j] + py[j]) + pz[j];
          if (vxnl) d = d - pxr;
          if (INT || ynl[j]) d = d - pyd;
          if (has_next) d = d - pzn;
          const float gv = step * (((sk + d) - c) - u * icc);
          g[j] = (INT || rin[j]) ? gv : 0.f;
          pzn_c[j] = pzn;
        }
        have_pz = has_next;
      }
      XG_L[xw] = g[kAfR - 1];
      __syncthreads();  // (1)
      if (lane == 0) {
        if (warp < narr && k + kAfMainLead <= kA_end) issue_main_array(k + kAfMainLead, warp, warp_map);
        if (warp == kAfWarps - 1 && k + 1 + kAfPzLead <= kpz_end) issue_pz(k + 1 + kAfPzLead);
      }

      // ---- stage B: p'(k) (kern_DescentSpatialFlow) and the total adjoint t(k)
      // of the new flows (incoming plus through the new divergence)
      float ppx_n[kAfR], ppy_n[kAfR], ppz_n[kAfR], tx_n[kAfR], ty_n[kAfR], tz_n[kAfR];
      {
        const float gup = XG_L[xw - 32];
#pragma unroll
        for (int j = 0; j < kAfR; ++j) {
          const float gxm = __shfl_up_sync(FULL, g[j], 1);
          const float gym = j ? g[j > 0 ? j - 1 : 0] : gup;
          const bool vin = doA && (INT || rin[j]);
          const bool vyp = INT || ypos[j];
          ppx_n[j] = (vin && vxpos) ? px[j] - (g[j] - gxm) : 0.f;
          ppy_n[j] = (vin && vyp) ? py[j] - (g[j] - gym) : 0.f;
          ppz_n[j] = (vin && (ST || k > 0)) ? pz[j] - (g[j] - gprev[j]) : 0.f;
          tx_n[j] = vin ? (Pbx[j] + dbp[j]) - (vxpos ? dbpl[j] : 0.f) : 0.f;
          ty_n[j] = vin ? (Pby[j] + dbp[j]) - (vyp ? dbpu[j] : 0.f) : 0.f;
          tz_n[j] = vin ? (Pbz[j] + dbp[j]) - ((ST || k > 0) ? dbp_prev[j] : 0.f) : 0.f;
          if (doA) {
            gprev[j] = g[j];
            dbp_prev[j] = dbp[j];
          }
        }
        XPPY_F[kb * kAfX + xw] = ppy_n[0];
        XTY_F[kb * kAfX + xw] = ty_n[0];
      }

      // ---- stage C: |p|, m(k-1) and the adjoint of the multiplier -> F2b(k-1)
      float m[kAfR], f2b[kAfR];
      {
        const float pdown = XPPY_F[(kb ^ 1) * kAfX + xw + 32];
        const float tdown = XTY_F[(kb ^ 1) * kAfX + xw + 32];
        const bool znl = ST || kc != G.vz - 1;
#pragma unroll
        for (int j = 0; j < kAfR; ++j) {
          const float pxr = __shfl_down_sync(FULL, ppx_c[j], 1);
          const float txr = __shfl_down_sync(FULL, tx_c[j], 1);
          const float pyd = j < kAfR - 1 ? ppy_c[j < kAfR - 1 ? j + 1 : j] : pdown;
          const float tyd = j < kAfR - 1 ? ty_c[j < kAfR - 1 ? j + 1 : j] : tdown;
          m[j] = 1.f;
          f2b[j] = 0.f;
          if (doC && (INT || rin[j])) {
            const bool vyp = INT || ypos[j], vyn = INT || ynl[j];
            float up = ppx_c[j] * ppx_c[j];
            float dn = vxnl ? pxr * pxr : 0.f;
            float F = up + dn;
            up = ppy_c[j] * ppy_c[j];
            dn = vyn ? pyd * pyd : 0.f;
            F = F + (up + dn);
            up = ppz_c[j] * ppz_c[j];
            dn = znl ? ppz_n[j] * ppz_n[j] : 0.f;
            F = F + (up + dn);
            const float h = 0.5f * F;
            const float lim = has_s ? alpha * S_c[j] : alpha;
            if (!(lim > 1.0e-18f && h < (lim * lim) * (1.0f - 0x1p-20f))) {  // else |p| <= lim exactly: m = 1
              const float Fm = sqrtf(h);
              if (Fm > lim) {
                float mb = 0.f;
                if (vxpos) mb = mb + (tx_c[j] * 0.5f) * ppx_c[j];
                if (vxnl) mb = mb + (txr * 0.5f) * pxr;
                if (vyp) mb = mb + (ty_c[j] * 0.5f) * ppy_c[j];
                if (vyn) mb = mb + (tyd * 0.5f) * pyd;
                if (ST || kc > 0) mb = mb + (tz_c[j] * 0.5f) * ppz_c[j];
                if (znl) mb = mb + (tz_n[j] * 0.5f) * ppz_n[j];
                m[j] = lim / Fm;
                f2b[j] = -mb * lim / (4.0f * Fm * Fm * Fm);
                if (rown[j] && (ST || kc >= zs) && kc < ze) asum += (double)(mb / Fm * (has_s ? S_c[j] : 1.0f));
              }
            }
          }
        }
        XM_L[xw] = m[kAfR - 1];
        XF_L[xw] = f2b[kAfR - 1];
      }
      if (threadIdx.x == 0) {  // the planes the next step's stage A reads
        if (k + 1 <= kA_end) wait_main0(k + 1);
        if (k + 2 < G.vz && k + 2 <= kpz_end) wait_pz0(k + 2);
      }
      __syncthreads();  // (2)
      if (stop) {
        k_stop = k;
        return false;
      }

      // ---- stage D: q(k-1), the adjoint of p'
      float qx_n[kAfR], qy_n[kAfR], qz_n[kAfR];
      {
        const float mup = XM_L[xw - 32], fup = XF_L[xw - 32];
#pragma unroll
        for (int j = 0; j < kAfR; ++j) {
          const float mxm = __shfl_up_sync(FULL, m[j], 1);
          const float fxm = __shfl_up_sync(FULL, f2b[j], 1);
          const float mym = j ? m[j > 0 ? j - 1 : 0] : mup;
          const float fym = j ? f2b[j > 0 ? j - 1 : 0] : fup;
          qx_n[j] = qy_n[j] = qz_n[j] = 0.f;
          if (doC && (INT || rin[j])) {
            qx_n[j] = vxpos ? (tx_c[j] * 0.5f) * (m[j] + mxm) + (2.0f * ppx_c[j]) * (f2b[j] + fxm) : 0.f;
            qy_n[j] = (INT || ypos[j]) ? (ty_c[j] * 0.5f) * (m[j] + mym) + (2.0f * ppy_c[j]) * (f2b[j] + fym) : 0.f;
            qz_n[j] = (ST || kc > 0) ? (tz_c[j] * 0.5f) * (m[j] + m_prev[j]) + (2.0f * ppz_c[j]) * (f2b[j] + f_prev[j])
                                      : 0.f;
          }
          if (doC) {
            m_prev[j] = m[j];
            f_prev[j] = f2b[j];
          }
        }
        XQY_F[(kb ^ 1) * kAfX + xw] = qy_n[0];  // plane k-1
      }

      // ---- stage E: gb(k-2), the adjoint of g, and dbo = step * gb
      float dbo[kAfR];
      {
        const float qdown = XQY_F[kb * kAfX + xw + 32];  // plane k-2
#pragma unroll
        for (int j = 0; j < kAfR; ++j) {
          const float qxr = __shfl_down_sync(FULL, qx_e[j], 1);
          const float qyd = j < kAfR - 1 ? qy_e[j < kAfR - 1 ? j + 1 : j] : qdown;
          dbo[j] = 0.f;
          if (doE && (INT || rin[j])) {
            float gb = -((qx_e[j] + qy_e[j]) + qz_e[j]);
            if (vxnl) gb = gb + qxr;
            if (INT || ynl[j]) gb = gb + qyd;
            if (ST || ko != G.vz - 1) gb = gb + qz_n[j];
            dbo[j] = step * gb;
            if (rown[j] && (ST || ko >= zs)) ogb[go + rowoff[j]] = gb;
          }
        }
        XD_L[kb * kAfX + xw] = dbo[kAfR - 1];  // plane k-2
      }

      // ---- stage F: adjoint of the old flows at k-3
      {
        const float dup = XD_L[(kb ^ 1) * kAfX + xw - 32];  // plane k-3
#pragma unroll
        for (int j = 0; j < kAfR; ++j) {
          const float dxl = __shfl_up_sync(FULL, dbo_f[j], 1);
          const float dyu = j ? dbo_f[j > 0 ? j - 1 : 0] : dup;
          if (doF && rown[j]) {
            const long long o = fo + rowoff[j];
            ox[o] = (qx_f[j] + dbo_f[j]) - (vxpos ? dxl : 0.f);
            oy[o] = (qy_f[j] + dbo_f[j]) - ((INT || ypos[j]) ? dyu : 0.f);
            oz[o] = (qz_f[j] + dbo_f[j]) - ((ST || kf > 0) ? dbo_ff[j] : 0.f);
          }
        }
      }

      // ---- rotate carries and ring positions
#pragma unroll
      for (int j = 0; j < kAfR; ++j) {
        ppx_c[j] = ppx_n[j];
        ppy_c[j] = ppy_n[j];
        ppz_c[j] = ppz_n[j];
        tx_c[j] = tx_n[j];
        ty_c[j] = ty_n[j];
        tz_c[j] = tz_n[j];
        S_c[j] = Sk[j];
        qx_f[j] = qx_e[j];
        qy_f[j] = qy_e[j];
        qz_f[j] = qz_e[j];
        qx_e[j] = qx_n[j];
        qy_e[j] = qy_n[j];
        qz_e[j] = qz_n[j];
        dbo_ff[j] = dbo_f[j];
        dbo_f[j] = dbo[j];
      }
      msi = msi + 1 == kAfMainSlots ? 0 : msi + 1;
      zsi = zsi + 1 == kAfPzSlots ? 0 : zsi + 1;
      cur = mslots + msi * (kAfMainArrays * kAfPlane);
      zc = zslots + zsi * kAfPlane;
      go += G.plane;
      fo += G.plane;
      return true;
    };
    const int k_lo = zs + 4, k_hi = min(ze + 1, G.vz - 2);
    int k = kstart;
    bool go_on = true;
    for (; go_on && k <= kend && k < k_lo; ++k) go_on = zstep(k, BoolTag<false>{});
    for (; go_on && k <= k_hi; ++k) go_on = zstep(k, BoolTag<true>{});
    for (; go_on && k <= kend; ++k) go_on = zstep(k, BoolTag<false>{});
  };
  if (interior) march(BoolTag<true>{});
  else march(BoolTag<false>{});
  const bool timed_out = stop != 0;

  // alpha gradient: block sum, one atomic per CTA
  for (int o = 16; o > 0; o >>= 1) asum += __shfl_down_sync(FULL, asum, o);
  if (lane == 0) red[warp] = asum;
  __syncthreads();
  if (warp == 0) {
    double v = lane < kAfWarps ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
    if (lane == 0 && v != 0.0) atomicAdd(V->alpha_grad, v);
  }
  if (timed_out && threadIdx.x == 0) {
    if (fp.error_flag) atomicOr(fp.error_flag, 2);
    // Copies still in flight into this CTA's shared memory must land before
    // it exits.  Up to step k_stop the main ring was filled to plane
    // k_stop + kAfMainLead and the pz ring to k_stop + 1 + kAfPzLead (the
    // initial issue: kstart - 1 + kAfMainLead, kstart + kAfPzLead), each slot
    // holding at most one pending phase: wait for the last plane issued into
    // each slot, with the default bound.
    const int ks = k_stop >= 0 ? k_stop : kstart;
    const int l_main = min(max(ks + kAfMainLead, kstart + kAfMainLead - 1), kA_end);
    const int l_pz = min(max(ks + 1 + kAfPzLead, kstart + kAfPzLead), kpz_end);
    for (int p = max(kstart, l_main - kAfMainSlots + 1); p <= l_main; ++p)
      mbar_wait_bounded(&mbars[(p - kstart) % kAfMainSlots], (unsigned)(((p - kstart) / kAfMainSlots) & 1),
                        kTmaWaitLimitNs);
    for (int p = max(kstart, l_pz - kAfPzSlots + 1); p <= l_pz; ++p)
      mbar_wait_bounded(&zbars[(p - kstart) % kAfPzSlots], (unsigned)(((p - kstart) / kAfPzSlots) & 1),
                        kTmaWaitLimitNs);
  }
}

}  // namespace hmf
