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
// z: thread (lane, row) = column x0-3+lane, row y0-3+row; x neighbours move
// by warp shuffles, y neighbours through small exchange planes in shared
// memory, z neighbours stay in registers.  Per plane k the CTA computes g,
// p' and the total new-flow adjoint t on plane k, m / F2b and q on k-1, gb on
// k-2 and the old-flow adjoints on k-3 (two __syncthreads per plane).  Input
// planes arrive by cp.async.bulk.tensor into mbarrier rings two planes ahead;
// one thread waits for them, before a barrier; every wait is bounded and a
// time-out sets the error flag.
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
constexpr int kAfThreads = 1024;            // 32 rows x 32 lanes
constexpr int kAfX = 34 * 32;               // exchange plane: rows -1 .. 32
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
};

__global__ void __launch_bounds__(kAfThreads, 1)
adj_flow_tma_kernel(const AdjFlowVertex* __restrict__ vertices, const AdjFlowParams fp) {
  extern __shared__ __align__(1024) unsigned char af_raw[];
  float* mslots = reinterpret_cast<float*>(af_raw);                      // [3][10][1216]
  float* zslots = mslots + kAfMainSlots * kAfMainArrays * kAfPlane;      // [4][1216]
  float* xp = zslots + kAfPzSlots * kAfPlane;                            // [11][34][32]
  uint64_t* mbars = reinterpret_cast<uint64_t*>(xp + kAfXPlanes * kAfX); // [3]
  uint64_t* zbars = mbars + kAfMainSlots;                                // [4]
  float* XG = xp;
  float* XPPY = xp + 1 * kAfX;  // [2]
  float* XTY = xp + 3 * kAfX;   // [2]
  float* XM = xp + 5 * kAfX;
  float* XF = xp + 6 * kAfX;
  float* XQY = xp + 7 * kAfX;   // [2]
  float* XD = xp + 9 * kAfX;    // [2]
  __shared__ int abort_cta;
  __shared__ double red[32];

  const int nv = fp.n_vertices;
  const FlowItem item = fp.items[blockIdx.x / nv];
  const FlowVolume FV = fp.vols[item.vol];
  const Geometry G = FV.G;
  const AdjFlowVertex* V = vertices + (size_t)item.vol * nv + (blockIdx.x % nv);
  const int lane = threadIdx.x & 31, row = threadIdx.x >> 5;
  const unsigned FULL = 0xffffffffu;
  const int ocols = FV.out_x, orows = FV.out_y;
  const int x0 = (item.tile % FV.tiles_x) * ocols;
  const int y0 = (item.tile / FV.tiles_x) * orows;
  const int xs = ((x0 + 1) / 4) * 4 - 4;  // x0 - 3 rounded down to a multiple of 4 (x0 >= 0)
  const int off = (x0 - 3) - xs;           // 0..3
  const int x = x0 - 3 + lane, y = y0 - 3 + row;
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
  const bool in = x >= 0 && x < G.vx && y >= 0 && y < G.vy;
  const bool xpos = x > 0, xnl = x != G.vx - 1, ypos = y > 0, ynl = y != G.vy - 1;
  const bool own = in && lane >= 3 && lane < 3 + ocols && row >= 3 && row < 3 + orows;
  const long long rowoff = (long long)y * G.pitch + x;
  const int si = row * kAfBoxX + off + lane;  // this thread's element in a staged plane
  const int xi = (row + 1) * 32 + lane;       // ... in an exchange plane

  if (threadIdx.x == 0) {
    abort_cta = fp.error_flag ? (*(volatile int*)fp.error_flag & 2) : 0;
    if (smem_addr(af_raw) & 127) {  // TMA destinations must be 128-byte aligned
      abort_cta = 1;
      if (fp.error_flag) atomicOr(fp.error_flag, 4);
    }
    for (int s = 0; s < kAfMainSlots; ++s) mbar_init(&mbars[s], 1);
    for (int s = 0; s < kAfPzSlots; ++s) mbar_init(&zbars[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  // exchange planes: rows -1 and 32 are read as zeros (never written)
  for (int i = threadIdx.x; i < kAfXPlanes * kAfX; i += kAfThreads) xp[i] = 0.f;
  __syncthreads();
  if (abort_cta) return;

  auto mslot = [&](int p) { return mslots + ((p - kstart) % kAfMainSlots) * (kAfMainArrays * kAfPlane); };
  auto zslot = [&](int p) { return zslots + ((p - kstart) % kAfPzSlots) * kAfPlane; };
  auto issue_main = [&](int p) {  // thread 0 only
    uint64_t* bar = &mbars[(p - kstart) % kAfMainSlots];
    float* dst = mslot(p);
    mbar_expect_tx(bar, (unsigned)(narr * kAfBoxX * kAfBoxY * 4));
    const int yy = y0 - 3;
    tma_load_plane(dst + 0 * kAfPlane, &V->px, xs, yy, p, bar);
    tma_load_plane(dst + 1 * kAfPlane, &V->py, xs, yy, p, bar);
    tma_load_plane(dst + 2 * kAfPlane, &V->s, xs, yy, p, bar);
    tma_load_plane(dst + 3 * kAfPlane, &V->c, xs, yy, p, bar);
    tma_load_plane(dst + 4 * kAfPlane, &V->u, xs, yy, p, bar);
    tma_load_plane(dst + 5 * kAfPlane, &V->pb[par][0], xs, yy, p, bar);
    tma_load_plane(dst + 6 * kAfPlane, &V->pb[par][1], xs, yy, p, bar);
    tma_load_plane(dst + 7 * kAfPlane, &V->pb[par][2], xs, yy, p, bar);
    tma_load_plane(dst + 8 * kAfPlane, &V->dbp, xs, yy, p, bar);
    if (has_s) tma_load_plane(dst + 9 * kAfPlane, &V->smooth, xs, yy, p, bar);
  };
  auto issue_pz = [&](int p) {  // thread 0 only
    uint64_t* bar = &zbars[(p - kstart) % kAfPzSlots];
    mbar_expect_tx(bar, (unsigned)(kAfBoxX * kAfBoxY * 4));
    tma_load_plane(zslot(p), &V->pz, xs, y0 - 3, p, bar);
  };
  // Thread 0 alone waits for the planes a step reads, just before a CTA
  // barrier that precedes the reads (the barrier extends its acquire to every
  // thread).  A wait that runs out raises `stop`, read by all after the
  // barrier: the CTA leaves the march, drains its copies and reports.
  __shared__ int stop;
  auto wait0 = [&](uint64_t* bar, unsigned parity) {  // thread 0 only
    if (stop) return;
    if (!mbar_wait_bounded(bar, parity, kTmaWaitLimitNs)) stop = 1;
  };
  auto wait_main0 = [&](int p) {
    wait0(&mbars[(p - kstart) % kAfMainSlots], (unsigned)(((p - kstart) / kAfMainSlots) & 1));
  };
  auto wait_pz0 = [&](int p) {
    wait0(&zbars[(p - kstart) % kAfPzSlots], (unsigned)(((p - kstart) / kAfPzSlots) & 1));
  };
  if (threadIdx.x == 0) {
    stop = 0;
    for (int p = kstart; p <= min(kstart + 1, kA_end); ++p) issue_main(p);
    for (int p = kstart; p <= min(kstart + 2, kpz_end); ++p) issue_pz(p);
    wait_main0(kstart);
    wait_pz0(kstart);
    if (kstart + 1 < G.vz) wait_pz0(kstart + 1);
  }
  __syncthreads();

  // A window whose 32 x 32 columns / rows lie strictly inside the volume (not
  // on its first or last column / row) needs none of the x / y boundary
  // masks; it runs a copy of the march with them folded away.
  const bool interior = x0 - 3 >= 1 && x0 + 28 <= G.vx - 2 && y0 - 3 >= 1 && y0 + 28 <= G.vy - 2;
  double asum = 0.0;

  auto march = [&](auto tag) {
    constexpr bool INT = decltype(tag)::value;
    const bool vin = INT || in, vxpos = INT || xpos, vxnl = INT || xnl, vypos = INT || ypos, vynl = INT || ynl;
    // carries (this thread's column)
    float gprev = 0.f, dbp_prev = 0.f;                                                          // plane k-1
    float ppx_c = 0.f, ppy_c = 0.f, ppz_c = 0.f, tx_c = 0.f, ty_c = 0.f, tz_c = 0.f, S_c = 0.f;  // plane k-1
    float m_prev = 1.f, f_prev = 0.f;                                                          // plane k-2
    float qx_e = 0.f, qy_e = 0.f, qz_e = 0.f;                                                  // q of plane k-2
    float qx_f = 0.f, qy_f = 0.f, qz_f = 0.f;                                                  // q of plane k-3
    float dbo_f = 0.f, dbo_ff = 0.f;                                                           // dbo of k-3, k-4
    float pzn_c = 0.f;
    bool have_pz = false;
    const float* cur = mslot(kstart);
    const float* zc = zslot(kstart);
    int msi = 0, zsi = 0;  // ring positions of plane k
    long long go = (long long)(kstart - 2) * G.plane + rowoff;      // gb output at plane k-2
    long long fo = (long long)(kstart - 3) * G.plane + rowoff;      // old-flow output at plane k-3

    for (int k = kstart; k <= kend; ++k) {
      const bool doA = k <= kA_end;
      const int kc = k - 1;
      const bool doC = kc >= kstart && kc <= min(ze, G.vz - 1);
      const int ko = k - 2;
      const bool doE = ko >= kstart && ko <= ze - 1;
      const int kf = k - 3;
      const bool doF = kf >= zs && kf < ze;
      const int kb = k & 1;  // exchange-plane parity of plane k

      // ---- stage A: g(k) (kern_CalcGradStep on the recomputed divergence)
      float g = 0.f, px = 0.f, py = 0.f, pz = 0.f, Pbx = 0.f, Pby = 0.f, Pbz = 0.f, dbp = 0.f, dbpl = 0.f,
            dbpu = 0.f, Sk = 0.f;
      if (doA) {
        const bool has_next = k + 1 < G.vz;
        const int znext = zsi + 1 == kAfPzSlots ? 0 : zsi + 1;
        const float* zn = zslots + znext * kAfPlane;
        px = cur[si];
        py = cur[kAfPlane + si];
        pz = have_pz ? pzn_c : zc[si];
        const float pxr = cur[si + 1];
        const float pyd = cur[kAfPlane + si + kAfBoxX];
        const float pzn = has_next ? zn[si] : 0.f;
        const float sk = cur[2 * kAfPlane + si], c = cur[3 * kAfPlane + si], u = cur[4 * kAfPlane + si];
        Pbx = cur[5 * kAfPlane + si];
        Pby = cur[6 * kAfPlane + si];
        Pbz = cur[7 * kAfPlane + si];
        dbp = cur[8 * kAfPlane + si];
        dbpl = (off + lane) > 0 ? cur[8 * kAfPlane + si - 1] : 0.f;
        dbpu = row > 0 ? cur[8 * kAfPlane + si - kAfBoxX] : 0.f;
        Sk = has_s ? cur[9 * kAfPlane + si] : 0.f;
        float d = (px + py) + pz;
        if (vxnl) d = d - pxr;
        if (vynl) d = d - pyd;
        if (has_next) d = d - pzn;
        const float gv = step * (((sk + d) - c) - u * icc);
        g = vin ? gv : 0.f;
        pzn_c = pzn;
        have_pz = has_next;
      }
      XG[xi] = g;
      __syncthreads();  // (1)
      if (threadIdx.x == 0) {
        if (k + 2 <= kA_end) issue_main(k + 2);
        if (k + 3 <= kpz_end) issue_pz(k + 3);
      }

      // ---- stage B: p'(k) (kern_DescentSpatialFlow) and the total adjoint t(k)
      // of the new flows (incoming plus through the new divergence)
      float ppx_n = 0.f, ppy_n = 0.f, ppz_n = 0.f, tx_n = 0.f, ty_n = 0.f, tz_n = 0.f;
      {
        const float gxm = __shfl_up_sync(FULL, g, 1);
        const float gym = XG[xi - 32];
        if (doA && vin) {
          ppx_n = vxpos ? px - (g - gxm) : 0.f;
          ppy_n = vypos ? py - (g - gym) : 0.f;
          ppz_n = k > 0 ? pz - (g - gprev) : 0.f;
          tx_n = (Pbx + dbp) - (vxpos ? dbpl : 0.f);
          ty_n = (Pby + dbp) - (vypos ? dbpu : 0.f);
          tz_n = (Pbz + dbp) - (k > 0 ? dbp_prev : 0.f);
        }
        if (doA) {
          gprev = g;
          dbp_prev = dbp;
        }
        XPPY[kb * kAfX + xi] = ppy_n;
        XTY[kb * kAfX + xi] = ty_n;
      }

      // ---- stage C: |p|, m(k-1) and the adjoint of the multiplier -> F2b(k-1)
      float m = 1.f, f2b = 0.f;
      {
        const float pxr = __shfl_down_sync(FULL, ppx_c, 1);
        const float txr = __shfl_down_sync(FULL, tx_c, 1);
        const float pyd = XPPY[(kb ^ 1) * kAfX + xi + 32];
        const float tyd = XTY[(kb ^ 1) * kAfX + xi + 32];
        if (doC && vin) {
          const bool znl = kc != G.vz - 1;
          float up = ppx_c * ppx_c;
          float dn = vxnl ? pxr * pxr : 0.f;
          float F = up + dn;
          up = ppy_c * ppy_c;
          dn = vynl ? pyd * pyd : 0.f;
          F = F + (up + dn);
          up = ppz_c * ppz_c;
          dn = znl ? ppz_n * ppz_n : 0.f;
          F = F + (up + dn);
          const float h = 0.5f * F;
          const float lim = has_s ? alpha * S_c : alpha;
          if (!(lim > 1.0e-18f && h < (lim * lim) * (1.0f - 0x1p-20f))) {  // else |p| <= lim exactly: m = 1
            const float Fm = sqrtf(h);
            if (Fm > lim) {
              float mb = 0.f;
              if (vxpos) mb = mb + (tx_c * 0.5f) * ppx_c;
              if (vxnl) mb = mb + (txr * 0.5f) * pxr;
              if (vypos) mb = mb + (ty_c * 0.5f) * ppy_c;
              if (vynl) mb = mb + (tyd * 0.5f) * pyd;
              if (kc > 0) mb = mb + (tz_c * 0.5f) * ppz_c;
              if (znl) mb = mb + (tz_n * 0.5f) * ppz_n;
              m = lim / Fm;
              f2b = -mb * lim / (4.0f * Fm * Fm * Fm);
              if (own && kc >= zs && kc < ze) asum += (double)(mb / Fm * (has_s ? S_c : 1.0f));
            }
          }
        }
        XM[xi] = m;
        XF[xi] = f2b;
      }
      if (threadIdx.x == 0) {  // the planes the next step's stage A reads
        if (k + 1 <= kA_end) wait_main0(k + 1);
        if (k + 2 < G.vz && k + 2 <= kpz_end) wait_pz0(k + 2);
      }
      __syncthreads();  // (2)
      if (stop) break;

      // ---- stage D: q(k-1), the adjoint of p'
      float qx_n = 0.f, qy_n = 0.f, qz_n = 0.f;
      {
        const float mxm = __shfl_up_sync(FULL, m, 1);
        const float fxm = __shfl_up_sync(FULL, f2b, 1);
        const float mym = XM[xi - 32];
        const float fym = XF[xi - 32];
        if (doC && vin) {
          qx_n = vxpos ? (tx_c * 0.5f) * (m + mxm) + (2.0f * ppx_c) * (f2b + fxm) : 0.f;
          qy_n = vypos ? (ty_c * 0.5f) * (m + mym) + (2.0f * ppy_c) * (f2b + fym) : 0.f;
          qz_n = kc > 0 ? (tz_c * 0.5f) * (m + m_prev) + (2.0f * ppz_c) * (f2b + f_prev) : 0.f;
        }
        if (doC) {
          m_prev = m;
          f_prev = f2b;
        }
        XQY[(kb ^ 1) * kAfX + xi] = qy_n;  // plane k-1
      }

      // ---- stage E: gb(k-2), the adjoint of g, and dbo = step * gb
      float dbo = 0.f;
      {
        const float qxr = __shfl_down_sync(FULL, qx_e, 1);
        const float qyd = XQY[kb * kAfX + xi + 32];  // plane k-2
        if (doE && vin) {
          float gb = -((qx_e + qy_e) + qz_e);
          if (vxnl) gb = gb + qxr;
          if (vynl) gb = gb + qyd;
          if (ko != G.vz - 1) gb = gb + qz_n;
          dbo = step * gb;
          if (own && ko >= zs) ogb[go] = gb;
        }
        XD[kb * kAfX + xi] = dbo;  // plane k-2
      }

      // ---- stage F: adjoint of the old flows at k-3
      {
        const float dxl = __shfl_up_sync(FULL, dbo_f, 1);
        const float dyu = XD[(kb ^ 1) * kAfX + xi - 32];  // plane k-3
        if (doF && own) {
          ox[fo] = (qx_f + dbo_f) - (vxpos ? dxl : 0.f);
          oy[fo] = (qy_f + dbo_f) - (vypos ? dyu : 0.f);
          oz[fo] = (qz_f + dbo_f) - (kf > 0 ? dbo_ff : 0.f);
        }
      }

      // ---- rotate carries and ring positions
      ppx_c = ppx_n;
      ppy_c = ppy_n;
      ppz_c = ppz_n;
      tx_c = tx_n;
      ty_c = ty_n;
      tz_c = tz_n;
      S_c = Sk;
      qx_f = qx_e;
      qy_f = qy_e;
      qz_f = qz_e;
      qx_e = qx_n;
      qy_e = qy_n;
      qz_e = qz_n;
      dbo_ff = dbo_f;
      dbo_f = dbo;
      msi = msi + 1 == kAfMainSlots ? 0 : msi + 1;
      zsi = zsi + 1 == kAfPzSlots ? 0 : zsi + 1;
      cur = mslots + msi * (kAfMainArrays * kAfPlane);
      zc = zslots + zsi * kAfPlane;
      go += G.plane;
      fo += G.plane;
    }
  };
  if (interior) march(BoolTag<true>{});
  else march(BoolTag<false>{});
  const bool timed_out = stop != 0;

  // alpha gradient: block sum, one atomic per CTA
  for (int o = 16; o > 0; o >>= 1) asum += __shfl_down_sync(FULL, asum, o);
  if (lane == 0) red[row] = asum;
  __syncthreads();
  if (row == 0) {
    double v = red[lane];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
    if (lane == 0 && v != 0.0) atomicAdd(V->alpha_grad, v);
  }
  if (timed_out) {
    if (fp.error_flag) atomicOr(fp.error_flag, 2);
  }
  if (threadIdx.x == 0) {
    // copies still in flight into this CTA's shared memory must land before it
    // exits: after a time-out wait (bounded) for the last plane of each slot
    if (timed_out) {
      for (int p = max(kstart, kA_end - kAfMainSlots + 1); p <= kA_end; ++p)
        mbar_wait_bounded(&mbars[(p - kstart) % kAfMainSlots], (unsigned)(((p - kstart) / kAfMainSlots) & 1),
                          kTmaWaitLimitNs);
      for (int p = max(kstart, kpz_end - kAfPzSlots + 1); p <= kpz_end; ++p)
        mbar_wait_bounded(&zbars[(p - kstart) % kAfPzSlots], (unsigned)(((p - kstart) / kAfPzSlots) & 1),
                          kTmaWaitLimitNs);
    }
  }
}

}  // namespace hmf
