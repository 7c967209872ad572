// The TMA-fed phase-field step's unit body (internal), shared by the
// single-step kernel (pf_tma.cu) and the batched serving kernel
// (pf_batch.cu).  See pf_tma.cu for the design.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "pfg_mbar.cuh"
#include "pfg_step.cuh"
#include "pfg_warp.cuh"

namespace pfg {

constexpr int kTmaMaxStages = 8;  // ring slots of a batched unit, at most
constexpr int kTmaMaxPlanes = 66;  // planes of a batched unit with its halo (z chunks <= 64)

// Wait for the phase with this parity to complete; false (and *err set to
// PFG_ERR_TIMEOUT) if the wait ran out.
__device__ __forceinline__ bool tma_wait(uint64_t* bar, unsigned parity, int* err,
                                         long long cycles = kWaitCycles) {
  if (mbar_wait_for(bar, parity, cycles)) return true;
  atomicExch(err, PFG_ERR_TIMEOUT);
  return false;
}

// Folded update of one element (see pfg_warp.cuh for the derivation).  The
// per-cell coefficients are k = (A1, B1, C1, W) with W = -C2 = 2 A cl w_x, and
// the anisotropy enters through cn = -cos^2 = m * rcp(-ee):
// C1 + C2 c2 (1 - c2) = C1 + W (cn + cn^2).  ee starts from 1e-30 instead of
// 0, so |e| = 0 gives m = 0, cn = 0 and cn + cn^2 = 0: the value of the
// reference's NaN-to-zero rule (cos^2 = 1), with no clamp.  For any gradient
// that matters, ee >= ~1e-14 and the 1e-30 is far below an ulp; rounding can
// leave m / ee a few ulps above 1, which changes the anisotropy term by a
// relative ~1e-7 instead of clamping it to 0.
struct LapConstsT {
  float ry, rz, nm;
};
template <bool ANISO>
__device__ __forceinline__ float tma_update_elem(const LapConstsT& L, float e, float xm, float xp,
                                                 float ym, float yp, float zm, float zp,
                                                 const float* d, const float4 k) {
  const float lap = fmaf(L.rz, zp + zm, fmaf(L.ry, yp + ym, fmaf(L.nm, e, xp + xm)));
  float u = k.z;
  if constexpr (ANISO) {
    const float ex = xp - xm, ey = yp - ym, ez = zp - zm;
    const float ee = fmaf(ex, ex, fmaf(ey, ey, fmaf(ez, ez, 1e-30f)));
    const float p0 = fmaf(d[0], ex, fmaf(d[1], ey, d[2] * ez));
    const float p1 = fmaf(d[3], ex, fmaf(d[4], ey, d[5] * ez));
    const float q0 = p0 * p0, q1 = p1 * p1;
    const float q2 = ee - q0 - q1;
    float m;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(m) : "f"(q0), "f"(q1), "f"(q2));
    const float cn = m * rcp_approx(-ee);
    u = fmaf(k.w, fmaf(cn, cn, cn), k.z);
  }
  return fmaf(u, lap, e * fmaf(k.y, e * e, k.x));
}

__device__ __forceinline__ float4 tma_fold(const PFConsts& c, const TempCoef& tc, float S) {
  if (tc.liquid != 0.f) return make_float4(0.f, 0.f, 0.f, 0.f);
  const float K = 4.f * S + tc.om2 - 1.f;
  const float clw = tc.cl * c.wx;
  return make_float4(1.f + tc.cg * K, -3.f * tc.cg, clw * (1.f + c.aniso), 2.f * c.aniso * clw);
}

// NC threads (256: two CTAs per SM, or 512: one CTA per SM with a tile
// twice as large).  VEC = 4 when num_oris % 4 == 0 (a cell is whole 16-byte
// vectors); VEC = 2 for other even num_oris with an even nx, even tile
// widths and Neumann x faces: each halo row is then copied from the even
// cell at or before x0 - 1 to the even cell at or after xe + 1, so that every
// bulk copy starts on a 16-byte boundary and moves a multiple of 16 bytes
// without leaving the grid row, and the tile's first cell sits at position
// x0 - base of the staged row.
// Launch plans the planner picks for the reference's large workloads, as
// compile-time constants: FIX = 1 is the 20-orientation case (every
// configuration of the reference uses num_oris = 20; 24 x 10 cell tiles,
// 6 cells x 5 lanes per warp row, 5 rows per warp), FIX = 2 the 30-orientation
// multi-track case (8-byte vectors, 16 x 9 tiles, 2 cells x 15 lanes per warp
// row, 9 rows per warp); both with 4 ring slots and 256 threads.  The host
// launches an instance only for exactly its plan; the tile arithmetic then
// folds into immediate offsets.
template <int FIX> struct FixedPlan;
template <> struct FixedPlan<1> {
  static constexpr int vec = 4, n = 20, tx = 24, ty = 10, rpw = 5, cpw = 6, wx = 4, tpc = 5;
  static constexpr int stages = 4, pitch = (tx + 2) * n, tslot = ((ty + 2) * (tx + 2) + 3) / 4 * 4;
};
template <> struct FixedPlan<2> {
  static constexpr int vec = 2, n = 30, tx = 16, ty = 9, rpw = 9, cpw = 2, wx = 8, tpc = 15;
  // 8-byte-vector rows carry two more cells (the even-aligned copy range)
  static constexpr int stages = 4, pitch = ((tx + 4) * n + 3) / 4 * 4;
  static constexpr int tslot = ((ty + 2) * (tx + 2) + 3) / 4 * 4;
};

// One work unit (a tile x z chunk) of the TMA-fed step.  BATCH: a unit of
// the batched serving kernel (pf_batch.cu), whose persistent CTAs run one
// unit after another: the barriers are invalidated and initialised again
// (reinit), the step's start time is t_batch and the clock is not advanced.
// err: the device error flag of the calling kernel.
template <bool ANISO, int TSRC, int NC, int VEC, int FIX, bool BATCH>
__device__ __forceinline__ void tma_unit(const StepArgs& a, int unit, const float* eta_in,
                                         float* eta_out, double t_batch, bool reinit, int* err) {
  static_assert(VEC == 4 || VEC == 2, "16- or 8-byte vectors");
  using FP = FixedPlan<FIX == 0 ? 1 : FIX>;
  static_assert(FIX == 0 || (FP::vec == VEC && NC == 256), "a fixed plan is a 256-thread plan");
  constexpr bool kFix = FIX != 0;
  // tile plan: compile-time constants under FIX, the launch arguments otherwise
  const int P_n = kFix ? FP::n : a.n, P_pitch = kFix ? FP::pitch : a.pitch;
  const int P_tx = kFix ? FP::tx : a.tx, P_ty = kFix ? FP::ty : a.ty;
  const int P_rpw = kFix ? FP::rpw : a.rpw, P_cpw = kFix ? FP::cpw : a.cpw;
  const int P_wx = kFix ? FP::wx : a.wx, P_tpc = kFix ? FP::tpc : a.tpc;
  const int P_stages = kFix ? FP::stages : a.stages, P_tslot = kFix ? FP::tslot : a.tslot;
  constexpr int kTQ = 3;  // temperature cells staged per thread and plane, at most
  extern __shared__ __align__(128) float smem[];
  const int S = P_stages;
  const int slot_floats = (P_ty + 2) * P_pitch;
  float* eta_s = smem;
  float* T_s = eta_s + (size_t)S * slot_floats;
  float4* cc = reinterpret_cast<float4*>(T_s + (size_t)S * P_tslot);  // [2][ty * tx]
  // the ring's barriers: after the coefficient buffer, or, for the batched
  // kernel's units (whose plans differ), at a fixed static place so that a
  // unit invalidates exactly the barriers the previous one initialised
  __shared__ uint64_t s_full_batch[kTmaMaxStages];
  uint64_t* full = BATCH ? s_full_batch : reinterpret_cast<uint64_t*>(cc + 2 * P_ty * P_tx);

  // ---- work unit
  const int per_plane = a.tiles_x * a.tiles_y;
  const int zi = unit / per_plane;
  const int rem = unit - zi * per_plane;
  const int byi = rem / a.tiles_x;
  const int bxi = rem - byi * a.tiles_x;
  const int x0 = bxi * P_tx, y0 = byi * P_ty;
  const int xe = min(x0 + P_tx, a.nx), ye = min(y0 + P_ty, a.ny);
  const int zb = zi * a.zc, ze = min(zb + a.zc, a.nz);
  const int txv = xe - x0, tyv = ye - y0;
  const bool tile_inner = x0 > 0 && xe < a.nx && y0 > 0 && ye < a.ny;
  const int n = P_n;
  const int nplanes = ze - zb + 2;  // planes zb-1 .. ze
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  __shared__ int s_abort;  // set by any thread whose wait ran out; read after a barrier
  __shared__ double s_t0;
  __shared__ long long s_step;
  __shared__ float s_beam[3];
  __shared__ uint64_t s_never;  // a barrier nothing arrives on (the wait probe)
  if (threadIdx.x == 0) {
    s_abort = 0;
    // expect-tx arrival of warp 0's lane 0 + one cp.async arrival per thread
    if (BATCH && reinit) {  // every phase of the previous unit has completed
      for (int s = 0; s < S; ++s) mbar_inval(&full[s]);
      mbar_inval(&s_never);
    }
    for (int s = 0; s < S; ++s) mbar_init(&full[s], 1 + NC);
    mbar_init(&s_never, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    double t = 0.0;
    if constexpr (TSRC != kTArray) {
      t = BATCH ? t_batch : a.clk_in->t;
      if (!BATCH && unit == 0 && a.clk_out) {
        a.clk_out->t = t + (double)a.dt;
        a.clk_out->step = a.clk_in->step + 1;
      }
    }
    s_t0 = t;
    s_step = (TSRC != kTArray && !BATCH) ? a.clk_in->step : 0;
    if constexpr (TSRC == kTHeat) {
      // beam position and power at mid-step, once per CTA
      laser_at(a.hp, t + 0.5 * (double)a.dt, &s_beam[0], &s_beam[1], &s_beam[2]);
    }
  }
  __syncthreads();
  const double t0 = s_t0;
  // batched units (moving gradient): the temperature of each of the unit's
  // planes, evaluated once (float64 arithmetic is slow on this GPU) rather
  // than by every thread at every plane
  __shared__ float s_Tq[kTmaMaxPlanes];
  if constexpr (BATCH && TSRC == kTQuench) {
    for (int j = threadIdx.x; j < nplanes; j += NC) {
      const double zc = a.q.z_first + (double)(zb - 1 + j) * (double)a.h_z;
      s_Tq[j] = (float)(a.q.T_base + a.q.grad * (zc - a.q.z0) - a.q.grad * a.q.vel * t0);
    }
    __syncthreads();
  }
  // the point source's record for this step (the same for every cell)
  pfg_point_source prec{};
  if constexpr (TSRC == kTPoint) prec = point_record(a.ps, s_step);
  float w_past = 0.f;
  if constexpr (TSRC == kTInterp) w_past = interp_weight(a.t_future, a.dt_coarse, t0 + (double)a.dt);

  // ---- staging: plane j (grid plane zb - 1 + j) into ring slot s.
  // Cells cx0 .. cx1-1 of each row land at positions dst_cell0 ..; cell x0 of
  // the tile is at position pos0.
  int cx0, cx1, dst_cell0, pos0;
  if constexpr (VEC == 4) {
    cx0 = max(x0 - 1, 0);
    cx1 = min(xe + 1, a.nx);
    dst_cell0 = cx0 - (x0 - 1);
    pos0 = 1;
  } else {  // x0, xe and nx even (host checks)
    cx0 = (x0 >= 2) ? x0 - 2 : 0;
    cx1 = (xe < a.nx) ? xe + 2 : a.nx;
    dst_cell0 = 0;
    pos0 = x0 - cx0;
  }
  const bool wrap_left = (x0 == 0) && a.bcx == PFG_BC_PERIODIC;
  const bool wrap_right = (xe == a.nx) && a.bcx == PFG_BC_PERIODIC;
  const int rows = tyv + 2;
  const unsigned row_bytes = (unsigned)((cx1 - cx0) * n * 4);
  const unsigned cell_bytes = (unsigned)(n * 4);
  const unsigned plane_bytes =
      (unsigned)rows * (row_bytes + (wrap_left ? cell_bytes : 0u) + (wrap_right ? cell_bytes : 0u));
  const int tp = P_tx + 2;
  const int gsy = a.nx + 2, gsz = (a.ny + 2) * (a.nx + 2);  // ghosted strides (host checks < 2^31)
  // this thread's temperature cells of a plane: offsets fixed for the unit
  int t_src[kTQ], t_dst[kTQ];
  {
    const int tcols = (TSRC == kTHeat) ? txv + 2 : txv;
    const int tcount = (TSRC == kTHeat) ? rows * tcols : tyv * txv;
    const uint64_t mg = div_magic(tcols);
#pragma unroll
    for (int q = 0; q < kTQ; ++q) {
      const int i = threadIdx.x + q * NC;
      const int r = fast_div(i, mg), c = i - r * tcols;
      const bool ok = (TSRC == kTHeat || TSRC == kTArray) && i < tcount;
      if constexpr (TSRC == kTHeat) {
        t_src[q] = ok ? (y0 + r) * gsy + x0 + c : -1;
        t_dst[q] = r * tp + c;
      } else {
        t_src[q] = ok ? (y0 + r) * a.nx + x0 + c : -1;
        t_dst[q] = (r + 1) * tp + c + 1;
      }
    }
  }
  auto stage = [&](int j, int s) {
    const int pz = zb - 1 + j;
    if (warp == 0) {
      const int gz = bc_index(pz, a.nz, a.bcz);
      float* es = eta_s + (size_t)s * slot_floats;
      if (lane == 0) mbar_arrive_expect_tx(&full[s], plane_bytes);
      __syncwarp();
      for (int r = lane; r < rows; r += 32) {
        const int gy = bc_index(y0 - 1 + r, a.ny, a.bcy);
        const float* src_row = eta_in + ((int64_t)gz * a.ny + gy) * a.nx * n;
        float* dst_row = es + r * P_pitch;
        tma_row(dst_row + dst_cell0 * n, src_row + (int64_t)cx0 * n, row_bytes, &full[s]);
        if (wrap_left) tma_row(dst_row, src_row + (int64_t)(a.nx - 1) * n, cell_bytes, &full[s]);
        if (wrap_right) tma_row(dst_row + (txv + 1) * n, src_row, cell_bytes, &full[s]);
      }
    }
    float* ts = T_s + (size_t)s * P_tslot;
    if constexpr (TSRC == kTHeat) {
      const float* tplane = a.T + (int64_t)(pz + 1) * gsz;
#pragma unroll
      for (int q = 0; q < kTQ; ++q)
        if (t_src[q] >= 0) cp_async<4>(ts + t_dst[q], tplane + t_src[q]);
    } else if constexpr (TSRC == kTArray) {
      if (pz >= 0 && pz < a.nz) {
        const float* tplane = a.T + (int64_t)pz * a.ny * a.nx;
#pragma unroll
        for (int q = 0; q < kTQ; ++q)
          if (t_src[q] >= 0) cp_async<4>(ts + t_dst[q], tplane + t_src[q]);
      }
    }
    cp_async_mbar_arrive_noinc(&full[s]);
  };

  // ---- lane -> (cell, orientation chunk)
  const int tpc = P_tpc;
  const int wxi = warp % P_wx, wyi = warp / P_wx;
  const int lc = lane / tpc, kk = lane - lc * tpc;
  const bool lane_active = lc < P_cpw;
  const int xs = wxi * P_cpw + (lane_active ? lc : 0);
  const bool col_valid = lane_active && xs < txv;
  const int xsp = xs + pos0;  // staged-row position of this lane's cell
  const int i0 = kk * VEC;
  // Neumann along x: the edge cell is its own neighbour
  const int gx = x0 + xs;
  const int off_xm = (gx == 0 && a.bcx == PFG_BC_NEUMANN) ? 0 : -n;
  const int off_xp = (gx == a.nx - 1 && a.bcx == PFG_BC_NEUMANN) ? 0 : n;

  float dl[ANISO ? 6 * VEC : 1];
  if constexpr (ANISO) {
    const int ib = min(i0, n - VEC);
#pragma unroll
    for (int v = 0; v < VEC; ++v)
#pragma unroll
      for (int j = 0; j < 6; ++j) dl[v * 6 + j] = a.dirs[((j / 3) * n + ib + v) * 3 + (j % 3)];
  }
  LapConstsT L;
  L.ry = a.pc.wy / a.pc.wx;
  L.rz = a.pc.wz / a.pc.wx;
  L.nm = -2.f * (1.f + L.ry + L.rz);

  float xl = 0.f, yl = 0.f, Pw = 0.f;
  if constexpr (TSRC == kTHeat) {
    xl = s_beam[0];
    yl = s_beam[1];
    Pw = s_beam[2];
  }

  // ---- this thread's cells for the per-cell work (at most two), fixed per unit
  const int ncell = tyv * txv;
  int c_eoff[2], c_toff[2], c_cc[2], c_g[2], c_hx[2], c_hy[2];
  bool c_ok[2];
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int i = threadIdx.x + q * NC;
    c_ok[q] = i < ncell;
    const int r = c_ok[q] ? i / txv : 0, c = c_ok[q] ? i - r * txv : 0;
    c_eoff[q] = (r + 1) * P_pitch + (c + pos0) * n;
    c_toff[q] = (r + 1) * tp + c + 1;
    c_cc[q] = r * P_tx + c;
    c_hx[q] = x0 + c;
    c_hy[q] = y0 + r;
    c_g[q] = (c_hy[q] + 1) * gsy + c_hx[q] + 1;
  }

  // per-cell coefficients of plane pz (in slot s) -> cc[buf]
  auto cell_coefs = [&](int s, int buf, int pz) {
    const float* es = eta_s + (size_t)s * slot_floats;
    const float* ts = T_s + (size_t)s * P_tslot;
    float4* cb = cc + (size_t)buf * P_ty * P_tx;
    TempCoef plane{};
    if constexpr (TSRC == kTQuench) {
      float Tz;
      if constexpr (BATCH) {
        Tz = s_Tq[pz - zb + 1];
      } else {
        const double zc = a.q.z_first + (double)pz * (double)a.h_z;
        Tz = (float)(a.q.T_base + a.q.grad * (zc - a.q.z0) - a.q.grad * a.q.vel * t0);
      }
      plane = temp_coefficients_fast(a.pc, Tz, a.dt);
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (!c_ok[q]) continue;
      const float* ce = es + c_eoff[q];
      float s0 = 0.f, s1 = 0.f;
      int k = 0;
      if constexpr (VEC == 4) {
        for (; k + 8 <= n; k += 8) {
          const float4 u = *reinterpret_cast<const float4*>(ce + k);
          const float4 v = *reinterpret_cast<const float4*>(ce + k + 4);
          s0 = fmaf(u.x, u.x, fmaf(u.y, u.y, fmaf(u.z, u.z, fmaf(u.w, u.w, s0))));
          s1 = fmaf(v.x, v.x, fmaf(v.y, v.y, fmaf(v.z, v.z, fmaf(v.w, v.w, s1))));
        }
        if (k < n) {
          const float4 u = *reinterpret_cast<const float4*>(ce + k);
          s0 = fmaf(u.x, u.x, fmaf(u.y, u.y, fmaf(u.z, u.z, fmaf(u.w, u.w, s0))));
        }
      } else {  // cells start on 8-byte boundaries only
        for (; k + 4 <= n; k += 4) {
          const float2 u = *reinterpret_cast<const float2*>(ce + k);
          const float2 v = *reinterpret_cast<const float2*>(ce + k + 2);
          s0 = fmaf(u.x, u.x, fmaf(u.y, u.y, s0));
          s1 = fmaf(v.x, v.x, fmaf(v.y, v.y, s1));
        }
        if (k < n) {
          const float2 u = *reinterpret_cast<const float2*>(ce + k);
          s0 = fmaf(u.x, u.x, fmaf(u.y, u.y, s0));
        }
      }
      TempCoef tc;
      if constexpr (TSRC == kTQuench) tc = plane;
      else if constexpr (TSRC == kTPoint)
        tc = temp_coefficients_fast(a.pc, point_source_T(a.ps, prec, c_hx[q], c_hy[q], pz), a.dt);
      else if constexpr (TSRC == kTInterp) {
        const int64_t ti = ((int64_t)pz * a.ny + c_hy[q]) * a.nx + c_hx[q];
        const float Tp = __ldg(a.T + ti), Tf = __ldg(a.T2 + ti);
        tc = temp_coefficients_fast(a.pc, w_past * Tp + (1.f - w_past) * Tf, a.dt);
      }
      else if constexpr (TSRC == kTHeat) {
        // compensated state (a.T_lo set): zeta from the exact pair
        tc = a.T_lo ? temp_coefficients_pair(
                          a.pc, ts[c_toff[q]],
                          __ldg(a.T_lo + (int64_t)(pz + 1) * gsz + c_g[q]), a.dt)
                    : temp_coefficients_fast(a.pc, ts[c_toff[q]], a.dt);
      }
      else tc = temp_coefficients_fast(a.pc, ts[c_toff[q]], a.dt);
      cb[c_cc[q]] = tma_fold(a.pc, tc, s0 + s1);
    }
  };

  // ---- prologue: planes 0 .. S-2 in flight (slot j), wait for planes 0, 1, 2
  int issued = 0;
  for (int j = 0; j < S - 1 && j < nplanes; ++j) { stage(j, j); issued = j + 1; }
  bool ok = true;
  // wait probe: a wait on a barrier that never completes runs out after
  // probe_wait cycles and takes the timeout path below
  if (a.probe_wait > 0) ok = tma_wait(&s_never, 0u, err, a.probe_wait);
  for (int j = 0; j < 3 && ok; ++j) ok = tma_wait(&full[j], 0u, err);  // S >= 4: first phase
  if (ok) cell_coefs(1, 0, zb);
  else s_abort = 1;

  const int64_t plane_elems = (int64_t)a.ny * a.nx * n;
  const int64_t row_elems = (int64_t)a.nx * n;
  const int64_t col_base = ((int64_t)y0 * a.nx + gx) * n + i0;
  const int r_begin = wyi * P_rpw;
  const int r_end = min(r_begin + P_rpw, tyv);
  // ring slots of planes m, m+1, m+2 and the phase parity of plane m+2,
  // rotated each iteration (plane j is in slot j % S)
  int s_prev = 0, s_cur = 1, s_next = 2;
  unsigned ph_next = 0;
  for (int z = zb; z < ze; ++z) {
    const int m = z - zb;
    if (ok) ok = tma_wait(&full[s_next], ph_next, err);
    if (!ok) *(volatile int*)&s_abort = 1;
    __syncthreads();  // cc[m & 1] complete; everyone finished iteration m-1
    if (*(volatile int*)&s_abort) break;  // uniform across the CTA
    // the slot of plane m-1 is free: fill it with plane m+S-1
    if (m + S - 1 < nplanes) {
      stage(m + S - 1, s_prev == 0 ? S - 1 : s_prev - 1);
      issued = m + S;
    }

    if constexpr (TSRC == kTHeat) {
      const float* tp_ = T_s + (size_t)s_prev * P_tslot;
      const float* tc_ = T_s + (size_t)s_cur * P_tslot;
      const float* tn_ = T_s + (size_t)s_next * P_tslot;
      const int zoff = (z + 1) * gsz;
      auto heat_cells = [&](auto faces) {
        constexpr bool F = decltype(faces)::value;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          if (!c_ok[q]) continue;
          const int o = c_toff[q];
          const int idx = zoff + c_g[q];
          const float Tn = heat_cell_update<int, F>(a.hc, tc_[o], tc_[o - 1], tc_[o + 1],
                                                    tc_[o - tp], tc_[o + tp], tp_[o], tn_[o],
                                                    c_hx[q], c_hy[q], z, xl, yl, Pw, a.dt,
                                                    a.T_out, idx, 1, gsy, gsz);
          a.T_out[idx] = Tn;
        }
      };
      // CTA-uniform: no cell of this tile plane touches a domain face.  With a
      // compensated state the heat update has run in its own kernel.
      if (a.T_lo) {
      } else if (tile_inner && z > 0 && z < a.nz - 1) heat_cells(std::false_type{});
      else heat_cells(std::true_type{});
    }
    if (z + 1 < ze) cell_coefs(s_next, (m + 1) & 1, z + 1);

    const float* e_cur = eta_s + (size_t)s_cur * slot_floats;
    const float* e_prev = eta_s + (size_t)s_prev * slot_floats;
    const float* e_next = eta_s + (size_t)s_next * slot_floats;
    const float4* ccb = cc + (size_t)(m & 1) * P_ty * P_tx;
    float* out_row = eta_out + ((int64_t)z * plane_elems + col_base + (int64_t)r_begin * row_elems);
    auto row_out = [&](int r, float* dst, const VecF<VEC>& c, const VecF<VEC>& xm,
                       const VecF<VEC>& xp, const VecF<VEC>& ym, const VecF<VEC>& yp,
                       const VecF<VEC>& zm, const VecF<VEC>& zp) {
      const float4 kc = ccb[r * P_tx + xs];
      VecF<VEC> out;
#pragma unroll
      for (int v = 0; v < VEC; ++v)
        out.v[v] = tma_update_elem<ANISO>(L, c.v[v], xm.v[v], xp.v[v], ym.v[v], yp.v[v], zm.v[v],
                                          zp.v[v], &dl[ANISO ? v * 6 : 0], kc);
      if (col_valid) out.store(dst);
    };
    int r = r_begin;
    // two rows at a time: rows r-1 .. r+2 of the plane are loaded once
    for (; r + 1 < r_end; r += 2, out_row += 2 * row_elems) {
      const int off = (r + 1) * P_pitch + xsp * n + i0;
      const int off2 = off + P_pitch;
      VecF<VEC> ym, c, c2, yp2, xm, xp, xm2, xp2, zm, zp, zm2, zp2;
      ym.load(e_cur + off - P_pitch);
      c.load(e_cur + off);
      c2.load(e_cur + off2);
      yp2.load(e_cur + off2 + P_pitch);
      xm.load(e_cur + off + off_xm);
      xp.load(e_cur + off + off_xp);
      xm2.load(e_cur + off2 + off_xm);
      xp2.load(e_cur + off2 + off_xp);
      zm.load(e_prev + off);
      zp.load(e_next + off);
      zm2.load(e_prev + off2);
      zp2.load(e_next + off2);
      row_out(r, out_row, c, xm, xp, ym, c2, zm, zp);
      row_out(r + 1, out_row + row_elems, c2, xm2, xp2, c, yp2, zm2, zp2);
    }
    if (r < r_end) {
      const int off = (r + 1) * P_pitch + xsp * n + i0;
      VecF<VEC> c, xm, xp, ym, yp, zm, zp;
      c.load(e_cur + off);
      xm.load(e_cur + off + off_xm);
      xp.load(e_cur + off + off_xp);
      ym.load(e_cur + off - P_pitch);
      yp.load(e_cur + off + P_pitch);
      zm.load(e_prev + off);
      zp.load(e_next + off);
      row_out(r, out_row, c, xm, xp, ym, yp, zm, zp);
    }
    // rotate the ring slots
    s_prev = s_cur;
    s_cur = s_next;
    s_next = (s_next + 1 == S) ? 0 : s_next + 1;
    if (s_next == 0) ph_next ^= 1u;
  }
  // drain: copies still in flight must land before the CTA's shared memory is
  // released (in a normal run every issued plane has been waited for
  // already).  After a timeout every slot still gets its full bound.
  cp_async_wait(0);
  if (threadIdx.x == 0) {
    for (int j = max(0, issued - S); j < issued; ++j)
      tma_wait(&full[j % S], (unsigned)((j / S) & 1), err);
  }
}

}  // namespace pfg
