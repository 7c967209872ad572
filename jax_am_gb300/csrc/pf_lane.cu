// Cell-per-lane TMA stencil step: the fast path for num_oris = 20 (every
// configuration of the reference), with 16-byte orientation vectors.
//
// Each thread owns one cell of a TX x TY tile (TX * TY = the CTA's threads:
// one cell per thread) and marches it through a chunk of z planes.  All per-cell work is
// done by the thread that owns the cell, in registers: the sum S of eta^2,
// zeta and the Arrhenius factor, the folded coefficients and the fused heat
// update.  Nothing per cell goes through shared memory, there are no
// shuffles, and all 32 lanes of a warp update cells.
//  * Staging.  Each halo row of a plane tile is one contiguous run of cells in
//    HBM, copied by one cp.async.bulk (TMA) transfer into a ring of plane
//    slots; the ghosted temperature tile goes through 4-byte cp.async copies
//    arriving on the same mbarrier.  Warp 0 issues the copies of a plane right
//    after the per-plane barrier; there is no producer warp.
//  * z in registers.  A thread keeps its own cell's eta (all orientations)
//    of plane z-1 in registers (read when that plane was the centre), so a
//    plane needs from shared memory the cell and its four x/y neighbours in
//    plane z and the cell above (z+1).  The plane below is never read again
//    once it has been the centre, so its slot is refilled one
//    iteration earlier than a stencil that reads z-1 from shared memory.
//  * The orientation loop is unrolled: the rotated cube axes of each
//    orientation are kernel parameters, read as constant-bank operands.
// Every wait is bounded; a wait that runs out sets the device error flag,
// the CTA waits for its copies in flight (each with the full bound) and
// returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "pfg_host.h"
#include "pfg_mbar.cuh"
#include "pfg_step.cuh"

namespace pfg {

__device__ int g_lane_device_error = 0;  // PFG_ERR_TIMEOUT once a bounded wait ran out

__device__ __forceinline__ bool lane_wait(uint64_t* bar, unsigned parity,
                                          long long cycles = kWaitCycles) {
  if (mbar_wait_for(bar, parity, cycles)) return true;
  atomicExch(&g_lane_device_error, PFG_ERR_TIMEOUT);
  return false;
}

// The moving gradient's temperature of plane z at time t
// (solidification/example.py:21-34), in float64 as the reference evaluates it.
__device__ __forceinline__ float quench_T(const StepArgs& a, int z, double t) {
  const double zc = a.q.z_first + (double)z * (double)a.h_z;
  return (float)(a.q.T_base + a.q.grad * (zc - a.q.z0) - a.q.grad * a.q.vel * t);
}

// Folded update of one element (allen_cahn.py:42-51,58,60-85 with the
// Euler step, :106-114).  Per cell, k = (A1, B1, C1, W):
//   eta' = e (A1 + B1 e^2) + (C1 + W (cn + cn^2)) lap'
// with A1 = 1 + cg K, B1 = -3 cg, C1 = cl wx (1 + A), W = 2 A cl wx,
// lap' = (xp + xm) + ry (yp + ym) + rz (zp + zm) - 2 (1 + ry + rz) e, and
// cn = -cos^2 of the smallest angle between the central difference and the
// orientation's cube axes: cos^4 + sin^4 = 1 - 2 c2 (1 - c2) with
// c2 = max_k (d_k . g)^2 / |g|^2 (allen_cahn.py:28-39); the third axis is
// orthogonal to the first two, so (d_2 . g)^2 = |g|^2 - q0 - q1.  |g|^2
// starts from 1e-30, so a zero gradient gives cn = 0: the reference's
// NaN-to-zero rule (c2 = 1 gives the same factor), with no clamp.
struct LaneLap {
  float ry, rz, nm;
};
template <bool ANISO>
__device__ __forceinline__ float lane_elem(const LaneLap& L, float e, float xm, float xp, float ym,
                                           float yp, float zm, float zp, float d00, float d01,
                                           float d02, float d10, float d11, float d12,
                                           const float4& k) {
  const float lap = fmaf(L.rz, zp + zm, fmaf(L.ry, yp + ym, fmaf(L.nm, e, xp + xm)));
  float u = k.z;
  if constexpr (ANISO) {
    const float gx = xp - xm, gy = yp - ym, gz = zp - zm;
    const float ee = fmaf(gx, gx, fmaf(gy, gy, fmaf(gz, gz, 1e-30f)));
    const float p0 = fmaf(d00, gx, fmaf(d01, gy, d02 * gz));
    const float p1 = fmaf(d10, gx, fmaf(d11, gy, d12 * gz));
    const float q0 = p0 * p0, q1 = p1 * p1;
    const float q2 = ee - q0 - q1;
    float m;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(m) : "f"(q0), "f"(q1), "f"(q2));
    const float cn = m * rcp_approx(-ee);
    u = fmaf(k.w, fmaf(cn, cn, cn), k.z);
  }
  return fmaf(u, lap, e * fmaf(k.y, e * e, k.x));
}

// Per-cell folded coefficients from the temperature part and S.
__device__ __forceinline__ float4 lane_fold(const PFConsts& c, const TempCoef& tc, float S) {
  if (tc.liquid != 0.f) return make_float4(0.f, 0.f, 0.f, 0.f);
  const float K = 4.f * S + tc.om2 - 1.f;
  const float clw = tc.cl * c.wx;
  return make_float4(1.f + tc.cg * K, -3.f * tc.cg, clw * (1.f + c.aniso), 2.f * c.aniso * clw);
}

__device__ __forceinline__ float4 lds4(const float* p) {
  return *reinterpret_cast<const float4*>(p);
}

template <int NV>
__device__ __forceinline__ void load_cell(float4 (&v)[NV], const float* p) {
#pragma unroll
  for (int i = 0; i < NV; ++i) v[i] = lds4(p + 4 * i);
}

__device__ __forceinline__ float comp(const float4& v, int q) {
  return q == 0 ? v.x : (q == 1 ? v.y : (q == 2 ? v.z : v.w));
}

// NV: 16-byte vectors per cell (num_oris = 4 NV); NC threads, MINB CTAs per
// SM; TX: tile width (16 or 32; the tile is TX x NC/TX cells); S: ring slots
// (3 or 4); COMP: the fused heat state is compensated (T = T + T_lo,
// double-float update).
//
// Ring: plane j (grid plane zb - 1 + j) sits in slot j % S and its copies
// complete phase (j / S) & 1 of that slot's barrier.  Iteration m (z =
// zb + m) reads plane m + 1 (the x/y neighbours) and plane m + 2 (the cell
// above); plane m was last read in iteration m - 1, so right after the
// barrier that opens iteration m its slot takes plane m + S.
template <int NV, bool ANISO, int TSRC, int NC, int MINB, int TX, int S, bool COMP>
__global__ void __launch_bounds__(NC, MINB) pf_lane_kernel(const __grid_constant__ StepArgs a) {
  static_assert(NC % TX == 0 && NC % 32 == 0, "whole rows, whole warps");
  constexpr int TY = NC / TX;
  constexpr int N = 4 * NV;
  constexpr int TPX = TX + 2, TPY = TY + 2;  // staged tile with its halo
  constexpr int ROWF = TPX * N;               // floats per staged row
  constexpr int SLOTF = TPY * ROWF;           // floats per eta slot
  constexpr int TSLOT = (TPX * TPY + 3) / 4 * 4;
  constexpr bool HEAT = TSRC == kTHeat;
  static_assert(S == 3 || S == 4, "3 or 4 plane slots");
  static_assert(!COMP || HEAT, "the compensated state is the fused heat state");
  extern __shared__ __align__(128) float smem[];
  float* eta_s = smem;
  float* T_s = eta_s + S * SLOTF;
  float* TL_s = T_s + S * TSLOT;  // low parts of the compensated temperature
  uint64_t* full = reinterpret_cast<uint64_t*>(TL_s + (COMP ? S * TSLOT : 0));

  // ---- work unit: (tile, z chunk), z chunk slowest
  const int per_plane = a.tiles_x * a.tiles_y;
  const int zi = blockIdx.x / per_plane;
  const int rem = blockIdx.x - zi * per_plane;
  const int byi = rem / a.tiles_x;
  const int bxi = rem - byi * a.tiles_x;
  const int x0 = bxi * TX, y0 = byi * TY;
  const int xe = min(x0 + TX, a.nx), ye = min(y0 + TY, a.ny);
  const int zb = zi * a.zc, ze = min(zb + a.zc, a.nz);
  const int txv = xe - x0, tyv = ye - y0;
  const bool tile_inner = x0 > 0 && xe < a.nx && y0 > 0 && ye < a.ny;
  const int nplanes = ze - zb + 2;  // planes zb-1 .. ze
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  __shared__ int s_abort;
  __shared__ double s_t0;
  __shared__ long long s_step;
  __shared__ float s_beam[5];  // xl, yl, P and the low parts of xl, yl
  // moving gradient: the temperature of plane z, evaluated by one thread a
  // plane ahead (float64 arithmetic is slow on this GPU), double-buffered
  __shared__ float s_Tq[2];
  __shared__ uint64_t s_never;  // a barrier nothing arrives on (the wait probe)
  if (threadIdx.x == 0) {
    s_abort = 0;
    // expect-tx arrival of warp 0's lane 0 (+ one cp.async arrival per thread)
    for (int s = 0; s < S; ++s) mbar_init(&full[s], 1 + (HEAT ? NC : 0));
    mbar_init(&s_never, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    double t = 0.0;
    if constexpr (TSRC != kTArray) {
      t = a.clk_in->t;
      if (blockIdx.x == 0 && a.clk_out) {
        a.clk_out->t = t + (double)a.dt;
        a.clk_out->step = a.clk_in->step + 1;
      }
    }
    s_t0 = t;
    if constexpr (TSRC == kTQuench) s_Tq[0] = quench_T(a, zb, t);
    s_step = (TSRC != kTArray) ? a.clk_in->step : 0;
    if constexpr (HEAT) {
      // beam centre and power at mid-step; the centre also as double-float
      double xd, yd;
      laser_at_d(a.hp, t + 0.5 * (double)a.dt, &xd, &yd, &s_beam[2]);
      s_beam[0] = (float)xd;
      s_beam[1] = (float)yd;
      s_beam[3] = (float)(xd - (double)s_beam[0]);
      s_beam[4] = (float)(yd - (double)s_beam[1]);
    }
  }
  __syncthreads();
  const double t0 = s_t0;
  pfg_point_source prec{};
  if constexpr (TSRC == kTPoint) prec = point_record(a.ps, s_step);
  float w_past = 0.f;
  if constexpr (TSRC == kTInterp) w_past = interp_weight(a.t_future, a.dt_coarse, t0 + (double)a.dt);

  // ---- staging of plane j into slot j % S: eta rows by warp 0 (TMA), the
  // ghosted temperature tile by every thread (cp.async)
  const int cx0 = max(x0 - 1, 0), cx1 = min(xe + 1, a.nx);
  const int dst_cell0 = cx0 - (x0 - 1);
  const bool wrap_left = (x0 == 0) && a.bcx == PFG_BC_PERIODIC;
  const bool wrap_right = (xe == a.nx) && a.bcx == PFG_BC_PERIODIC;
  const int rows = tyv + 2;
  const unsigned row_bytes = (unsigned)((cx1 - cx0) * N * 4);
  const unsigned cell_bytes = (unsigned)(N * 4);
  const unsigned plane_bytes =
      (unsigned)rows * (row_bytes + (wrap_left ? cell_bytes : 0u) + (wrap_right ? cell_bytes : 0u));
  const int gsy = a.nx + 2, gsz = (a.ny + 2) * (a.nx + 2);  // ghosted strides (host checks < 2^31)
  // this thread's ghosted temperature cells of a staged plane (at most two):
  // offsets from the tile's first ghosted cell and in the slot, or -1
  int t_src[2], t_dst[2];
  if constexpr (HEAT) {
    const int tcols = txv + 2;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int i = threadIdx.x + q * NC;
      const int r = i / tcols, c = i - r * tcols;
      t_src[q] = r < rows ? r * gsy + c : -1;
      t_dst[q] = r * TPX + c;
    }
  }
  auto stage = [&](int j) {
    const int s = j % S;
    const int pz = zb - 1 + j;
    if (warp == 0) {
      const int gz = bc_index(pz, a.nz, a.bcz);
      float* es = eta_s + s * SLOTF;
      if (lane == 0) mbar_arrive_expect_tx(&full[s], plane_bytes);
      __syncwarp();
      if (lane < rows) {
        const int gy = bc_index(y0 - 1 + lane, a.ny, a.bcy);
        const float* src_row = a.eta_in + ((int64_t)gz * a.ny + gy) * a.nx * N;
        float* dst_row = es + lane * ROWF;
        tma_row(dst_row + dst_cell0 * N, src_row + (int64_t)cx0 * N, row_bytes, &full[s]);
        if (wrap_left) tma_row(dst_row, src_row + (int64_t)(a.nx - 1) * N, cell_bytes, &full[s]);
        if (wrap_right) tma_row(dst_row + (txv + 1) * N, src_row, cell_bytes, &full[s]);
      }
    }
    if constexpr (HEAT) {
      float* ts = T_s + s * TSLOT;
      const float* tplane = a.T + (int64_t)(pz + 1) * gsz + (int64_t)y0 * gsy + x0;
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        if (t_src[q] >= 0) {
          cp_async<4>(ts + t_dst[q], tplane + t_src[q]);
          if constexpr (COMP)
            cp_async<4>(TL_s + s * TSLOT + t_dst[q], a.T_lo + (tplane - a.T) + t_src[q]);
        }
      }
      cp_async_mbar_arrive_noinc(&full[s]);
    }
  };

  // ---- this thread's cell
  // a warp owns an 8 x 4 block of cells (rows of 8 lanes): its cells and
  // their neighbours span fewer grains than a 16 x 2 strip, so more of its
  // orientation vectors are exact zeros (1.4 % faster than 16 x 2); a row of
  // 8 lanes at an 80-byte stride reads shared memory without bank conflicts
  const int tr = ((threadIdx.x >> 5) / (TX / 8)) * 4 + ((threadIdx.x & 31) >> 3);
  const int tc = ((threadIdx.x >> 5) % (TX / 8)) * 8 + (threadIdx.x & 7);
  const bool valid = tr < tyv && tc < txv;
  const bool warp_on = ((threadIdx.x >> 5) / (TX / 8)) * 4 < tyv;  // some row of this warp is in the tile
  const int gx = x0 + tc, gy = y0 + tr;
  const int own = (tr + 1) * ROWF + (tc + 1) * N;  // staged offset of the cell
  // Neumann along x: the edge cell is its own neighbour (its halo is not staged)
  const int oxm = (gx == 0 && a.bcx == PFG_BC_NEUMANN) ? 0 : -N;
  const int oxp = (gx == a.nx - 1 && a.bcx == PFG_BC_NEUMANN) ? 0 : N;
  const int town = (tr + 1) * TPX + tc + 1;  // staged temperature offset
  const int g_own = (gy + 1) * gsy + gx + 1;  // ghosted index within a plane
  const int64_t cell0 = (int64_t)gy * a.nx + gx;  // cell index within a plane
  const int64_t plane_cells = (int64_t)a.ny * a.nx;

  LaneLap L;
  L.ry = a.pc.wy / a.pc.wx;
  L.rz = a.pc.wz / a.pc.wx;
  L.nm = -2.f * (1.f + L.ry + L.rz);
  float xl = 0.f, yl = 0.f, Pw = 0.f;
  DF xld{0.f, 0.f}, yld{0.f, 0.f};
  if constexpr (HEAT) {
    xl = s_beam[0];
    yl = s_beam[1];
    Pw = s_beam[2];
    if constexpr (COMP) {
      xld = DF{s_beam[0], s_beam[3]};
      yld = DF{s_beam[1], s_beam[4]};
    }
  }

  // ---- prologue: planes 0 .. S-1 in flight; planes 0, 1, 2 waited for
  int issued = 0;
  for (int j = 0; j < S && j < nplanes; ++j) {
    stage(j);
    issued = j + 1;
  }
  bool ok = true;
  // wait probe: a wait on a barrier that never completes runs out after
  // probe_wait cycles and takes the timeout path
  if (a.probe_wait > 0) ok = lane_wait(&s_never, 0u, a.probe_wait);
  for (int j = 0; j < 3 && ok; ++j) ok = lane_wait(&full[j], 0u);
  if (!ok) s_abort = 1;

  // The cell's eta and temperature of plane z-1 are carried in registers
  // (that plane's slot is refilled while plane z is computed); plane z's come
  // from its slot.  (Unrolling the z loop to rotate register sets instead of
  // copying them makes the loop body overflow the instruction cache.)
  float4 zm[NV], cc[NV];
  float Tzm = 0.f, Tc = 0.f;
  float Lzm = 0.f, Lc = 0.f;  // their low parts (COMP)
  if (ok) {
    load_cell<NV>(zm, eta_s + 0 * SLOTF + own);
    if constexpr (HEAT) Tzm = T_s[0 * TSLOT + town];
    if constexpr (COMP) Lzm = TL_s[0 * TSLOT + town];
  }
  // per-cell temperature array: the value of the next plane is loaded one
  // plane ahead
  float Tnext = 0.f;
  if constexpr (TSRC == kTArray) {
    if (valid) Tnext = __ldg(a.T + (int64_t)zb * plane_cells + cell0);
  }
  float* out = a.eta_out + ((int64_t)zb * plane_cells + cell0) * N;

  for (int z = zb; z < ze; ++z) {
    const int m = z - zb;
    const int s1 = (m + 1) % S, s2 = (m + 2) % S;  // slots of planes z and z + 1
    if (m > 0 && ok) ok = lane_wait(&full[s2], (unsigned)(((m + 2) / S) & 1));
    if (!ok) *(volatile int*)&s_abort = 1;
    __syncthreads();  // everyone finished plane z - 1; the slot of plane m is free
    if (*(volatile int*)&s_abort) break;  // uniform across the CTA
    if (m + S < nplanes) {
      stage(m + S);
      issued = m + S + 1;
    }
    // read in the next iteration, after its barrier
    if constexpr (TSRC == kTQuench)
      if (threadIdx.x == 0 && z + 1 < ze) s_Tq[(m + 1) & 1] = quench_T(a, z + 1, t0);
    const float* e1 = eta_s + s1 * SLOTF;
    const float* e2 = eta_s + s2 * SLOTF;
    load_cell<NV>(cc, e1 + own);
    float Tzp = 0.f, Lzp = 0.f;
    if constexpr (HEAT) {
      Tc = T_s[s1 * TSLOT + town];
      Tzp = T_s[s2 * TSLOT + town];
    }
    if constexpr (COMP) {
      Lc = TL_s[s1 * TSLOT + town];
      Lzp = TL_s[s2 * TSLOT + town];
    }
    if (warp_on) {
      // ---- temperature at the start of the step, and the heat update
      float Tcell;
      if constexpr (HEAT) {
        const float* t1 = T_s + s1 * TSLOT;
        const float Txm = t1[town - 1], Txp = t1[town + 1];
        const float Tym = t1[town - TPX], Typ = t1[town + TPX];
        const int idx = (z + 1) * gsz + g_own;
        const bool face_plane = !(tile_inner && z > 0 && z < a.nz - 1);  // CTA-uniform
        if constexpr (COMP) {
          const float* l1 = TL_s + s1 * TSLOT;
          const DF c{Tc, Lc};
          DF n[6] = {DF{Txm, l1[town - 1]},   DF{Txp, l1[town + 1]}, DF{Tym, l1[town - TPX]},
                     DF{Typ, l1[town + TPX]}, DF{Tzm, Lzm},         DF{Tzp, Lzp}};
          const bool on_face = face_plane && (gx == 0 || gx == a.nx - 1 || gy == 0 ||
                                              gy == a.ny - 1 || z == 0 || z == a.nz - 1);
          const float tmax = fmaxf(fmaxf(fmaxf(Tc, Txm), fmaxf(Txp, Tym)),
                                   fmaxf(fmaxf(Typ, Tzm), Tzp));
          DF Tn = c;
          // warp-uniform choice: DF arithmetic where the temperature is far
          // from ambient or the beam heats the top face
          if (__any_sync(0xffffffffu, valid && (tmax > a.hd.hot || z == a.nz - 1))) {
            if (valid)
              Tn = heat_update_df_accurate(a.hc, a.hd, c, n, gx, gy, z, xld, yld, Pw, a.T_out,
                                           a.T_lo_out, idx, 1, gsy, gsz);
          } else if (__any_sync(0xffffffffu, on_face && valid)) {
            if (valid)
              Tn = heat_update_df_near_ambient<true>(a.hc, c, n, gx, gy, z, xl, yl, Pw, a.dt,
                                                     a.T_out, a.T_lo_out, idx, 1, gsy, gsz);
          } else {
            Tn = heat_update_df_near_ambient<false>(a.hc, c, n, gx, gy, z, xl, yl, Pw, a.dt,
                                                    a.T_out, a.T_lo_out, idx, 1, gsy, gsz);
          }
          if (valid) {
            a.T_out[idx] = Tn.h;
            a.T_lo_out[idx] = Tn.l;
          }
        } else {
          float Tn;
          if (!face_plane)
            Tn = heat_cell_update<int, false>(a.hc, Tc, Txm, Txp, Tym, Typ, Tzm, Tzp, gx, gy, z,
                                              xl, yl, Pw, a.dt, a.T_out, idx, 1, gsy, gsz);
          else if (valid)
            Tn = heat_cell_update<int, true>(a.hc, Tc, Txm, Txp, Tym, Typ, Tzm, Tzp, gx, gy, z, xl,
                                             yl, Pw, a.dt, a.T_out, idx, 1, gsy, gsz);
          else
            Tn = 0.f;
          if (valid) a.T_out[idx] = Tn;
        }
        Tcell = Tc;
      } else if constexpr (TSRC == kTArray) {
        Tcell = Tnext;
        if (valid && z + 1 < ze) Tnext = __ldg(a.T + (int64_t)(z + 1) * plane_cells + cell0);
      } else if constexpr (TSRC == kTQuench) {
        Tcell = s_Tq[m & 1];
      } else if constexpr (TSRC == kTPoint) {
        Tcell = point_source_T(a.ps, prec, gx, gy, z);
      } else {  // kTInterp
        const int64_t ti = (int64_t)z * plane_cells + cell0;
        const float Tp = valid ? __ldg(a.T + ti) : 0.f, Tf = valid ? __ldg(a.T2 + ti) : 0.f;
        Tcell = w_past * Tp + (1.f - w_past) * Tf;
      }
      // ---- per-cell coefficients
      float s_a = 0.f, s_b = 0.f;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const float4 u = cc[v];
        s_a = fmaf(u.x, u.x, fmaf(u.y, u.y, s_a));
        s_b = fmaf(u.z, u.z, fmaf(u.w, u.w, s_b));
      }
      TempCoef tcf;
      if constexpr (COMP) tcf = temp_coefficients_pair(a.pc, Tcell, Lc, a.dt);
      else tcf = temp_coefficients_fast(a.pc, Tcell, a.dt);
      const float4 k = lane_fold(a.pc, tcf, s_a + s_b);
      // the skip below needs finite coefficients in every cell of the warp
      const bool kfinite = __all_sync(0xffffffffu, !valid || (isfinite(k.x) && isfinite(k.y) &&
                                                               isfinite(k.z) && isfinite(k.w)));
      // ---- element updates, one 16-byte vector of orientations at a time
      const float* p1 = e1 + own;
      const float* p2 = e2 + own;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const float4 xm = lds4(p1 + oxm + 4 * v), xp = lds4(p1 + oxp + 4 * v);
        const float4 ym = lds4(p1 - ROWF + 4 * v), yp = lds4(p1 + ROWF + 4 * v);
        const float4 zp = lds4(p2 + 4 * v);
        // Exact zeros: an orientation that is zero (+0.0) at every cell of
        // the warp and at all their six neighbours stays exactly zero
        // (gradient, Laplacian and local term vanish, and the update of +0.0
        // is +0.0 with finite coefficients), so the warp skips its
        // arithmetic.  Grain interiors and the far side of an interface are
        // such zeros.  The test is per pair of orientations (0.8 % faster
        // than per vector of four): the cells' own values (in registers)
        // first, the neighbours only when those are zero across the warp.
        float r[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int h = 0; h < 2; ++h) {  // orientations 4v + 2h, 4v + 2h + 1
          auto pr = [&](const float4& u) {
            return h == 0 ? (__float_as_uint(u.x) | __float_as_uint(u.y))
                          : (__float_as_uint(u.z) | __float_as_uint(u.w));
          };
          bool work = !kfinite || __any_sync(0xffffffffu, (pr(cc[v]) | pr(zm[v])) != 0u);
          if (!work)
            work = __any_sync(0xffffffffu,
                              (pr(xm) | pr(xp) | pr(ym) | pr(yp) | pr(zp)) != 0u);
          if (work)
#pragma unroll
            for (int q = 2 * h; q < 2 * h + 2; ++q) {
              const int o = 4 * v + q;  // orientation
              r[q] = lane_elem<ANISO>(L, comp(cc[v], q), comp(xm, q), comp(xp, q), comp(ym, q),
                                      comp(yp, q), comp(zm[v], q), comp(zp, q),
                                      a.dirs[o * 3 + 0], a.dirs[o * 3 + 1], a.dirs[o * 3 + 2],
                                      a.dirs[(N + o) * 3 + 0], a.dirs[(N + o) * 3 + 1],
                                      a.dirs[(N + o) * 3 + 2], k);
            }
        }
        if (valid) *reinterpret_cast<float4*>(out + 4 * v) = make_float4(r[0], r[1], r[2], r[3]);
      }
    }
    out += plane_cells * N;
    // plane z is the next plane's z - 1
#pragma unroll
    for (int v = 0; v < NV; ++v) zm[v] = cc[v];
    Tzm = Tc;
    Lzm = Lc;
  }
  // drain: copies still in flight must land before the CTA's shared memory is
  // released (in a normal run every issued plane has been waited for
  // already); after a timeout every slot still gets its full bound
  if constexpr (HEAT) cp_async_wait(0);
  if (threadIdx.x == 0) {
    for (int j = max(0, issued - S); j < issued; ++j)
      lane_wait(&full[j % S], (unsigned)((j / S) & 1));
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

constexpr int kLaneNV = 5;   // num_oris = 20
constexpr int kLaneNC = 256;  // threads per CTA: one cell each
constexpr int kLaneCTAs = 2;  // CTAs per SM
constexpr int kLaneTX = 16;   // 16 x 16 tiles
constexpr int kLaneS = 4;    // ring slots

// Shared memory of one CTA: the eta ring, the temperature ring (high and
// low parts), the barriers.
static size_t lane_smem(int n, int tx, int slots) {
  const int ty = kLaneNC / tx;
  const size_t slot = (size_t)(ty + 2) * (tx + 2) * n * 4;
  const size_t tslot = (size_t)(((tx + 2) * (ty + 2) + 3) / 4 * 4) * 4;
  return (size_t)slots * (slot + 2 * tslot) + (size_t)slots * sizeof(uint64_t);
}

bool plan_lane_tiles(int nx, int ny, int nz, int n, int sm_count, int max_smem_per_sm,
                     int max_smem_per_block, int zchunks_override, TilePlan* out) {
  if (n != 4 * kLaneNV) return false;
  // ghosted temperature offsets are 32-bit in this kernel
  if ((int64_t)(nx + 2) * (ny + 2) * (nz + 2) >= ((int64_t)1 << 31)) return false;
  const int tx = kLaneTX, ty = kLaneNC / tx, S = kLaneS;
  const size_t smem = lane_smem(n, tx, S);
  // kLaneCTAs CTAs per SM: the dynamic shared memory plus the static variables and
  // the per-CTA reservation
  if (kLaneCTAs * (smem + 1024 + 128) > (size_t)max_smem_per_sm ||
      smem > (size_t)max_smem_per_block)
    return false;
  TilePlan t{};
  t.vec = 4;
  t.tpc = 1;
  t.tx = tx;
  t.ty = ty;
  t.cpw = 8;        // a warp owns 8 x 4 cells
  t.wx = tx / 8;
  t.rpw = 4;
  t.rs = kLaneNC;
  t.stages = S;
  t.pitch = (tx + 2) * n;
  t.tslot = ((tx + 2) * (ty + 2) + 3) / 4 * 4;
  t.tiles_x = (nx + tx - 1) / tx;
  t.tiles_y = (ny + ty - 1) / ty;
  const long tiles = (long)t.tiles_x * t.tiles_y;
  const long slots_gpu = (long)kLaneCTAs * sm_count;
  // z chunks: a wave of CTAs lasts about (planes per unit + 1/2) plane times
  // (the prologue); pick the chunking with the fewest plane times in all
  int best_zc = nz;
  double best = 1e300;
  for (int zch = 1; zch <= std::max(1, nz / 4); ++zch) {
    const int zc = (nz + zch - 1) / zch;
    const long units = tiles * ((nz + zc - 1) / zc);
    const double cost = (double)((units + slots_gpu - 1) / slots_gpu) * (zc + 0.5);
    if (cost < best - 1e-9) {
      best = cost;
      best_zc = zc;
    }
  }
  if (zchunks_override > 0) best_zc = (nz + std::min(zchunks_override, nz) - 1) /
                                      std::min(zchunks_override, nz);
  t.zc = best_zc;
  t.zchunks = (nz + t.zc - 1) / t.zc;
  t.units = tiles * t.zchunks;
  t.smem = smem;
  if (t.units >= (1L << 31)) return false;
  *out = t;
  return true;
}

template <bool ANISO, int TSRC, bool COMP>
static cudaError_t launch_lane_t(const StepArgs& a, const TilePlan& t, cudaStream_t s) {
  auto k = pf_lane_kernel<kLaneNV, ANISO, TSRC, kLaneNC, kLaneCTAs, kLaneTX, kLaneS, COMP>;
  static int configured[64] = {0};
  const int dev = device_info().device;
  if (dev < 0 || dev >= 64 || configured[dev] < (int)t.smem) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)t.smem);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64) configured[dev] = (int)t.smem;
  }
  k<<<(unsigned)t.units, kLaneNC, t.smem, s>>>(a);
  return cudaGetLastError();
}

template <int TSRC>
cudaError_t launch_lane_kernel(const StepArgs& a, const TilePlan& t, cudaStream_t s) {
  if (a.n != 4 * kLaneNV || t.tx != kLaneTX || t.stages != kLaneS) return cudaErrorInvalidValue;
  if constexpr (TSRC == kTHeat) {
    if (a.T_lo)
      return (a.pc.aniso > 0.f) ? launch_lane_t<true, TSRC, true>(a, t, s)
                                : launch_lane_t<false, TSRC, true>(a, t, s);
  }
  return (a.pc.aniso > 0.f) ? launch_lane_t<true, TSRC, false>(a, t, s)
                            : launch_lane_t<false, TSRC, false>(a, t, s);
}

template cudaError_t launch_lane_kernel<kTArray>(const StepArgs&, const TilePlan&, cudaStream_t);
template cudaError_t launch_lane_kernel<kTHeat>(const StepArgs&, const TilePlan&, cudaStream_t);
template cudaError_t launch_lane_kernel<kTQuench>(const StepArgs&, const TilePlan&, cudaStream_t);
template cudaError_t launch_lane_kernel<kTPoint>(const StepArgs&, const TilePlan&, cudaStream_t);
template cudaError_t launch_lane_kernel<kTInterp>(const StepArgs&, const TilePlan&, cudaStream_t);

int read_lane_device_error(int clear) {
  int v = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, g_lane_device_error, sizeof(int));
  if (e != cudaSuccess) return record_cuda(e);
  if (clear && v) {
    const int zero = 0;
    e = cudaMemcpyToSymbol(g_lane_device_error, &zero, sizeof(int));
    if (e != cudaSuccess) return record_cuda(e);
  }
  return v;
}

}  // namespace pfg
