// Warp-per-cells z-marching unit of the phase-field step: the body shared by
// the single-job kernel (pf_fast.cu) and the batched serving kernel
// (pf_batch.cu).  Internal to the library.
#pragma once

#include <cuda_runtime.h>

#include "pfg_step.cuh"

namespace pfg {

// Folded per-cell coefficients of one Euler step.  With K = 4 S + 2 (1 - zeta)^2 - 1,
// cg = -dt Lg m_g / ad_hoc and cl = dt Lg kappa_g ad_hoc, the update
//   eta' = eta + cg eta (K - 3 eta^2) + cl a Lap(eta)
// is evaluated as
//   eta' = eta (A1 + B1 eta^2) + (C1 + C2 t) Lap'(eta)
// with A1 = 1 + cg K, B1 = -3 cg, Lap' = Lap / w_x (w_d = 1 / h_d^2),
// a = 1 + A (cos^4 + sin^4) = (1 + A) - 2 A t, t = c2 (1 - c2), c2 = cos^2,
// C1 = cl w_x (1 + A), C2 = -2 A cl w_x.  Liquid forcing sets all four to 0.
struct LapConsts {
  float ry, rz, nm;  // w_y / w_x, w_z / w_x, -2 (1 + ry + rz)
};

__device__ __forceinline__ float4 fold_coefficients(const PFConsts& c, const TempCoef& tc,
                                                    float S) {
  if (tc.liquid != 0.f) return make_float4(0.f, 0.f, 0.f, 0.f);
  const float K = 4.f * S + tc.om2 - 1.f;
  const float clw = tc.cl * c.wx;
  return make_float4(1.f + tc.cg * K, -3.f * tc.cg, clw * (1.f + c.aniso), -2.f * c.aniso * clw);
}

// One element: e and its six neighbours; d = the first two rotated cube axes
// of this orientation (the third follows from sum_k (d_k . e)^2 = |e|^2).
template <bool ANISO>
__device__ __forceinline__ float update_elem(const LapConsts& L, float e, float xm, float xp,
                                             float ym, float yp, float zm, float zp,
                                             const float* d, const float4 k) {
  const float lap = fmaf(L.rz, zp + zm, fmaf(L.ry, yp + ym, fmaf(L.nm, e, xp + xm)));
  float u = k.z;
  if constexpr (ANISO) {
    const float ex = xp - xm, ey = yp - ym, ez = zp - zm;
    const float ee = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
    const float p0 = fmaf(d[0], ex, fmaf(d[1], ey, d[2] * ez));
    const float p1 = fmaf(d[3], ex, fmaf(d[4], ey, d[5] * ez));
    const float q0 = p0 * p0, q1 = p1 * p1;
    const float q2 = ee - q0 - q1;
    // |e| = 0 gives 0 * inf = NaN and fminf(NaN, 1) = 1: the reference's
    // NaN-angle-to-zero rule; rounding above 1 is clamped the same way
    const float c2 = fminf(fmaxf(fmaxf(q0, q1), q2) * rcp_approx(ee), 1.f);
    u = fmaf(k.w, fmaf(-c2, c2, c2), k.z);
  }
  return fmaf(u, lap, e * fmaf(k.y, e * e, k.x));
}

// floor(i / d) for 0 <= i < 2^32 / d, with magic = ceil(2^32 / d) held in 64 bits
// (d = 1 needs 2^32).
__device__ __forceinline__ uint64_t div_magic(int d) {
  return ((uint64_t)1 << 32) / (uint64_t)d + (((((uint64_t)1 << 32) % (uint64_t)d) != 0) ? 1 : 0);
}
__device__ __forceinline__ int fast_div(int i, uint64_t magic) {
  return (int)(((uint64_t)(unsigned)i * magic) >> 32);
}

template <int VEC, int TSRC>
__device__ __forceinline__ void stage_plane_w(const StepArgs& a, float* eta_s, float* T_s,
                                              int slot, int pz, int x0, int y0, int txv, int tyv,
                                              int cx0, int row_chunks, int dst_cell0,
                                              uint64_t magic_rc, uint64_t magic_tx2,
                                              uint64_t magic_txv) {
  const int n = a.n, nx = a.nx, ny = a.ny;
  const int gz = bc_index(pz, a.nz, a.bcz);
  float* es = eta_s + (size_t)slot * (a.ty + 2) * a.pitch;
  const int rows = tyv + 2;
  const int total = rows * row_chunks;
  for (int i = threadIdx.x; i < total; i += kThreads) {
    const int r = fast_div(i, magic_rc);
    const int q = i - r * row_chunks;
    const int gy = bc_index(y0 - 1 + r, ny, a.bcy);
    const float* src = a.eta_in + (((int64_t)gz * ny + gy) * nx + cx0) * n + q * VEC;
    cp_async<VEC * 4>(es + r * a.pitch + dst_cell0 * n + q * VEC, src);
  }
  // halo cells outside the grid: copy of the boundary cell (Neumann) or the
  // wrapped cell (periodic)
  const int tpc = a.tpc;
  if (x0 == 0) {
    const int sx = bc_index(-1, nx, a.bcx);
    for (int i = threadIdx.x; i < rows * tpc; i += kThreads) {
      const int r = i / tpc, q = i - r * tpc;
      const int gy = bc_index(y0 - 1 + r, ny, a.bcy);
      cp_async<VEC * 4>(es + r * a.pitch + q * VEC,
                        a.eta_in + (((int64_t)gz * ny + gy) * nx + sx) * n + q * VEC);
    }
  }
  if (x0 + txv == nx) {
    const int sx = bc_index(nx, nx, a.bcx);
    for (int i = threadIdx.x; i < rows * tpc; i += kThreads) {
      const int r = i / tpc, q = i - r * tpc;
      const int gy = bc_index(y0 - 1 + r, ny, a.bcy);
      cp_async<VEC * 4>(es + r * a.pitch + (txv + 1) * n + q * VEC,
                        a.eta_in + (((int64_t)gz * ny + gy) * nx + sx) * n + q * VEC);
    }
  }
  float* ts = T_s + (size_t)slot * a.tslot;
  const int tp = a.tx + 2;
  if constexpr (TSRC == kTHeat) {
    const int cols = txv + 2;
    const int64_t gsy = nx + 2, gsz = (int64_t)(ny + 2) * (nx + 2);
    for (int i = threadIdx.x; i < rows * cols; i += kThreads) {
      const int r = fast_div(i, magic_tx2), c = i - r * cols;
      cp_async<4>(ts + r * tp + c, a.T + (int64_t)(pz + 1) * gsz + (int64_t)(y0 + r) * gsy + x0 + c);
    }
  } else if constexpr (TSRC == kTArray) {
    if (pz >= 0 && pz < a.nz) {
      for (int i = threadIdx.x; i < tyv * txv; i += kThreads) {
        const int r = fast_div(i, magic_txv), c = i - r * txv;
        cp_async<4>(ts + (r + 1) * tp + c + 1, a.T + ((int64_t)pz * ny + y0 + r) * nx + x0 + c);
      }
    }
  }
}

// One work unit (a tile and a chunk of z planes) of the step described by
// `a`, started at simulation time t0, using `smem` as the staging ring.
template <int VEC, bool ANISO, int TSRC>
__device__ __forceinline__ void warp_unit(const StepArgs& a, int unit, double t0, float* smem) {
  const int S = a.stages;
  const int slot_floats = (a.ty + 2) * a.pitch;
  float* eta_s = smem;
  float* T_s = eta_s + (size_t)S * slot_floats;
  float4* cc = reinterpret_cast<float4*>(T_s + (size_t)S * a.tslot);  // [2][ty * tx]

  // ---- work unit
  const int per_plane = a.tiles_x * a.tiles_y;
  const int zi = unit / per_plane;
  const int rem = unit - zi * per_plane;
  const int byi = rem / a.tiles_x;
  const int bxi = rem - byi * a.tiles_x;
  const int x0 = bxi * a.tx, y0 = byi * a.ty;
  const int xe = min(x0 + a.tx, a.nx), ye = min(y0 + a.ty, a.ny);
  const int zb = zi * a.zc, ze = min(zb + a.zc, a.nz);
  const int txv = xe - x0, tyv = ye - y0;
  const int n = a.n, tpc = a.tpc;

  // ---- lane -> (cell, orientation chunk)
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wxi = warp % a.wx, wyi = warp / a.wx;
  const int lc = lane / tpc, k = lane - lc * tpc;
  const bool lane_active = lc < a.cpw;
  const int xs = wxi * a.cpw + (lane_active ? lc : 0);
  const bool col_valid = lane_active && xs < txv;
  const int i0 = k * VEC;

  float dl[ANISO ? 6 * VEC : 1];
  if constexpr (ANISO) {
    const int ib = min(i0, n - VEC);
#pragma unroll
    for (int v = 0; v < VEC; ++v)
#pragma unroll
      for (int j = 0; j < 6; ++j) dl[v * 6 + j] = a.dirs[((j / 3) * n + ib + v) * 3 + (j % 3)];
  }
  LapConsts L;
  L.ry = a.pc.wy / a.pc.wx;
  L.rz = a.pc.wz / a.pc.wx;
  L.nm = -2.f * (1.f + L.ry + L.rz);

  // ---- staging geometry (fixed per tile)
  const int cx0 = max(x0 - 1, 0), cx1 = min(xe + 1, a.nx);
  const int row_chunks = (cx1 - cx0) * tpc;
  const int dst_cell0 = cx0 - (x0 - 1);
  const uint64_t magic_rc = div_magic(row_chunks);
  const uint64_t magic_tx2 = div_magic(txv + 2);
  const uint64_t magic_txv = div_magic(txv);

  // ---- beam at mid-step (float64, evaluated by one thread: float64
  // arithmetic is slow on this GPU); point-source record of this step
  __shared__ float s_beam_w[3];
  // moving gradient: the temperature of plane pz in s_Tw[(pz - zb) & 1],
  // evaluated by one thread a barrier ahead of its use
  __shared__ float s_Tw[2];
  auto quench_T = [&](int pz) {
    const double zc = a.q.z_first + (double)pz * (double)a.h_z;
    return (float)(a.q.T_base + a.q.grad * (zc - a.q.z0) - a.q.grad * a.q.vel * t0);
  };
  if (threadIdx.x == 0) {
    if constexpr (TSRC == kTHeat)
      laser_at(a.hp, t0 + 0.5 * (double)a.dt, &s_beam_w[0], &s_beam_w[1], &s_beam_w[2]);
    if constexpr (TSRC == kTQuench) {
      s_Tw[0] = quench_T(zb);
      s_Tw[1] = quench_T(zb + 1);
    }
  }
  float xl = 0.f, yl = 0.f, Pw = 0.f;  // read after the prologue's barrier
  pfg_point_source prec{};
  if constexpr (TSRC == kTPoint) prec = point_record(a.ps, a.clk_in->step);
  float w_past = 0.f;
  if constexpr (TSRC == kTInterp) w_past = interp_weight(a.t_future, a.dt_coarse, t0 + (double)a.dt);

  auto stage = [&](int slot, int pz) {
    stage_plane_w<VEC, TSRC>(a, eta_s, T_s, slot, pz, x0, y0, txv, tyv, cx0, row_chunks,
                             dst_cell0, magic_rc, magic_tx2, magic_txv);
  };

  // per-cell coefficients of the plane staged in `slot` -> cc[buf]:
  // (cg, cl, K = 4 S + 2 (1 - zeta)^2 - 1, liquid) with S = sum_i eta_i^2
  auto cell_coefs = [&](int slot, int buf, int pz) {
    const float* es = eta_s + (size_t)slot * slot_floats;
    const float* ts = T_s + (size_t)slot * a.tslot;
    float4* cb = cc + (size_t)buf * a.ty * a.tx;
    TempCoef plane{};
    if constexpr (TSRC == kTQuench) plane = temp_coefficients_fast(a.pc, s_Tw[(pz - zb) & 1], a.dt);
    for (int i = threadIdx.x; i < tyv * txv; i += kThreads) {
      const int r = fast_div(i, magic_txv), c = i - r * txv;
      const float* ce = es + (r + 1) * a.pitch + (c + 1) * n;
      float s0 = 0.f, s1 = 0.f;
      int q = 0;
      for (; q + 2 * VEC <= n; q += 2 * VEC) {
        VecF<VEC> u, v;
        u.load(ce + q);
        v.load(ce + q + VEC);
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
          s0 = fmaf(u.v[e], u.v[e], s0);
          s1 = fmaf(v.v[e], v.v[e], s1);
        }
      }
      for (; q < n; q += VEC) {
        VecF<VEC> u;
        u.load(ce + q);
#pragma unroll
        for (int e = 0; e < VEC; ++e) s0 = fmaf(u.v[e], u.v[e], s0);
      }
      const float S_ = s0 + s1;
      TempCoef tc;
      if constexpr (TSRC == kTQuench) tc = plane;
      else if constexpr (TSRC == kTPoint)
        tc = temp_coefficients_fast(a.pc, point_source_T(a.ps, prec, x0 + c, y0 + r, pz), a.dt);
      else if constexpr (TSRC == kTInterp) {
        const int64_t ti = ((int64_t)pz * a.ny + y0 + r) * a.nx + x0 + c;
        const float Tp = __ldg(a.T + ti), Tf = __ldg(a.T2 + ti);
        tc = temp_coefficients_fast(a.pc, w_past * Tp + (1.f - w_past) * Tf, a.dt);
      }
      else tc = temp_coefficients_fast(a.pc, ts[(r + 1) * (a.tx + 2) + c + 1], a.dt);
      cb[r * a.tx + c] = fold_coefficients(a.pc, tc, S_);
    }
  };

  // ---- prologue
  for (int p = 0; p < S - 1; ++p) {
    const int pz = zb - 1 + p;
    if (pz <= ze) stage(p % S, pz);
    cp_async_commit();
  }
  cp_async_wait(S - 4);
  __syncthreads();
  if constexpr (TSRC == kTHeat) {
    xl = s_beam_w[0];
    yl = s_beam_w[1];
    Pw = s_beam_w[2];
  }
  cell_coefs(1, 0, zb);  // plane zb sits in slot 1

  const int64_t plane_elems = (int64_t)a.ny * a.nx * n;
  for (int z = zb; z < ze; ++z) {
    const int m = z - zb;
    cp_async_wait(S - 4);
    __syncthreads();
    {
      const int pz = z + S - 2;
      if (pz <= ze) stage((m + S - 1) % S, pz);
      cp_async_commit();
    }
    // read by cell_coefs(z + 2) after the next barrier
    if constexpr (TSRC == kTQuench)
      if (threadIdx.x == 0 && z + 2 < ze) s_Tw[(m + 2) & 1] = quench_T(z + 2);
    const int s_prev = m % S, s_cur = (m + 1) % S, s_next = (m + 2) % S;

    // ---- per-cell work: heat update of plane z, coefficients of plane z+1
    if constexpr (TSRC == kTHeat) {
      const float* tp_ = T_s + (size_t)s_prev * a.tslot;
      const float* tc_ = T_s + (size_t)s_cur * a.tslot;
      const float* tn_ = T_s + (size_t)s_next * a.tslot;
      const int tp = a.tx + 2;
      const int64_t sy = a.nx + 2, sz = (int64_t)(a.ny + 2) * (a.nx + 2);
      for (int i = threadIdx.x; i < tyv * txv; i += kThreads) {
        const int r = fast_div(i, magic_txv), c = i - r * txv;
        const int o = (r + 1) * tp + c + 1;
        const int gx = x0 + c, gy = y0 + r;
        const int64_t idx = (int64_t)(z + 1) * sz + (int64_t)(gy + 1) * sy + gx + 1;
        const float Tn = heat_cell_update(a.hc, tc_[o], tc_[o - 1], tc_[o + 1], tc_[o - tp],
                                          tc_[o + tp], tp_[o], tn_[o], gx, gy, z, xl, yl, Pw,
                                          a.dt, a.T_out, idx, (int64_t)1, sy, sz);
        a.T_out[idx] = Tn;
      }
    }
    if (z + 1 < ze) cell_coefs(s_next, (m + 1) & 1, z + 1);

    // ---- element pass
    const float* e_cur = eta_s + (size_t)s_cur * slot_floats;
    const float* e_prev = eta_s + (size_t)s_prev * slot_floats;
    const float* e_next = eta_s + (size_t)s_next * slot_floats;
    const float4* ccb = cc + (size_t)(m & 1) * a.ty * a.tx;
    auto row_update = [&](int r, const VecF<VEC>& c, const VecF<VEC>& xm, const VecF<VEC>& xp,
                          const VecF<VEC>& ym, const VecF<VEC>& yp, const VecF<VEC>& zm,
                          const VecF<VEC>& zp) {
      const float4 kc = ccb[r * a.tx + xs];
      VecF<VEC> out;
#pragma unroll
      for (int v = 0; v < VEC; ++v)
        out.v[v] = update_elem<ANISO>(L, c.v[v], xm.v[v], xp.v[v], ym.v[v], yp.v[v], zm.v[v],
                                      zp.v[v], &dl[ANISO ? v * 6 : 0], kc);
      if (col_valid) {
        const int64_t g = (int64_t)z * plane_elems +
                          ((int64_t)(y0 + r) * a.nx + (x0 + xs)) * n + i0;
        out.store(a.eta_out + g);
      }
    };
    const int r_begin = wyi * a.rpw;
    const int r_end = min(r_begin + a.rpw, tyv);
    int r = r_begin;
    for (; r + 1 < r_end; r += 2) {
      // two rows share their y neighbours: rows r-1 .. r+2 are loaded once
      const int off = (r + 1) * a.pitch + (xs + 1) * n + i0;
      const int off2 = off + a.pitch;
      VecF<VEC> ym, c, c2, yp2, xm, xp, xm2, xp2, zm, zp, zm2, zp2;
      ym.load(e_cur + off - a.pitch);
      c.load(e_cur + off);
      c2.load(e_cur + off2);
      yp2.load(e_cur + off2 + a.pitch);
      xm.load(e_cur + off - n);
      xp.load(e_cur + off + n);
      xm2.load(e_cur + off2 - n);
      xp2.load(e_cur + off2 + n);
      zm.load(e_prev + off);
      zp.load(e_next + off);
      zm2.load(e_prev + off2);
      zp2.load(e_next + off2);
      row_update(r, c, xm, xp, ym, c2, zm, zp);
      row_update(r + 1, c2, xm2, xp2, c, yp2, zm2, zp2);
    }
    if (r < r_end) {
      const int off = (r + 1) * a.pitch + (xs + 1) * n + i0;
      VecF<VEC> c, xm, xp, ym, yp, zm, zp;
      c.load(e_cur + off);
      xm.load(e_cur + off - n);
      xp.load(e_cur + off + n);
      ym.load(e_cur + off - a.pitch);
      yp.load(e_cur + off + a.pitch);
      zm.load(e_prev + off);
      zp.load(e_next + off);
      row_update(r, c, xm, xp, ym, yp, zm, zp);
    }
  }
  cp_async_wait(0);
}

}  // namespace pfg
