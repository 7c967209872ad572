// Warp-per-cells z-marching phase-field step (the fast path for sm_103a).
//
// Same arithmetic as pf_step.cu's generic kernel, organised for instruction
// throughput:
//  * Each warp owns `cpw` whole cells of a tile row: `tpc` = num_oris / VEC
//    consecutive lanes per cell, VEC orientations per lane.  The per-cell sum
//    S = sum_i eta_i^2 is a segmented warp-shuffle reduction over those lanes.
//  * Per-cell temperature coefficients (tanh, exp, divisions) for plane z+1
//    are computed while plane z is updated, so one __syncthreads per plane
//    separates staging, coefficients and the element pass.
//  * The element arithmetic runs on packed pairs of orientations with the
//    Blackwell f32x2 FMA/ADD/MUL instructions; the anisotropy needs one MUFU
//    reciprocal per element and no arccos.
//  * Staging copies each halo row as one contiguous run of VEC-float chunks
//    (no per-chunk index division); halo cells outside the grid are copied
//    separately from the boundary cell (Neumann) or the wrapped cell
//    (periodic).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "pfg_host.h"
#include "pfg_step.cuh"

namespace pfg {

__device__ __forceinline__ float2 f2(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.f), a); }

struct PairConsts {
  float2 wx, wy, wz, m2w;  // 1/h^2 per axis and -2 sum(1/h^2)
  float2 A, one, neg3;
};

// One explicit Euler update of a pair of orientations of one cell:
//   eta + cg * eta (K - 3 eta^2) + cl * a * Lap(eta)
// d points at the 9 direction pairs (3 cube axes x 3 components).
template <bool ANISO>
__device__ __forceinline__ float2 update_pair(const PairConsts& P, float2 e, float2 xm, float2 xp,
                                              float2 ym, float2 yp, float2 zm, float2 zp,
                                              const float2* d, float2 K, float2 cg, float2 cl) {
  const float2 sx = add2(xp, xm), sy = add2(yp, ym), sz = add2(zp, zm);
  const float2 lap = fma2(P.wx, sx, fma2(P.wy, sy, fma2(P.wz, sz, mul2(P.m2w, e))));
  float2 a = P.one;
  if constexpr (ANISO) {
    const float2 ex = sub2(xp, xm), ey = sub2(yp, ym), ez = sub2(zp, zm);
    const float2 ee = fma2(ex, ex, fma2(ey, ey, mul2(ez, ez)));
    float2 p0 = fma2(d[0], ex, fma2(d[1], ey, mul2(d[2], ez)));
    float2 p1 = fma2(d[3], ex, fma2(d[4], ey, mul2(d[5], ez)));
    float2 p2 = fma2(d[6], ex, fma2(d[7], ey, mul2(d[8], ez)));
    p0 = mul2(p0, p0);
    p1 = mul2(p1, p1);
    p2 = mul2(p2, p2);
    const float2 m = make_float2(fmaxf(fmaxf(p0.x, p1.x), p2.x), fmaxf(fmaxf(p0.y, p1.y), p2.y));
    // |e| = 0 gives 0 * inf = NaN here and fminf(NaN, 1) = 1: the reference's
    // NaN-angle-to-zero rule; rounding above 1 is clamped to 1 as well
    float2 c2 = mul2(m, make_float2(__fdividef(1.f, ee.x), __fdividef(1.f, ee.y)));
    c2 = make_float2(fminf(c2.x, 1.f), fminf(c2.y, 1.f));
    const float2 s2 = sub2(P.one, c2);
    a = fma2(P.A, fma2(c2, c2, mul2(s2, s2)), P.one);
  }
  const float2 g = mul2(e, fma2(P.neg3, mul2(e, e), K));
  return fma2(mul2(cl, a), lap, fma2(cg, g, e));
}

template <bool ANISO>
__device__ __forceinline__ float update_one(const PFConsts& c, float e, float xm, float xp,
                                            float ym, float yp, float zm, float zp,
                                            const float* d, float K, float cg, float cl) {
  const float lap = c.wx * (xp + xm) + (c.wy * (yp + ym) + (c.wz * (zp + zm) -
                    2.f * (c.wx + c.wy + c.wz) * e));
  float a = 1.f;
  if constexpr (ANISO) {
    const float ex = xp - xm, ey = yp - ym, ez = zp - zm;
    const float ee = ex * ex + ey * ey + ez * ez;
    const float p0 = d[0] * ex + d[1] * ey + d[2] * ez;
    const float p1 = d[3] * ex + d[4] * ey + d[5] * ez;
    const float p2 = d[6] * ex + d[7] * ey + d[8] * ez;
    const float m = fmaxf(fmaxf(p0 * p0, p1 * p1), p2 * p2);
    const float c2 = fminf(m * __fdividef(1.f, ee), 1.f);
    const float s2 = 1.f - c2;
    a = 1.f + c.aniso * (c2 * c2 + s2 * s2);
  }
  const float g = e * (K - 3.f * e * e);
  return e + cg * g + (cl * a) * lap;
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

template <int VEC, bool ANISO, int TSRC>
__global__ void __launch_bounds__(kThreads, 2) pf_warp_kernel(const __grid_constant__ StepArgs a) {
  extern __shared__ __align__(16) float smem[];
  const int S = a.stages;
  const int slot_floats = (a.ty + 2) * a.pitch;
  float* eta_s = smem;
  float* T_s = eta_s + (size_t)S * slot_floats;
  float4* cc = reinterpret_cast<float4*>(T_s + (size_t)S * a.tslot);  // [2][ty * tx]

  // ---- work unit
  const int per_plane = a.tiles_x * a.tiles_y;
  const int zi = blockIdx.x / per_plane;
  const int rem = blockIdx.x - zi * per_plane;
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

  constexpr int NP = (VEC >= 2) ? VEC / 2 : 1;  // orientation pairs per lane
  float2 dpair[ANISO && VEC >= 2 ? 9 * NP : 1];
  float dsc[ANISO && VEC == 1 ? 9 : 1];
  if constexpr (ANISO) {
    const int ib = min(i0, n - VEC);
    if constexpr (VEC >= 2) {
#pragma unroll
      for (int p = 0; p < NP; ++p)
#pragma unroll
        for (int j = 0; j < 9; ++j) {
          const int ax = j / 3, dd = j % 3;
          dpair[p * 9 + j] = make_float2(a.dirs[(ax * n + ib + 2 * p) * 3 + dd],
                                         a.dirs[(ax * n + ib + 2 * p + 1) * 3 + dd]);
        }
    } else {
#pragma unroll
      for (int j = 0; j < 9; ++j) dsc[j] = a.dirs[((j / 3) * n + ib) * 3 + (j % 3)];
    }
  }
  PairConsts P;
  P.wx = f2(a.pc.wx); P.wy = f2(a.pc.wy); P.wz = f2(a.pc.wz);
  P.m2w = f2(-2.f * (a.pc.wx + a.pc.wy + a.pc.wz));
  P.A = f2(a.pc.aniso); P.one = f2(1.f); P.neg3 = f2(-3.f);

  // ---- staging geometry (fixed per tile)
  const int cx0 = max(x0 - 1, 0), cx1 = min(xe + 1, a.nx);
  const int row_chunks = (cx1 - cx0) * tpc;
  const int dst_cell0 = cx0 - (x0 - 1);
  const uint64_t magic_rc = div_magic(row_chunks);
  const uint64_t magic_tx2 = div_magic(txv + 2);
  const uint64_t magic_txv = div_magic(txv);

  // ---- clock and beam
  float xl = 0.f, yl = 0.f, Pw = 0.f;
  double t0 = 0.0;
  if constexpr (TSRC != kTArray) {
    t0 = a.clk_in->t;
    if constexpr (TSRC == kTHeat) laser_at(a.hp, t0 + 0.5 * (double)a.dt, &xl, &yl, &Pw);
    if (blockIdx.x == 0 && threadIdx.x == 0 && a.clk_out) {
      a.clk_out->t = t0 + (double)a.dt;
      a.clk_out->step = a.clk_in->step + 1;
    }
  }

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
    if constexpr (TSRC == kTQuench) {
      const double zc = a.q.z_first + (double)pz * (double)a.h_z;
      const float Tz = (float)(a.q.T_base + a.q.grad * (zc - a.q.z0) - a.q.grad * a.q.vel * t0);
      plane = temp_coefficients(a.pc, Tz, a.dt);
    }
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
      else tc = temp_coefficients(a.pc, ts[(r + 1) * (a.tx + 2) + c + 1], a.dt);
      cb[r * a.tx + c] = make_float4(tc.cg, tc.cl, 4.f * S_ + tc.om2 - 1.f, tc.liquid);
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
                                          a.dt, a.T_out, idx, 1, sy, sz);
        a.T_out[idx] = Tn;
      }
    }
    if (z + 1 < ze) cell_coefs(s_next, (m + 1) & 1, z + 1);

    // ---- element pass
    const float* e_cur = eta_s + (size_t)s_cur * slot_floats;
    const float* e_prev = eta_s + (size_t)s_prev * slot_floats;
    const float* e_next = eta_s + (size_t)s_next * slot_floats;
    const float4* ccb = cc + (size_t)(m & 1) * a.ty * a.tx;
    const bool force = a.pc.force != 0;
    auto row_update = [&](int r, const VecF<VEC>& c, const VecF<VEC>& xm, const VecF<VEC>& xp,
                          const VecF<VEC>& ym, const VecF<VEC>& yp, const VecF<VEC>& zm,
                          const VecF<VEC>& zp) {
      const float4 tc = ccb[r * a.tx + xs];
      VecF<VEC> out;
      if constexpr (VEC >= 2) {
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          const float2 o2 = update_pair<ANISO>(
              P, make_float2(c.v[2 * p], c.v[2 * p + 1]),
              make_float2(xm.v[2 * p], xm.v[2 * p + 1]), make_float2(xp.v[2 * p], xp.v[2 * p + 1]),
              make_float2(ym.v[2 * p], ym.v[2 * p + 1]), make_float2(yp.v[2 * p], yp.v[2 * p + 1]),
              make_float2(zm.v[2 * p], zm.v[2 * p + 1]), make_float2(zp.v[2 * p], zp.v[2 * p + 1]),
              &dpair[ANISO ? p * 9 : 0], f2(tc.z), f2(tc.x), f2(tc.y));
          out.v[2 * p] = o2.x;
          out.v[2 * p + 1] = o2.y;
        }
      } else {
        out.v[0] = update_one<ANISO>(a.pc, c.v[0], xm.v[0], xp.v[0], ym.v[0], yp.v[0], zm.v[0],
                                     zp.v[0], dsc, tc.z, tc.x, tc.y);
      }
      if (force && tc.w != 0.f) {
#pragma unroll
        for (int v = 0; v < VEC; ++v) out.v[v] = 0.f;
      }
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

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

// Plan overrides for tuning sweeps (0 = automatic).
static int g_tune_wx = 0, g_tune_rpw = 0, g_tune_stages = 0, g_tune_zchunks = 0;

int set_tune(int key, int value) {
  if (value < 0) return PFG_ERR_PARAM;
  switch (key) {
    case 0: if (value && value != 1 && value != 2 && value != 4 && value != 8) return PFG_ERR_PARAM;
            g_tune_wx = value; return PFG_OK;
    case 1: if (value > 32) return PFG_ERR_PARAM;
            g_tune_rpw = value; return PFG_OK;
    case 2: if (value && (value < 4 || value > 6)) return PFG_ERR_PARAM;
            g_tune_stages = value; return PFG_OK;
    case 3: g_tune_zchunks = value; return PFG_OK;
    default: return PFG_ERR_PARAM;
  }
}

bool plan_warp_tiles(int nx, int ny, int nz, int n, int sm_count, int max_smem_per_sm,
                     TilePlan* out) {
  TilePlan t{};
  t.vec = vec_width(n);
  t.tpc = n / t.vec;
  if (t.tpc > 32) return false;
  t.cpw = 32 / t.tpc;
  t.stages = g_tune_stages ? g_tune_stages : 4;
  const size_t budget = (size_t)max_smem_per_sm / 2 - 2048;  // two CTAs per SM
  const long concurrent = 2L * sm_count;
  double best = 1e30;
  for (int wx = 1; wx <= 8; wx *= 2) {
    if (g_tune_wx && wx != g_tune_wx) continue;
    const int wy = 8 / wx;
    const int tx = wx * t.cpw;
    if (!g_tune_wx && wx > 1 && (wx / 2) * t.cpw >= nx) continue;  // a narrower tile covers x
    for (int rpw = 1; rpw <= 32; ++rpw) {
      if (g_tune_rpw && rpw != g_tune_rpw) continue;
      const int ty = wy * rpw;
      if (!g_tune_rpw && rpw > 1 && wy * (rpw - 1) >= ny) break;
      const int pitch = ((tx + 2) * n + 3) / 4 * 4;
      const int tslot = ((ty + 2) * (tx + 2) + 3) / 4 * 4;
      const size_t smem = (size_t)t.stages * ((size_t)(ty + 2) * pitch + tslot) * 4 +
                          (size_t)2 * ty * tx * 16;
      if (smem > budget) break;
      const long tiles = (long)((nx + tx - 1) / tx) * ((ny + ty - 1) / ty);
      const double cover = (double)tiles * tx * ty / ((double)nx * ny);
      const double halo = (double)(tx + 2) * (ty + 2) / ((double)tx * ty);
      // wave quantisation of the units this tile gives
      long zch = (4 * concurrent + tiles - 1) / tiles;
      zch = std::max(1L, std::min(zch, (long)std::max(1, nz / 8)));
      const long zc = (nz + zch - 1) / zch;
      const double waves = (double)(tiles * ((nz + zc - 1) / zc)) / (double)concurrent;
      const double wave_eff = waves / std::ceil(waves);
      const double score = cover * (0.75 + 0.25 * halo) / wave_eff;
      if (score < best - 1e-9) {
        best = score;
        t.tx = tx; t.ty = ty; t.wx = wx; t.rpw = rpw;
        t.pitch = pitch; t.tslot = tslot; t.smem = smem;
      }
    }
  }
  if (best >= 1e30) return false;
  t.rs = 0;
  t.tiles_x = (nx + t.tx - 1) / t.tx;
  t.tiles_y = (ny + t.ty - 1) / t.ty;
  const long tiles = (long)t.tiles_x * t.tiles_y;
  long zch = (4 * concurrent + tiles - 1) / tiles;
  zch = std::max(1L, std::min(zch, (long)std::max(1, nz / 8)));
  if (g_tune_zchunks) zch = std::min<long>(g_tune_zchunks, nz);
  t.zc = (int)((nz + zch - 1) / zch);
  t.zchunks = (nz + t.zc - 1) / t.zc;
  t.units = tiles * t.zchunks;
  *out = t;
  return true;
}

template <int VEC, bool ANISO, int TSRC>
static cudaError_t launch_w(const StepArgs& a, const TilePlan& t, cudaStream_t s) {
  auto k = pf_warp_kernel<VEC, ANISO, TSRC>;
  static int configured[64] = {0};
  const int dev = device_info().device;
  if (dev < 0 || dev >= 64 || configured[dev] < (int)t.smem) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)t.smem);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64) configured[dev] = (int)t.smem;
  }
  k<<<(unsigned)t.units, kThreads, t.smem, s>>>(a);
  return cudaGetLastError();
}

template <int TSRC>
cudaError_t launch_warp_kernel(const StepArgs& a, const TilePlan& t, cudaStream_t s) {
  const bool an = a.pc.aniso > 0.f;
  switch (t.vec) {
    case 4: return an ? launch_w<4, true, TSRC>(a, t, s) : launch_w<4, false, TSRC>(a, t, s);
    case 2: return an ? launch_w<2, true, TSRC>(a, t, s) : launch_w<2, false, TSRC>(a, t, s);
    default: return an ? launch_w<1, true, TSRC>(a, t, s) : launch_w<1, false, TSRC>(a, t, s);
  }
}

template cudaError_t launch_warp_kernel<kTArray>(const StepArgs&, const TilePlan&, cudaStream_t);
template cudaError_t launch_warp_kernel<kTHeat>(const StepArgs&, const TilePlan&, cudaStream_t);
template cudaError_t launch_warp_kernel<kTQuench>(const StepArgs&, const TilePlan&, cudaStream_t);

}  // namespace pfg
