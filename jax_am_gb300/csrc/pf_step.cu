// Phase-field (and fused heat + phase-field) explicit step for sm_103a.
//
// Layout: eta (nz, ny, nx, n) float32, orientation innermost, exactly the
// reference's (N, num_oris) array (allen_cahn.py:60).  A CTA owns a tile of
// TX x TY cells in the x-y plane and marches through a range of z planes.
// Each plane of the tile plus a one-cell halo is staged in shared memory by
// cp.async copies into a ring of `stages` plane slots, so every eta byte is
// read from HBM about once and the six neighbours come from shared memory.
// The boundary condition is applied while staging: a halo cell outside the
// grid is filled with the edge cell (Neumann, allen_cahn.py:61-66) or the
// wrapped cell (periodic), so the arithmetic has no boundary branches.
//
// Work split inside a CTA: every thread owns one (cell column, orientation
// chunk of VEC floats) of the tile and loops over the tile's rows; a per-cell
// pass first reduces S = sum eta_i^2 and evaluates zeta, the Arrhenius
// mobility and (fused variant) the heat update of each cell.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>

#include "pfg_device.cuh"
#include "pfg_host.h"
#include "pfg_step.cuh"

namespace pfg {

template <int VEC>
__device__ __forceinline__ void stage_copy(float* dst, const float* src) {
  cp_async<VEC * 4>(dst, src);
}

// Issue the cp.async copies of plane `pz` (grid z index, may be -1 or nz) of
// this tile into ring slot `slot`.
template <int VEC, int TSRC>
__device__ __forceinline__ void stage_plane(const StepArgs& a, float* eta_s, float* T_s, int slot,
                                            int pz, int x0, int y0, int xe, int ye,
                                            const int* col_off, const int* col_ok, int ncol) {
  const int gz = bc_index(pz, a.nz, a.bcz);
  float* es = eta_s + (size_t)slot * (a.ty + 2) * a.pitch;
  const int rows = ye - y0 + 2;  // halo row, interior rows, halo row
  for (int r = 0; r < rows; ++r) {
    const int gy = bc_index(y0 - 1 + r, a.ny, a.bcy);
    const float* src_row = a.eta_in + ((int64_t)gz * a.ny + gy) * a.nx * a.n;
    float* dst_row = es + r * a.pitch;
    for (int c = 0; c < ncol; ++c) {
      if (col_ok[c]) {
        const int sidx = threadIdx.x + c * kThreads;  // chunk index within the row
        stage_copy<VEC>(dst_row + sidx * VEC, src_row + col_off[c]);
      }
    }
  }
  float* ts = T_s + (size_t)slot * a.tslot;
  const int tcols = xe - x0 + 2;
  if constexpr (TSRC == kTHeat) {
    // ghosted temperature: halo = neighbouring interior cells or old ghosts
    const int gzp = pz + 1;  // ghosted plane index, 0..nz+1
    const int64_t sy = a.nx + 2, sz = (int64_t)(a.ny + 2) * (a.nx + 2);
    for (int i = threadIdx.x; i < rows * tcols; i += kThreads) {
      const int r = i / tcols, xs = i - r * tcols;
      const int64_t src = gzp * sz + (int64_t)(y0 + r) * sy + (x0 + xs);
      cp_async<4>(ts + r * (a.tx + 2) + xs, a.T + src);
    }
  } else if constexpr (TSRC == kTArray) {
    if (pz >= 0 && pz < a.nz) {
      const int icols = xe - x0, irows = ye - y0;
      for (int i = threadIdx.x; i < irows * icols; i += kThreads) {
        const int r = i / icols, xs = i - r * icols;
        const int64_t src = ((int64_t)pz * a.ny + (y0 + r)) * a.nx + (x0 + xs);
        cp_async<4>(ts + (r + 1) * (a.tx + 2) + xs + 1, a.T + src);
      }
    }
  }
}

template <int VEC, bool ANISO, int TSRC>
__global__ void __launch_bounds__(kThreads)
pf_zmarch_kernel(const __grid_constant__ StepArgs a) {
  extern __shared__ __align__(16) float smem[];
  float* eta_s = smem;
  float* T_s = eta_s + (size_t)a.stages * (a.ty + 2) * a.pitch;
  CellCoef* cc = reinterpret_cast<CellCoef*>(T_s + (size_t)a.stages * a.tslot);

  // ---- work unit: tile (bx, by) and z chunk
  const int unit = blockIdx.x;
  const int per_plane = a.tiles_x * a.tiles_y;
  const int zi = unit / per_plane;
  const int rem = unit - zi * per_plane;
  const int byi = rem / a.tiles_x;
  const int bxi = rem - byi * a.tiles_x;
  const int x0 = bxi * a.tx, y0 = byi * a.ty;
  const int xe = min(x0 + a.tx, a.nx), ye = min(y0 + a.ty, a.ny);
  const int zb = zi * a.zc, ze = min(zb + a.zc, a.nz);
  const int txv = xe - x0, tyv = ye - y0;
  const int n = a.n;

  // ---- staging map: this thread's chunks within a halo row (fixed per tile)
  constexpr int MAXC = 3;
  int col_off[MAXC], col_ok[MAXC];
  const int row_chunks = (txv + 2) * a.tpc;
  int ncol = 0;
#pragma unroll
  for (int c = 0; c < MAXC; ++c) {
    const int sidx = threadIdx.x + c * kThreads;
    col_ok[c] = 0;
    col_off[c] = 0;
    if (sidx < row_chunks) {
      const int xs = sidx / a.tpc, k = sidx - xs * a.tpc;
      const int gx = bc_index(x0 - 1 + xs, a.nx, a.bcx);
      col_off[c] = gx * n + k * VEC;
      col_ok[c] = 1;
      ncol = c + 1;
    }
  }

  // ---- compute map: (row phase ry, column xs, chunk k)
  const int cols = a.tx * a.tpc;
  const int ry = threadIdx.x / cols;
  const int j = threadIdx.x - ry * cols;
  const int my_xs = j / a.tpc;
  const int my_k = j - my_xs * a.tpc;
  const bool computes = (ry < a.rs) && (my_xs < txv);
  const int i0 = my_k * VEC;

  float dir[ANISO ? 9 * VEC : 1];
  if constexpr (ANISO) {
#pragma unroll
    for (int v = 0; v < VEC; ++v) {
      const int i = min(i0 + v, n - 1);
#pragma unroll
      for (int ax = 0; ax < 3; ++ax)
#pragma unroll
        for (int d = 0; d < 3; ++d) dir[v * 9 + ax * 3 + d] = a.dirs[(ax * n + i) * 3 + d];
    }
  }

  // fused: beam at mid-step; quench: start-of-step time
  float xl = 0.f, yl = 0.f, P = 0.f;
  double t0 = 0.0;
  pfg_point_source prec{};
  if constexpr (TSRC == kTPoint) prec = point_record(a.ps, a.clk_in->step);
  if constexpr (TSRC != kTArray) {
    t0 = a.clk_in->t;
    if constexpr (TSRC == kTHeat) laser_at(a.hp, t0 + 0.5 * (double)a.dt, &xl, &yl, &P);
    if (blockIdx.x == 0 && threadIdx.x == 0 && a.clk_out) {
      a.clk_out->t = t0 + (double)a.dt;
      a.clk_out->step = a.clk_in->step + 1;
    }
  }

  const int S = a.stages;
  // ---- prologue: planes zb-1 .. zb+S-3
  for (int p = 0; p < S - 1; ++p) {
    const int pz = zb - 1 + p;
    if (pz <= ze) stage_plane<VEC, TSRC>(a, eta_s, T_s, p % S, pz, x0, y0, xe, ye, col_off,
                                         col_ok, ncol);
    cp_async_commit();
  }

  const int64_t plane_elems = (int64_t)a.ny * a.nx * n;
  for (int z = zb; z < ze; ++z) {
    const int m = z - zb;
    cp_async_wait(S - 4);
    __syncthreads();
    {
      const int pz = z + S - 2;
      if (pz <= ze) stage_plane<VEC, TSRC>(a, eta_s, T_s, (m + S - 1) % S, pz, x0, y0, xe, ye,
                                           col_off, col_ok, ncol);
      cp_async_commit();
    }
    const int sm = (m + 1) % S, s_prev = m % S, s_next = (m + 2) % S;
    const float* e_cur = eta_s + (size_t)sm * (a.ty + 2) * a.pitch;
    const float* e_prev = eta_s + (size_t)s_prev * (a.ty + 2) * a.pitch;
    const float* e_next = eta_s + (size_t)s_next * (a.ty + 2) * a.pitch;
    const float* t_cur = T_s + (size_t)sm * a.tslot;
    TempCoef plane_tc{};
    if constexpr (TSRC == kTQuench) {
      // the moving gradient is constant over a z plane
      const double zc = a.q.z_first + (double)z * (double)a.h_z;
      const float Tz = (float)(a.q.T_base + a.q.grad * (zc - a.q.z0) - a.q.grad * a.q.vel * t0);
      plane_tc = temp_coefficients(a.pc, Tz, a.dt);
    }

    // ---- per-cell pass
    for (int cidx = threadIdx.x; cidx < tyv * txv; cidx += kThreads) {
      const int r = cidx / txv, xs = cidx - r * txv;
      const float* ce = e_cur + (r + 1) * a.pitch + (xs + 1) * n;
      float s = 0.f;
      for (int i = 0; i < n; i += VEC) {
        VecF<VEC> q;
        q.load(ce + i);
#pragma unroll
        for (int v = 0; v < VEC; ++v) s = fmaf(q.v[v], q.v[v], s);
      }
      const int tp = a.tx + 2;
      float Tc = 0.f;
      if constexpr (TSRC == kTQuench) {
        cc[r * a.tx + xs] = cell_coefficients(plane_tc, s);
      } else if constexpr (TSRC == kTPoint) {
        Tc = point_source_T(a.ps, prec, x0 + xs, y0 + r, z);
        cc[r * a.tx + xs] = cell_coefficients(temp_coefficients(a.pc, Tc, a.dt), s);
      } else if constexpr (TSRC == kTInterp) {
        const float w = interp_weight(a.t_future, a.dt_coarse, t0 + (double)a.dt);
        const int64_t ti = ((int64_t)z * a.ny + y0 + r) * a.nx + x0 + xs;
        Tc = w * a.T[ti] + (1.f - w) * a.T2[ti];
        cc[r * a.tx + xs] = cell_coefficients(temp_coefficients(a.pc, Tc, a.dt), s);
      } else {
        Tc = t_cur[(r + 1) * tp + xs + 1];
        cc[r * a.tx + xs] = cell_coefficients(temp_coefficients(a.pc, Tc, a.dt), s);
      }
      if constexpr (TSRC == kTHeat) {
        const float* t_prev = T_s + (size_t)s_prev * a.tslot;
        const float* t_next = T_s + (size_t)s_next * a.tslot;
        const int o = (r + 1) * tp + xs + 1;
        const int gx = x0 + xs, gy = y0 + r;
        const int64_t sy = a.nx + 2, sz = (int64_t)(a.ny + 2) * (a.nx + 2);
        const int64_t idx = (int64_t)(z + 1) * sz + (int64_t)(gy + 1) * sy + gx + 1;
        const float Tn = heat_cell_update(a.hc, Tc, t_cur[o - 1], t_cur[o + 1], t_cur[o - tp],
                                          t_cur[o + tp], t_prev[o], t_next[o], gx, gy, z, xl, yl,
                                          P, a.dt, a.T_out, idx, (int64_t)1, sy, sz);
        a.T_out[idx] = Tn;
      }
    }
    __syncthreads();

    // ---- element pass
    if (computes) {
      for (int r = ry; r < tyv; r += a.rs) {
        const int off = (r + 1) * a.pitch + (my_xs + 1) * n + i0;
        VecF<VEC> c, xm, xp, ym, yp, zm, zp;
        c.load(e_cur + off);
        xm.load(e_cur + off - n);
        xp.load(e_cur + off + n);
        ym.load(e_cur + off - a.pitch);
        yp.load(e_cur + off + a.pitch);
        zm.load(e_prev + off);
        zp.load(e_next + off);
        const CellCoef k = cc[r * a.tx + my_xs];
        VecF<VEC> out;
#pragma unroll
        for (int v = 0; v < VEC; ++v) {
          const float e = c.v[v];
          const float lap = a.pc.wx * ((xp.v[v] - e) + (xm.v[v] - e)) +
                            a.pc.wy * ((yp.v[v] - e) + (ym.v[v] - e)) +
                            a.pc.wz * ((zp.v[v] - e) + (zm.v[v] - e));
          float aniso = 1.f;
          if constexpr (ANISO) {
            aniso = aniso_factor(a.pc.aniso, xp.v[v] - xm.v[v], yp.v[v] - ym.v[v],
                                 zp.v[v] - zm.v[v], &dir[v * 9]);
          }
          float o = e + k.cg * (e * (k.K - 3.f * e * e)) + k.cl * (aniso * lap);
          out.v[v] = (k.liquid != 0.f) ? 0.f : o;
        }
        const int64_t g = (int64_t)z * plane_elems +
                          ((int64_t)(y0 + r) * a.nx + (x0 + my_xs)) * n + i0;
        out.store(a.eta_out + g);
      }
    }
  }
  cp_async_wait(0);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

PFConsts make_pf_consts(const pfg_pf_params& p) {
  PFConsts c;
  c.wx = 1.f / (p.h_x * p.h_x);
  c.wy = 1.f / (p.h_y * p.h_y);
  c.wz = 1.f / (p.h_z * p.h_z);
  c.T_liq = p.T_liquidus;
  c.inv_T_liq = 1.f / p.T_liquidus;
  {
    // thresholds of the sign of fl(Tc / T_liq) - 1 (float division, as the
    // device would do it); a handful of steps from T_liq in each direction
    const volatile float tl = p.T_liquidus;
    float hi = tl, lo = tl;
    for (int i = 0; i < 64 && !((float)(hi / tl) > 1.f); ++i) hi = nextafterf(hi, INFINITY);
    for (int i = 0; i < 64 && !((float)(lo / tl) < 1.f); ++i) lo = nextafterf(lo, -INFINITY);
    c.zeta_hi = hi;
    c.zeta_lo = lo;
  }
  c.neg_Qg_over_R = -p.Qg / p.gas_const;
  c.L0 = p.L0;
  c.mg_ad = p.m_g / p.ad_hoc;
  c.kappa_ad = p.kappa_g * p.ad_hoc;
  c.aniso = p.anisotropy;
  c.liquid_limit = p.T_liquidus + p.liquid_shift;
  c.force = p.force_liquid_zero;
  return c;
}

PointConsts make_point_consts(const pfg_point_sources& s, const pfg_pf_params& p) {
  PointConsts c;
  c.T_ambient = s.T_ambient;
  c.inv_2pi_kappa = (float)(1.0 / (2.0 * 3.14159265358979323846 * (double)s.kappa));
  c.inv_2alpha = (float)(1.0 / (2.0 * (double)s.alpha));
  c.T_clip = s.T_clip;
  c.x_first = s.x_first; c.y_first = s.y_first; c.z_first = s.z_first;
  c.hx = p.h_x; c.hy = p.h_y; c.hz = p.h_z;
  c.table = s.table;
  c.num_records = s.num_records;
  return c;
}

static int check_point_sources(const pfg_point_sources* s) {
  if (!s || !s->table) return PFG_ERR_NULL;
  if (reinterpret_cast<uintptr_t>(s->table) % 8 != 0) return PFG_ERR_ALIGN;
  if (s->num_records < 1 || !(s->alpha > 0.f) || !(s->kappa > 0.f)) return PFG_ERR_PARAM;
  return PFG_OK;
}

__global__ void __launch_bounds__(kThreads) point_T_kernel(const PointConsts c,
                                                           const pfg_clock* clk, float* T,
                                                           int nx, int ny, int nz) {
  const pfg_point_source r = point_record(c, clk->step);
  const int64_t N = (int64_t)nx * ny * nz;
  const int64_t xy = (int64_t)nx * ny;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int z = (int)(i / xy);
    const int64_t rem = i - (int64_t)z * xy;
    const int y = (int)(rem / nx), x = (int)(rem - (int64_t)y * nx);
    T[i] = point_source_T(c, r, x, y, z);
  }
}

HeatConsts make_heat_consts(const pfg_heat_params& h) {
  HeatConsts c;
  c.nx = h.nx; c.ny = h.ny; c.nz = h.nz;
  c.dx = h.dx; c.dy = h.dy; c.dz = h.dz;
  c.dx2 = h.dx * h.dx; c.dy2 = h.dy * h.dy; c.dz2 = h.dz * h.dz;
  c.rdx2 = 1.f / c.dx2; c.rdy2 = 1.f / c.dy2; c.rdz2 = 1.f / c.dz2;
  c.inv_rho = 1.f / h.rho;
  c.rho = h.rho;
  c.h = h.h_conv;
  c.sb_eps = (float)((double)h.sigma_sb * (double)h.emissivity);
  c.T0 = h.T0;
  const float t02 = h.T0 * h.T0;
  c.T0_4 = t02 * t02;
  c.Ts = h.Ts; c.Tl = h.Tl;
  c.latent = h.latent;
  c.beam_coef = (float)(2.0 * (double)h.absorptivity / 3.14159265358979323846 /
                        ((double)h.beam_radius * (double)h.beam_radius));
  c.two_over_r2 = (float)(2.0 / ((double)h.beam_radius * (double)h.beam_radius));
  c.x_first = h.x_first;
  c.y_first = h.y_first;
  return c;
}

static DF df_split(double v) {
  const float h = (float)v;
  return DF{h, (float)(v - (double)h)};
}

// The DF constants of the compensated heat update, from the float32
// parameters (so the device evaluates exactly the model those values
// define) and the reference's literal coefficients (gamma.py:12-15).
HeatDF make_heat_df(const pfg_heat_params& h, float dt) {
  HeatDF d;
  d.k1 = df_split(0.0163);
  d.k0 = df_split(4.5847);
  d.c1 = df_split(0.2441);
  d.c0 = df_split(338.39);
  d.latent = df_split((double)h.latent);
  const double r = (double)h.beam_radius;
  d.beam_coef = df_split(2.0 * (double)h.absorptivity / 3.14159265358979323846 / (r * r));
  d.two_over_r2 = df_split(2.0 / (r * r));
  d.sb_eps = df_split((double)h.sigma_sb * (double)h.emissivity);
  const double t0 = (double)h.T0;
  d.T0_4 = df_split(t0 * t0 * t0 * t0);
  d.rd2[0] = df_split(1.0 / ((double)h.dx * (double)h.dx));
  d.rd2[1] = df_split(1.0 / ((double)h.dy * (double)h.dy));
  d.rd2[2] = df_split(1.0 / ((double)h.dz * (double)h.dz));
  d.dt = DF{dt, 0.f};
  d.hot = h.T0 + 50.f;
  return d;
}

int vec_width(int n) { return (n % 4 == 0) ? 4 : (n % 2 == 0) ? 2 : 1; }

TilePlan plan_tiles(int nx, int ny, int nz, int n, int sm_count, int max_smem_per_sm,
                    int max_smem_per_block) {
  TilePlan t;
  t.vec = vec_width(n);
  t.tpc = n / t.vec;
  t.tx = std::max(1, std::min(kThreads / t.tpc, nx));
  t.rs = std::max(1, kThreads / (t.tx * t.tpc));
  t.stages = 4;
  t.pitch = ((t.tx + 2) * n + 3) / 4 * 4;
  // rows: as many as fit two CTAs per SM, a multiple of rs, at most 16 and ny
  auto smem_for = [&](int ty) {
    const int tslot = ((ty + 2) * (t.tx + 2) + 3) / 4 * 4;
    return (size_t)t.stages * ((size_t)(ty + 2) * t.pitch + tslot) * 4 +
           (size_t)ty * t.tx * sizeof(CellCoef);
  };
  const size_t budget2 = (size_t)max_smem_per_sm / 2 - 1024;
  int ty = std::min(ny, std::max(t.rs, 16 / t.rs * t.rs));
  while (ty > 1 && smem_for(ty) > budget2) --ty;
  if (smem_for(ty) > (size_t)max_smem_per_block) ty = 1;
  t.ty = ty;
  t.tslot = ((ty + 2) * (t.tx + 2) + 3) / 4 * 4;
  t.smem = smem_for(ty);
  t.tiles_x = (nx + t.tx - 1) / t.tx;
  t.tiles_y = (ny + t.ty - 1) / t.ty;
  const int per_sm = std::max(1, (int)(max_smem_per_sm / (t.smem + 1024)));
  const long concurrent = (long)sm_count * std::min(per_sm, 2);
  const long tiles = (long)t.tiles_x * t.tiles_y;
  // enough units for ~4 waves, but z chunks of at least 8 planes
  long zch = (4 * concurrent + tiles - 1) / tiles;
  zch = std::max(1L, std::min(zch, (long)std::max(1, nz / 8)));
  t.zc = (int)((nz + zch - 1) / zch);
  t.zchunks = (nz + t.zc - 1) / t.zc;
  t.units = tiles * t.zchunks;
  return t;
}

template <int VEC, bool ANISO, int TSRC>
static cudaError_t launch_t(const StepArgs& a, const TilePlan& t, cudaStream_t s) {
  auto k = pf_zmarch_kernel<VEC, ANISO, TSRC>;
  // opt in to the dynamic shared memory this plan needs (once per size and device)
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

template <bool ANISO, int TSRC>
static cudaError_t launch_v(const StepArgs& a, const TilePlan& t, cudaStream_t s) {
  switch (t.vec) {
    case 4: return launch_t<4, ANISO, TSRC>(a, t, s);
    case 2: return launch_t<2, ANISO, TSRC>(a, t, s);
    default: return launch_t<1, ANISO, TSRC>(a, t, s);
  }
}

template <int TSRC>
static cudaError_t launch_a(const StepArgs& a, const TilePlan& t, cudaStream_t s) {
  return (a.pc.aniso > 0.f) ? launch_v<true, TSRC>(a, t, s) : launch_v<false, TSRC>(a, t, s);
}

void fill_step_args(StepArgs& a, const pfg_pf_params& p, const TilePlan& t, float dt);
static void fill_common(StepArgs& a, const pfg_pf_params& p, const TilePlan& t, float dt) {
  fill_step_args(a, p, t, dt);
}

void fill_step_args(StepArgs& a, const pfg_pf_params& p, const TilePlan& t, float dt) {
  a.nx = p.nx; a.ny = p.ny; a.nz = p.nz; a.n = p.num_oris;
  a.bcx = p.bc_x; a.bcy = p.bc_y; a.bcz = p.bc_z;
  a.dt = dt;
  a.pc = make_pf_consts(p);
  a.tx = t.tx; a.ty = t.ty; a.zc = t.zc; a.stages = t.stages; a.pitch = t.pitch;
  a.tslot = t.tslot; a.tpc = t.tpc; a.rs = t.rs;
  a.tiles_x = t.tiles_x; a.tiles_y = t.tiles_y; a.zchunks = t.zchunks;
  a.h_z = p.h_z;
  a.probe_wait = g_probe_wait;
  for (int i = 0; i < 3 * p.num_oris * 3; ++i) a.dirs[i] = p.grain_dirs[i];
}

int check_pf_params(const pfg_pf_params* p) {
  if (!p) return PFG_ERR_NULL;
  if (p->nx < 1 || p->ny < 1 || p->nz < 1) return PFG_ERR_SHAPE;
  if (p->num_oris < 1 || p->num_oris > PFG_MAX_ORIS) return PFG_ERR_SHAPE;
  if (!(p->h_x > 0.f) || !(p->h_y > 0.f) || !(p->h_z > 0.f)) return PFG_ERR_PARAM;
  if (!(p->ad_hoc != 0.f) || !(p->gas_const != 0.f) || !(p->T_liquidus > 0.f)) return PFG_ERR_PARAM;
  const int bcs[3] = {p->bc_x, p->bc_y, p->bc_z};
  for (int b : bcs)
    if (b != PFG_BC_NEUMANN && b != PFG_BC_PERIODIC) return PFG_ERR_PARAM;
  return PFG_OK;
}

int check_heat_params(const pfg_heat_params* h) {
  if (!h) return PFG_ERR_NULL;
  if (h->nx < 1 || h->ny < 1 || h->nz < 1) return PFG_ERR_SHAPE;
  if (!(h->dx > 0.f) || !(h->dy > 0.f) || !(h->dz > 0.f)) return PFG_ERR_PARAM;
  if (!(h->rho > 0.f) || !(h->Tl > h->Ts) || !(h->beam_radius > 0.f)) return PFG_ERR_PARAM;
  if (h->num_segments < 0 || h->num_segments > PFG_MAX_SEGMENTS) return PFG_ERR_PARAM;
  return PFG_OK;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

int g_kernel_variant = 0;

TilePlan plan_for_current_device(const pfg_pf_params& p) {
  const DeviceInfo& d = device_info();
  return plan_tiles(p.nx, p.ny, p.nz, p.num_oris, d.sm_count, d.smem_per_sm, d.smem_per_block);
}

static bool plan_lane(const pfg_pf_params& p, TilePlan* t) {
  const DeviceInfo& d = device_info();
  return plan_lane_tiles(p.nx, p.ny, p.nz, p.num_oris, d.sm_count, d.smem_per_sm,
                         d.smem_per_block, g_tune_zchunks, t);
}

// Plan and launch one step: the cell-per-lane kernel (num_oris = 20), else
// the TMA-fed kernel, else the warp-per-cells kernel when the orientation
// count allows it (num_oris / VEC <= 32), otherwise the generic kernel.
template <int TSRC>
static cudaError_t dispatch(StepArgs& a, const pfg_pf_params& p, float dt, cudaStream_t s) {
  const DeviceInfo& d = device_info();
  TilePlan t;
  const int v = g_kernel_variant;
  if (v == 0 && plan_lane(p, &t)) {
    fill_common(a, p, t, dt);
    a.cpw = t.cpw; a.wx = t.wx; a.rpw = t.rpw;
    return launch_lane_kernel<TSRC>(a, t, s);
  }
  if ((v == 0 || v == 3) &&
      plan_tma_tiles(p.nx, p.ny, p.nz, p.num_oris, p.bc_x, d.sm_count, d.smem_per_sm, &t)) {
    fill_common(a, p, t, dt);
    a.cpw = t.cpw; a.wx = t.wx; a.rpw = t.rpw;
    return launch_tma_kernel<TSRC>(a, t, s);
  }
  if ((v == 0 || v == 2 || v == 3) &&
      plan_warp_tiles(p.nx, p.ny, p.nz, p.num_oris, d.sm_count, d.smem_per_sm, &t)) {
    fill_common(a, p, t, dt);
    a.cpw = t.cpw; a.wx = t.wx; a.rpw = t.rpw;
    return launch_warp_kernel<TSRC>(a, t, s);
  }
  t = plan_for_current_device(p);
  fill_common(a, p, t, dt);
  return launch_a<TSRC>(a, t, s);
}

}  // namespace pfg

using namespace pfg;

extern "C" int pfg_tune(int key, int value) { return set_tune(key, value); }

extern "C" int pfg_describe_plan(const pfg_pf_params* p, int32_t* out) {
  int st = check_pf_params(p);
  if (st) return st;
  if (!out) return PFG_ERR_NULL;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  const DeviceInfo& d = device_info();
  TilePlan t;
  int kernel;
  const int variant = g_kernel_variant;
  if (variant == 0 && plan_lane(*p, &t)) {
    kernel = 4;
  } else if ((variant == 0 || variant == 3) &&
      plan_tma_tiles(p->nx, p->ny, p->nz, p->num_oris, p->bc_x, d.sm_count, d.smem_per_sm, &t)) {
    kernel = 3;
  } else if ((variant == 0 || variant == 2 || variant == 3) &&
             plan_warp_tiles(p->nx, p->ny, p->nz, p->num_oris, d.sm_count, d.smem_per_sm, &t)) {
    kernel = 2;
  } else {
    t = plan_for_current_device(*p);
    kernel = 1;
    t.wx = 0; t.rpw = 0;
  }
  const int32_t v[12] = {kernel, t.vec, t.tpc, t.tx, t.ty, t.wx, t.rpw, t.stages, t.zc,
                         (int32_t)t.units, (int32_t)t.smem, d.sm_count};
  for (int i = 0; i < 12; ++i) out[i] = v[i];
  return PFG_OK;
}

extern "C" int pfg_fixed_plan(const pfg_pf_params* p) {
  int st = check_pf_params(p);
  if (st) return -st;
  if (!device_info().ok) return -PFG_ERR_NO_DEVICE;
  const DeviceInfo& d = device_info();
  TilePlan t;
  const int variant = g_kernel_variant;
  if (variant == 0 && plan_lane(*p, &t)) return 0;
  if ((variant == 0 || variant == 3) &&
      plan_tma_tiles(p->nx, p->ny, p->nz, p->num_oris, p->bc_x, d.sm_count, d.smem_per_sm, &t))
    return fixed_plan_index(p->num_oris, t);
  return 0;
}

extern "C" int pfg_device_error(int clear) {
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  const int v = read_device_error(clear);
  const int w = read_lane_device_error(clear);
  const int b = read_batch_device_error(clear);
  if (v < 0) return v;
  if (w < 0) return w;
  if (b < 0) return b;
  return v ? v : (w ? w : b);
}

extern "C" int pfg_set_kernel_variant(int variant) {
  if (variant < 0 || variant > 3) return PFG_ERR_PARAM;
  g_kernel_variant = variant;
  return PFG_OK;
}

extern "C" int pfg_pf_step(const pfg_pf_params* p, const float* eta_in, float* eta_out,
                           const float* T, float dt, void* stream) {
  int st = check_pf_params(p);
  if (st) return st;
  if (!eta_in || !eta_out || !T) return PFG_ERR_NULL;
  if (!aligned16(eta_in) || !aligned16(eta_out)) return PFG_ERR_ALIGN;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  StepArgs a{};
  a.eta_in = eta_in; a.eta_out = eta_out; a.T = T; a.T_out = nullptr;
  a.clk_in = nullptr; a.clk_out = nullptr;
  return record_cuda(dispatch<kTArray>(a, *p, dt, static_cast<cudaStream_t>(stream)));
}

extern "C" int pfg_pf_step_quench(const pfg_pf_params* p, const pfg_quench* q,
                                  const float* eta_in, float* eta_out, const pfg_clock* clk_in,
                                  pfg_clock* clk_out, float dt, void* stream) {
  int st = check_pf_params(p);
  if (st) return st;
  if (!q || !eta_in || !eta_out || !clk_in) return PFG_ERR_NULL;
  if (clk_in == clk_out) return PFG_ERR_PARAM;
  if (!aligned16(eta_in) || !aligned16(eta_out)) return PFG_ERR_ALIGN;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  StepArgs a{};
  a.eta_in = eta_in; a.eta_out = eta_out; a.T = nullptr; a.T_out = nullptr;
  a.clk_in = clk_in; a.clk_out = clk_out;
  a.q = *q;
  return record_cuda(dispatch<kTQuench>(a, *p, dt, static_cast<cudaStream_t>(stream)));
}

extern "C" int pfg_pf_step_point_source(const pfg_pf_params* p, const pfg_point_sources* src,
                                        const float* eta_in, float* eta_out,
                                        const pfg_clock* clk_in, pfg_clock* clk_out, float dt,
                                        void* stream) {
  int st = check_pf_params(p);
  if (st) return st;
  st = check_point_sources(src);
  if (st) return st;
  if (!eta_in || !eta_out || !clk_in) return PFG_ERR_NULL;
  if (clk_in == clk_out) return PFG_ERR_PARAM;
  if (!aligned16(eta_in) || !aligned16(eta_out)) return PFG_ERR_ALIGN;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  StepArgs a{};
  a.eta_in = eta_in; a.eta_out = eta_out; a.T = nullptr; a.T_out = nullptr;
  a.clk_in = clk_in; a.clk_out = clk_out;
  a.ps = make_point_consts(*src, *p);
  return record_cuda(dispatch<kTPoint>(a, *p, dt, static_cast<cudaStream_t>(stream)));
}

extern "C" int pfg_pf_step_interp(const pfg_pf_params* p, const pfg_interp* w,
                                  const float* T_past, const float* T_future,
                                  const float* eta_in, float* eta_out, const pfg_clock* clk_in,
                                  pfg_clock* clk_out, float dt, void* stream) {
  int st = check_pf_params(p);
  if (st) return st;
  if (!w || !T_past || !T_future || !eta_in || !eta_out || !clk_in) return PFG_ERR_NULL;
  if (clk_in == clk_out) return PFG_ERR_PARAM;
  if (!(w->dt_coarse > 0.0)) return PFG_ERR_PARAM;
  if (!aligned16(eta_in) || !aligned16(eta_out)) return PFG_ERR_ALIGN;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  StepArgs a{};
  a.eta_in = eta_in; a.eta_out = eta_out; a.T = T_past; a.T2 = T_future; a.T_out = nullptr;
  a.clk_in = clk_in; a.clk_out = clk_out;
  a.t_future = w->t_future;
  a.dt_coarse = w->dt_coarse;
  return record_cuda(dispatch<kTInterp>(a, *p, dt, static_cast<cudaStream_t>(stream)));
}

// (nx, ny, nz) z-fastest -> (nz, ny, nx) x-fastest, 32 x 32 tiles of (x, z)
// through shared memory for each y.
__global__ void __launch_bounds__(256) transpose_xyz_kernel(int nx, int ny, int nz,
                                                             const float* __restrict__ src,
                                                             float* __restrict__ dst) {
  __shared__ float tile[32][33];
  const int z0 = blockIdx.x * 32, x0 = blockIdx.y * 32, y = blockIdx.z;
  for (int k = threadIdx.y; k < 32; k += 8) {  // read rows of x, z fastest
    const int x = x0 + k, z = z0 + threadIdx.x;
    if (x < nx && z < nz) tile[k][threadIdx.x] = src[((int64_t)x * ny + y) * nz + z];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += 8) {  // write rows of z, x fastest
    const int z = z0 + k, x = x0 + threadIdx.x;
    if (x < nx && z < nz) dst[((int64_t)z * ny + y) * nx + x] = tile[threadIdx.x][k];
  }
}

extern "C" int pfg_transpose_xyz(int32_t nx, int32_t ny, int32_t nz, const float* T_xyz,
                                 float* T_zyx, void* stream) {
  if (nx < 1 || ny < 1 || nz < 1 || ny > 65535) return PFG_ERR_SHAPE;
  if (!T_xyz || !T_zyx) return PFG_ERR_NULL;
  if (T_xyz == T_zyx) return PFG_ERR_PARAM;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  const dim3 grid((unsigned)((nz + 31) / 32), (unsigned)((nx + 31) / 32), (unsigned)ny);
  transpose_xyz_kernel<<<grid, dim3(32, 8), 0, static_cast<cudaStream_t>(stream)>>>(nx, ny, nz,
                                                                                    T_xyz, T_zyx);
  return record_cuda(cudaGetLastError());
}

extern "C" int pfg_point_source_T(const pfg_pf_params* p, const pfg_point_sources* src,
                                  const pfg_clock* clk, float* T_out, void* stream) {
  int st = check_pf_params(p);
  if (st) return st;
  st = check_point_sources(src);
  if (st) return st;
  if (!clk || !T_out) return PFG_ERR_NULL;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  const int64_t N = (int64_t)p->nx * p->ny * p->nz;
  const int64_t want = (N + kThreads - 1) / kThreads;
  const int64_t cap = (int64_t)device_info().sm_count * 8;
  const int grid = (int)(want < cap ? want : cap);
  point_T_kernel<<<grid, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      make_point_consts(*src, *p), clk, T_out, p->nx, p->ny, p->nz);
  return record_cuda(cudaGetLastError());
}

extern "C" int pfg_heat_pf_step(const pfg_pf_params* p, const pfg_heat_params* h,
                                const float* eta_in, float* eta_out, const float* Tg_in,
                                float* Tg_out, const pfg_clock* clk_in, pfg_clock* clk_out,
                                float dt, void* stream) {
  int st = check_pf_params(p);
  if (st) return st;
  st = check_heat_params(h);
  if (st) return st;
  if (h->nx != p->nx || h->ny != p->ny || h->nz != p->nz) return PFG_ERR_SHAPE;
  if (p->bc_x || p->bc_y || p->bc_z) return PFG_ERR_PARAM;  // heat faces are not periodic
  if (h->layout != PFG_LAYOUT_ZYX) return PFG_ERR_PARAM;
  if (!eta_in || !eta_out || !Tg_in || !Tg_out || !clk_in) return PFG_ERR_NULL;
  if (clk_in == clk_out) return PFG_ERR_PARAM;
  if (!aligned16(eta_in) || !aligned16(eta_out)) return PFG_ERR_ALIGN;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  StepArgs a{};
  a.eta_in = eta_in; a.eta_out = eta_out; a.T = Tg_in; a.T_out = Tg_out;
  a.clk_in = clk_in; a.clk_out = clk_out;
  a.hc = make_heat_consts(*h);
  a.hp = *h;
  return record_cuda(dispatch<kTHeat>(a, *p, dt, static_cast<cudaStream_t>(stream)));
}

extern "C" int pfg_heat_pf_step_comp_supported(const pfg_pf_params* p) {
  int st = check_pf_params(p);
  if (st) return -st;
  if (!device_info().ok) return -PFG_ERR_NO_DEVICE;
  if ((int64_t)(p->nx + 2) * (p->ny + 2) * (p->nz + 2) >= ((int64_t)1 << 31)) return 0;
  const DeviceInfo& d = device_info();
  TilePlan t;
  const int v = g_kernel_variant;
  if (v == 0 && plan_lane(*p, &t)) return 1;
  return ((v == 0 || v == 3) && plan_tma_tiles(p->nx, p->ny, p->nz, p->num_oris, p->bc_x,
                                               d.sm_count, d.smem_per_sm, &t))
             ? 1
             : 0;
}

extern "C" int pfg_heat_pf_step_comp(const pfg_pf_params* p, const pfg_heat_params* h,
                                     const float* eta_in, float* eta_out, const float* Tg_in,
                                     const float* Tlo_in, float* Tg_out, float* Tlo_out,
                                     const pfg_clock* clk_in, pfg_clock* clk_out, float dt,
                                     void* stream) {
  int st = check_pf_params(p);
  if (st) return st;
  st = check_heat_params(h);
  if (st) return st;
  if (h->nx != p->nx || h->ny != p->ny || h->nz != p->nz) return PFG_ERR_SHAPE;
  if (p->bc_x || p->bc_y || p->bc_z) return PFG_ERR_PARAM;  // heat faces are not periodic
  if (h->layout != PFG_LAYOUT_ZYX) return PFG_ERR_PARAM;
  if (!eta_in || !eta_out || !Tg_in || !Tg_out || !Tlo_in || !Tlo_out || !clk_in)
    return PFG_ERR_NULL;
  if (clk_in == clk_out || Tg_in == Tg_out || Tlo_in == Tlo_out) return PFG_ERR_PARAM;
  if (!aligned16(eta_in) || !aligned16(eta_out)) return PFG_ERR_ALIGN;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  // ghosted offsets are 32-bit in the compensated kernels
  if ((int64_t)(p->nx + 2) * (p->ny + 2) * (p->nz + 2) >= ((int64_t)1 << 31))
    return PFG_ERR_SHAPE;
  const DeviceInfo& d = device_info();
  const int v = g_kernel_variant;
  StepArgs a{};
  a.eta_in = eta_in; a.eta_out = eta_out; a.T = Tg_in; a.T_out = Tg_out;
  a.T_lo = Tlo_in; a.T_lo_out = Tlo_out;
  a.clk_in = clk_in; a.clk_out = clk_out;
  a.hc = make_heat_consts(*h);
  a.hd = make_heat_df(*h, dt);
  a.hp = *h;
  const cudaStream_t cs = static_cast<cudaStream_t>(stream);
  TilePlan t;
  if (v == 0 && plan_lane(*p, &t)) {  // the heat update inside the stencil
    fill_common(a, *p, t, dt);
    a.cpw = t.cpw; a.wx = t.wx; a.rpw = t.rpw;
    return record_cuda(launch_lane_kernel<kTHeat>(a, t, cs));
  }
  if ((v == 0 || v == 3) &&
      plan_tma_tiles(p->nx, p->ny, p->nz, p->num_oris, p->bc_x, d.sm_count, d.smem_per_sm, &t)) {
    // the compensated heat update in its own kernel, then the phase field
    // with the start-of-step pair (both read only the old state)
    fill_common(a, *p, t, dt);
    a.cpw = t.cpw; a.wx = t.wx; a.rpw = t.rpw;
    cudaError_t e = launch_heat_comp(a, cs);
    if (e != cudaSuccess) return record_cuda(e);
    return record_cuda(launch_tma_kernel<kTHeat>(a, t, cs));
  }
  return PFG_ERR_PARAM;
}
