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
//  * The per-cell constants are folded so that one element costs 10 FP32
//    operations (33 with anisotropy, which needs one MUFU reciprocal and no
//    arccos); liquid forcing is folded into the constants as well.
//  * Staging copies each halo row as one contiguous run of VEC-float chunks
//    (no per-chunk index division); halo cells outside the grid are copied
//    separately from the boundary cell (Neumann) or the wrapped cell
//    (periodic).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "pfg_host.h"
#include "pfg_step.cuh"
#include "pfg_warp.cuh"

namespace pfg {

template <int VEC, bool ANISO, int TSRC>
__global__ void __launch_bounds__(kThreads, 2) pf_warp_kernel(const __grid_constant__ StepArgs a) {
  extern __shared__ __align__(16) float smem[];
  double t0 = 0.0;
  if constexpr (TSRC != kTArray) {
    t0 = a.clk_in->t;
    if (blockIdx.x == 0 && threadIdx.x == 0 && a.clk_out) {
      a.clk_out->t = t0 + (double)a.dt;
      a.clk_out->step = a.clk_in->step + 1;
    }
  }
  warp_unit<VEC, ANISO, TSRC>(a, blockIdx.x, t0, smem);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

extern int g_tma_consumers;
extern int g_cfd_cells_per_thread;
extern int g_fixed_plans;
// Plan overrides for tuning sweeps (0 = automatic).
static int g_tune_wx = 0, g_tune_rpw = 0, g_tune_stages = 0;
int g_tune_zchunks = 0;  // pfg_tune key 3 (every z-marching planner)
long long g_probe_wait = 0;  // pfg_tune key 8: cycles of the wait probe, 0 = off

int set_tune(int key, int value) {
  if (value < 0) return PFG_ERR_PARAM;
  switch (key) {
    case 0: if (value && value != 1 && value != 2 && value != 4 && value != 8 && value != 16)
              return PFG_ERR_PARAM;
            g_tune_wx = value; return PFG_OK;
    case 1: if (value > 32) return PFG_ERR_PARAM;
            g_tune_rpw = value; return PFG_OK;
    case 2: if (value && (value < 4 || value > 6)) return PFG_ERR_PARAM;
            g_tune_stages = value; return PFG_OK;
    case 3: g_tune_zchunks = value; return PFG_OK;
    case 5: if (value && value != 256 && value != 512) return PFG_ERR_PARAM;
            g_tma_consumers = value ? value : 256; return PFG_OK;
    case 6: if (value > 16) return PFG_ERR_PARAM;
            g_cfd_cells_per_thread = value ? value : 4; return PFG_OK;
    case 7: if (value > 1) return PFG_ERR_PARAM;
            g_fixed_plans = value ? 0 : 1; return PFG_OK;
    case 8: g_probe_wait = value; return PFG_OK;
    default: return PFG_ERR_PARAM;
  }
}

bool plan_warp_tiles(int nx, int ny, int nz, int n, int sm_count, int max_smem_per_sm,
                     TilePlan* out) {
  return plan_warp_tiles_budget(nx, ny, nz, n, sm_count,
                                (size_t)max_smem_per_sm / 2 - 2048, out);
}

bool plan_warp_tiles_budget(int nx, int ny, int nz, int n, int sm_count, size_t budget,
                            TilePlan* out) {
  return plan_warp_tiles_ex(nx, ny, nz, n, sm_count, budget, 8, 2, 1 << 30, out);
}

// warps: warps that own cells (the tile is wx * cpw by (warps / wx) * rpw cells);
// ctas_per_sm: for the wave count (0: the units share the GPU with other work,
// as in the batched step, so waves are not counted); max_cells: cap on tile
// cells.
bool plan_warp_tiles_ex(int nx, int ny, int nz, int n, int sm_count, size_t budget, int warps,
                        int ctas_per_sm, int max_cells, TilePlan* out, int extra_cells,
                        bool even_tx) {
  TilePlan t{};
  t.vec = vec_width(n);
  t.tpc = n / t.vec;
  if (t.tpc > 32) return false;
  t.cpw = 32 / t.tpc;
  t.stages = g_tune_stages ? g_tune_stages : 4;
  const long concurrent = (long)ctas_per_sm * sm_count;
  double best = 1e30;
  for (int wx = 1; wx <= warps; wx *= 2) {
    if (g_tune_wx && wx != g_tune_wx) continue;
    const int wy = warps / wx;
    const int tx = wx * t.cpw;
    if (!g_tune_wx && wx > 1 && (wx / 2) * t.cpw >= nx) continue;  // a narrower tile covers x
    if (even_tx && tx % 2 != 0) continue;
    for (int rpw = 1; rpw <= 32; ++rpw) {
      if (g_tune_rpw && rpw != g_tune_rpw) continue;
      const int ty = wy * rpw;
      if (!g_tune_rpw && rpw > 1 && wy * (rpw - 1) >= ny) break;
      const int pitch = ((tx + 2 + extra_cells) * n + 3) / 4 * 4;
      const int tslot = ((ty + 2) * (tx + 2) + 3) / 4 * 4;
      const size_t smem = (size_t)t.stages * ((size_t)(ty + 2) * pitch + tslot) * 4 +
                          (size_t)2 * ty * tx * 16;
      if (smem > budget || tx * ty > max_cells) break;
      const long tiles = (long)((nx + tx - 1) / tx) * ((ny + ty - 1) / ty);
      const double cover = (double)tiles * tx * ty / ((double)nx * ny);
      const double halo = (double)(tx + 2) * (ty + 2) / ((double)tx * ty);
      // wave quantisation of the units this tile gives
      long zch = (4 * concurrent + tiles - 1) / tiles;
      zch = std::max(1L, std::min(zch, (long)std::max(1, nz / 8)));
      const long zc = (nz + zch - 1) / zch;
      const double waves = (double)(tiles * ((nz + zc - 1) / zc)) / (double)concurrent;
      const double wave_eff = concurrent > 0 ? waves / std::ceil(waves) : 1.0;
      // measured on GB300: halo columns cost about twice what halo rows cost
      // (every staged row carries its two x-halo cells)
      const double hx = (double)(tx + 2) / tx, hy = (double)(ty + 2) / ty;
      const double score = cover * hx * hx * hy / wave_eff;
      (void)halo;
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
template cudaError_t launch_warp_kernel<kTPoint>(const StepArgs&, const TilePlan&, cudaStream_t);
template cudaError_t launch_warp_kernel<kTInterp>(const StepArgs&, const TilePlan&, cudaStream_t);

}  // namespace pfg
