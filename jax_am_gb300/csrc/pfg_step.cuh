// Arguments of the stencil step kernels (internal).
#pragma once

#include "pfg_device.cuh"

namespace pfg {

// Where the phase field takes its temperature from.
enum TSource { kTArray = 0, kTHeat = 1, kTQuench = 2, kTPoint = 3, kTInterp = 4 };

struct __align__(16) StepArgs {
  int nx, ny, nz, n;
  int bcx, bcy, bcz;
  float dt;
  PFConsts pc;
  // tiling (generic kernel: rs rows in flight; warp-cell kernel: wx x wy warps,
  // cpw cells per warp, rpw rows per warp)
  int tx, ty, zc, stages, pitch, tslot, tpc, rs;
  int tiles_x, tiles_y, zchunks;
  int cpw, wx, rpw;
  // buffers
  const float* eta_in;
  float* eta_out;
  const float* T;  // per-cell T (pf only) or ghosted Tg (fused)
  float* T_out;    // ghosted Tg_out (fused) or nullptr
  const pfg_clock* clk_in;
  pfg_clock* clk_out;
  HeatConsts hc;
  HeatDF hd;           // compensated heat update constants (fused, T_lo set)
  const float* T_lo;   // low parts of the compensated ghosted T (or nullptr)
  float* T_lo_out;
  pfg_heat_params hp;  // tool path (fused)
  pfg_quench q;        // moving gradient (quench)
  PointConsts ps;      // moving point source
  const float* T2;     // interpolation: T_future (T holds T_past)
  double t_future, dt_coarse;
  float h_z;
  long long probe_wait;  // > 0: the wait probe (pfg_tune key 8), cycles
  float dirs[3 * PFG_MAX_ORIS * 3];
};


struct TilePlan;
int set_tune(int key, int value);
// Warp-per-cells kernel (pf_fast.cu).
bool plan_warp_tiles(int nx, int ny, int nz, int n, int sm_count, int max_smem_per_sm,
                     TilePlan* out);
bool plan_warp_tiles_budget(int nx, int ny, int nz, int n, int sm_count, size_t budget,
                            TilePlan* out);
bool plan_warp_tiles_ex(int nx, int ny, int nz, int n, int sm_count, size_t budget, int warps,
                        int ctas_per_sm, int max_cells, TilePlan* out, int extra_cells = 0,
                        bool even_tx = false);
template <int TSRC>
cudaError_t launch_warp_kernel(const StepArgs& a, const TilePlan& t, cudaStream_t s);
void fill_step_args(StepArgs& a, const pfg_pf_params& p, const TilePlan& t, float dt);
// TMA-fed kernel (pf_tma.cu), num_oris % 4 == 0.
bool plan_tma_tiles(int nx, int ny, int nz, int n, int bcx, int sm_count, int max_smem_per_sm,
                    TilePlan* out);
template <int TSRC>
cudaError_t launch_tma_kernel(const StepArgs& a, const TilePlan& t, cudaStream_t s);
// Which compile-time plan of the TMA-fed kernel (1 or 2) a TMA plan uses, or 0.
int fixed_plan_index(int n, const TilePlan& t);
// Cell-per-lane TMA kernel (pf_lane.cu), num_oris = 20.
bool plan_lane_tiles(int nx, int ny, int nz, int n, int sm_count, int max_smem_per_sm,
                     int max_smem_per_block, int zchunks_override, TilePlan* out);
template <int TSRC>
cudaError_t launch_lane_kernel(const StepArgs& a, const TilePlan& t, cudaStream_t s);
// Compensated heat step alone (heat_comp.cu): a.T, a.T_lo -> a.T_out,
// a.T_lo_out, the beam at mid-step from a.clk_in (the fused compensated step
// of the kernels other than the cell-per-lane one).
cudaError_t launch_heat_comp(const StepArgs& a, cudaStream_t s);
// The device error flags (PFG_ERR_TIMEOUT after a bounded wait ran out) of
// the TMA-fed and the cell-per-lane kernels, or a negative pfg_status if one
// cannot be read; clear != 0 resets it.
int read_device_error(int clear);
int read_lane_device_error(int clear);
int read_batch_device_error(int clear);
extern int g_tune_zchunks;
extern long long g_probe_wait;

}  // namespace pfg
