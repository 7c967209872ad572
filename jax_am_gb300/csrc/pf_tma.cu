// TMA-fed phase-field step: the fast path when num_oris is a multiple of 4.
//
// Same tiling and arithmetic as the warp-per-cells kernel (warps own whole
// cells, per-cell coefficients one plane ahead, folded element update), with
// the staging done by the Tensor Memory Accelerator:
//  * Each halo row of a plane tile is one contiguous run of cells in HBM and
//    is copied into shared memory by one cp.async.bulk (TMA) transfer that
//    completes on the slot's mbarrier (expect-tx bytes).  The temperature
//    tile (4-byte cells, unaligned rows) goes through ordinary cp.async copies
//    that arrive on the same barrier.
//  * All threads compute; after the per-plane barrier (which every thread
//    passes anyway for the coefficient buffer) warp 0 issues the copies of
//    the plane S-1 ahead into the slot everyone has just finished with, so no
//    producer warp and no "empty" barriers are needed and the CTA keeps the
//    full register budget (16 warps per SM).
//  * Neumann halo cells along x are never copied: the stencil offset of the
//    edge cell points at itself.  Periodic halo cells are copied by TMA.
// Every wait is bounded (about one second of clock64 cycles); a wait that
// runs out sets the library's device error flag, the CTA drains its copies in
// flight and returns.
#include <cuda_runtime.h>

#include <type_traits>

#include <algorithm>
#include <cmath>

#include "pfg_host.h"
#include "pfg_mbar.cuh"
#include "pfg_step.cuh"
#include "pfg_tma.cuh"
#include "pfg_warp.cuh"

namespace pfg {

__device__ int g_pfg_device_error = 0;  // PFG_ERR_TIMEOUT once a bounded wait ran out

template <bool ANISO, int TSRC, int NC, int VEC, int FIX>
__global__ void __launch_bounds__(NC, NC == 256 ? 2 : 1)
pf_tma_kernel(const __grid_constant__ StepArgs a) {
  tma_unit<ANISO, TSRC, NC, VEC, FIX, false>(a, blockIdx.x, a.eta_in, a.eta_out, 0.0, false,
                                             &g_pfg_device_error);
}


// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

int g_tma_consumers = 256;  // threads per CTA: 256 (two CTAs per SM) or 512 (one per SM)

bool plan_tma_tiles(int nx, int ny, int nz, int n, int bcx, int sm_count, int max_smem_per_sm,
                    TilePlan* out) {
  // 16-byte vectors, or 8-byte vectors with the aligned-row conditions above
  const bool vec2 = (n % 4 == 2) && (nx % 2 == 0) && bcx == PFG_BC_NEUMANN &&
                    g_tma_consumers == 256;
  if (n % 4 != 0 && !vec2) return false;
  // ghosted temperature offsets are 32-bit in this kernel
  if ((int64_t)(nx + 2) * (ny + 2) * (nz + 2) >= ((int64_t)1 << 31)) return false;
  TilePlan t{};
  const int warps = g_tma_consumers / 32;
  const int ctas = g_tma_consumers == 256 ? 2 : 1;
  const size_t budget = (size_t)max_smem_per_sm / ctas - 2048 - 6 * sizeof(uint64_t) - 64;
  // VEC = 2 rows carry up to two more cells (the even-aligned copy range)
  if (!plan_warp_tiles_ex(nx, ny, nz, n, sm_count, budget, warps, ctas, 2 * g_tma_consumers, &t,
                          vec2 ? 2 : 0, vec2))
    return false;
  // each thread stages at most three temperature cells of a plane
  if ((t.tx + 2) * (t.ty + 2) > 3 * g_tma_consumers) return false;
  // the ring's barriers sit after the coefficient buffer
  t.smem += (size_t)t.stages * sizeof(uint64_t);
  t.rs = g_tma_consumers;  // threads of this plan
  *out = t;
  return true;
}

template <bool ANISO, int TSRC, int NC, int VEC, int FIX = 0>
static cudaError_t launch_tma_t(const StepArgs& a, const TilePlan& t, cudaStream_t s) {
  auto k = pf_tma_kernel<ANISO, TSRC, NC, VEC, FIX>;
  static int configured[64] = {0};
  const int dev = device_info().device;
  if (dev < 0 || dev >= 64 || configured[dev] < (int)t.smem) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)t.smem);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64) configured[dev] = (int)t.smem;
  }
  k<<<(unsigned)t.units, NC, t.smem, s>>>(a);
  return cudaGetLastError();
}

// the plan is exactly FixedPlan<FIX>
template <int FIX>
static bool plan_is(int n, const TilePlan& t) {
  using FP = FixedPlan<FIX>;
  return t.rs == 256 && t.vec == FP::vec && n == FP::n && t.tx == FP::tx && t.ty == FP::ty &&
         t.rpw == FP::rpw && t.cpw == FP::cpw && t.wx == FP::wx && t.tpc == FP::tpc &&
         t.stages == FP::stages && t.pitch == FP::pitch && t.tslot == FP::tslot;
}

extern int g_fixed_plans;
int fixed_plan_index(int n, const TilePlan& t) {
  if (!g_fixed_plans) return 0;
  return plan_is<1>(n, t) ? 1 : (plan_is<2>(n, t) ? 2 : 0);
}

// ... and the launch arguments carry exactly that plan
template <int FIX>
static bool is_fixed_plan(const StepArgs& a, const TilePlan& t) {
  using FP = FixedPlan<FIX>;
  return t.rs == 256 && t.vec == FP::vec && a.n == FP::n && t.tx == FP::tx && t.ty == FP::ty &&
         t.rpw == FP::rpw && t.cpw == FP::cpw && t.wx == FP::wx && t.tpc == FP::tpc &&
         t.stages == FP::stages && t.pitch == FP::pitch && t.tslot == FP::tslot &&
         a.pitch == FP::pitch && a.tx == FP::tx && a.ty == FP::ty && a.rpw == FP::rpw &&
         a.cpw == FP::cpw && a.wx == FP::wx && a.tpc == FP::tpc && a.stages == FP::stages &&
         a.tslot == FP::tslot;
}

int g_fixed_plans = 1;  // pfg_tune key 7: 0 runs every plan through the run-time-plan instance

template <int TSRC>
cudaError_t launch_tma_kernel(const StepArgs& a, const TilePlan& t, cudaStream_t s) {
  if (g_fixed_plans && is_fixed_plan<1>(a, t))
    return (a.pc.aniso > 0.f) ? launch_tma_t<true, TSRC, 256, 4, 1>(a, t, s)
                              : launch_tma_t<false, TSRC, 256, 4, 1>(a, t, s);
  if (g_fixed_plans && is_fixed_plan<2>(a, t))
    return (a.pc.aniso > 0.f) ? launch_tma_t<true, TSRC, 256, 2, 2>(a, t, s)
                              : launch_tma_t<false, TSRC, 256, 2, 2>(a, t, s);
  if (t.rs == 512)
    return (a.pc.aniso > 0.f) ? launch_tma_t<true, TSRC, 512, 4>(a, t, s)
                              : launch_tma_t<false, TSRC, 512, 4>(a, t, s);
  if (t.vec == 2)
    return (a.pc.aniso > 0.f) ? launch_tma_t<true, TSRC, 256, 2>(a, t, s)
                              : launch_tma_t<false, TSRC, 256, 2>(a, t, s);
  return (a.pc.aniso > 0.f) ? launch_tma_t<true, TSRC, 256, 4>(a, t, s)
                            : launch_tma_t<false, TSRC, 256, 4>(a, t, s);
}

template cudaError_t launch_tma_kernel<kTArray>(const StepArgs&, const TilePlan&, cudaStream_t);
template cudaError_t launch_tma_kernel<kTHeat>(const StepArgs&, const TilePlan&, cudaStream_t);
template cudaError_t launch_tma_kernel<kTQuench>(const StepArgs&, const TilePlan&, cudaStream_t);
template cudaError_t launch_tma_kernel<kTPoint>(const StepArgs&, const TilePlan&, cudaStream_t);
template cudaError_t launch_tma_kernel<kTInterp>(const StepArgs&, const TilePlan&, cudaStream_t);

int read_device_error(int clear) {
  int v = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, g_pfg_device_error, sizeof(int));
  if (e != cudaSuccess) return record_cuda(e);
  if (clear && v) {
    const int zero = 0;
    e = cudaMemcpyToSymbol(g_pfg_device_error, &zero, sizeof(int));
    if (e != cudaSuccess) return record_cuda(e);
  }
  return v;
}

}  // namespace pfg
