// Run-time diagnostics of a phase-field state, reduced on the device.
//
// The reference's only observability on this path is PFSolver.inspect_sol
// (allen_cahn.py:165-180): percentage of cells whose argmax orientation
// changed, percentage of cells at or above the liquidus, max T and a NaN
// check.  This computes those counts plus the float64 free energy and
// per-orientation mass in one pass.  One warp handles one cell at a time,
// lanes spanning the orientations, so loads are coalesced and the argmax and
// sums are warp shuffles.  Per-block partial records go to a caller-provided
// scratch buffer; a second one-block kernel folds them in a fixed order, so
// the result is bit-reproducible.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "pfg_device.cuh"
#include "pfg_host.h"

namespace pfg {

struct DiagPartial {
  double energy;
  double max_T;
  long long changed, liquid, nonfinite, pad;
  double mass[PFG_MAX_ORIS];
};

struct DiagArgs {
  int nx, ny, nz, n;
  int bcx, bcy, bcz;
  int T_ghosted;
  double wx, wy, wz;  // 1/h per axis
  double m_g, kappa_half, vol, T_liq;
  const float* eta;
  const float* T;
  const int32_t* argmax0;
  int32_t* argmax_out;
  DiagPartial* partials;
};

constexpr int kDiagBlocks = 296;  // 2 x 148..152 SMs; fixed so results do not depend on the GPU

__device__ __forceinline__ bool argmax_better(float a, int ia, float b, int ib) {
  // np.argmax semantics: the first NaN wins, otherwise the first maximum
  const bool na = isnan(a), nb = isnan(b);
  if (na || nb) return na && (!nb || ia < ib);
  return a > b || (a == b && ia < ib);
}

__global__ void __launch_bounds__(256) pf_diag_kernel(const __grid_constant__ DiagArgs a) {
  __shared__ double s_mass[8][PFG_MAX_ORIS];
  __shared__ double s_energy[8], s_maxT[8];
  __shared__ long long s_cnt[8][3];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long ncell = (long long)a.nx * a.ny * a.nz;
  const long long gwarp = (long long)blockIdx.x * 8 + warp;
  const long long nwarps = (long long)gridDim.x * 8;
  const int n = a.n;
  double mass0 = 0.0, mass1 = 0.0, energy = 0.0, maxT = -INFINITY;
  long long changed = 0, liquid = 0, nonfinite = 0;
  const int64_t sy = (int64_t)a.nx * n, sz = (int64_t)a.ny * a.nx * n;
  for (long long c = gwarp; c < ncell; c += nwarps) {
    const int x = (int)(c % a.nx);
    const int y = (int)((c / a.nx) % a.ny);
    const int z = (int)(c / ((long long)a.nx * a.ny));
    const float* e = a.eta + c * n;
    const float v0 = (lane < n) ? e[lane] : 0.f;
    const float v1 = (lane + 32 < n) ? e[lane + 32] : 0.f;
    if (lane < n && !isfinite(v0)) ++nonfinite;
    if (lane + 32 < n && !isfinite(v1)) ++nonfinite;
    mass0 += v0;
    mass1 += v1;
    // argmax over the cell's orientations
    float best = (lane < n) ? v0 : -INFINITY;
    int bi = (lane < n) ? lane : 1 << 30;
    if (lane + 32 < n && argmax_better(v1, lane + 32, best, bi)) { best = v1; bi = lane + 32; }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (argmax_better(ob, oi, best, bi)) { best = ob; bi = oi; }
    }
    // local energy terms (allen_cahn.py:42-49) in float64
    const double d0 = v0, d1 = v1;
    double s2 = d0 * d0 + d1 * d1;
    double s4 = d0 * d0 * d0 * d0 + d1 * d1 * d1 * d1;
    // gradient energy: forward differences, zero across a Neumann face
    double g2 = 0.0;
    {
      const int xn = (x + 1 < a.nx) ? x + 1 : (a.bcx ? 0 : x);
      const int yn = (y + 1 < a.ny) ? y + 1 : (a.bcy ? 0 : y);
      const int zn = (z + 1 < a.nz) ? z + 1 : (a.bcz ? 0 : z);
      const float* ex = a.eta + (int64_t)z * sz + (int64_t)y * sy + (int64_t)xn * n;
      const float* ey = a.eta + (int64_t)z * sz + (int64_t)yn * sy + (int64_t)x * n;
      const float* ez = a.eta + (int64_t)zn * sz + (int64_t)y * sy + (int64_t)x * n;
      if (lane < n) {
        const double gx = ((double)ex[lane] - d0) * a.wx, gy = ((double)ey[lane] - d0) * a.wy,
                     gz = ((double)ez[lane] - d0) * a.wz;
        g2 += gx * gx + gy * gy + gz * gz;
      }
      if (lane + 32 < n) {
        const double gx = ((double)ex[lane + 32] - d1) * a.wx,
                     gy = ((double)ey[lane + 32] - d1) * a.wy,
                     gz = ((double)ez[lane + 32] - d1) * a.wz;
        g2 += gx * gx + gy * gy + gz * gz;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s2 += __shfl_xor_sync(0xffffffffu, s2, o);
      s4 += __shfl_xor_sync(0xffffffffu, s4, o);
      g2 += __shfl_xor_sync(0xffffffffu, g2, o);
    }
    if (lane == 0) {
      float T;
      if (a.T_ghosted) {
        const int64_t gsy = a.nx + 2, gsz = (int64_t)(a.ny + 2) * (a.nx + 2);
        T = a.T[(int64_t)(z + 1) * gsz + (int64_t)(y + 1) * gsy + x + 1];
      } else {
        T = a.T[c];
      }
      const double Tc = (T > 2000.f) ? 2000.0 : (double)T;
      const double zeta = 0.5 * (1.0 - tanh(1e10 * (Tc / a.T_liq - 1.0)));
      const double om = 1.0 - zeta;
      const double f_loc = a.m_g * ((s4 / 4.0 - s2 / 2.0) + (s2 * s2 - s4) + om * om * s2);
      energy += (f_loc + a.kappa_half * g2) * a.vol;
      if ((double)T >= a.T_liq) ++liquid;
      if ((double)T > maxT || isnan(T)) maxT = isnan(maxT) ? maxT : (double)T;
      if (a.argmax_out) a.argmax_out[c] = bi;
      if (a.argmax0 && a.argmax0[c] != bi) ++changed;
    }
  }
  // block reduction
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nonfinite += __shfl_xor_sync(0xffffffffu, nonfinite, o);
  if (lane < n) s_mass[warp][lane] = mass0;
  if (lane + 32 < n) s_mass[warp][lane + 32] = mass1;
  if (lane == 0) {
    s_energy[warp] = energy;
    s_maxT[warp] = maxT;
    s_cnt[warp][0] = changed;
    s_cnt[warp][1] = liquid;
    s_cnt[warp][2] = nonfinite;
  }
  __syncthreads();
  DiagPartial* out = a.partials + blockIdx.x;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double m = 0.0;
    for (int w = 0; w < 8; ++w) m += s_mass[w][i];
    out->mass[i] = m;
  }
  if (threadIdx.x == 0) {
    double en = 0.0, mt = -INFINITY;
    long long c0 = 0, c1 = 0, c2 = 0;
    for (int w = 0; w < 8; ++w) {
      en += s_energy[w];
      if (s_maxT[w] > mt || isnan(s_maxT[w])) mt = isnan(mt) ? mt : s_maxT[w];
      c0 += s_cnt[w][0];
      c1 += s_cnt[w][1];
      c2 += s_cnt[w][2];
    }
    out->energy = en;
    out->max_T = mt;
    out->changed = c0;
    out->liquid = c1;
    out->nonfinite = c2;
  }
}

__global__ void __launch_bounds__(256)
pf_diag_finish_kernel(const DiagPartial* __restrict__ parts, int nparts, int n, long long ncell,
                      pfg_diag* __restrict__ out) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double m = 0.0;
    for (int b = 0; b < nparts; ++b) m += parts[b].mass[i];
    out->mass[i] = m;
  }
  for (int i = n + threadIdx.x; i < PFG_MAX_ORIS; i += blockDim.x) out->mass[i] = 0.0;
  if (threadIdx.x == 0) {
    double en = 0.0, mt = -INFINITY;
    long long c0 = 0, c1 = 0, c2 = 0;
    for (int b = 0; b < nparts; ++b) {
      en += parts[b].energy;
      if (parts[b].max_T > mt || isnan(parts[b].max_T)) mt = isnan(mt) ? mt : parts[b].max_T;
      c0 += parts[b].changed;
      c1 += parts[b].liquid;
      c2 += parts[b].nonfinite;
    }
    out->energy = en;
    out->max_T = mt;
    out->n_cells = ncell;
    out->n_ori_changed = c0;
    out->n_liquid = c1;
    out->n_nonfinite = c2;
  }
}

int diag_blocks(const pfg_pf_params& p) {
  const long long ncell = (long long)p.nx * p.ny * p.nz;
  const long long need = (ncell + 7) / 8;
  return (int)(need < kDiagBlocks ? need : kDiagBlocks);
}

int launch_diag(const pfg_pf_params* p, const float* eta, const float* T, int T_ghosted,
                const int32_t* argmax0, int32_t* argmax_out, void* scratch,
                pfg_diag* out, cudaStream_t s) {
  DiagArgs a{};
  a.nx = p->nx; a.ny = p->ny; a.nz = p->nz; a.n = p->num_oris;
  a.bcx = p->bc_x; a.bcy = p->bc_y; a.bcz = p->bc_z;
  a.T_ghosted = T_ghosted;
  a.wx = 1.0 / p->h_x; a.wy = 1.0 / p->h_y; a.wz = 1.0 / p->h_z;
  a.m_g = p->m_g;
  a.kappa_half = 0.5 * (double)p->kappa_g;
  a.vol = (double)p->h_x * p->h_y * p->h_z;
  a.T_liq = p->T_liquidus;
  a.eta = eta; a.T = T; a.argmax0 = argmax0; a.argmax_out = argmax_out;
  a.partials = static_cast<DiagPartial*>(scratch);
  const int nb = diag_blocks(*p);
  pf_diag_kernel<<<nb, 256, 0, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return record_cuda(e);
  pf_diag_finish_kernel<<<1, 256, 0, s>>>(a.partials, nb, p->num_oris,
                                          (long long)p->nx * p->ny * p->nz, out);
  return record_cuda(cudaGetLastError());
}

}  // namespace pfg

using namespace pfg;

extern "C" int64_t pfg_pf_diag_scratch_bytes(const pfg_pf_params* p) {
  if (check_pf_params(p)) return -1;
  return (int64_t)diag_blocks(*p) * (int64_t)sizeof(DiagPartial);
}

extern "C" int pfg_pf_diag(const pfg_pf_params* p, const float* eta, const float* T,
                           int T_ghosted, const int32_t* argmax0, int32_t* argmax_out,
                           void* scratch, int64_t scratch_bytes, pfg_diag* out, void* stream) {
  int st = check_pf_params(p);
  if (st) return st;
  if (!eta || !T || !scratch || !out) return PFG_ERR_NULL;
  if (scratch_bytes < pfg_pf_diag_scratch_bytes(p)) return PFG_ERR_CAPACITY;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  return launch_diag(p, eta, T, T_ghosted, argmax0, argmax_out, scratch, out,
                     static_cast<cudaStream_t>(stream));
}

// ---------------------------------------------------------------------------
// Diagnostics that allocate nothing.
//
// Some callers cannot hand this library a scratch buffer or let it call
// cudaMalloc: a host framework that owns all device memory and gives a plugin
// only the buffers it planned ahead of time (an XLA custom call, a fixed
// arena in a real-time control loop), or a binding from a language that has
// no CUDA allocator.  pfg_pf_diag_noalloc keeps the per-block partial records
// in the file-scope array below instead.  It holds PFG_DIAG_NOALLOC_RECORDS
// records (165,760 bytes); every GPU that loads the library keeps it until the
// process exits.
// ---------------------------------------------------------------------------
namespace pfg {

static_assert(PFG_DIAG_NOALLOC_RECORDS >= kDiagBlocks,
              "the static array must hold the partials of the largest reduction");
static __device__ __align__(256) DiagPartial g_diag_noalloc_partials[PFG_DIAG_NOALLOC_RECORDS];

// Device address of g_diag_noalloc_partials on the current device, looked up
// once per device (in host code the symbol name is only a host-side handle).
static int noalloc_partials(void** out) {
  static void* addr[64] = {nullptr};
  static std::mutex mu;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return record_cuda(e);
  if (dev < 0 || dev >= 64) return PFG_ERR_NO_DEVICE;
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_diag_noalloc_partials);
    if (e != cudaSuccess) return record_cuda(e);
    addr[dev] = p;
  }
  *out = addr[dev];
  return PFG_OK;
}

}  // namespace pfg

extern "C" int pfg_pf_diag_noalloc(const pfg_pf_params* p, const float* eta, const float* T,
                                   int T_ghosted, const int32_t* argmax0, int32_t* argmax_out,
                                   pfg_diag* out, void* stream) {
  int st = check_pf_params(p);
  if (st) return st;
  if (!eta || !T || !out) return PFG_ERR_NULL;
  // every block of the reduction writes one record; they must all fit
  if ((int64_t)diag_blocks(*p) * (int64_t)sizeof(DiagPartial) >
      (int64_t)sizeof(g_diag_noalloc_partials))
    return PFG_ERR_CAPACITY;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  void* partials = nullptr;
  st = noalloc_partials(&partials);
  if (st) return st;
  // each block overwrites its whole record before the finishing kernel reads
  // it, and records past this call's block count are never read, so nothing
  // left over from an earlier call needs clearing
  return launch_diag(p, eta, T, T_ghosted, argmax0, argmax_out, partials, out,
                     static_cast<cudaStream_t>(stream));
}
