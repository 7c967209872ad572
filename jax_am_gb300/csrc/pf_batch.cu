// Batched serving step: many independent directional-solidification jobs,
// one launch advancing every active job by one step.
//
// The encoded table (host-built by pfg_batch_encode, copied to the device by
// the caller) holds a header and one record per job: the job's full step
// arguments (grid, tile plan, physics, grain directions), its double buffer,
// start time and step counters, and the prefix sum of work units.  A fixed
// grid of persistent CTAs (two per SM) walks the units of all jobs; each unit
// is a tile x z-chunk of one job, processed by the single-job kernels' unit
// bodies: the TMA-fed body (pfg_tma.cuh) for orientation counts that are a
// multiple of 4 (the server pads every job to one), else the cp.async
// warp-per-cells body (pfg_warp.cuh).  A unit's job arguments are copied to
// shared memory, and the TMA-fed body's ring barriers, in static shared
// memory, are invalidated and initialised again for every unit.  Because the
// grid and the table's address never
// change, a graph of K launches (k = 0 .. K-1) is captured once and replayed
// while the host rewrites the table between replays (admitting and retiring
// jobs: continuous batching).
//
// Units are handed out dynamically: each CTA takes the next unit from a
// counter in the table header, and the encoder orders the jobs by unit cost,
// largest first, so that units of very different sizes (jobs differ tenfold
// in tile and column size) still finish together.  The last CTA of a launch
// to run out of units resets the counter for the next launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <utility>
#include <vector>

#include "pfg_host.h"
#include "pfg_step.cuh"
#include "pfg_tma.cuh"
#include "pfg_warp.cuh"

namespace pfg {

struct BatchJobDev {
  StepArgs args;
  float* eta[2];
  double t0;
  long long base_step, target_steps;
  long long unit_begin;
  int units, vec, aniso;
  int body;  // 1: the TMA-fed unit body (num_oris % 4 == 0), 0: warp-per-cells
};

struct BatchHeader {
  int num_jobs, pad;
  long long total_units;
  unsigned long long next_unit;  // dynamic unit counter (zero between launches)
  unsigned int done_ctas;        // CTAs of this launch that ran out of units
  int pad2;
};
static_assert(sizeof(BatchHeader) % 16 == 0, "job records follow the header 16-byte aligned");

constexpr int kBatchVersion = 2;
constexpr int kBatchCachedJobs = 256;  // job tables up to this size are searched in shared memory

__device__ int g_batch_device_error = 0;  // PFG_ERR_TIMEOUT once a bounded wait ran out

__global__ void __launch_bounds__(kThreads, 2)
pf_batch_kernel(BatchHeader* __restrict__ hdr, int k) {
  extern __shared__ __align__(128) float smem[];
  __shared__ __align__(16) StepArgs s_args;
  __shared__ int s_job;
  __shared__ long long s_unit;
  __shared__ int s_begin[kBatchCachedJobs];  // the jobs' first units (host keeps them < 2^31)
  const BatchJobDev* jobs = reinterpret_cast<const BatchJobDev*>(hdr + 1);
  const long long total = hdr->total_units;
  const int nj = hdr->num_jobs;
  const bool cached = nj <= kBatchCachedJobs;
  if (cached)
    for (int i = threadIdx.x; i < nj; i += blockDim.x) s_begin[i] = (int)jobs[i].unit_begin;
  __syncthreads();
  bool tma_barriers = false;  // this CTA's TMA-unit barriers are initialised
  for (;;) {
    if (threadIdx.x == 0) {
      const long long u = (long long)atomicAdd(&hdr->next_unit, 1ULL);
      s_unit = u;
      if (u < total) {
        int lo = 0, hi = nj - 1;  // last job whose first unit is <= u
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if ((cached ? (long long)s_begin[mid] : jobs[mid].unit_begin) <= u) lo = mid;
          else hi = mid - 1;
        }
        s_job = lo;
      }
    }
    __syncthreads();
    const long long u = s_unit;
    if (u >= total) break;  // uniform across the CTA
    const BatchJobDev& J = jobs[s_job];
    const long long step = J.base_step + k;
    if (step < J.target_steps && J.body == 1) {  // uniform over the CTA
      {  // the job's arguments into shared memory (3 % faster than reading the table)
        const int4* src = reinterpret_cast<const int4*>(&J.args);
        int4* dst = reinterpret_cast<int4*>(&s_args);
        for (int i = threadIdx.x; i < (int)(sizeof(StepArgs) / 16); i += kThreads) dst[i] = src[i];
        __syncthreads();
      }
      const double t0 = J.t0 + (double)step * (double)J.args.dt;
      const int unit = (int)(u - J.unit_begin);
      const float* ein = J.eta[step & 1];
      float* eout = J.eta[(step + 1) & 1];
      if (J.aniso)
        tma_unit<true, kTQuench, kThreads, 4, 0, true>(s_args, unit, ein, eout, t0, tma_barriers,
                                                       &g_batch_device_error);
      else
        tma_unit<false, kTQuench, kThreads, 4, 0, true>(s_args, unit, ein, eout, t0, tma_barriers,
                                                        &g_batch_device_error);
      tma_barriers = true;
    } else if (step < J.target_steps) {  // uniform over the CTA
      // the job's arguments into shared memory, then this step's buffers
      const int4* src = reinterpret_cast<const int4*>(&J.args);
      int4* dst = reinterpret_cast<int4*>(&s_args);
      for (int i = threadIdx.x; i < (int)(sizeof(StepArgs) / 16); i += kThreads) dst[i] = src[i];
      __syncthreads();
      if (threadIdx.x == 0) {
        s_args.eta_in = J.eta[step & 1];
        s_args.eta_out = J.eta[(step + 1) & 1];
      }
      __syncthreads();
      const double t0 = J.t0 + (double)step * (double)s_args.dt;
      const int unit = (int)(u - J.unit_begin);
      const int vec = J.vec;
      if (J.aniso) {
        if (vec == 4) warp_unit<4, true, kTQuench>(s_args, unit, t0, smem);
        else if (vec == 2) warp_unit<2, true, kTQuench>(s_args, unit, t0, smem);
        else warp_unit<1, true, kTQuench>(s_args, unit, t0, smem);
      } else {
        if (vec == 4) warp_unit<4, false, kTQuench>(s_args, unit, t0, smem);
        else if (vec == 2) warp_unit<2, false, kTQuench>(s_args, unit, t0, smem);
        else warp_unit<1, false, kTQuench>(s_args, unit, t0, smem);
      }
    }
    __syncthreads();  // shared memory is reused by the next unit
  }
  // the last CTA out resets the counter: every CTA has stopped taking units
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&hdr->done_ctas, 1u) == gridDim.x - 1) {
      atomicExch(&hdr->next_unit, 0ULL);
      atomicExch(&hdr->done_ctas, 0u);
    }
  }
}

static_assert(sizeof(StepArgs) % 16 == 0, "StepArgs is copied as int4");

// After a replay of k_steps launches: every job's base_step += k_steps (the
// host keeps the same count, so the table needs no rewrite between replays).
__global__ void pf_batch_advance_kernel(BatchHeader* __restrict__ hdr, int k_steps) {
  BatchJobDev* jobs = reinterpret_cast<BatchJobDev*>(hdr + 1);
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < hdr->num_jobs;
       j += gridDim.x * blockDim.x)
    jobs[j].base_step += k_steps;
}

// Dynamic shared memory of every batch launch: two CTAs per SM, less the
// kernel's static shared memory.
static size_t batch_smem_budget(const DeviceInfo& d) {
  return (size_t)d.smem_per_sm / 2 - 2048 - sizeof(StepArgs) - 64 - kBatchCachedJobs * sizeof(int);
}

}  // namespace pfg

using namespace pfg;

namespace pfg {
int read_batch_device_error(int clear) {
  int v = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, g_batch_device_error, sizeof(int));
  if (e != cudaSuccess) return record_cuda(e);
  if (clear && v) {
    const int zero = 0;
    e = cudaMemcpyToSymbol(g_batch_device_error, &zero, sizeof(int));
    if (e != cudaSuccess) return record_cuda(e);
  }
  return v;
}
}  // namespace pfg

extern "C" int64_t pfg_batch_table_bytes(int num_jobs) {
  if (num_jobs < 0) return -1;
  return (int64_t)sizeof(BatchHeader) + (int64_t)num_jobs * (int64_t)sizeof(BatchJobDev);
}

extern "C" int pfg_batch_encode(const pfg_batch_job* jobs, int num_jobs, void* table,
                                int64_t table_bytes, int64_t* total_units) {
  if (num_jobs < 0) return PFG_ERR_PARAM;
  if (!table || (num_jobs > 0 && !jobs)) return PFG_ERR_NULL;
  if (table_bytes < pfg_batch_table_bytes(num_jobs)) return PFG_ERR_CAPACITY;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  const DeviceInfo& d = device_info();
  const size_t budget = batch_smem_budget(d);
  BatchHeader* hdr = static_cast<BatchHeader*>(table);
  BatchJobDev* out = reinterpret_cast<BatchJobDev*>(hdr + 1);
  std::vector<TilePlan> plans((size_t)num_jobs);
  std::vector<int> bodies((size_t)num_jobs, 0);
  std::vector<std::pair<double, int>> order((size_t)num_jobs);
  for (int j = 0; j < num_jobs; ++j) {
    const pfg_batch_job& J = jobs[j];
    int st = check_pf_params(&J.params);
    if (st) return st;
    if (!J.eta[0] || !J.eta[1]) return PFG_ERR_NULL;
    if (!aligned16(J.eta[0]) || !aligned16(J.eta[1])) return PFG_ERR_ALIGN;
    if (J.eta[0] == J.eta[1] || J.target_steps < 0 || J.base_step < 0) return PFG_ERR_PARAM;
    TilePlan& t = plans[(size_t)j];
    // tiles chosen for cover and halo only: the batch has units enough to
    // fill the GPU whatever their count.  num_oris % 4 == 0: the TMA-fed
    // body (at most two cells per thread in its per-cell pass, 16-byte
    // vectors, ring barriers in static shared memory)
    bool tma = false;
    if (J.params.num_oris % 4 == 0 &&
        plan_warp_tiles_ex(J.params.nx, J.params.ny, J.params.nz, J.params.num_oris, d.sm_count,
                           budget - 64, kThreads / 32, 0, 2 * kThreads, &t) &&
        t.vec == 4 && t.stages <= kTmaMaxStages &&
        std::min(J.params.nz, 64) + 2 <= kTmaMaxPlanes) {
      t.rs = kThreads;
      tma = true;
    } else if (!plan_warp_tiles_ex(J.params.nx, J.params.ny, J.params.nz, J.params.num_oris,
                                   d.sm_count, budget, kThreads / 32, 0, 1 << 30, &t)) {
      return PFG_ERR_SHAPE;  // orientation count the warp-per-cells body cannot take
    }
    bodies[(size_t)j] = tma ? 1 : 0;
    // units of whole z columns (or 64-plane chunks), so that few halo planes
    // are read twice
    const int zch = std::max(1, (J.params.nz + 63) / 64);
    t.zc = (J.params.nz + zch - 1) / zch;
    t.zchunks = (J.params.nz + t.zc - 1) / t.zc;
    t.units = (long)t.tiles_x * t.tiles_y * t.zchunks;
    // bytes a unit moves: its tile with halo, its planes with halo, n floats
    const double cost = (double)(t.tx + 2) * (t.ty + 2) * (t.zc + 2) * J.params.num_oris;
    order[(size_t)j] = {-cost, j};
  }
  // largest units first (stable: equal costs keep the caller's order)
  std::stable_sort(order.begin(), order.end(),
                   [](const std::pair<double, int>& x, const std::pair<double, int>& y) {
                     return x.first < y.first;
                   });
  long long units = 0;
  for (int r = 0; r < num_jobs; ++r) {
    const int j = order[(size_t)r].second;
    const pfg_batch_job& J = jobs[j];
    const TilePlan& t = plans[(size_t)j];
    BatchJobDev& D = out[r];
    std::memset(&D, 0, sizeof(D));
    fill_step_args(D.args, J.params, t, J.dt);
    D.args.cpw = t.cpw; D.args.wx = t.wx; D.args.rpw = t.rpw;
    D.args.q = J.quench;
    D.args.clk_in = nullptr; D.args.clk_out = nullptr;
    D.eta[0] = J.eta[0]; D.eta[1] = J.eta[1];
    D.t0 = J.t0;
    D.base_step = J.base_step;
    D.target_steps = J.target_steps;
    D.unit_begin = units;
    D.units = (int)t.units;
    D.vec = t.vec;
    D.aniso = J.params.anisotropy > 0.f ? 1 : 0;
    D.body = bodies[(size_t)j];
    units += t.units;
  }
  if (units >= ((long long)1 << 31)) return PFG_ERR_CAPACITY;  // unit indices are 32-bit
  hdr->num_jobs = num_jobs;
  hdr->pad = kBatchVersion;
  hdr->total_units = units;
  hdr->next_unit = 0;
  hdr->done_ctas = 0;
  hdr->pad2 = 0;
  if (total_units) *total_units = units;
  return PFG_OK;
}

extern "C" int pfg_batch_step(void* device_table, int k, void* stream) {
  if (!device_table) return PFG_ERR_NULL;
  if (k < 0) return PFG_ERR_PARAM;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  const DeviceInfo& d = device_info();
  const size_t smem = batch_smem_budget(d);
  static int configured[64] = {0};
  const int dev = d.device;
  if (dev < 0 || dev >= 64 || configured[dev] < (int)smem) {
    cudaError_t e = cudaFuncSetAttribute(pf_batch_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return record_cuda(e);
    if (dev >= 0 && dev < 64) configured[dev] = (int)smem;
  }
  pf_batch_kernel<<<2 * d.sm_count, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(
      static_cast<BatchHeader*>(device_table), k);
  return record_cuda(cudaGetLastError());
}

extern "C" int pfg_batch_advance(void* device_table, int k_steps, void* stream) {
  if (!device_table) return PFG_ERR_NULL;
  if (k_steps < 0) return PFG_ERR_PARAM;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  pf_batch_advance_kernel<<<1, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<BatchHeader*>(device_table), k_steps);
  return record_cuda(cudaGetLastError());
}
