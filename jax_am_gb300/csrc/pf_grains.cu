// Grain segmentation of a phase-field state on the device.
//
// The reference's post-processing (jax_am/phase_field/utils.py:181-310)
// finds the grains of a solution by a breadth-first search on the host: two
// face-adjacent cells belong to the same grain when both are solid
// (T < T_liquidus) and have the same argmax orientation; grains are listed by
// orientation, then in the order the search meets them (increasing smallest
// cell index); each grain's volume and PCA aspect ratio follow from its cells'
// centres.
//
// Here the components come from a lock-free union-find over the cell grid:
//  1. every solid cell starts as its own root (liquid cells are -1);
//  2. each solid cell unites with its +x, +y, +z neighbours of the same
//     orientation (Playne and Hawick's merge: find both roots, hang the larger
//     root under the smaller with atomicMin, retry if that root moved);
//  3. every cell's label is replaced by its root.
// A root is therefore the smallest cell index of its component -- the cell at
// which the reference's search starts that grain.  Roots are then numbered in
// increasing index order (a block-wise scan), and one pass adds each cell's
// count and first and second coordinate moments into its grain's record
// (exact 64-bit integers, aggregated per warp before the atomics).  The
// caller orders the records by (orientation, first cell) to obtain the
// reference's order, and computes volumes and aspect ratios from the moments.
//
// Termination: a label only ever decreases and never drops below its own
// root's index, and a non-root always points to a smaller index, so every find
// walks a strictly decreasing chain and every merge retry sees a smaller root.
#include <cuda_runtime.h>

#include <cstdint>

#include "pfg_host.h"
#include "pfg_step.cuh"

namespace pfg {

constexpr int kGrainThreads = 256;
constexpr int kScanItems = 8;                           // cells per thread in the numbering pass
constexpr int kScanChunk = kGrainThreads * kScanItems;  // cells per numbering block

struct GrainArgs {
  int nx, ny, nz;
  int T_ghosted;
  float T_liq;
  const int32_t* ori;
  const float* T;
  int32_t* L;        // labels (N)
  int32_t* id;       // grain number of each root (N; only roots are written)
  int32_t* chunk;    // roots per numbering chunk, then their exclusive offsets
  int32_t* out_of_cell;
  pfg_grain* grains;
  int64_t max_grains;
  int64_t* num_grains;
};

__device__ __forceinline__ int find_root(const int32_t* L, int x) {
  int y = __ldcg(L + x);
  while (y != x) {
    x = y;
    y = __ldcg(L + x);
  }
  return x;
}

__device__ __forceinline__ void merge(int32_t* L, int a, int b) {
  bool done;
  do {
    a = find_root(L, a);
    b = find_root(L, b);
    if (a < b) {
      const int old = atomicMin(L + b, a);
      done = (old == b);
      b = old;
    } else if (b < a) {
      const int old = atomicMin(L + a, b);
      done = (old == a);
      a = old;
    } else {
      done = true;
    }
  } while (!done);
}

__global__ void __launch_bounds__(kGrainThreads) grain_init_kernel(const GrainArgs a) {
  const int N = a.nx * a.ny * a.nz;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    float T;
    if (a.T_ghosted) {
      const int xy = a.nx * a.ny;
      const int z = i / xy, r = i - z * xy, y = r / a.nx, x = r - y * a.nx;
      T = a.T[((int64_t)(z + 1) * (a.ny + 2) + (y + 1)) * (a.nx + 2) + x + 1];
    } else {
      T = a.T[i];
    }
    a.L[i] = (T < a.T_liq) ? i : -1;  // NaN T is not solid, as in the reference's compare
  }
}

__global__ void __launch_bounds__(kGrainThreads) grain_merge_kernel(const GrainArgs a) {
  const int N = a.nx * a.ny * a.nz;
  const int xy = a.nx * a.ny;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    if (__ldcg(a.L + i) < 0) continue;
    const int z = i / xy, r = i - z * xy, y = r / a.nx, x = r - y * a.nx;
    const int o = a.ori[i];
    if (x + 1 < a.nx && __ldcg(a.L + i + 1) >= 0 && a.ori[i + 1] == o) merge(a.L, i, i + 1);
    if (y + 1 < a.ny && __ldcg(a.L + i + a.nx) >= 0 && a.ori[i + a.nx] == o)
      merge(a.L, i, i + a.nx);
    if (z + 1 < a.nz && __ldcg(a.L + i + xy) >= 0 && a.ori[i + xy] == o) merge(a.L, i, i + xy);
  }
}

__global__ void __launch_bounds__(kGrainThreads) grain_compress_kernel(const GrainArgs a) {
  const int N = a.nx * a.ny * a.nz;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    if (__ldcg(a.L + i) >= 0) a.L[i] = find_root(a.L, i);
  }
}

// exclusive prefix sum of v over the block; *total receives the block's sum
__device__ __forceinline__ int block_exclusive_scan(int v, int* total) {
  __shared__ int s_warp[kGrainThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) s_warp[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    int w = (lane < kGrainThreads / 32) ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    if (lane < kGrainThreads / 32) s_warp[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  const int before = (warp > 0) ? s_warp[warp - 1] : 0;
  *total = s_warp[kGrainThreads / 32 - 1];
  __syncthreads();  // s_warp is reused by the next call
  return before + inc - v;
}

// roots per chunk of kScanChunk cells
__global__ void __launch_bounds__(kGrainThreads) grain_count_kernel(const GrainArgs a) {
  const int N = a.nx * a.ny * a.nz;
  const int base = blockIdx.x * kScanChunk + threadIdx.x * kScanItems;
  int c = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int i = base + k;
    if (i < N && a.L[i] == i) ++c;
  }
  int total;
  block_exclusive_scan(c, &total);
  if (threadIdx.x == 0) a.chunk[blockIdx.x] = total;
}

// exclusive offsets of the chunk counts (one block) and the grain count
__global__ void __launch_bounds__(kGrainThreads) grain_offsets_kernel(const GrainArgs a,
                                                                      int nchunks) {
  int carry = 0;
  for (int b0 = 0; b0 < nchunks; b0 += kGrainThreads) {
    const int b = b0 + threadIdx.x;
    const int v = (b < nchunks) ? a.chunk[b] : 0;
    int total;
    const int ex = block_exclusive_scan(v, &total);
    if (b < nchunks) a.chunk[b] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) *a.num_grains = carry;
}

// number the roots and start their records
__global__ void __launch_bounds__(kGrainThreads) grain_number_kernel(const GrainArgs a) {
  const int N = a.nx * a.ny * a.nz;
  const int base = blockIdx.x * kScanChunk + threadIdx.x * kScanItems;
  int c = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int i = base + k;
    if (i < N && a.L[i] == i) ++c;
  }
  int total;
  int g = a.chunk[blockIdx.x] + block_exclusive_scan(c, &total);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int i = base + k;
    if (i < N && a.L[i] == i) {
      a.id[i] = g;
      if (g < a.max_grains) {
        pfg_grain& G = a.grains[g];
        G.first_cell = i;
        G.ori = a.ori[i];
        G.reserved = 0;
        G.cells = 0;
        for (int d = 0; d < 3; ++d) G.sum[d] = 0;
        for (int d = 0; d < 6; ++d) G.sum2[d] = 0;
      }
      ++g;
    }
  }
}

// per-cell grain number and the grains' moments
__global__ void __launch_bounds__(kGrainThreads) grain_moments_kernel(const GrainArgs a) {
  const int N = a.nx * a.ny * a.nz;
  const int xy = a.nx * a.ny;
  const int lane = threadIdx.x & 31;
  const int stride = gridDim.x * blockDim.x;
  // the loop bound is uniform across the warp so that every lane takes part
  // in the warp-wide aggregation below
  const int first = blockIdx.x * blockDim.x + (threadIdx.x & ~31);
  for (int w0 = first; w0 < N; w0 += stride) {
    const int i = w0 + lane;
    int g = -1;
    long long v[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (i < N) {
      const int root = __ldcg(a.L + i);
      if (root >= 0) {
        g = a.id[root];
        const long long z = i / xy, r = i - z * xy, y = r / a.nx, x = r - y * a.nx;
        v[0] = 1;
        v[1] = x; v[2] = y; v[3] = z;
        v[4] = x * x; v[5] = y * y; v[6] = z * z;
        v[7] = x * y; v[8] = x * z; v[9] = y * z;
      }
      if (a.out_of_cell) a.out_of_cell[i] = g;
    }
    // one group of lanes with the same grain at a time
    unsigned pending = __ballot_sync(0xffffffffu, g >= 0);
    while (pending) {
      const int leader = __ffs(pending) - 1;
      const int gl = __shfl_sync(0xffffffffu, g, leader);
      const bool mine = (g == gl);
      pending &= ~__ballot_sync(0xffffffffu, mine);
      long long s[10];
#pragma unroll
      for (int k = 0; k < 10; ++k) {
        long long t = mine ? v[k] : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        s[k] = t;
      }
      if (lane == leader && gl < a.max_grains) {
        pfg_grain& G = a.grains[gl];
        unsigned long long* p = reinterpret_cast<unsigned long long*>(&G.cells);
        atomicAdd(p, (unsigned long long)s[0]);
        for (int d = 0; d < 3; ++d)
          atomicAdd(reinterpret_cast<unsigned long long*>(&G.sum[d]), (unsigned long long)s[1 + d]);
        for (int d = 0; d < 6; ++d)
          atomicAdd(reinterpret_cast<unsigned long long*>(&G.sum2[d]),
                    (unsigned long long)s[4 + d]);
      }
    }
  }
}

static int grain_grid(int64_t N) {
  const DeviceInfo& d = device_info();
  const int64_t want = (N + kGrainThreads - 1) / kGrainThreads;
  const int64_t cap = (int64_t)d.sm_count * 8;
  return (int)(want < cap ? (want > 0 ? want : 1) : cap);
}

static int64_t chunk_count(int64_t N) { return (N + kScanChunk - 1) / kScanChunk; }

}  // namespace pfg

using namespace pfg;

// scratch: labels (N), root numbers (N), chunk counts, each 256-byte aligned
static int64_t align256(int64_t b) { return (b + 255) / 256 * 256; }

extern "C" int64_t pfg_grain_scratch_bytes(const pfg_pf_params* p) {
  if (check_pf_params(p)) return -1;
  const int64_t N = (int64_t)p->nx * p->ny * p->nz;
  return 2 * align256(N * 4) + align256(chunk_count(N) * 4);
}

extern "C" int pfg_grains(const pfg_pf_params* p, const int32_t* ori, const float* T,
                          int T_ghosted, int32_t* grain_of_cell, pfg_grain* grains,
                          int64_t max_grains, int64_t* num_grains, void* scratch,
                          int64_t scratch_bytes, void* stream) {
  int st = check_pf_params(p);
  if (st) return st;
  if (!ori || !T || !num_grains || !scratch || (max_grains > 0 && !grains)) return PFG_ERR_NULL;
  if (max_grains < 0) return PFG_ERR_PARAM;
  if (reinterpret_cast<uintptr_t>(grains) % 8 != 0) return PFG_ERR_ALIGN;
  const int64_t N = (int64_t)p->nx * p->ny * p->nz;
  // 32-bit cell labels, with room for the last block's and grid's index ranges
  if (N >= ((int64_t)1 << 31) - ((int64_t)1 << 22)) return PFG_ERR_SHAPE;
  if (scratch_bytes < pfg_grain_scratch_bytes(p)) return PFG_ERR_CAPACITY;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  GrainArgs a{};
  a.nx = p->nx; a.ny = p->ny; a.nz = p->nz;
  a.T_ghosted = T_ghosted;
  a.T_liq = p->T_liquidus;
  a.ori = ori; a.T = T;
  char* sp = static_cast<char*>(scratch);
  a.L = reinterpret_cast<int32_t*>(sp);
  a.id = reinterpret_cast<int32_t*>(sp + align256(N * 4));
  a.chunk = reinterpret_cast<int32_t*>(sp + 2 * align256(N * 4));
  a.out_of_cell = grain_of_cell;
  a.grains = grains;
  a.max_grains = max_grains;
  a.num_grains = num_grains;
  const int grid = grain_grid(N);
  const int nchunks = (int)chunk_count(N);
  grain_init_kernel<<<grid, kGrainThreads, 0, s>>>(a);
  grain_merge_kernel<<<grid, kGrainThreads, 0, s>>>(a);
  grain_compress_kernel<<<grid, kGrainThreads, 0, s>>>(a);
  grain_count_kernel<<<nchunks, kGrainThreads, 0, s>>>(a);
  grain_offsets_kernel<<<1, kGrainThreads, 0, s>>>(a, nchunks);
  grain_number_kernel<<<nchunks, kGrainThreads, 0, s>>>(a);
  grain_moments_kernel<<<grid, kGrainThreads, 0, s>>>(a);
  return record_cuda(cudaGetLastError());
}
