// Run-time diagnostics of a phase-field state, reduced on the device.
//
// The reference's only observability on this path is PFSolver.inspect_sol
// (allen_cahn.py:165-180): percentage of cells whose argmax orientation
// changed, percentage of cells at or above the liquidus, max T and a NaN
// check.  This computes those counts plus the free energy and the
// per-orientation mass in one pass over eta.
//
// Layout of the work: a group of G lanes (G a power of two, 4 G >= n) owns one
// cell, each lane a fixed set of up to four orientations (a 16-byte vector
// when n % 4 == 0), so a warp covers 32 / G cells per iteration with coalesced
// loads, and each lane keeps the running mass of its own orientations in
// registers.  Per-cell sums (sum eta^2, sum eta^4, gradient energy, argmax)
// are FP32 butterflies over the group.
//
// Precision.  GB300 issues FP64 at a small fraction of its FP32 rate, so no
// FP64 instruction runs per element or per cell: the mass and the energy are
// accumulated per thread with compensated FP32 sums (Knuth's TwoSum: the
// rounding error of every addition is carried in a second word), which is as
// accurate as FP64 accumulation for these sums, and the per-thread (hi, lo)
// pairs are folded in FP64 at the end of the block.  The per-cell local and
// gradient energy densities are evaluated in FP32 (a few roundings, relative
// error ~1e-7 of the cell's energy).  Per-block partial records go to a
// caller-provided scratch buffer; a second one-block kernel folds them in a
// fixed order, so the result is bit-reproducible.
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

// n / d for 0 <= n < 2^31 as (umulhi(n, m) + n) >> s, with s = ceil(log2 d)
// and m = floor(2^32 (2^s - d) / d) + 1 (Granlund and Montgomery's
// round-up multiplier; the sum stays below 2^32 because n < 2^31).
struct FastDiv {
  uint32_t m;
  int s;
};
static FastDiv make_fastdiv(int d) {
  int s = 0;
  while ((1LL << s) < (long long)d) ++s;
  const uint64_t m = ((uint64_t)1 << 32) * (((uint64_t)1 << s) - (uint64_t)d) / (uint64_t)d + 1;
  return FastDiv{(uint32_t)m, s};
}
__device__ __forceinline__ int fast_div(int n, FastDiv f) {
  return (int)((__umulhi((uint32_t)n, f.m) + (uint32_t)n) >> f.s);
}

struct DiagArgs {
  int nx, ny, nz, n;
  FastDiv div_x, div_xy;  // by nx and by nx * ny
  int bcx, bcy, bcz;
  int T_ghosted;
  float gwx, gwy, gwz;  // kappa_g / 2 / h_d^2: the gradient energy weight per axis
  float m_g, vol;
  // T_liq (double) compared with float T exactly: T >= T_liq <=> T >= tl_ge
  // (the smallest float >= T_liq); T == T_liq <=> T == tl_eq (NaN when T_liq
  // is not a float)
  float tl_ge, tl_eq;
  const float* eta;
  const float* T;
  const int32_t* argmax0;
  int32_t* argmax_out;
  DiagPartial* partials;
};

constexpr int kDiagBlocks = 296;  // 2 x 148..152 SMs; fixed so results do not depend on the GPU
constexpr int kDiagThreads = 512;

__device__ __forceinline__ bool argmax_better(float a, int ia, float b, int ib) {
  // np.argmax semantics: the first NaN wins, otherwise the first maximum
  const bool na = isnan(a), nb = isnan(b);
  if (na || nb) return na && (!nb || ia < ib);
  return a > b || (a == b && ia < ib);
}

// Compensated running sum: hi + lo is the sum of everything added, to within
// the rounding of lo (Knuth's TwoSum gives the exact error of each addition).
struct CSum {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float s = __fadd_rn(hi, x);
    const float bp = __fsub_rn(s, hi);
    const float ap = __fsub_rn(s, bp);
    const float err = __fadd_rn(__fsub_rn(hi, ap), __fsub_rn(x, bp));
    hi = s;
    lo = __fadd_rn(lo, err);
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// Lane's orientation v (0..3) of its group slot g: vector layout (n % 4 == 0)
// holds 4 g .. 4 g + 3, strided layout g, g + G, g + 2 G, g + 3 G.
template <int G, bool VEC4>
__device__ __forceinline__ int ori_of(int g, int v) {
  return VEC4 ? 4 * g + v : g + G * v;
}

template <int G, bool VEC4>
__device__ __forceinline__ void load4(const float* p, int g, int n, float (&out)[4]) {
  if constexpr (VEC4) {
    if (4 * g < n) {
      const float4 u = __ldg(reinterpret_cast<const float4*>(p) + g);
      out[0] = u.x; out[1] = u.y; out[2] = u.z; out[3] = u.w;
    } else {
      out[0] = out[1] = out[2] = out[3] = 0.f;
    }
  } else {
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int i = g + G * v;
      out[v] = (i < n) ? __ldg(p + i) : 0.f;
    }
  }
}

__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// Cell iterations between a group's L2 prefetch and its load of that cell:
// keeps several lines per warp in flight without holding them in registers.
constexpr int kDiagPrefetch = 4;

template <int G, bool VEC4>
__global__ void __launch_bounds__(kDiagThreads)
pf_diag_kernel(const __grid_constant__ DiagArgs a) {
  constexpr int kWarps = kDiagThreads / 32;
  constexpr int kCellsPerWarp = 32 / G;
  __shared__ double s_mass[kWarps][PFG_MAX_ORIS];
  __shared__ double s_energy[kWarps], s_maxT[kWarps];
  __shared__ long long s_cnt[kWarps][3];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane & (G - 1);          // slot within the cell's group
  const int cw = lane / G;               // cell within the warp
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (cw * G));
  const int n = a.n;
  const int ncell = a.nx * a.ny * a.nz;  // host checks < 2^31
  const int64_t sy = (int64_t)a.nx * n;
  const int64_t sz = (int64_t)a.ny * a.nx * n;
  const int stride = gridDim.x * kWarps * kCellsPerWarp;

  CSum mass[4], energy;
  float maxT = -INFINITY;
  int changed = 0, liquid = 0, nonfinite = 0;

  for (int c = (blockIdx.x * kWarps + warp) * kCellsPerWarp + cw; c < ncell; c += stride) {
    const int xy = a.nx * a.ny;
    const int z = c / xy;
    const int r = c - z * xy;
    const int y = r / a.nx;
    const int x = r - y * a.nx;
    const float* e = a.eta + (int64_t)c * n;
    {
      const int64_t cp = (int64_t)c + (int64_t)kDiagPrefetch * stride;
      if (cp < ncell && 4 * g < n) prefetch_l2(a.eta + cp * n + 4 * g);
    }
    const int64_t dx = (x + 1 < a.nx) ? n : (a.bcx ? -(int64_t)(a.nx - 1) * n : 0);
    const int64_t dy = (y + 1 < a.ny) ? sy : (a.bcy ? -(int64_t)(a.ny - 1) * sy : 0);
    const int64_t dz = (z + 1 < a.nz) ? sz : (a.bcz ? -(int64_t)(a.nz - 1) * sz : 0);
    float v[4], ex[4], ey[4], ez[4];
    load4<G, VEC4>(e, g, n, v);
    load4<G, VEC4>(e + dx, g, n, ex);
    load4<G, VEC4>(e + dy, g, n, ey);
    load4<G, VEC4>(e + dz, g, n, ez);
    float s2 = 0.f, s4 = 0.f, g2 = 0.f, best = -INFINITY;
    int bi = 1 << 30;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int i = ori_of<G, VEC4>(g, k);
      if (i < n) {
        if (!isfinite(v[k])) ++nonfinite;
        mass[k].add(v[k]);
        const float q = v[k] * v[k];
        s2 += q;
        s4 = fmaf(q, q, s4);
        const float gx = ex[k] - v[k], gy = ey[k] - v[k], gz = ez[k] - v[k];
        g2 = fmaf(a.gwx * gx, gx, fmaf(a.gwy * gy, gy, fmaf(a.gwz * gz, gz, g2)));
        if (argmax_better(v[k], i, best, bi)) { best = v[k]; bi = i; }
      }
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
      s2 += __shfl_xor_sync(gmask, s2, o);
      s4 += __shfl_xor_sync(gmask, s4, o);
      g2 += __shfl_xor_sync(gmask, g2, o);
      const float ob = __shfl_xor_sync(gmask, best, o);
      const int oi = __shfl_xor_sync(gmask, bi, o);
      if (argmax_better(ob, oi, best, bi)) { best = ob; bi = oi; }
    }
    if (g == 0) {
      float T;
      if (a.T_ghosted) {
        const int64_t gsy = a.nx + 2, gsz = (int64_t)(a.ny + 2) * (a.nx + 2);
        T = a.T[(int64_t)(z + 1) * gsz + (int64_t)(y + 1) * gsy + x + 1];
      } else {
        T = a.T[c];
      }
      // 1 - zeta of allen_cahn.py:56-57: the tanh is +-1 unless T_c == T_liq
      // (a float32 T differs from T_liq by at least 7e-8 relative, times 1e10)
      const float Tc = fminf(T, 2000.f);
      const float om = isnan(T) ? T : (Tc == a.tl_eq ? 0.5f : (Tc >= a.tl_ge ? 1.f : 0.f));
      const float f_loc =
          a.m_g * ((0.25f * s4 - 0.5f * s2) + fmaf(s2, s2, -s4) + om * om * s2);
      energy.add((f_loc + g2) * a.vol);
      if (T >= a.tl_ge) ++liquid;
      if (T > maxT || isnan(T)) maxT = isnan(maxT) ? maxT : T;
      if (a.argmax_out) a.argmax_out[c] = bi;
      if (a.argmax0 && a.argmax0[c] != bi) ++changed;
    }
  }

  // ---- block reduction (fixed order): warp butterflies, then warps in order
  double m[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) m[k] = mass[k].value();
  double en = energy.value();
  double mt = (double)maxT;
  long long c0 = changed, c1 = liquid, c2 = nonfinite;
#pragma unroll
  for (int o = 16; o >= G; o >>= 1) {  // lanes with the same slot hold the same orientations
#pragma unroll
    for (int k = 0; k < 4; ++k) m[k] += __shfl_xor_sync(0xffffffffu, m[k], o);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    en += __shfl_xor_sync(0xffffffffu, en, o);
    const double om = __shfl_xor_sync(0xffffffffu, mt, o);
    if (om > mt || isnan(om)) mt = isnan(mt) ? mt : om;
    c0 += __shfl_xor_sync(0xffffffffu, c0, o);
    c1 += __shfl_xor_sync(0xffffffffu, c1, o);
    c2 += __shfl_xor_sync(0xffffffffu, c2, o);
  }
  if (lane < G) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int i = ori_of<G, VEC4>(lane, k);
      if (i < n) s_mass[warp][i] = m[k];
    }
  }
  if (lane == 0) {
    s_energy[warp] = en;
    s_maxT[warp] = mt;
    s_cnt[warp][0] = c0;
    s_cnt[warp][1] = c1;
    s_cnt[warp][2] = c2;
  }
  __syncthreads();
  DiagPartial* out = a.partials + blockIdx.x;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double s = 0.0;
    for (int w = 0; w < kWarps; ++w) s += s_mass[w][i];
    out->mass[i] = s;
  }
  if (threadIdx.x == 0) {
    double e2 = 0.0, t2 = -INFINITY;
    long long d0 = 0, d1 = 0, d2 = 0;
    for (int w = 0; w < kWarps; ++w) {
      e2 += s_energy[w];
      if (s_maxT[w] > t2 || isnan(s_maxT[w])) t2 = isnan(t2) ? t2 : s_maxT[w];
      d0 += s_cnt[w][0];
      d1 += s_cnt[w][1];
      d2 += s_cnt[w][2];
    }
    out->energy = e2;
    out->max_T = t2;
    out->changed = d0;
    out->liquid = d1;
    out->nonfinite = d2;
  }
}

// Folds the per-block partial records in a fixed order, so the result is
// bit-reproducible.  Scalars: thread t folds records t, t + 256 in order, then
// a fixed binary tree over the 256 threads.  Masses: thread (g, i) of
// G = 256 / n groups folds records g, g + G, ... of orientation i in order,
// then thread i folds the G group sums in order.  Every chain is short, so
// the slow float64 pipe and the load latency are paid a few dozen times, not
// once per record.
constexpr int kFinishThreads = 256;

__device__ __forceinline__ double nan_max(double a, double b) {
  return isnan(a) ? a : (isnan(b) ? b : (b > a ? b : a));
}

__global__ void __launch_bounds__(kFinishThreads)
pf_diag_finish_kernel(const DiagPartial* __restrict__ parts, int nparts, int n, long long ncell,
                      pfg_diag* __restrict__ out) {
  __shared__ double s_en[kFinishThreads], s_mt[kFinishThreads];
  __shared__ long long s_cnt[kFinishThreads][3];
  __shared__ double s_mass[kFinishThreads];  // [group][orientation], G * n <= 256
  const int t = threadIdx.x;
  double en = 0.0, mt = -INFINITY;
  long long c0 = 0, c1 = 0, c2 = 0;
  for (int b = t; b < nparts; b += kFinishThreads) {
    const DiagPartial& p = parts[b];
    en += p.energy;
    mt = nan_max(mt, p.max_T);
    c0 += p.changed;
    c1 += p.liquid;
    c2 += p.nonfinite;
  }
  s_en[t] = en;
  s_mt[t] = mt;
  s_cnt[t][0] = c0;
  s_cnt[t][1] = c1;
  s_cnt[t][2] = c2;
  const int G = kFinishThreads / n;  // n <= 64: at least 4 groups
  if (t < G * n) {
    const int g = t / n, i = t - g * n;
    double m = 0.0;
#pragma unroll 8
    for (int b = g; b < nparts; b += G) m += parts[b].mass[i];
    s_mass[t] = m;
  }
  __syncthreads();
  for (int half = kFinishThreads / 2; half > 0; half >>= 1) {
    if (t < half) {
      s_en[t] += s_en[t + half];
      s_mt[t] = nan_max(s_mt[t], s_mt[t + half]);
      s_cnt[t][0] += s_cnt[t + half][0];
      s_cnt[t][1] += s_cnt[t + half][1];
      s_cnt[t][2] += s_cnt[t + half][2];
    }
    __syncthreads();
  }
  if (t < n) {
    double m = 0.0;
    for (int g = 0; g < G; ++g) m += s_mass[g * n + t];
    out->mass[t] = m;
  }
  for (int i = n + t; i < PFG_MAX_ORIS; i += kFinishThreads) out->mass[i] = 0.0;
  if (t == 0) {
    out->energy = s_en[0];
    out->max_T = s_mt[0];
    out->n_cells = ncell;
    out->n_ori_changed = s_cnt[0][0];
    out->n_liquid = s_cnt[0][1];
    out->n_nonfinite = s_cnt[0][2];
  }
}

// lanes per cell: the smallest power of two G with 4 G >= n (n <= 64)
static int diag_group(int n) {
  int g = 1;
  while (4 * g < n) g *= 2;
  return g;
}

int diag_blocks(const pfg_pf_params& p) {
  const long long ncell = (long long)p.nx * p.ny * p.nz;
  const long long per_block = (kDiagThreads / 32) * (32 / diag_group(p.num_oris));
  const long long need = (ncell + per_block - 1) / per_block;
  return (int)(need < kDiagBlocks ? need : kDiagBlocks);
}

template <int G>
static void launch_diag_g(const DiagArgs& a, int nb, cudaStream_t s) {
  if (a.n % 4 == 0) pf_diag_kernel<G, true><<<nb, kDiagThreads, 0, s>>>(a);
  else pf_diag_kernel<G, false><<<nb, kDiagThreads, 0, s>>>(a);
}

// ---------------------------------------------------------------------------
// The metrics of the reference's inspect_sol only (argmax changes, liquid
// cells, max T, non-finite values).  With no per-orientation sums to keep,
// one lane takes a whole cell and scans its orientations in order, so the
// argmax needs no shuffles.  A warp works on 32 consecutive cells at a time:
// their 32 n floats are contiguous in eta, so the warp first copies them to
// its own shared-memory slice with fully coalesced 16-byte loads (every load
// instruction moves 512 contiguous bytes), then each lane reads its cell from
// shared memory (a cell of n = 20 floats is 5 vectors: an odd stride, so the
// reads are free of bank conflicts).  Partial records as for pf_diag_kernel,
// with zero energy and mass.
// ---------------------------------------------------------------------------
// Up to 32 warps per block, two blocks per SM: the chunk loads of 64 warps
// per SM in flight, as the blocks are capped at the partial-record count.
constexpr int kInspectMaxWarps = 32;
constexpr int kInspectSmemBudget = 100 * 1024;  // per block, opted in above 48 KB

// warps of an inspect block: as many as keep 32 cells per warp, plus the
// kernel's static shared memory, within kInspectSmemBudget
static int inspect_warps(int n) {
  const int w = (kInspectSmemBudget - 2048) / (32 * 4 * n);
  return w < kInspectMaxWarps ? (w < 1 ? 1 : w) : kInspectMaxWarps;
}

template <bool VEC4>
__global__ void __launch_bounds__(32 * kInspectMaxWarps, 2)
pf_inspect_kernel(const __grid_constant__ DiagArgs a) {
  extern __shared__ float4 s_cells[];  // per warp: 32 cells of n floats
  constexpr int kWarps = kInspectMaxWarps;
  __shared__ double s_maxT[kWarps];
  __shared__ long long s_cnt[kWarps][3];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int n = a.n;
  const int ncell = a.nx * a.ny * a.nz;  // < 2^31 (host checks)
  const int xy = a.nx * a.ny;
  const int64_t gsy = a.nx + 2, gsz = (int64_t)(a.ny + 2) * (a.nx + 2);
  float* ws = reinterpret_cast<float*>(s_cells) + (size_t)warp * 32 * n;
  float maxT = -INFINITY;
  int changed = 0, liquid = 0, nonfinite = 0;
  const int nchunks = (int)(((int64_t)ncell + 31) / 32);
  for (int ch = blockIdx.x * nwarps + warp; ch < nchunks; ch += gridDim.x * nwarps) {
    const int c0 = ch * 32;
    const int cells = min(32, ncell - c0);
    // the lane's T is loaded together with the chunk, not after it
    float T = 0.f;
    if (lane < cells) {
      const int c = c0 + lane;
      int64_t ti = c;
      if (a.T_ghosted) {
        const int z = c / xy, r = c - z * xy, y = r / a.nx, x = r - y * a.nx;
        ti = (int64_t)(z + 1) * gsz + (int64_t)(y + 1) * gsy + x + 1;
      }
      T = __ldg(a.T + ti);
    }
    if constexpr (VEC4) {
      const float4* src = reinterpret_cast<const float4*>(a.eta + (int64_t)c0 * n);
      float4* dst = reinterpret_cast<float4*>(ws);
      const int tot = cells * (n >> 2);
#pragma unroll 4
      for (int j = lane; j < tot; j += 32) dst[j] = __ldg(src + j);
    } else {
      const float* src = a.eta + (int64_t)c0 * n;
      const int tot = cells * n;
#pragma unroll 4
      for (int j = lane; j < tot; j += 32) ws[j] = __ldg(src + j);
    }
    __syncwarp();
    if (lane < cells) {
      const int c = c0 + lane;
      const float* e = ws + lane * n;
      // Fast scan: the first maximum by strict '>' (exact for finite values),
      // and bad = sum of q * 0, which turns NaN at any NaN or infinity (the
      // library is built without fast-math, so q * 0 is not folded to 0).
      float best = -INFINITY, bad = 0.f;
      int bi = 0;
      auto fast = [&](float q, int i) {
        bad = fmaf(q, 0.f, bad);
        if (q > best) { best = q; bi = i; }
      };
      if constexpr (VEC4) {
        const float4* e4 = reinterpret_cast<const float4*>(e);
        for (int k = 0; k < (n >> 2); ++k) {
          const float4 u = e4[k];
          fast(u.x, 4 * k);
          fast(u.y, 4 * k + 1);
          fast(u.z, 4 * k + 2);
          fast(u.w, 4 * k + 3);
        }
      } else {
        for (int i = 0; i < n; ++i) fast(e[i], i);
      }
      if (isnan(bad)) {  // a non-finite value: np.argmax's rules (first NaN wins) and the count
        best = -INFINITY;
        bi = 1 << 30;
        for (int i = 0; i < n; ++i) {
          const float q = e[i];
          if (!isfinite(q)) ++nonfinite;
          if (argmax_better(q, i, best, bi)) { best = q; bi = i; }
        }
      }
      if (T >= a.tl_ge) ++liquid;
      if (T > maxT || isnan(T)) maxT = isnan(maxT) ? maxT : T;
      if (a.argmax_out) a.argmax_out[c] = bi;
      if (a.argmax0 && __ldg(a.argmax0 + c) != bi) ++changed;
    }
    __syncwarp();  // the slice is rewritten by the next chunk
  }
  double mt = (double)maxT;
  long long c0 = changed, c1 = liquid, c2 = nonfinite;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double om = __shfl_xor_sync(0xffffffffu, mt, o);
    if (om > mt || isnan(om)) mt = isnan(mt) ? mt : om;
    c0 += __shfl_xor_sync(0xffffffffu, c0, o);
    c1 += __shfl_xor_sync(0xffffffffu, c1, o);
    c2 += __shfl_xor_sync(0xffffffffu, c2, o);
  }
  if (lane == 0) {
    s_maxT[warp] = mt;
    s_cnt[warp][0] = c0;
    s_cnt[warp][1] = c1;
    s_cnt[warp][2] = c2;
  }
  __syncthreads();
  DiagPartial* out = a.partials + blockIdx.x;
  for (int i = threadIdx.x; i < n; i += blockDim.x) out->mass[i] = 0.0;
  if (threadIdx.x == 0) {
    double t2 = -INFINITY;
    long long d0 = 0, d1 = 0, d2 = 0;
    for (int w = 0; w < nwarps; ++w) {
      if (s_maxT[w] > t2 || isnan(s_maxT[w])) t2 = isnan(t2) ? t2 : s_maxT[w];
      d0 += s_cnt[w][0];
      d1 += s_cnt[w][1];
      d2 += s_cnt[w][2];
    }
    out->energy = 0.0;
    out->max_T = t2;
    out->changed = d0;
    out->liquid = d1;
    out->nonfinite = d2;
  }
}

// ---------------------------------------------------------------------------
// The full record (free energy, per-orientation mass and the inspect metrics)
// with one lane per cell, for num_oris a multiple of 4 up to 20.  A warp takes
// 32 consecutive cells at a time: their n floats are contiguous, so it stages
// them in its shared-memory slice with 16-byte cp.async copies (the next
// chunk's copies in flight while this one is reduced), then each lane reduces
// its cell's orientations in order: sum eta^2, sum eta^4, the gradient energy
// against the forward neighbours (x + 1 from the staged chunk where it is in
// it, y + 1 and z + 1 from L2), the argmax, and the per-orientation mass in
// the lane's own compensated sums.  No per-cell shuffles.  Per-block partial
// records as for pf_diag_kernel.
// ---------------------------------------------------------------------------
constexpr int kCellWarps = 8;
constexpr int kCellMaxVec = 5;  // n <= 20 (the per-lane mass sums fit in registers)

template <int NV>  // num_oris = 4 NV
__global__ void __launch_bounds__(32 * kCellWarps, 2)
pf_diag_cells_kernel(const __grid_constant__ DiagArgs a) {
  extern __shared__ float4 s_chunks[];  // per warp: two chunks of 32 cells
  __shared__ double s_mass[kCellWarps][4 * kCellMaxVec];
  __shared__ double s_energy[kCellWarps], s_maxT[kCellWarps];
  __shared__ long long s_cnt[kCellWarps][3];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int n = 4 * NV, nv = NV;
  const int ncell = a.nx * a.ny * a.nz;  // < 2^31 (host checks)
  const int xy = a.nx * a.ny;
  const int64_t gsy = a.nx + 2, gsz = (int64_t)(a.ny + 2) * (a.nx + 2);
  float4* buf0 = s_chunks + (size_t)warp * 2 * 32 * nv;
  float4* buf1 = buf0 + 32 * nv;
  const float4* eta4 = reinterpret_cast<const float4*>(a.eta);
  const int nchunks = (int)(((int64_t)ncell + 31) / 32);
  const int cstride = gridDim.x * kCellWarps;

  float mh[n], ml[n];  // compensated mass per orientation
#pragma unroll
  for (int i = 0; i < n; ++i) mh[i] = ml[i] = 0.f;
  CSum energy;
  float maxT = -INFINITY;
  int changed = 0, liquid = 0, nonfinite = 0;

  // the chunk's y + 1 and z + 1 neighbours are the 32 cells nx and nx * ny
  // further on: their 128-byte lines (at most 21 for n <= 20) are prefetched
  // into L1 one chunk ahead, so the lanes' 16-byte loads of them hit L1
  const int64_t nbytes = (int64_t)ncell * n * 4;
  const char* eta_b = reinterpret_cast<const char*>(a.eta);
  auto prefetch_span = [&](int64_t cell0) {
    const int64_t b0 = (cell0 * n * 4) & ~(int64_t)127;
    const int64_t b = b0 + (int64_t)lane * 128;
    if (lane * 128 < 32 * n * 4 + 128 && b < nbytes)
      asm volatile("prefetch.global.L1 [%0];" ::"l"(eta_b + b));
  };
  auto stage = [&](int chunk, float4* dst) {
    const int c0 = chunk * 32;
    const int tot = min(32, ncell - c0) * nv;
    const float4* src = eta4 + (int64_t)c0 * nv;
    for (int j = lane; j < tot; j += 32) cp_async<16>(dst + j, src + j);
    prefetch_span((int64_t)c0 + a.nx);
    prefetch_span((int64_t)c0 + xy);
  };
  int ch = blockIdx.x * kCellWarps + warp;
  if (ch < nchunks) stage(ch, buf0);
  cp_async_commit();
  for (int it = 0; ch < nchunks; ch += cstride, ++it) {
    float4* cur = (it & 1) ? buf1 : buf0;
    float4* nxt = (it & 1) ? buf0 : buf1;
    if (ch + cstride < nchunks) stage(ch + cstride, nxt);
    cp_async_commit();
    cp_async_wait(1);  // this chunk has landed; the next may stay in flight
    __syncwarp();
    const int c0 = ch * 32;
    const int cells = min(32, ncell - c0);
    if (lane < cells) {
      const int c = c0 + lane;
      const int z = fast_div(c, a.div_xy), r = c - z * xy, y = fast_div(r, a.div_x);
      const int x = r - y * a.nx;
      const int64_t ti = a.T_ghosted ? (int64_t)(z + 1) * gsz + (int64_t)(y + 1) * gsy + x + 1
                                     : (int64_t)c;
      const float T = __ldg(a.T + ti);
      // forward neighbours under the boundary conditions (-1: the cell itself)
      const int cx = (x + 1 < a.nx) ? c + 1 : (a.bcx ? c - (a.nx - 1) : -1);
      const int cy = (y + 1 < a.ny) ? c + a.nx : (a.bcy ? c - (a.ny - 1) * a.nx : -1);
      const int cz = (z + 1 < a.nz) ? c + xy : (a.bcz ? c - (a.nz - 1) * xy : -1);
      const float4* e = cur + lane * nv;
      const float4* ex = (cx == c + 1 && lane + 1 < cells) ? cur + (lane + 1) * nv
                                                            : eta4 + (int64_t)(cx < 0 ? c : cx) * nv;
      const float4* ey = eta4 + (int64_t)(cy < 0 ? c : cy) * nv;
      const float4* ez = eta4 + (int64_t)(cz < 0 ? c : cz) * nv;
      float s2 = 0.f, s4 = 0.f, gxx = 0.f, gyy = 0.f, gzz = 0.f, best = -INFINITY;
      int bi = 0;
#pragma unroll
      for (int v = 0; v < nv; ++v) {
        {
          const float4 u = e[v];
          const float4 X = (cx < 0) ? u : ex[v];
          const float4 Y = (cy < 0) ? u : __ldg(ey + v);
          const float4 Z = (cz < 0) ? u : __ldg(ez + v);
          const float uu[4] = {u.x, u.y, u.z, u.w}, xx[4] = {X.x, X.y, X.z, X.w};
          const float yy[4] = {Y.x, Y.y, Y.z, Y.w}, zz[4] = {Z.x, Z.y, Z.z, Z.w};
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const float q = uu[k];
            const int i = 4 * v + k;
            if (q > best) { best = q; bi = i; }
            {  // mass: compensated sum (TwoSum)
              const float sum = __fadd_rn(mh[i], q);
              const float bp = __fsub_rn(sum, mh[i]);
              const float ap = __fsub_rn(sum, bp);
              ml[i] = __fadd_rn(ml[i], __fadd_rn(__fsub_rn(mh[i], ap), __fsub_rn(q, bp)));
              mh[i] = sum;
            }
            const float qq = q * q;
            s2 += qq;
            s4 = fmaf(qq, qq, s4);
            const float gx = xx[k] - q, gy = yy[k] - q, gz = zz[k] - q;
            gxx = fmaf(gx, gx, gxx);
            gyy = fmaf(gy, gy, gyy);
            gzz = fmaf(gz, gz, gzz);
          }
        }
      }
      const float g2 = fmaf(a.gwx, gxx, fmaf(a.gwy, gyy, a.gwz * gzz));
      // A non-finite value makes the sum of squares non-finite (so can a
      // finite value above 2^64; the exact pass below then finds no
      // non-finite value and the same argmax): np.argmax's rules (the first
      // NaN wins) and the count
      if (!isfinite(s2)) {
        const float* ef = reinterpret_cast<const float*>(e);
        best = -INFINITY;
        bi = 1 << 30;
        for (int i = 0; i < n; ++i) {
          const float q = ef[i];
          if (!isfinite(q)) ++nonfinite;
          if (argmax_better(q, i, best, bi)) { best = q; bi = i; }
        }
      }
      // 1 - zeta of allen_cahn.py:56-57, as pf_diag_kernel
      const float Tc = fminf(T, 2000.f);
      const float om = isnan(T) ? T : (Tc == a.tl_eq ? 0.5f : (Tc >= a.tl_ge ? 1.f : 0.f));
      const float f_loc =
          a.m_g * ((0.25f * s4 - 0.5f * s2) + fmaf(s2, s2, -s4) + om * om * s2);
      energy.add((f_loc + g2) * a.vol);
      if (T >= a.tl_ge) ++liquid;
      if (T > maxT || isnan(T)) maxT = isnan(maxT) ? maxT : T;
      if (a.argmax_out) a.argmax_out[c] = bi;
      if (a.argmax0 && __ldg(a.argmax0 + c) != bi) ++changed;
    }
    __syncwarp();  // this buffer is restaged in the next iteration but one
  }
  cp_async_wait(0);

  // ---- block reduction (fixed order): lanes by butterflies, then warps in order
  double en = energy.value(), mt = (double)maxT;
  long long k0 = changed, k1 = liquid, k2 = nonfinite;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    en += __shfl_xor_sync(0xffffffffu, en, o);
    const double om = __shfl_xor_sync(0xffffffffu, mt, o);
    if (om > mt || isnan(om)) mt = isnan(mt) ? mt : om;
    k0 += __shfl_xor_sync(0xffffffffu, k0, o);
    k1 += __shfl_xor_sync(0xffffffffu, k1, o);
    k2 += __shfl_xor_sync(0xffffffffu, k2, o);
  }
#pragma unroll
  for (int i = 0; i < n; ++i) {
    {
      double m = (double)mh[i] + (double)ml[i];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) m += __shfl_xor_sync(0xffffffffu, m, o);
      if (lane == 0) s_mass[warp][i] = m;
    }
  }
  if (lane == 0) {
    s_energy[warp] = en;
    s_maxT[warp] = mt;
    s_cnt[warp][0] = k0;
    s_cnt[warp][1] = k1;
    s_cnt[warp][2] = k2;
  }
  __syncthreads();
  DiagPartial* out = a.partials + blockIdx.x;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double sm = 0.0;
    for (int w = 0; w < kCellWarps; ++w) sm += s_mass[w][i];
    out->mass[i] = sm;
  }
  if (threadIdx.x == 0) {
    double e2 = 0.0, t2 = -INFINITY;
    long long d0 = 0, d1 = 0, d2 = 0;
    for (int w = 0; w < kCellWarps; ++w) {
      e2 += s_energy[w];
      if (s_maxT[w] > t2 || isnan(s_maxT[w])) t2 = isnan(t2) ? t2 : s_maxT[w];
      d0 += s_cnt[w][0];
      d1 += s_cnt[w][1];
      d2 += s_cnt[w][2];
    }
    out->energy = e2;
    out->max_T = t2;
    out->changed = d0;
    out->liquid = d1;
    out->nonfinite = d2;
  }
}

template <int NV>
static cudaError_t launch_diag_cells_t(const DiagArgs& a, int nb, size_t smem, cudaStream_t s) {
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(pf_diag_cells_kernel<NV>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  pf_diag_cells_kernel<NV><<<nb, 32 * kCellWarps, smem, s>>>(a);
  return cudaSuccess;
}

static cudaError_t launch_diag_cells(const DiagArgs& a, int nb, size_t smem, cudaStream_t s) {
  switch (a.n / 4) {
    case 1: return launch_diag_cells_t<1>(a, nb, smem, s);
    case 2: return launch_diag_cells_t<2>(a, nb, smem, s);
    case 3: return launch_diag_cells_t<3>(a, nb, smem, s);
    case 4: return launch_diag_cells_t<4>(a, nb, smem, s);
    default: return launch_diag_cells_t<5>(a, nb, smem, s);
  }
}

int launch_diag(const pfg_pf_params* p, const float* eta, const float* T, int T_ghosted,
                const int32_t* argmax0, int32_t* argmax_out, void* scratch,
                pfg_diag* out, cudaStream_t s, bool full = true) {
  // cell indices are 32-bit in the reduction
  if ((int64_t)p->nx * p->ny * p->nz >= ((int64_t)1 << 31)) return PFG_ERR_SHAPE;
  DiagArgs a{};
  a.nx = p->nx; a.ny = p->ny; a.nz = p->nz; a.n = p->num_oris;
  a.div_x = make_fastdiv(p->nx);
  a.div_xy = make_fastdiv(p->nx * p->ny);
  a.bcx = p->bc_x; a.bcy = p->bc_y; a.bcz = p->bc_z;
  a.T_ghosted = T_ghosted;
  a.gwx = (float)(0.5 * (double)p->kappa_g / ((double)p->h_x * p->h_x));
  a.gwy = (float)(0.5 * (double)p->kappa_g / ((double)p->h_y * p->h_y));
  a.gwz = (float)(0.5 * (double)p->kappa_g / ((double)p->h_z * p->h_z));
  a.m_g = (float)p->m_g;
  a.vol = (float)((double)p->h_x * p->h_y * p->h_z);
  {
    const double tl = p->T_liquidus;
    float f = (float)tl;
    if ((double)f < tl) f = nextafterf(f, INFINITY);
    a.tl_ge = f;
    a.tl_eq = ((double)(float)tl == tl) ? (float)tl : NAN;
  }
  a.eta = eta; a.T = T; a.argmax0 = argmax0; a.argmax_out = argmax_out;
  a.partials = static_cast<DiagPartial*>(scratch);
  int nb = diag_blocks(*p);
  if (!full) {
    // no more blocks than partial records in the scratch (diag_blocks) or
    // than chunks of 32 cells per warp
    const int w = inspect_warps(a.n);
    const long long nchunks = ((long long)a.nx * a.ny * a.nz + 31) / 32;
    const long long need = (nchunks + w - 1) / w;
    nb = (int)(need < nb ? (need < 1 ? 1 : need) : nb);
    const size_t smem = (size_t)w * 32 * a.n * sizeof(float);
    const void* fn = (a.n % 4 == 0) ? (const void*)pf_inspect_kernel<true>
                                    : (const void*)pf_inspect_kernel<false>;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem);
      if (e != cudaSuccess) return record_cuda(e);
    }
    if (a.n % 4 == 0) pf_inspect_kernel<true><<<nb, 32 * w, smem, s>>>(a);
    else pf_inspect_kernel<false><<<nb, 32 * w, smem, s>>>(a);
  } else if (a.n % 4 == 0 && a.n <= 4 * kCellMaxVec) {
    // the lane-per-cell record: no more blocks than partial records or than
    // chunks of 32 cells per warp
    const long long nchunks = ((long long)a.nx * a.ny * a.nz + 31) / 32;
    const long long need = (nchunks + kCellWarps - 1) / kCellWarps;
    nb = (int)(need < nb ? (need < 1 ? 1 : need) : nb);
    const size_t smem = (size_t)kCellWarps * 2 * 32 * a.n * sizeof(float);
    cudaError_t e = launch_diag_cells(a, nb, smem, s);
    if (e != cudaSuccess) return record_cuda(e);
  } else switch (diag_group(a.n)) {
    case 1: launch_diag_g<1>(a, nb, s); break;
    case 2: launch_diag_g<2>(a, nb, s); break;
    case 4: launch_diag_g<4>(a, nb, s); break;
    case 8: launch_diag_g<8>(a, nb, s); break;
    default: launch_diag_g<16>(a, nb, s); break;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return record_cuda(e);
  pf_diag_finish_kernel<<<1, kFinishThreads, 0, s>>>(a.partials, nb, p->num_oris,
                                          (long long)p->nx * p->ny * p->nz, out);
  return record_cuda(cudaGetLastError());
}

}  // namespace pfg

using namespace pfg;

extern "C" int64_t pfg_pf_diag_scratch_bytes(const pfg_pf_params* p) {
  if (check_pf_params(p)) return -1;
  return (int64_t)diag_blocks(*p) * (int64_t)sizeof(DiagPartial);
}

extern "C" int pfg_pf_inspect(const pfg_pf_params* p, const float* eta, const float* T,
                              int T_ghosted, const int32_t* argmax0, int32_t* argmax_out,
                              void* scratch, int64_t scratch_bytes, pfg_diag* out, void* stream) {
  int st = check_pf_params(p);
  if (st) return st;
  if (!eta || !T || !scratch || !out) return PFG_ERR_NULL;
  if (scratch_bytes < pfg_pf_diag_scratch_bytes(p)) return PFG_ERR_CAPACITY;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  return launch_diag(p, eta, T, T_ghosted, argmax0, argmax_out, scratch, out,
                     static_cast<cudaStream_t>(stream), false);
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
