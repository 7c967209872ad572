// TMA-fed phase-field step: the fast path when num_oris is a multiple of 4.
//
// Same tiling and arithmetic as pf_fast.cu (warps own whole cells, per-cell
// coefficients one plane ahead, folded element update), with the staging
// moved to a producer warp:
//  * Each halo row of a plane tile is one contiguous run of cells in HBM; the
//    producer copies it into shared memory with one cp.async.bulk (TMA)
//    transfer that completes on the slot's "full" mbarrier (expect-tx bytes).
//    The temperature tile (4-byte cells, unaligned rows) goes through
//    ordinary cp.async copies that arrive on the same barrier.
//  * The eight consumer warps wait on "full", release the slot on "empty"
//    after their last use of the plane, and synchronise among themselves
//    with a named barrier only for the per-cell coefficient buffer.
//  * Neumann halo cells along x are never copied: the stencil offset of the
//    edge cell points at itself.  Periodic halo cells are copied by TMA.
// Every wait is bounded (about one second of clock64 cycles); a wait that
// runs out sets the library's device error flag, the CTA drains its copies in
// flight and returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "pfg_host.h"
#include "pfg_step.cuh"

namespace pfg {

__device__ int g_pfg_device_error = 0;  // PFG_ERR_TIMEOUT once a bounded wait ran out

constexpr int kConsumers = 256;                 // eight consumer warps
constexpr int kTmaThreads = kConsumers + 32;    // plus one producer warp
constexpr long long kWaitCycles = 2000000000LL;  // ~1 s at 2 GHz

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void cp_async_mbar_arrive_noinc(uint64_t* bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];\n" ::"r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Wait for the phase with this parity to complete; false if the wait ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > kWaitCycles) {
      atomicExch(&g_pfg_device_error, PFG_ERR_TIMEOUT);
      return false;
    }
  }
  return true;
}
__device__ __forceinline__ void tma_row(void* dst, const void* src, unsigned bytes,
                                        uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void consumer_sync() {
  asm volatile("bar.sync 1, %0;\n" ::"n"(kConsumers) : "memory");
}

// Folded update of one element (see pf_fast.cu for the derivation).
struct LapConstsT {
  float ry, rz, nm;
};
template <bool ANISO>
__device__ __forceinline__ float tma_update_elem(const LapConstsT& L, float e, float xm, float xp,
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
    const float c2 = fminf(fmaxf(fmaxf(q0, q1), q2) * __fdividef(1.f, ee), 1.f);
    u = fmaf(k.w, fmaf(-c2, c2, c2), k.z);
  }
  return fmaf(u, lap, e * fmaf(k.y, e * e, k.x));
}

__device__ __forceinline__ float4 tma_fold(const PFConsts& c, const TempCoef& tc, float S) {
  if (tc.liquid != 0.f) return make_float4(0.f, 0.f, 0.f, 0.f);
  const float K = 4.f * S + tc.om2 - 1.f;
  const float clw = tc.cl * c.wx;
  return make_float4(1.f + tc.cg * K, -3.f * tc.cg, clw * (1.f + c.aniso), -2.f * c.aniso * clw);
}

template <bool ANISO, int TSRC>
__global__ void __launch_bounds__(kTmaThreads, 2) pf_tma_kernel(const __grid_constant__ StepArgs a) {
  constexpr int VEC = 4;
  extern __shared__ __align__(128) float smem[];
  const int S = a.stages;
  const int slot_floats = (a.ty + 2) * a.pitch;
  float* eta_s = smem;
  float* T_s = eta_s + (size_t)S * slot_floats;
  float4* cc = reinterpret_cast<float4*>(T_s + (size_t)S * a.tslot);  // [2][ty * tx]
  uint64_t* full = reinterpret_cast<uint64_t*>(cc + 2 * a.ty * a.tx);
  uint64_t* empty = full + S;

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
  const int n = a.n;
  const int nplanes = ze - zb + 2;  // planes zb-1 .. ze
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  __shared__ int s_abort;  // set by any consumer whose wait ran out; read after a barrier
  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1 + 32);  // producer's expect-tx arrival + 32 cp.async arrivals
      mbar_init(&empty[s], kConsumers / 32);
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();

  double t0 = 0.0;
  if constexpr (TSRC != kTArray) {
    t0 = a.clk_in->t;
    if (blockIdx.x == 0 && threadIdx.x == 0 && a.clk_out) {
      a.clk_out->t = t0 + (double)a.dt;
      a.clk_out->step = a.clk_in->step + 1;
    }
  }

  if (warp == kConsumers / 32) {
    // =================== producer warp ===================
    const int cx0 = max(x0 - 1, 0), cx1 = min(xe + 1, a.nx);
    const int dst_cell0 = cx0 - (x0 - 1);
    const bool wrap_left = (x0 == 0) && a.bcx == PFG_BC_PERIODIC;
    const bool wrap_right = (xe == a.nx) && a.bcx == PFG_BC_PERIODIC;
    const int rows = tyv + 2;
    const unsigned row_bytes = (unsigned)((cx1 - cx0) * n * 4);
    const unsigned cell_bytes = (unsigned)(n * 4);
    const unsigned plane_bytes =
        (unsigned)rows * (row_bytes + (wrap_left ? cell_bytes : 0u) + (wrap_right ? cell_bytes : 0u));
    const int tp = a.tx + 2;
    int issued = 0;
    bool ok = true;
    for (int j = 0; j < nplanes && ok; ++j) {
      const int s = j % S, k = j / S;
      if (k > 0) ok = mbar_wait(&empty[s], (unsigned)((k - 1) & 1));
      if (!ok) break;
      const int pz = zb - 1 + j;
      const int gz = bc_index(pz, a.nz, a.bcz);
      float* es = eta_s + (size_t)s * slot_floats;
      if (lane == 0) mbar_arrive_expect_tx(&full[s], plane_bytes);
      __syncwarp();
      for (int r = lane; r < rows; r += 32) {
        const int gy = bc_index(y0 - 1 + r, a.ny, a.bcy);
        const float* src_row = a.eta_in + ((int64_t)gz * a.ny + gy) * a.nx * n;
        float* dst_row = es + r * a.pitch;
        tma_row(dst_row + dst_cell0 * n, src_row + (int64_t)cx0 * n, row_bytes, &full[s]);
        if (wrap_left) tma_row(dst_row, src_row + (int64_t)(a.nx - 1) * n, cell_bytes, &full[s]);
        if (wrap_right)
          tma_row(dst_row + (txv + 1) * n, src_row, cell_bytes, &full[s]);
      }
      float* ts = T_s + (size_t)s * a.tslot;
      if constexpr (TSRC == kTHeat) {
        const int cols = txv + 2;
        const int64_t gsy = a.nx + 2, gsz = (int64_t)(a.ny + 2) * (a.nx + 2);
        for (int i = lane; i < rows * cols; i += 32) {
          const int r = i / cols, c = i - r * cols;
          cp_async<4>(ts + r * tp + c, a.T + (int64_t)(pz + 1) * gsz + (int64_t)(y0 + r) * gsy + x0 + c);
        }
      } else if constexpr (TSRC == kTArray) {
        if (pz >= 0 && pz < a.nz) {
          for (int i = lane; i < tyv * txv; i += 32) {
            const int r = i / txv, c = i - r * txv;
            cp_async<4>(ts + (r + 1) * tp + c + 1,
                        a.T + ((int64_t)pz * a.ny + y0 + r) * a.nx + x0 + c);
          }
        }
      }
      cp_async_mbar_arrive_noinc(&full[s]);
      issued = j + 1;
    }
    // drain: every copy issued must have landed before the CTA's shared
    // memory can be released.  Only the latest use of each slot can still be
    // in flight (earlier uses completed before the slot was refilled), and a
    // barrier can only be asked about its latest phase.
    for (int j = max(0, issued - S); j < issued; ++j) {
      if (!mbar_wait(&full[j % S], (unsigned)((j / S) & 1))) break;
    }
    return;
  }

  // =================== consumer warps ===================
  const int tpc = a.tpc;
  const int wxi = warp % a.wx, wyi = warp / a.wx;
  const int lc = lane / tpc, kk = lane - lc * tpc;
  const bool lane_active = lc < a.cpw;
  const int xs = wxi * a.cpw + (lane_active ? lc : 0);
  const bool col_valid = lane_active && xs < txv;
  const int i0 = kk * VEC;
  // Neumann along x: the edge cell is its own neighbour
  const int gx = x0 + xs;
  const int off_xm = (gx == 0 && a.bcx == PFG_BC_NEUMANN) ? 0 : -n;
  const int off_xp = (gx == a.nx - 1 && a.bcx == PFG_BC_NEUMANN) ? 0 : n;

  float dl[ANISO ? 6 * VEC : 1];
  if constexpr (ANISO) {
    const int ib = min(i0, n - VEC);
#pragma unroll
    for (int v = 0; v < VEC; ++v)
#pragma unroll
      for (int j = 0; j < 6; ++j) dl[v * 6 + j] = a.dirs[((j / 3) * n + ib + v) * 3 + (j % 3)];
  }
  LapConstsT L;
  L.ry = a.pc.wy / a.pc.wx;
  L.rz = a.pc.wz / a.pc.wx;
  L.nm = -2.f * (1.f + L.ry + L.rz);

  float xl = 0.f, yl = 0.f, Pw = 0.f;
  if constexpr (TSRC == kTHeat) laser_at(a.hp, t0 + 0.5 * (double)a.dt, &xl, &yl, &Pw);

  const int ncell = tyv * txv;
  // per-cell coefficients of plane pz (in slot s) -> cc[buf]
  auto cell_coefs = [&](int s, int buf, int pz) {
    const float* es = eta_s + (size_t)s * slot_floats;
    const float* ts = T_s + (size_t)s * a.tslot;
    float4* cb = cc + (size_t)buf * a.ty * a.tx;
    TempCoef plane{};
    if constexpr (TSRC == kTQuench) {
      const double zc = a.q.z_first + (double)pz * (double)a.h_z;
      const float Tz = (float)(a.q.T_base + a.q.grad * (zc - a.q.z0) - a.q.grad * a.q.vel * t0);
      plane = temp_coefficients_fast(a.pc, Tz, a.dt);
    }
    for (int i = threadIdx.x; i < ncell; i += kConsumers) {
      const int r = i / txv, c = i - r * txv;
      const float* ce = es + (r + 1) * a.pitch + (c + 1) * n;
      float s0 = 0.f, s1 = 0.f;
      int q = 0;
      for (; q + 8 <= n; q += 8) {
        const float4 u = *reinterpret_cast<const float4*>(ce + q);
        const float4 v = *reinterpret_cast<const float4*>(ce + q + 4);
        s0 = fmaf(u.x, u.x, fmaf(u.y, u.y, fmaf(u.z, u.z, fmaf(u.w, u.w, s0))));
        s1 = fmaf(v.x, v.x, fmaf(v.y, v.y, fmaf(v.z, v.z, fmaf(v.w, v.w, s1))));
      }
      for (; q < n; q += 4) {
        const float4 u = *reinterpret_cast<const float4*>(ce + q);
        s0 = fmaf(u.x, u.x, fmaf(u.y, u.y, fmaf(u.z, u.z, fmaf(u.w, u.w, s0))));
      }
      TempCoef tc;
      if constexpr (TSRC == kTQuench) tc = plane;
      else tc = temp_coefficients_fast(a.pc, ts[(r + 1) * (a.tx + 2) + c + 1], a.dt);
      cb[r * a.tx + c] = tma_fold(a.pc, tc, s0 + s1);
    }
  };

  bool ok = true;
  // prologue: planes zb-1, zb, zb+1 (slots 0, 1, 2 of their first use)
  for (int j = 0; j < 3 && ok; ++j) ok = mbar_wait(&full[j % S], (unsigned)((j / S) & 1));
  if (ok) cell_coefs(1 % S, 0, zb);
  else s_abort = 1;

  const int64_t plane_elems = (int64_t)a.ny * a.nx * n;
  for (int z = zb; z < ze; ++z) {
    const int m = z - zb;
    const int j_next = m + 2;
    if (ok) ok = mbar_wait(&full[j_next % S], (unsigned)((j_next / S) & 1));
    if (!ok) *(volatile int*)&s_abort = 1;
    consumer_sync();  // cc[m & 1] complete; everyone finished iteration m-1
    if (*(volatile int*)&s_abort) break;  // uniform across the consumer warps
    const int s_prev = m % S, s_cur = (m + 1) % S, s_next = j_next % S;

    if constexpr (TSRC == kTHeat) {
      const float* tp_ = T_s + (size_t)s_prev * a.tslot;
      const float* tc_ = T_s + (size_t)s_cur * a.tslot;
      const float* tn_ = T_s + (size_t)s_next * a.tslot;
      const int tp = a.tx + 2;
      const int64_t sy = a.nx + 2, sz = (int64_t)(a.ny + 2) * (a.nx + 2);
      for (int i = threadIdx.x; i < ncell; i += kConsumers) {
        const int r = i / txv, c = i - r * txv;
        const int o = (r + 1) * tp + c + 1;
        const int hx = x0 + c, hy = y0 + r;
        const int64_t idx = (int64_t)(z + 1) * sz + (int64_t)(hy + 1) * sy + hx + 1;
        const float Tn = heat_cell_update(a.hc, tc_[o], tc_[o - 1], tc_[o + 1], tc_[o - tp],
                                          tc_[o + tp], tp_[o], tn_[o], hx, hy, z, xl, yl, Pw,
                                          a.dt, a.T_out, idx, 1, sy, sz);
        a.T_out[idx] = Tn;
      }
    }
    if (z + 1 < ze) cell_coefs(s_next, (m + 1) & 1, z + 1);

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
        out.v[v] = tma_update_elem<ANISO>(L, c.v[v], xm.v[v], xp.v[v], ym.v[v], yp.v[v], zm.v[v],
                                          zp.v[v], &dl[ANISO ? v * 6 : 0], kc);
      if (col_valid) {
        const int64_t g = (int64_t)z * plane_elems + ((int64_t)(y0 + r) * a.nx + gx) * n + i0;
        out.store(a.eta_out + g);
      }
    };
    const int r_end = min(wyi * a.rpw + a.rpw, tyv);
    for (int r = wyi * a.rpw; r < r_end; ++r) {
      const int off = (r + 1) * a.pitch + (xs + 1) * n + i0;
      VecF<VEC> c, xm, xp, ym, yp, zm, zp;
      c.load(e_cur + off);
      xm.load(e_cur + off + off_xm);
      xp.load(e_cur + off + off_xp);
      ym.load(e_cur + off - a.pitch);
      yp.load(e_cur + off + a.pitch);
      zm.load(e_prev + off);
      zp.load(e_next + off);
      row_update(r, c, xm, xp, ym, yp, zm, zp);
    }
    // plane z-1 (slot s_prev) is no longer needed by this warp
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s_prev]);
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

bool plan_tma_tiles(int nx, int ny, int nz, int n, int sm_count, int max_smem_per_sm,
                    TilePlan* out) {
  if (n % 4 != 0) return false;
  TilePlan t{};
  if (!plan_warp_tiles(nx, ny, nz, n, sm_count, max_smem_per_sm, &t)) return false;
  // the ring's barriers sit after the coefficient buffer
  t.smem += (size_t)2 * t.stages * sizeof(uint64_t);
  *out = t;
  return true;
}

template <bool ANISO, int TSRC>
static cudaError_t launch_tma_t(const StepArgs& a, const TilePlan& t, cudaStream_t s) {
  auto k = pf_tma_kernel<ANISO, TSRC>;
  static int configured[64] = {0};
  const int dev = device_info().device;
  if (dev < 0 || dev >= 64 || configured[dev] < (int)t.smem) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)t.smem);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64) configured[dev] = (int)t.smem;
  }
  k<<<(unsigned)t.units, kTmaThreads, t.smem, s>>>(a);
  return cudaGetLastError();
}

template <int TSRC>
cudaError_t launch_tma_kernel(const StepArgs& a, const TilePlan& t, cudaStream_t s) {
  return (a.pc.aniso > 0.f) ? launch_tma_t<true, TSRC>(a, t, s) : launch_tma_t<false, TSRC>(a, t, s);
}

template cudaError_t launch_tma_kernel<kTArray>(const StepArgs&, const TilePlan&, cudaStream_t);
template cudaError_t launch_tma_kernel<kTHeat>(const StepArgs&, const TilePlan&, cudaStream_t);
template cudaError_t launch_tma_kernel<kTQuench>(const StepArgs&, const TilePlan&, cudaStream_t);

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
