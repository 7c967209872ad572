// Compensated explicit heat step on the ghosted (nz+2, ny+2, nx+2) field
// held as two float32 arrays whose sum is the temperature
// (jax_am/cfd/gamma.py:9-61: update_mat, BC_thermal, laplace, update_T).
//
// The fused compensated step of the cell-per-lane kernel evaluates the same
// update inside the phase-field stencil; for the other stencil kernels
// (num_oris != 20) the compensated step runs this kernel first and then the
// phase field with the start-of-step temperature pair.  Both kernels read the
// old state only, so the order of the two launches does not matter.
//
// A thread owns one (x, y) column and marches kChunk cells along z, carrying
// the values of planes z - 1 and z (high and low parts) in registers; per
// cell it loads the cell above and the four in-plane neighbours.  The
// arithmetic is that of the fused kernel, choosing per warp as it does:
// wherever a cell of the warp or one of its neighbours is above T0 + 50 K,
// or on the beam-heated top plane, the whole update is double-float
// (heat_update_df_accurate); elsewhere the coefficients and face fluxes are
// float32 on the exact Laplacian of the pairs (heat_update_df_near_ambient).
#include <cuda_runtime.h>

#include "pfg_host.h"
#include "pfg_step.cuh"

namespace pfg {

constexpr int kHeatCompChunk = 8;  // cells marched per thread along z

__global__ void __launch_bounds__(256, 4)
heat_comp_kernel(const __grid_constant__ StepArgs a) {
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  // The beam enters only the top face: blocks whose z range ends below the
  // top plane neither need it nor wait for its (float64) evaluation.
  __shared__ float s_beam[5];  // xl, yl, P and the low parts of xl, yl
  const bool top = min((int)(blockIdx.y + 1) * kHeatCompChunk, nz) == nz;  // block-uniform
  if (top) {
    if (threadIdx.x == 0) {
      // the beam centre and power at mid-step, the centre also as double-float
      double xd, yd;
      laser_at_d(a.hp, a.clk_in->t + 0.5 * (double)a.dt, &xd, &yd, &s_beam[2]);
      s_beam[0] = (float)xd;
      s_beam[1] = (float)yd;
      s_beam[3] = (float)(xd - (double)s_beam[0]);
      s_beam[4] = (float)(yd - (double)s_beam[1]);
    }
    __syncthreads();
  }
  const float xl = top ? s_beam[0] : 0.f, yl = top ? s_beam[1] : 0.f;
  const float Pw = top ? s_beam[2] : 0.f;
  const DF xld{xl, top ? s_beam[3] : 0.f}, yld{yl, top ? s_beam[4] : 0.f};

  const int t = blockIdx.x * blockDim.x + threadIdx.x;  // host keeps nx * ny < 2^31
  const bool valid = t < nx * ny;
  // a spare lane shadows the last column (every lane takes part in the votes)
  const int tc = valid ? t : nx * ny - 1;
  const int gy = tc / nx, gx = tc - gy * nx;
  const int z0 = blockIdx.y * kHeatCompChunk, z1 = min(z0 + kHeatCompChunk, nz);
  const int gsy = nx + 2, gsz = (ny + 2) * gsy;  // host keeps the ghosted size < 2^31
  int idx = (z0 + 1) * gsz + (gy + 1) * gsy + gx + 1;
  const float* Th = a.T;
  const float* Tl = a.T_lo;
  float Tzm = __ldg(Th + idx - gsz), Lzm = __ldg(Tl + idx - gsz);
  float Tc = __ldg(Th + idx), Lc = __ldg(Tl + idx);
  const bool side = gx == 0 || gx == nx - 1 || gy == 0 || gy == ny - 1;
  // the next plane's loads are issued one plane ahead (the loop body is not
  // unrolled: the double-float update is long)
  float q[10];
  auto load_plane = [&](int i) {
    q[0] = __ldg(Th + i + gsz);
    q[1] = __ldg(Tl + i + gsz);
    q[2] = __ldg(Th + i - 1);
    q[3] = __ldg(Th + i + 1);
    q[4] = __ldg(Th + i - gsy);
    q[5] = __ldg(Th + i + gsy);
    q[6] = __ldg(Tl + i - 1);
    q[7] = __ldg(Tl + i + 1);
    q[8] = __ldg(Tl + i - gsy);
    q[9] = __ldg(Tl + i + gsy);
  };
  load_plane(idx);
#pragma unroll 1
  for (int z = z0; z < z1; ++z, idx += gsz) {
    const float Tzp = q[0], Lzp = q[1];
    const float Txm = q[2], Txp = q[3], Tym = q[4], Typ = q[5];
    const DF c{Tc, Lc};
    DF n[6] = {DF{Txm, q[6]}, DF{Txp, q[7]}, DF{Tym, q[8]}, DF{Typ, q[9]}, DF{Tzm, Lzm},
               DF{Tzp, Lzp}};
    if (z + 1 < z1) load_plane(idx + gsz);  // block-uniform
    const bool on_face = side || z == 0 || z == nz - 1;
    const float tmax =
        fmaxf(fmaxf(fmaxf(Tc, Txm), fmaxf(Txp, Tym)), fmaxf(fmaxf(Typ, Tzm), Tzp));
    DF Tn = c;
    // warp-uniform choice, as in the fused kernel
    if (__any_sync(0xffffffffu, valid && (tmax > a.hd.hot || z == nz - 1))) {
      if (valid)
        Tn = heat_update_df_accurate(a.hc, a.hd, c, n, gx, gy, z, xld, yld, Pw, a.T_out,
                                     a.T_lo_out, idx, 1, gsy, gsz);
    } else if (__any_sync(0xffffffffu, on_face && valid)) {
      if (valid)
        Tn = heat_update_df_near_ambient<true>(a.hc, c, n, gx, gy, z, xl, yl, Pw, a.dt, a.T_out,
                                               a.T_lo_out, idx, 1, gsy, gsz);
    } else {
      Tn = heat_update_df_near_ambient<false>(a.hc, c, n, gx, gy, z, xl, yl, Pw, a.dt, a.T_out,
                                              a.T_lo_out, idx, 1, gsy, gsz);
    }
    if (valid) {
      a.T_out[idx] = Tn.h;
      a.T_lo_out[idx] = Tn.l;
    }
    Tzm = Tc;
    Lzm = Lc;
    Tc = Tzp;
    Lc = Lzp;
  }
}

cudaError_t launch_heat_comp(const StepArgs& a, cudaStream_t s) {
  if ((long long)a.nx * a.ny >= (1LL << 31)) return cudaErrorInvalidValue;
  if ((a.nz + kHeatCompChunk - 1) / kHeatCompChunk > 65535) return cudaErrorInvalidValue;
  const dim3 grid((unsigned)(((long long)a.nx * a.ny + 255) / 256),
                  (unsigned)((a.nz + kHeatCompChunk - 1) / kHeatCompChunk), 1);
  heat_comp_kernel<<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace pfg
