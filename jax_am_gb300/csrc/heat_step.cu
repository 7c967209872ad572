// Explicit finite-difference heat step on the ghosted field (jax_am/cfd/gamma.py:55-61).
// One thread per interior cell; the six neighbours are read straight from the
// ghosted array (a neighbour across a face is the previous ghost value).  The
// field may be in either axis order: threadIdx.x runs along the unit-stride
// axis so loads stay coalesced.
#include <cuda_runtime.h>

#include "pfg_device.cuh"
#include "pfg_host.h"

namespace pfg {

template <bool XYZ>
__global__ void __launch_bounds__(256)
heat_step_kernel(const __grid_constant__ HeatConsts H, const float* __restrict__ Tg_in,
                 float* __restrict__ Tg_out, float xl, float yl, float P, float dt) {
  // (f, m, s) = fastest, middle, slowest thread axes
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = blockIdx.y * blockDim.y + threadIdx.y;
  const int s = blockIdx.z;
  const int gx = XYZ ? s : f, gy = m, gz = XYZ ? f : s;
  if (gx >= H.nx || gy >= H.ny || gz >= H.nz) return;
  int64_t sx, sy, sz;
  if (XYZ) {  // (nx+2, ny+2, nz+2), z fastest: the reference's order
    sz = 1; sy = H.nz + 2; sx = (int64_t)(H.ny + 2) * (H.nz + 2);
  } else {    // (nz+2, ny+2, nx+2), x fastest
    sx = 1; sy = H.nx + 2; sz = (int64_t)(H.ny + 2) * (H.nx + 2);
  }
  const int64_t idx = (int64_t)(gx + 1) * sx + (int64_t)(gy + 1) * sy + (int64_t)(gz + 1) * sz;
  const float Tc = __ldg(Tg_in + idx);
  const float Tn = heat_cell_update(H, Tc, __ldg(Tg_in + idx - sx), __ldg(Tg_in + idx + sx),
                                    __ldg(Tg_in + idx - sy), __ldg(Tg_in + idx + sy),
                                    __ldg(Tg_in + idx - sz), __ldg(Tg_in + idx + sz), gx, gy, gz,
                                    xl, yl, P, dt, Tg_out, idx, sx, sy, sz);
  Tg_out[idx] = Tn;
}

}  // namespace pfg

using namespace pfg;

extern "C" int pfg_heat_step(const pfg_heat_params* h, const float* Tg_in, float* Tg_out,
                             float xl, float yl, float power, float dt, void* stream) {
  int st = check_heat_params(h);
  if (st) return st;
  if (h->layout != PFG_LAYOUT_ZYX && h->layout != PFG_LAYOUT_XYZ) return PFG_ERR_PARAM;
  if (!Tg_in || !Tg_out) return PFG_ERR_NULL;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  const HeatConsts H = make_heat_consts(*h);
  const bool xyz = h->layout == PFG_LAYOUT_XYZ;
  const int nf = xyz ? h->nz : h->nx, ns = xyz ? h->nx : h->nz;
  dim3 block(32, 8, 1);
  dim3 grid((nf + 31) / 32, (h->ny + 7) / 8, ns);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (xyz)
    heat_step_kernel<true><<<grid, block, 0, s>>>(H, Tg_in, Tg_out, xl, yl, power, dt);
  else
    heat_step_kernel<false><<<grid, block, 0, s>>>(H, Tg_in, Tg_out, xl, yl, power, dt);
  return record_cuda(cudaGetLastError());
}
