// Explicit finite-difference heat step on the ghosted field (jax_am/cfd/gamma.py:55-61).
// A thread owns one (fast, middle) position and marches kHeatChunk cells along
// the slowest axis, keeping the previous, current and next values of that axis
// in registers: per cell it loads the next value and the four in-plane
// neighbours (a neighbour across a face is the previous ghost value).  The
// field may be in either axis order; consecutive threads take consecutive
// cells of the unit-stride axis, so loads stay coalesced.  A warp whose whole
// chunk touches no domain face runs the update with the face code compiled
// out and steps pointers instead of recomputing indices.
#include <cuda_runtime.h>

#include <type_traits>

#include "pfg_device.cuh"
#include "pfg_host.h"

namespace pfg {

constexpr int kHeatChunk = 8;  // cells marched per thread along the slowest axis

template <bool XYZ>
__global__ void __launch_bounds__(256, 8)
heat_step_kernel(const __grid_constant__ HeatConsts H, const float* __restrict__ Tg_in,
                 float* __restrict__ Tg_out, float xl, float yl, float P, float dt) {
  // fast / middle / slow axis extents (XYZ: z, y, x; ZYX: x, y, z)
  const int nf = XYZ ? H.nz : H.nx, nm = H.ny, ns = XYZ ? H.nx : H.nz;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;  // host keeps nf * nm < 2^31
  const bool valid = t < nf * nm;
  const int m = t / nf, f = t - m * nf;
  const int s0 = blockIdx.y * kHeatChunk;
  // The face-free update runs when no cell of the whole warp's chunk touches a
  // domain face; the vote keeps that branch warp-uniform (every lane of the
  // 256-thread block is present at the vote).
  const bool interior =
      __all_sync(0xffffffffu, !valid || (f > 0 && f < nf - 1 && m > 0 && m < nm - 1)) &&
      s0 > 0 && s0 + kHeatChunk < ns;
  if (!valid) return;
  // ghosted strides: unit along the fast axis (host keeps the ghosted size < 2^31)
  const int sm = nf + 2, ss = (nm + 2) * (nf + 2);
  int idx = (s0 + 1) * ss + (m + 1) * sm + (f + 1);
  float prev = __ldg(Tg_in + idx - ss), cur = __ldg(Tg_in + idx);
  auto cell = [&](int s, auto faces) {
    constexpr bool F = decltype(faces)::value;
    const float next = __ldg(Tg_in + idx + ss);
    const float fm = __ldg(Tg_in + idx - 1), fp = __ldg(Tg_in + idx + 1);
    const float mm = __ldg(Tg_in + idx - sm), mp = __ldg(Tg_in + idx + sm);
    const int gx = XYZ ? s : f, gy = m, gz = XYZ ? f : s;
    const int sx = XYZ ? ss : 1, sz = XYZ ? 1 : ss;
    const float Tn = XYZ ? heat_cell_update<int, F>(H, cur, prev, next, mm, mp, fm, fp, gx, gy,
                                                    gz, xl, yl, P, dt, Tg_out, idx, sx, sm, sz)
                         : heat_cell_update<int, F>(H, cur, fm, fp, mm, mp, prev, next, gx, gy,
                                                    gz, xl, yl, P, dt, Tg_out, idx, sx, sm, sz);
    Tg_out[idx] = Tn;
    prev = cur;
    cur = next;
    idx += ss;
  };
  if (interior) {  // 5 loads, no face tests; pointer steps instead of index arithmetic
    const float* p = Tg_in + idx;
    float* q = Tg_out + idx;
#pragma unroll
    for (int k = 0; k < kHeatChunk; ++k) {
      const float next = __ldg(p + ss);
      const float fm = __ldg(p - 1), fp = __ldg(p + 1);
      const float mm = __ldg(p - sm), mp = __ldg(p + sm);
      const float Tn =
          XYZ ? heat_cell_update<int, false>(H, cur, prev, next, mm, mp, fm, fp, 0, 0, 0, xl, yl,
                                             P, dt, Tg_out, 0, 0, 0, 0)
              : heat_cell_update<int, false>(H, cur, fm, fp, mm, mp, prev, next, 0, 0, 0, xl, yl,
                                             P, dt, Tg_out, 0, 0, 0, 0);
      *q = Tn;
      prev = cur;
      cur = next;
      p += ss;
      q += ss;
    }
  } else if (s0 + kHeatChunk <= ns) {  // a whole chunk: unrolled, loads issued ahead
#pragma unroll
    for (int k = 0; k < kHeatChunk; ++k) cell(s0 + k, std::true_type{});
  } else {
    for (int s = s0; s < ns; ++s) cell(s, std::true_type{});
  }
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
  if ((int64_t)(h->nx + 2) * (h->ny + 2) * (h->nz + 2) >= ((int64_t)1 << 31)) return PFG_ERR_SHAPE;
  const HeatConsts H = make_heat_consts(*h);
  const bool xyz = h->layout == PFG_LAYOUT_XYZ;
  const int nf = xyz ? h->nz : h->nx, ns = xyz ? h->nx : h->nz;
  if ((ns + kHeatChunk - 1) / kHeatChunk > 65535) return PFG_ERR_SHAPE;
  dim3 block(256, 1, 1);
  dim3 grid((unsigned)((nf * h->ny + 255) / 256), (unsigned)((ns + kHeatChunk - 1) / kHeatChunk), 1);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (xyz)
    heat_step_kernel<true><<<grid, block, 0, s>>>(H, Tg_in, Tg_out, xl, yl, power, dt);
  else
    heat_step_kernel<false><<<grid, block, 0, s>>>(H, Tg_in, Tg_out, xl, yl, power, dt);
  return record_cuda(cudaGetLastError());
}
