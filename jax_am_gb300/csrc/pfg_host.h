// Host-side internals shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "pf_gb300.h"

namespace pfg {

struct DeviceInfo {
  bool ok;
  int device;
  int sm_count;
  int smem_per_sm;     // bytes of shared memory per SM
  int smem_per_block;  // opt-in maximum per CTA
  int cc_major, cc_minor;
};

// Properties of the current device, cached per device.
const DeviceInfo& device_info();

// Record a CUDA error for pfg_last_cuda_error() and map it to a pfg_status.
int record_cuda(cudaError_t e);

// Tiling of the z-marching stencil kernel.
struct TilePlan {
  int cpw, wx, rpw;  // warp kernel: cells per warp, warps along x, rows per warp
  int vec;       // floats per thread chunk (4, 2 or 1: the largest dividing num_oris)
  int tpc;       // chunks per cell = num_oris / vec
  int tx, ty;    // tile cells along x and y
  int rs;        // rows processed concurrently by one CTA
  int stages;    // plane slots in the shared-memory ring
  int pitch;     // floats per staged row (tx + 2 cells, padded to 4)
  int tslot;     // floats per staged temperature plane
  int zc;        // planes per work unit
  int tiles_x, tiles_y, zchunks;
  long units;    // CTAs launched
  size_t smem;   // dynamic shared memory per CTA
};

TilePlan plan_tiles(int nx, int ny, int nz, int n, int sm_count, int max_smem_per_sm,
                    int max_smem_per_block);
TilePlan plan_for_current_device(const pfg_pf_params& p);
int check_pf_params(const pfg_pf_params* p);
int check_heat_params(const pfg_heat_params* h);
bool aligned16(const void* p);
int vec_width(int n);
// 0: pick the warp kernel when it applies; 1: always the generic kernel.
extern int g_kernel_variant;

}  // namespace pfg
