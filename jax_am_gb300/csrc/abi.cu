// Library information, error reporting and the per-device property cache.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "pfg_host.h"

namespace pfg {

static thread_local char g_last_error[256] = "";

int record_cuda(cudaError_t e) {
  if (e == cudaSuccess) return PFG_OK;
  std::strncpy(g_last_error, cudaGetErrorString(e), sizeof(g_last_error) - 1);
  g_last_error[sizeof(g_last_error) - 1] = '\0';
  return PFG_ERR_LAUNCH;
}

const DeviceInfo& device_info() {
  static DeviceInfo cache[64];
  static bool filled[64] = {false};
  static std::mutex mu;
  static DeviceInfo none = {false, -1, 0, 0, 0, 0, 0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return none;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (!filled[dev]) {
    DeviceInfo d{};
    d.device = dev;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) == cudaSuccess) {
      d.ok = prop.major >= 10;
      d.sm_count = prop.multiProcessorCount;
      d.smem_per_sm = (int)prop.sharedMemPerMultiprocessor;
      d.smem_per_block = (int)prop.sharedMemPerBlockOptin;
      d.cc_major = prop.major;
      d.cc_minor = prop.minor;
    } else {
      cudaGetLastError();
      d.ok = false;
    }
    cache[dev] = d;
    filled[dev] = true;
  }
  return cache[dev];
}

}  // namespace pfg

extern "C" int pfg_abi_version(void) { return PFG_ABI_VERSION; }

extern "C" const char* pfg_last_cuda_error(void) { return pfg::g_last_error; }

extern "C" const char* pfg_status_string(int status) {
  switch (status) {
    case PFG_OK: return "ok";
    case PFG_ERR_SHAPE: return "bad shape: grid extent < 1 or num_oris outside [1, 64]";
    case PFG_ERR_NULL: return "a required pointer is NULL";
    case PFG_ERR_ALIGN: return "a device pointer is not 16-byte aligned";
    case PFG_ERR_PARAM: return "a parameter is out of its domain";
    case PFG_ERR_LAUNCH: return "CUDA launch failed";
    case PFG_ERR_TIMEOUT: return "a bounded device-side wait ran out";
    case PFG_ERR_CAPACITY: return "a table or scratch buffer is too small";
    case PFG_ERR_NO_DEVICE: return "no usable sm_103 device";
    default: return "unknown status";
  }
}

extern "C" int64_t pfg_struct_size(int which) {
  switch (which) {
    case 0: return (int64_t)sizeof(pfg_pf_params);
    case 1: return (int64_t)sizeof(pfg_segment);
    case 2: return (int64_t)sizeof(pfg_heat_params);
    case 3: return (int64_t)sizeof(pfg_clock);
    case 4: return (int64_t)sizeof(pfg_diag);
    case 5: return (int64_t)sizeof(pfg_quench);
    case 6: return (int64_t)sizeof(pfg_batch_job);
    case 7: return (int64_t)sizeof(pfg_grain);
    case 8: return (int64_t)sizeof(pfg_point_source);
    case 9: return (int64_t)sizeof(pfg_point_sources);
    case 10: return (int64_t)sizeof(pfg_interp);
    case 11: return (int64_t)sizeof(pfg_cfd_grid);
    case 12: return (int64_t)sizeof(pfg_linclip);
    case 13: return (int64_t)sizeof(pfg_cfd_energy);
    case 14: return (int64_t)sizeof(pfg_cfd_flow);
    case 15: return (int64_t)sizeof(pfg_cfd_stats);
    default: return -1;
  }
}
