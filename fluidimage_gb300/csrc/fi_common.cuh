// Shared helpers of the fluidimage_gb300 CUDA library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/fluidimage_gb300.h"

namespace fi {

// Last error message of the calling host thread (returned by fi_last_error()).
void set_error(const char* fmt, ...);

// Counts kernel launches made by the library (fi_launch_count()).
void add_launches(int k);

// Checks a CUDA call inside an entry point; returns FI_ERR_CUDA on failure.
#define FI_CUDA_TRY(call)                                                     \
  do {                                                                        \
    cudaError_t fi_err_ = (call);                                             \
    if (fi_err_ != cudaSuccess) {                                             \
      ::fi::set_error("%s: %s (%s:%d)", #call, cudaGetErrorString(fi_err_),   \
                      __FILE__, __LINE__);                                    \
      return FI_ERR_CUDA;                                                     \
    }                                                                         \
  } while (0)

#define FI_REQUIRE(cond, ...)                                                 \
  do {                                                                        \
    if (!(cond)) {                                                            \
      ::fi::set_error(__VA_ARGS__);                                           \
      return FI_ERR_INVALID;                                                  \
    }                                                                         \
  } while (0)

// Raises a kernel's dynamic shared-memory limit to at least `bytes` (above the 48 KB
// default) on the current device, calling the runtime only when the limit has to
// grow there.  The attribute is per device, so the call site's record keeps the
// limit set so far for each device, read and written under one mutex so that host
// threads launching concurrently never lower it.
inline std::mutex& smem_limit_mutex() {
  static std::mutex m;
  return m;
}
constexpr int FI_SMEM_DEVICES = 64;
struct SmemLimit {
  size_t bytes[FI_SMEM_DEVICES] = {};
};
template <typename Kernel>
inline cudaError_t raise_smem_limit(Kernel* kernel, size_t bytes, SmemLimit& rec) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  int dev = 0;
  const cudaError_t ed = cudaGetDevice(&dev);
  if (ed != cudaSuccess) return ed;
  std::lock_guard<std::mutex> lock(smem_limit_mutex());
  const bool cached = dev >= 0 && dev < FI_SMEM_DEVICES;
  if (cached && bytes <= rec.bytes[dev]) return cudaSuccess;
  const cudaError_t e =
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess && cached) rec.bytes[dev] = bytes;
  return e;
}

inline int check_launch(const char* what, int kernels = 1) {
  add_launches(kernels);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s launch failed: %s", what, cudaGetErrorString(e));
    return FI_ERR_CUDA;
  }
  return FI_OK;
}

// Pixel loads for the three image element types.
__device__ __forceinline__ float load_px(const void* im, int dtype, int64_t idx) {
  switch (dtype) {
    case FI_U8: return (float)__ldg(reinterpret_cast<const uint8_t*>(im) + idx);
    case FI_U16: return (float)__ldg(reinterpret_cast<const uint16_t*>(im) + idx);
    default: return __ldg(reinterpret_cast<const float*>(im) + idx);
  }
}

__device__ __forceinline__ int load_px_int(const void* im, int dtype, int64_t idx) {
  return (dtype == FI_U8) ? (int)__ldg(reinterpret_cast<const uint8_t*>(im) + idx)
                          : (int)__ldg(reinterpret_cast<const uint16_t*>(im) + idx);
}

// Order-preserving float <-> uint32 keys (for atomicMin over floats).
__device__ __forceinline__ uint32_t float_to_key(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_to_float(uint32_t k) {
  uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  return __uint_as_float(u);
}

// Python/numpy floor division by 2 for int32.
__device__ __forceinline__ int floordiv2(int v) { return (v >= 0) ? (v / 2) : -((-v + 1) / 2); }

// Effective [s, e) of a numpy slice arr[start:stop] (step 1) on an axis of length L.
__host__ __device__ __forceinline__ void slice_bounds(int start, int stop, int L, int* s, int* e) {
  int a = start < 0 ? (start + L < 0 ? 0 : start + L) : (start > L ? L : start);
  int b = stop < 0 ? (stop + L < 0 ? 0 : stop + L) : (stop > L ? L : stop);
  *s = a;
  *e = b > a ? b : a;
}

}  // namespace fi
