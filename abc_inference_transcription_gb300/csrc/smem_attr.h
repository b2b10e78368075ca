// smem_attr.h — raising a kernel's dynamic shared-memory limit once per device.
//
// cudaFuncAttributeMaxDynamicSharedMemorySize is a per-device setting: a
// process with contexts on several GPUs must set it on each of them before
// the first launch there that needs more than 48 KiB.  One bit per device
// index (devices 0..63) records where it has been set; beyond 64 devices the
// call is simply repeated (it is idempotent and cheap).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

namespace abc {

template <typename Kernel>
inline cudaError_t set_smem_once(std::atomic<uint64_t>& done, Kernel kernel, int bytes) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint64_t bit = (dev >= 0 && dev < 64) ? (uint64_t(1) << dev) : 0;
  if (bit && (done.load() & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess && bit) done.fetch_or(bit);
  return e;
}

}  // namespace abc
