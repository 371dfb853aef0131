// Kernel entry points instantiated in their own translation units (compiled in
// parallel): the persistent transport kernel per precision and block size, and the
// plain per-ray kernel.
#pragma once

#include <cstddef>
#include <cuda_runtime.h>

#include "mcrt_plain.cuh"
#include "mcrt_transport.cuh"

namespace mcrt {

struct KInfo {
  void (*fn)(KParams);
  size_t shared_static;  // bytes of the static shared-memory part (before the tables)
  size_t state_bytes;    // bytes of one photon's state in the pool
};

// FP32: block sizes 128, 256, 512. FP64: 128, 256. Returns false otherwise.
bool kernel_info_fp32(int bs, KInfo& k);
bool kernel_info_fp64(int bs, KInfo& k);
cudaError_t launch_transport(const KInfo& k, int blocks, int bs, size_t smem, cudaStream_t st,
                             const KParams& p);
cudaError_t launch_plain(int fp64, int blocks, cudaStream_t st, const PlainParams& p);

}  // namespace mcrt
