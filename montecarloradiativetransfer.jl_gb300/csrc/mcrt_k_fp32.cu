// FP32 instantiations of the persistent transport kernel.
#include "mcrt_kernels.h"

namespace mcrt {

// Bins per lane: 4 RT polar angles (8 for the 256-thread shape, which amortises the
// per-event setup over more bins and measured 2% faster), 2 CB bins; at most 128
// registers per thread.
bool kernel_info_fp32(int bs, KInfo& k) {
  k.state_bytes = sizeof(PState<float>);
  switch (bs) {
    case 128:
      k.fn = k_transport<float, 128, 4, 2, 4>;
      k.shared_static = sizeof(Shared<float, 128>);
      return true;
    case 256:
      k.fn = k_transport<float, 256, 8, 2, 2>;
      k.shared_static = sizeof(Shared<float, 256>);
      return true;
    case 512:
      k.fn = k_transport<float, 512, 4, 2, 1>;
      k.shared_static = sizeof(Shared<float, 512>);
      return true;
    case 768:  // one block per SM with 24 warps, at most 85 registers per thread
      k.fn = k_transport<float, 768, 4, 2, 1>;
      k.shared_static = sizeof(Shared<float, 768>);
      return true;
  }
  return false;
}

cudaError_t launch_transport(const KInfo& k, int blocks, int bs, size_t smem, cudaStream_t st,
                             const KParams& p) {
  void* args[] = {const_cast<KParams*>(&p)};
  return cudaLaunchKernel(reinterpret_cast<const void*>(k.fn), dim3(blocks), dim3(bs), args, smem, st);
}

}  // namespace mcrt
