// Instantiations of the plain per-ray kernel.
#include "mcrt_kernels.h"

namespace mcrt {

cudaError_t launch_plain(int fp64, int blocks, cudaStream_t st, const PlainParams& p) {
  if (fp64)
    k_plain<double><<<blocks, 256, 0, st>>>(p);
  else
    k_plain<float><<<blocks, 256, 0, st>>>(p);
  return cudaGetLastError();
}

}  // namespace mcrt
