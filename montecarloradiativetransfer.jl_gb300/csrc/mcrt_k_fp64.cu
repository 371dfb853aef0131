// FP64 instantiations of the persistent transport kernel.
#include "mcrt_kernels.h"

namespace mcrt {

// Bins per lane: 2 RT polar angles, 1 CB bin (doubles take twice the registers).
bool kernel_info_fp64(int bs, KInfo& k) {
  k.state_bytes = sizeof(PState<double>);
  switch (bs) {
    case 128:
      k.fn = k_transport<double, 128, 2, 1, 2>;
      k.shared_static = sizeof(Shared<double, 128>);
      return true;
    case 256:
      k.fn = k_transport<double, 256, 2, 1, 1>;
      k.shared_static = sizeof(Shared<double, 256>);
      return true;
  }
  return false;
}

}  // namespace mcrt
