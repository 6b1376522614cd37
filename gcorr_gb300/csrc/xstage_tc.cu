// tcgen05 tensor-core X-stage (FP16 channelised data, FP32 accumulation in TMEM).
#include "gxc_internal.h"

namespace gxc {

int xstage_tensor_supported(int nant) { (void)nant; return 0; }

cudaError_t launch_xstage_tensor(const void *, int, int, int, int, int, float2 *, float2 *, cudaStream_t) {
  return cudaErrorNotSupported;
}

}  // namespace gxc
