// Decode probe of the F-stage kernels: the same kernel templates as the
// production launcher (fstage_kernels.cuh), instantiated with DBG = true so
// that every decoded input sample is also written out before the fringe
// rotation.  It lets a test compare the GPU unpack of 2-bit real and 8-bit
// complex windows, at any offset the delay model produces, bit for bit with
// the reference's level table and byte layout (fxkernel/src/fxkernel.cpp:15-28,
// :443-487).  process() never launches these kernels.
#include "fstage_kernels.cuh"
#include "gxc_internal.h"

namespace gxc {

cudaError_t launch_fstage_probe(const Job &job, const float2 *twiddles, int t0, int nt, int T, void *chan,
                                int chan_type, float out_scale, float2 *probe, cudaStream_t s) {
  if (nt <= 0) return cudaSuccess;
  const FParams prm = fstage_params(job, twiddles, t0, T, chan, out_scale, probe);
  // FP16 / FP8 output at 16384 and 32768 points runs the FP16-buffer kernel; every other
  // shape runs a kernel template whose decode does not depend on the output type, probed
  // here with FP32 output (chan must then hold T FFTs of FP32 channelised data)
  if (chan_type != CHAN_F32 && job.log2F >= 14) {
    if (job.log2F == 14)
      return job.is_complex ? launch_fstage_h<14, __half2, true, true>(prm, nt, s)
                            : launch_fstage_h<14, __half2, false, true>(prm, nt, s);
    return job.is_complex ? launch_fstage_h<15, __half2, true, true>(prm, nt, s)
                          : launch_fstage_h<15, __half2, false, true>(prm, nt, s);
  }
  return job.is_complex ? launch_fstage_l<float2, true, true>(prm, nt, s)
                        : launch_fstage_l<float2, false, true>(prm, nt, s);
}

}  // namespace gxc
