// Internal declarations shared by the libgxcorr translation units.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>
#include <stdint.h>
#include <stddef.h>

#include "gxc.h"

namespace gxc {

// Channels per channel tile of the channelised layout [ctile][t][stream][CW].
constexpr int CW = 16;

// Per-(antenna, FFT) geometry record, produced by the geometry kernel from the
// delay polynomial (fxkernel/src/fxkernel.cpp:288-309, :425-440).  The phase
// constants of the F-stage are evaluated there in FP64, once per (antenna, FFT),
// reduced mod 1 turn and rounded to FP32 (fxkernel.cpp:503-535, :600-630).
struct Geom {
  float c0;      // fringe phase at the first sample, turns, in [0, 1)
  float c1;      // fringe phase slope, turns per sample
  float cstep;   // phase advance of one coarse rotator-table entry, turns
  float cf;      // fractional-sample correction, turns per channel
  int offset;    // first sample of the FFT window in the antenna stream
  int valid;     // 0 = flagged (window outside the buffer)
  int pad[2];
};
static_assert(sizeof(Geom) == 32, "Geom layout");

// Launch-time description of one sub-integration for the device kernels.
struct Job {
  const uint8_t *const *inputs;  // device array of nant device pointers
  const double *poly;            // [nant][3]
  const double *fso;             // [nant]
  Geom *geom;                    // [nant][nfft]
  int nant, nchan, nfft, F, log2F;
  int is_complex;                // 0: 2-bit real, 1: 8-bit complex
  int rotator;                   // GXC_ROTATOR_*
  int stride, substride;         // fringe rotator table split: F = stride * substride
  int fsub, fstride;             // frac-delay table split: nchan = fstride * fsub
  int fractional_lo;             // fxkernel.cpp:67-71
  double lo_hz, bw_hz, Ts;
  long long maxoffset;           // (nfft-1)*F
  // optional per-antenna frame validity (e.g. from a VDIF depacketiser): device array of nant
  // pointers to uint8 [nframes] (a null entry = all valid); an FFT whose window touches an
  // invalid frame is flagged.  fvalid == nullptr: no frame flags.
  const uint8_t *const *fvalid;
  long long samples_per_frame;
};

// Channelised-data element types.
// FP8: E4M3 pairs (re, im), two bytes per complex value.
enum ChanType { CHAN_F32 = 0, CHAN_F16 = 1, CHAN_F8 = 2 };
inline size_t chan_elem_bytes(int chan_type) { return chan_type == CHAN_F32 ? 8 : chan_type == CHAN_F16 ? 4 : 2; }
inline int chan_type_of(int precision) {
  return precision == GXC_PRECISION_FP32 ? CHAN_F32 : precision == GXC_PRECISION_FP16 ? CHAN_F16 : CHAN_F8;
}

// fstage.cu
cudaError_t launch_geometry(const Job &job, cudaStream_t s);
cudaError_t launch_counts(const Job &job, int autos, int32_t *counts, uint8_t *valid_flags, cudaStream_t s);
cudaError_t make_twiddles(int F, float2 **out);
// cscale (FP8 output only): per-channel output scale [nchan] replacing out_scale, or null.
cudaError_t launch_fstage(const Job &job, const float2 *twiddles, int t0, int nt, int T, void *chan, int chan_type,
                          float out_scale, cudaStream_t s, const float *cscale = nullptr);
int fstage_supported(int F);
// fstage_probe.cu: the F-stage of FFTs [t0, t0+nt) with every decoded input sample also written to
// probe [nant][2][nfft][F] (complex float) before the fringe rotation.  chan must hold T FFTs of
// FP32 channelised data.
cudaError_t launch_fstage_probe(const Job &job, const float2 *twiddles, int t0, int nt, int T, void *chan,
                                int chan_type, float out_scale, float2 *probe, cudaStream_t s);

// fstage_tc.cu: the tensor-core F-stage (8192-point windows, 2-bit real, FP16 / FP8 output).
int fstage_tc_supported(const Job &job, int chan_type);
cudaError_t make_fstage_tc_tables(void **out);  // its constant operands (cudaMalloc'd; caller frees)
// probe non-null: the decode probe (every decoded sample also written to probe [nant][2][nfft][F]).
cudaError_t launch_fstage_tc(const Job &job, const void *tables, int t0, int nt, int T, void *chan, int chan_type,
                             float out_scale, cudaStream_t s, const float *cscale = nullptr,
                             float2 *probe = nullptr);
cudaError_t fstage_tc_take_error(int *flag);

// xstage_fp32.cu: accumulates visibilities of FFTs [0, nt) of the block into
// the compensated (sum, comp) accumulators in the output layout.
cudaError_t launch_xstage_cuda_core(const void *chan, int chan_type, int nant, int nchan, int T, int nt, int autos,
                                    const int2 *pairs, float2 *vsum, float2 *vcomp, cudaStream_t s);
// Device table of (J, K) 2-antenna tile pairs, J <= K, J-major (cudaMalloc'd; caller frees).
cudaError_t make_tile_pairs(int nant, int2 **out);

cudaError_t launch_xstage_cuda_core_pairs(const void *chan, int chan_type, int nant, int nchan, int T, int nt,
                                          int autos, const int2 *pairs, float2 *vsum, float2 *vcomp,
                                          cudaStream_t s);

// xstage_tc.cu: tcgen05 tensor-core X-stage over FP16 channelised data.
// FP16 data: kind::f16 MMAs; FP32 data: kind::tf32 MMAs on a hi/lo split (FP32-accurate products).
// split_e >= 0 (FP32 data whose scale is known, e.g. the F-stage's output): the FP32 path uses
// an FP16 hi/lo split of the values times 2^-split_e; split_e < 0: the TF32 hi/lo split.
// kparts_max = 2 with plane > 0: the FP16 / FP8 kernel splits the block's FFTs across two CTAs
// per channel group when the groups are fewer than the SMs (3: whenever the block is long enough),
// the second CTA accumulating into vsum/vcomp + plane (a second plane the caller allocated, zeroed
// and sums at the end).
cudaError_t launch_xstage_tensor(const void *chan, int chan_type, int nant, int nchan, int T, int nt, int autos,
                                 float2 *vsum, float2 *vcomp, cudaStream_t s, int split_e = -1,
                                 int kparts_max = 1, size_t plane = 0);
int xstage_tensor_supported(int nant);
int xstage_tensor_channels_per_cta(int nant, int chan_type);
int xstage_tensor_fits(int nant, int nchan, int chan_type);
cudaError_t xstage_tensor_take_error(int *flag);

// gxc_api.cu: process() with its host->device input copies ordered behind copy_wait (when not
// null) and followed by a record of copy_done (when not null).  nchunk > 0: the device input
// arrives in chunks, bytes [0, chunk_end[j]) of every antenna once chunk_ev[j] has completed; each
// F-stage launch waits only for the chunk that holds its windows (gxc_input_bytes_for_ffts).
gxc_status process_chained(gxc_handle *h, void *stream, cudaEvent_t copy_wait, cudaEvent_t copy_done,
                           int nchunk = 0, const cudaEvent_t *chunk_ev = nullptr,
                           const long long *chunk_end = nullptr);

// Output baseline index of antennas j <= k (crosses in fxkernel order, then autos).
__host__ __device__ inline int baseline_index(int j, int k, int nant) {
  if (j == k) return nant * (nant - 1) / 2 + j;
  return j * nant - j * (j + 1) / 2 + (k - j - 1);
}

// Compensated accumulation acc += x (TwoSum): sum holds the running total,
// comp the accumulated rounding error; the result is sum + comp.
__device__ inline void two_sum_add(float &sum, float &comp, float x) {
  float t = sum + x;
  float bp = t - sum;
  float e = (sum - (t - bp)) + (x - bp);
  sum = t;
  comp += e;
}

}  // namespace gxc
