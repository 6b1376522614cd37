// gxc_xcorr: the X-stage alone, on already-channelised data in the layout of
// the reference GPU X kernels (gcorr/src/gxkernel.h:30-44 antIdx/accumIdx,
// gcorr/src/gxkernel.cu:518-585 CCAH3): ants[(ant*2 + pol)*nfft*fftwidth + f*fftwidth + chan].
// The data is re-laid into the engine's [ctile][T][stream][16] layout block by
// block, cross-multiplied by the CUDA-core or tensor-core X-stage, and each
// product divided by nfft as CCAH3 does.
#include <stdio.h>
#include <string.h>

#include <string>

#include "gxc_internal.h"

using namespace gxc;

namespace {

template <typename OutT>
__device__ __forceinline__ OutT cvt(float2 v);
template <> __device__ __forceinline__ float2 cvt<float2>(float2 v) { return v; }
template <> __device__ __forceinline__ __half2 cvt<__half2>(float2 v) { return __floats2half2_rn(v.x, v.y); }
template <> __device__ __forceinline__ __nv_fp8x2_e4m3 cvt<__nv_fp8x2_e4m3>(float2 v) { return __nv_fp8x2_e4m3(v); }

// ants (gcorr layout) -> chan [ctile][T][nstream][CW] for FFTs [t0, t0+nt)
template <typename OutT>
__global__ void relayout_kernel(const float2 *__restrict__ ants, int nstream, int nfft, int nchan, int fftwidth,
                                int t0, int nt, int T, OutT *__restrict__ chan) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t total = (size_t)nt * nstream * nchan;
  if (i >= total) return;
  const int c = (int)(i % nchan);
  const size_t r = i / nchan;
  const int s = (int)(r % nstream);
  const int t = (int)(r / nstream);
  const float2 v = ants[(size_t)s * nfft * fftwidth + (size_t)(t0 + t) * fftwidth + c];
  chan[(((size_t)(c >> 4) * T + t) * nstream + s) * CW + (c & 15)] = cvt<OutT>(v);
}

__global__ void divide_kernel(const float2 *__restrict__ vsum, const float2 *__restrict__ vcomp, size_t n,
                              float nfft, float2 *__restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float2 s = vsum[i], c = vcomp[i];
  out[i] = make_float2((s.x + c.x) / nfft, (s.y + c.y) / nfft);
}

bool is_device(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

namespace gxc {

// Runs the X-stage over ants with the given scratch buffers (device memory):
//   chan: block buffer of T*nstream*nchan elements (float2 or half2),
//   vsum, vcomp: nbl*4*nchan float2 each.
gxc_status xcorr_run(const float2 *ants, int nant, int nfft, int nchan, int fftwidth, int precision, int engine,
                     int autos, float2 *out, void *chan, int T, const int2 *pairs, float2 *vsum, float2 *vcomp,
                     cudaStream_t s, std::string *msg) {
  const int nstream = 2 * nant;
  const int nbl = nant * (nant - 1) / 2 + (autos ? nant : 0);
  const size_t nvis = (size_t)nbl * 4 * nchan;
  const int ct = chan_type_of(precision);
  cudaError_t e = cudaMemsetAsync(vsum, 0, nvis * sizeof(float2), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(vcomp, 0, nvis * sizeof(float2), s);
  for (int t0 = 0; e == cudaSuccess && t0 < nfft; t0 += T) {
    const int nt = (nfft - t0) < T ? (nfft - t0) : T;
    const size_t total = (size_t)nt * nstream * nchan;
    const unsigned blocks = (unsigned)((total + 255) / 256);
    if (ct == CHAN_F32)
      relayout_kernel<float2><<<blocks, 256, 0, s>>>(ants, nstream, nfft, nchan, fftwidth, t0, nt, T, (float2 *)chan);
    else if (ct == CHAN_F8)
      relayout_kernel<__nv_fp8x2_e4m3><<<blocks, 256, 0, s>>>(ants, nstream, nfft, nchan, fftwidth, t0, nt, T,
                                                              (__nv_fp8x2_e4m3 *)chan);
    else
      relayout_kernel<__half2><<<blocks, 256, 0, s>>>(ants, nstream, nfft, nchan, fftwidth, t0, nt, T,
                                                      (__half2 *)chan);
    e = cudaGetLastError();
    if (e != cudaSuccess) break;
    if (engine == GXC_XENGINE_TENSOR)
      e = launch_xstage_tensor(chan, ct, nant, nchan, T, nt, autos, vsum, vcomp, s);
    else
      e = launch_xstage_cuda_core(chan, ct, nant, nchan, T, nt, autos, pairs, vsum, vcomp, s);
  }
  if (e == cudaSuccess && nvis) {
    divide_kernel<<<(unsigned)((nvis + 255) / 256), 256, 0, s>>>(vsum, vcomp, nvis, (float)nfft, out);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    if (msg) *msg = std::string("gxc_xcorr: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? GXC_ERR_OUT_OF_MEMORY : GXC_ERR_CUDA;
  }
  return GXC_OK;
}

gxc_status xcorr_check(int nant, int nfft, int nchan, int fftwidth, int precision, int *engine, std::string *msg) {
  if (nant < 1 || nfft < 1 || nchan < 16 || (nchan % CW) || fftwidth < nchan) {
    *msg = "gxc_xcorr: need nant >= 1, nfft >= 1, nchan >= 16 and a multiple of 16, fftwidth >= nchan";
    return GXC_ERR_INVALID_ARGUMENT;
  }
  if (precision != GXC_PRECISION_FP32 && precision != GXC_PRECISION_FP16 && precision != GXC_PRECISION_FP8) {
    *msg = "gxc_xcorr: precision must be FP32, FP16 or FP8";
    return GXC_ERR_INVALID_ARGUMENT;
  }
  const int ct = chan_type_of(precision);
  const bool tc_ok = xstage_tensor_fits(nant, nchan, ct) != 0;
  if (*engine == GXC_XENGINE_AUTO) *engine = tc_ok ? GXC_XENGINE_TENSOR : GXC_XENGINE_CUDA_CORE;
  if (*engine == GXC_XENGINE_TENSOR && !tc_ok) {
    *msg = "gxc_xcorr: the tensor-core X-stage needs nant <= 64 (FP16), <= 32 (FP32, FP8) and nchan a multiple "
           "of its channel tile";
    return GXC_ERR_UNSUPPORTED;
  }
  return GXC_OK;
}

}  // namespace gxc

extern "C" gxc_status gxc_xcorr(const float *ants, int nant, int nfft, int nchan, int fftwidth, int precision,
                                int x_engine, int autos, float *accum, void *stream) {
  std::string msg;
  int engine = x_engine;
  if (!ants || !accum) return GXC_ERR_INVALID_ARGUMENT;
  gxc_status st = xcorr_check(nant, nfft, nchan, fftwidth, precision, &engine, &msg);
  if (st != GXC_OK) {
    fprintf(stderr, "%s\n", msg.c_str());
    return st;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int nbl = nant * (nant - 1) / 2 + (autos ? nant : 0);
  const size_t nvis = (size_t)nbl * 4 * nchan;
  const size_t nin = (size_t)2 * nant * nfft * fftwidth;
  const size_t esz = chan_elem_bytes(chan_type_of(precision));
  int T = nfft < 1024 ? nfft : 1024;
  // scratch: channelised block, accumulators, device copies of host buffers
  void *chan = nullptr;
  float2 *vsum = nullptr, *vcomp = nullptr, *dants = nullptr, *dout = nullptr;
  int2 *pairs = nullptr;
  const bool ants_dev = is_device(ants), out_dev = is_device(accum);
  cudaError_t e = cudaMalloc(&chan, (size_t)T * 2 * nant * nchan * esz);
  if (e == cudaSuccess) e = make_tile_pairs(nant, &pairs);
  if (e == cudaSuccess) e = cudaMalloc((void **)&vsum, nvis * sizeof(float2) + 16);
  if (e == cudaSuccess) e = cudaMalloc((void **)&vcomp, nvis * sizeof(float2) + 16);
  if (e == cudaSuccess && !ants_dev) e = cudaMalloc((void **)&dants, nin * sizeof(float2));
  if (e == cudaSuccess && !out_dev) e = cudaMalloc((void **)&dout, nvis * sizeof(float2) + 16);
  if (e == cudaSuccess && !ants_dev) e = cudaMemcpyAsync(dants, ants, nin * sizeof(float2), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    st = xcorr_run(ants_dev ? (const float2 *)ants : dants, nant, nfft, nchan, fftwidth, precision, engine, autos,
                   out_dev ? (float2 *)accum : dout, chan, T, pairs, vsum, vcomp, s, &msg);
    if (st == GXC_OK && !out_dev)
      e = cudaMemcpyAsync(accum, dout, nvis * sizeof(float2), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  if (st == GXC_OK && e == cudaSuccess && engine == GXC_XENGINE_TENSOR) {
    int flag = 0;
    e = xstage_tensor_take_error(&flag);
    if (e == cudaSuccess && flag) st = GXC_ERR_TIMEOUT;
  }
  cudaFree(chan);
  cudaFree(pairs);
  cudaFree(vsum);
  cudaFree(vcomp);
  cudaFree(dants);
  cudaFree(dout);
  if (st != GXC_OK) {
    if (!msg.empty()) fprintf(stderr, "%s\n", msg.c_str());
    return st;
  }
  if (e != cudaSuccess) {
    fprintf(stderr, "gxc_xcorr: %s\n", cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? GXC_ERR_OUT_OF_MEMORY : GXC_ERR_CUDA;
  }
  return GXC_OK;
}
