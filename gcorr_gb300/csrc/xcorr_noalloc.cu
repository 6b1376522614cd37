// gxc_xcorr_noalloc: the X-stage of gxc_xcorr for callers that must not
// allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is off limits, e.g. a host
// callback or a real-time ingest thread that may not block on the allocator
// (cudaMalloc can synchronise the device), a process whose GPU memory is
// carved up and capped by someone else, or a plugin inside a framework that
// owns all device allocations.  Such callers own their input and output
// buffers already; what gxc_xcorr would allocate on their behalf is scratch.
// Here that scratch is one file-scope device array of fixed size, so the call
// allocates nothing.
//
// The array (GXC_XCORR_NOALLOC_SCRATCH_BYTES) exists on every GPU that loads
// this library, for the life of the process.  Host code cannot use its name
// as a device address, so the first call on each device looks the address up
// with cudaGetSymbolAddress (with that device current) and caches it; make
// that first call at initialisation, before any stream capture and outside any
// thread that must not block (it may load this module's device code, which
// allocates the array).  A cudaDeviceReset invalidates the cached address:
// calls after one are not supported.  All calls share the array and
// leave their data in it: accumulators are cleared at the start of every call,
// and calls that overlap on the GPU (different streams, or concurrent host
// threads) race on it.
#include <mutex>
#include <stdio.h>
#include <string>

#include "gxc_internal.h"

#define GXC_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_xcorr_scratch[GXC_XCORR_NOALLOC_SCRATCH_BYTES];

using namespace gxc;

namespace {

std::mutex g_scratch_mu;
void *g_scratch_ptr[GXC_NOALLOC_MAX_DEVICES] = {};

// Device address of the scratch array on the current device (looked up once per device).
cudaError_t scratch_address(void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= GXC_NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_xcorr_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Tile-pair table J <= K over ceil(nant/2) antenna tiles, J-major, written on the device.
__global__ void pairs_kernel(int nat, int2 *pairs) {
  const int J = blockIdx.x;
  for (int K = J + threadIdx.x; K < nat; K += blockDim.x) {
    const int q = J * nat - J * (J - 1) / 2 + (K - J);
    pairs[q] = make_int2(J, K);
  }
}

template <typename OutT>
__device__ __forceinline__ OutT cvt(float2 v);
template <> __device__ __forceinline__ float2 cvt<float2>(float2 v) { return v; }
template <> __device__ __forceinline__ __half2 cvt<__half2>(float2 v) { return __floats2half2_rn(v.x, v.y); }
template <> __device__ __forceinline__ __nv_fp8x2_e4m3 cvt<__nv_fp8x2_e4m3>(float2 v) { return __nv_fp8x2_e4m3(v); }

// ants[(ant*2+pol)*nfft*fftwidth + f*fftwidth + c] -> [ctile][T][stream][16] for FFTs [t0, t0+nt)
template <typename OutT>
__global__ void relayout_noalloc_kernel(const float2 *__restrict__ ants, int nstream, int nfft, int nchan,
                                        int fftwidth, int t0, int nt, int T, OutT *__restrict__ chan) {
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

__global__ void divide_noalloc_kernel(const float2 *__restrict__ vsum, const float2 *__restrict__ vcomp, size_t n,
                                      float nfft, float2 *__restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float2 s = vsum[i], c = vcomp[i];
  out[i] = make_float2((s.x + c.x) / nfft, (s.y + c.y) / nfft);
}

// Device memory of the current device (whose scratch array the call uses), or managed memory.
bool on_device(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  int cur = -1;
  if (cudaGetDevice(&cur) != cudaSuccess) return false;
  return a.type == cudaMemoryTypeDevice && a.device == cur;
}

gxc_status fail(gxc_status st, const std::string &msg) {
  fprintf(stderr, "gxc_xcorr_noalloc: %s\n", msg.c_str());
  return st;
}

}  // namespace

extern "C" gxc_status gxc_xcorr_noalloc(const float *ants, int nant, int nfft, int nchan, int fftwidth,
                                        int precision, int autos, float *accum, void *stream) {
  if (!ants || !accum) return fail(GXC_ERR_INVALID_ARGUMENT, "null buffer");
  if (nant < 1 || nfft < 1 || nchan < 16 || (nchan % CW) || fftwidth < nchan)
    return fail(GXC_ERR_INVALID_ARGUMENT,
                "need nant >= 1, nfft >= 1, nchan >= 16 and a multiple of 16, fftwidth >= nchan");
  if (precision != GXC_PRECISION_FP32 && precision != GXC_PRECISION_FP16)
    return fail(GXC_ERR_UNSUPPORTED, "precision must be FP32 or FP16");
  if (!on_device(ants) || !on_device(accum))
    return fail(GXC_ERR_INVALID_ARGUMENT,
                "ants and accum must be device memory of the current device (nothing is staged)");

  const int nstream = 2 * nant;
  const int nat = (nant + 1) / 2;
  const int npairs = nat * (nat + 1) / 2;
  const int nbl = nant * (nant - 1) / 2 + (autos ? nant : 0);
  const size_t nvis = (size_t)nbl * 4 * nchan;
  const size_t esz = chan_elem_bytes(chan_type_of(precision));
  const int ct = chan_type_of(precision);
  // scratch layout: [pair table][sum][comp][channelised block of T FFTs]
  const size_t off_sum = align256(sizeof(int2) * (size_t)npairs);
  const size_t off_comp = off_sum + align256(sizeof(float2) * nvis);
  const size_t off_chan = off_comp + align256(sizeof(float2) * nvis);
  const size_t per_fft = (size_t)nstream * nchan * esz;
  const size_t limit = GXC_XCORR_NOALLOC_SCRATCH_BYTES;
  if (off_chan + per_fft > limit)
    return fail(GXC_ERR_INVALID_ARGUMENT,
                "problem too large for the fixed scratch (" + std::to_string(limit >> 20) +
                    " MiB): accumulators of nbl*4*nchan complex values plus one FFT of channelised data must fit");
  size_t T = (limit - off_chan) / per_fft;
  if (T > (size_t)nfft) T = (size_t)nfft;

  void *base = nullptr;
  cudaError_t e = scratch_address(&base);
  if (e != cudaSuccess) return fail(GXC_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  unsigned char *sc = (unsigned char *)base;
  int2 *pairs = (int2 *)sc;
  float2 *vsum = (float2 *)(sc + off_sum);
  float2 *vcomp = (float2 *)(sc + off_comp);
  void *chan = sc + off_chan;
  cudaStream_t s = (cudaStream_t)stream;

  pairs_kernel<<<nat, 64, 0, s>>>(nat, pairs);
  e = cudaGetLastError();
  if (e == cudaSuccess && nvis) e = cudaMemsetAsync(vsum, 0, sizeof(float2) * nvis, s);
  if (e == cudaSuccess && nvis) e = cudaMemsetAsync(vcomp, 0, sizeof(float2) * nvis, s);
  for (int t0 = 0; e == cudaSuccess && t0 < nfft; t0 += (int)T) {
    const int nt = (nfft - t0) < (int)T ? (nfft - t0) : (int)T;
    const size_t total = (size_t)nt * nstream * nchan;
    const unsigned blocks = (unsigned)((total + 255) / 256);
    if (ct == CHAN_F32)
      relayout_noalloc_kernel<float2><<<blocks, 256, 0, s>>>((const float2 *)ants, nstream, nfft, nchan, fftwidth,
                                                              t0, nt, (int)T, (float2 *)chan);
    else
      relayout_noalloc_kernel<__half2><<<blocks, 256, 0, s>>>((const float2 *)ants, nstream, nfft, nchan, fftwidth,
                                                               t0, nt, (int)T, (__half2 *)chan);
    e = cudaGetLastError();
    if (e == cudaSuccess)
      e = launch_xstage_cuda_core_pairs(chan, ct, nant, nchan, (int)T, nt, autos, pairs, vsum, vcomp, s);
  }
  if (e == cudaSuccess && nvis) {
    divide_noalloc_kernel<<<(unsigned)((nvis + 255) / 256), 256, 0, s>>>(vsum, vcomp, nvis, (float)nfft,
                                                                         (float2 *)accum);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return fail(GXC_ERR_CUDA, cudaGetErrorString(e));
  return GXC_OK;
}
