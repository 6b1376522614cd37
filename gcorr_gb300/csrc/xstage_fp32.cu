// CUDA-core X-stage: per-channel conjugate-multiply-accumulate over all
// baselines (autos included) and the four pol products, FP32 arithmetic.
//
// Restates the baseline loop of FxKernel::process (fxkernel/src/fxkernel.cpp:328-355,
// ippsAddProduct_32fc of X_j,l with conj(X_k,m)) and plays the role of the
// reference GPU X kernels (gcorr/src/gxkernel.cu:518-585, CCAH3) as the plain-FP32
// GPU X-stage.  Flagged FFTs arrive as zeros from the F-stage, so the sum over
// the block needs no masking; counts are applied at finalisation.
//
// Layout in: channelised [ctile][T][nstream][CW] (float2 or half2), stream s = 2*ant + pol.
// Work split: a CTA owns one channel tile (CW = 16 channels) and a group of
// antenna-tile pairs; a thread owns one channel and one pair of 2-antenna tiles
// (J <= K), i.e. a 2x2 block of antenna baselines x 4 products = 16 complex
// accumulators, reused over TT FFTs staged in shared memory.
#include <vector>

#include "gxc_internal.h"

namespace gxc {

template <typename InT> __device__ __forceinline__ float2 ld_c(const InT *p);
template <> __device__ __forceinline__ float2 ld_c<float2>(const float2 *p) { return *p; }
template <> __device__ __forceinline__ float2 ld_c<__half2>(const __half2 *p) { return __half22float2(*p); }
template <> __device__ __forceinline__ float2 ld_c<__nv_fp8x2_e4m3>(const __nv_fp8x2_e4m3 *p) {
  return static_cast<float2>(*p);
}

// x * conj(y) accumulated into a
__device__ __forceinline__ void cmac_conj(float2 &a, float2 x, float2 y) {
  a.x = fmaf(x.x, y.x, fmaf(x.y, y.y, a.x));
  a.y = fmaf(x.y, y.x, fmaf(-x.x, y.y, a.y));
}

template <typename InT>
__global__ void xstage_cc_kernel(const InT *__restrict__ chan, int nant, int nchan, int T, int nt, int autos,
                                 const int2 *__restrict__ tile_pairs, int npairs, int pairs_per_cta, int TT,
                                 float2 *__restrict__ vsum, float2 *__restrict__ vcomp) {
  extern __shared__ unsigned char xsm_raw[];
  InT *xs = reinterpret_cast<InT *>(xsm_raw);  // [TT][nstream][CW]
  const int nstream = 2 * nant;
  const int ctile = blockIdx.y;
  const int c = threadIdx.x & (CW - 1);
  const int pl = threadIdx.x >> 4;
  const int tp = blockIdx.x * pairs_per_cta + pl;
  const bool has_pair = (pl < pairs_per_cta) && (tp < npairs);
  int J = 0, K = 0;
  if (has_pair) {
    const int2 jk = tile_pairs[tp];
    J = jk.x;
    K = jk.y;
  }
  // streams of the four antennas 2J, 2J+1, 2K, 2K+1 (two pols each)
  const int sj0 = 4 * J, sk0 = 4 * K;
  const bool j1ok = (2 * J + 1) < nant, k1ok = (2 * K + 1) < nant;

  float2 acc[2][2][4];
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++)
#pragma unroll
      for (int p = 0; p < 4; p++) acc[a][b][p] = make_float2(0.f, 0.f);

  const InT *src = chan + (size_t)ctile * T * nstream * CW;
  const int row = nstream * CW;  // elements per FFT in this tile
  for (int t0 = 0; t0 < nt; t0 += TT) {
    const int tt_n = min(TT, nt - t0);
    // cooperative, contiguous, 16-byte vector copy of [tt_n][nstream][CW]
    {
      const size_t bytes = (size_t)tt_n * row * sizeof(InT);
      const int4 *g4 = reinterpret_cast<const int4 *>(src + (size_t)t0 * row);
      int4 *s4 = reinterpret_cast<int4 *>(xs);
      const int n4 = (int)(bytes / 16);
      for (int i = threadIdx.x; i < n4; i += blockDim.x) s4[i] = __ldg(&g4[i]);
    }
    __syncthreads();
    if (has_pair) {
      for (int tt = 0; tt < tt_n; tt++) {
        const InT *r = xs + (size_t)tt * row + c;
        float2 xj[2][2], xk[2][2];
        xj[0][0] = ld_c(r + (sj0 + 0) * CW);
        xj[0][1] = ld_c(r + (sj0 + 1) * CW);
        xj[1][0] = j1ok ? ld_c(r + (sj0 + 2) * CW) : make_float2(0.f, 0.f);
        xj[1][1] = j1ok ? ld_c(r + (sj0 + 3) * CW) : make_float2(0.f, 0.f);
        xk[0][0] = ld_c(r + (sk0 + 0) * CW);
        xk[0][1] = ld_c(r + (sk0 + 1) * CW);
        xk[1][0] = k1ok ? ld_c(r + (sk0 + 2) * CW) : make_float2(0.f, 0.f);
        xk[1][1] = k1ok ? ld_c(r + (sk0 + 3) * CW) : make_float2(0.f, 0.f);
#pragma unroll
        for (int a = 0; a < 2; a++)
#pragma unroll
          for (int b = 0; b < 2; b++)
#pragma unroll
            for (int l = 0; l < 2; l++)
#pragma unroll
              for (int m = 0; m < 2; m++) cmac_conj(acc[a][b][2 * l + m], xj[a][l], xk[b][m]);
      }
    }
    __syncthreads();
  }
  if (!has_pair) return;
  const int cg = ctile * CW + c;
  if (cg >= nchan) return;
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++) {
      const int j = 2 * J + a, k = 2 * K + b;
      if (j >= nant || k >= nant || j > k) continue;
      if (j == k && !autos) continue;
      const int bl = baseline_index(j, k, nant);
#pragma unroll
      for (int p = 0; p < 4; p++) {
        const size_t o = ((size_t)bl * 4 + p) * nchan + cg;
        float2 s = vsum[o], e = vcomp[o];
        two_sum_add(s.x, e.x, acc[a][b][p].x);
        two_sum_add(s.y, e.y, acc[a][b][p].y);
        vsum[o] = s;
        vcomp[o] = e;
      }
    }
}

// Tile-pair table J <= K over ceil(nant/2) antenna tiles, J-major, in device memory.
cudaError_t make_tile_pairs(int nant, int2 **out) {
  const int nat = (nant + 1) / 2;
  const int npairs = nat * (nat + 1) / 2;
  std::vector<int2> h((size_t)npairs);
  int q = 0;
  for (int J = 0; J < nat; J++)
    for (int K = J; K < nat; K++) h[(size_t)q++] = make_int2(J, K);
  cudaError_t e = cudaMalloc((void **)out, sizeof(int2) * (size_t)npairs);
  if (e == cudaSuccess) e = cudaMemcpy(*out, h.data(), sizeof(int2) * (size_t)npairs, cudaMemcpyHostToDevice);
  return e;
}

cudaError_t launch_xstage_cuda_core(const void *chan, int chan_type, int nant, int nchan, int T, int nt, int autos,
                                    const int2 *pairs, float2 *vsum, float2 *vcomp, cudaStream_t s) {
  return launch_xstage_cuda_core_pairs(chan, chan_type, nant, nchan, T, nt, autos, pairs, vsum, vcomp, s);
}

// Same launch with a caller-provided tile-pair table (J <= K over ceil(nant/2)
// antenna tiles, J-major), for callers that keep the table in their own memory.
cudaError_t launch_xstage_cuda_core_pairs(const void *chan, int chan_type, int nant, int nchan, int T, int nt,
                                          int autos, const int2 *pairs, float2 *vsum, float2 *vcomp,
                                          cudaStream_t s) {
  if (nt <= 0) return cudaSuccess;
  const int nat = (nant + 1) / 2;
  const int npairs = nat * (nat + 1) / 2;
  const int nstream = 2 * nant;
  const size_t esz = chan_elem_bytes(chan_type);
  const int pairs_per_cta = npairs < 64 ? npairs : 64;
  const int threads = pairs_per_cta * CW;
  int TT = (int)(65536 / ((size_t)nstream * CW * esz));
  if (TT < 1) TT = 1;
  if (TT > 32) TT = 32;
  const size_t smem = (size_t)TT * nstream * CW * esz;
  dim3 grid((unsigned)((npairs + pairs_per_cta - 1) / pairs_per_cta), (unsigned)((nchan + CW - 1) / CW));
  cudaError_t e;
  if (chan_type == CHAN_F32) {
    auto k = xstage_cc_kernel<float2>;
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, threads, smem, s>>>((const float2 *)chan, nant, nchan, T, nt, autos, pairs, npairs, pairs_per_cta, TT,
                                   vsum, vcomp);
  } else if (chan_type == CHAN_F8) {
    auto k = xstage_cc_kernel<__nv_fp8x2_e4m3>;
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, threads, smem, s>>>((const __nv_fp8x2_e4m3 *)chan, nant, nchan, T, nt, autos, pairs, npairs,
                                   pairs_per_cta, TT, vsum, vcomp);
  } else {
    auto k = xstage_cc_kernel<__half2>;
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, threads, smem, s>>>((const __half2 *)chan, nant, nchan, T, nt, autos, pairs, npairs, pairs_per_cta, TT,
                                   vsum, vcomp);
  }
  return cudaGetLastError();
}

}  // namespace gxc
