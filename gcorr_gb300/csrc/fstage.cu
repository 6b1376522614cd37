// F-stage of the FX correlator: per-(antenna, FFT) geometry, validity counts,
// twiddle tables, and the launcher of the fused channelising kernels
// (fstage_kernels.cuh: unpack -> fringe rotation -> FFT -> fractional-sample-delay
// correction -> cast -> write in the X-stage layout).
//
// Reference path restated: fxkernel/src/fxkernel.cpp:276-325 (station loop of
// process()), :425-440 getStationDelay, :443-487 unpack, :498-567 fringerotate,
// :569-580 dofft, :595-634 fracSampleCorrect.
#include <cooperative_groups.h>
#include <math.h>
#include <stdlib.h>
#include <type_traits>
#include <vector>

#include "fstage_kernels.cuh"
#include "gxc_internal.h"

namespace gxc {

// ----------------------------------------------------------------- geometry
// One thread per (antenna, FFT).  FP64 with explicit round-to-nearest
// operations so the integer/fractional split matches the CPU reference bit
// for bit (no FMA contraction): fxkernel.cpp:432-439 and :289-309.
__global__ void geometry_kernel(Job job) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long total = (long long)job.nant * job.nfft;
  if (idx >= total) return;
  const int ant = (int)(idx / job.nfft);
  const int i = (int)(idx % job.nfft);
  const double *p = job.poly + 3 * ant;
  const double fso = job.fso[ant];
  const double fi = (double)i, fh = fi + 0.5, f1 = fi + 1.0;
  const double d0 = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(p[0], fi), fi), __dmul_rn(p[1], fi)), p[2]);
  const double d1 = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(p[0], fh), fh), __dmul_rn(p[1], fh)), p[2]);
  const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(p[0], f1), f1), __dmul_rn(p[1], f1)), p[2]);
  const double a = __dsub_rn(d2, d0);
  const double b = __dadd_rn(d0, __ddiv_rn(__dsub_rn(d1, __dadd_rn(__dmul_rn(a, 0.5), d0)), 3.0));
  const double mean = __dadd_rn(__dmul_rn(a, 0.5), b);
  const double ndf = __ddiv_rn(__dsub_rn(mean, fso), job.Ts);
  Geom g;
  g.c0 = g.c1 = g.cstep = g.cf = 0.0f;
  g.offset = 0;
  g.valid = 0;
  g.pad[0] = g.pad[1] = 0;
  if (fabs(ndf) < 1.0e9) {  // false for NaN/Inf: flagged instead of undefined int()
    const int nd = __double2int_rz(__dadd_rn(ndf, 0.5));
    double frac = -__dmul_rn(__dsub_rn(ndf, (double)nd), job.Ts);
    long long off = (long long)i * job.F - nd;
    if (off == -1) { off++; frac = __dadd_rn(frac, job.Ts); }
    if (off == job.maxoffset + 1) { off--; frac = __dsub_rn(frac, job.Ts); }
    // Phase constants (fxkernel.cpp:503-535): phase(n) = LO*(b + a*n/F) turns, the
    // integer-sample part of b removed and the rest reduced mod 1 turn in FP64.
    const int intdelay = __double2int_rz(b);
    const double br = b - (double)intdelay;
    double c0 = br * job.lo_hz;
    if (job.fractional_lo) c0 += (job.lo_hz - trunc(job.lo_hz)) * (double)intdelay;
    c0 -= floor(c0);
    const double c1 = a * job.lo_hz / (double)job.F;  // turns per sample
    // coarse step: the reference advances its step table by `stride` samples per
    // entry (fxkernel.cpp:112) while applying it every `substride` samples;
    // FXKERNEL mode keeps that, EXACT uses the true step.
    const double stepmul = (job.rotator == GXC_ROTATOR_FXKERNEL) ? (double)job.stride : (double)job.substride;
    g.c0 = (float)c0;
    g.c1 = (float)c1;
    g.cstep = (float)(c1 * stepmul);
    // fractional-sample correction exp(+2 pi i c bw/nchan frac) (fxkernel.cpp:171-175,600-630)
    g.cf = (float)(job.bw_hz / (double)job.nchan * frac);
    if (off >= 0 && off <= job.maxoffset) {
      g.offset = (int)off;
      g.valid = 1;
      const uint8_t *fv = job.fvalid ? job.fvalid[ant] : nullptr;
      if (fv) {
        const long long f1 = (off + job.F - 1) / job.samples_per_frame;
        for (long long f = off / job.samples_per_frame; f <= f1; f++)
          if (!fv[f]) g.valid = 0;
      }
    }
  }
  job.geom[idx] = g;
}

cudaError_t launch_geometry(const Job &job, cudaStream_t s) {
  const long long total = (long long)job.nant * job.nfft;
  const int threads = 256;
  const long long blocks = (total + threads - 1) / threads;
  geometry_kernel<<<(unsigned)blocks, threads, 0, s>>>(job);
  return cudaGetLastError();
}

// ------------------------------------------------------------------- counts
// counts[bl] = number of FFTs where both antennas are valid (fxkernel.cpp:352),
// plus the antValid flags exported as uint8 [nant][nfft].
__global__ void counts_kernel(const Geom *__restrict__ geom, int nant, int nfft, int autos, int32_t *counts,
                              uint8_t *valid_flags) {
  const int bl = blockIdx.x;
  const int ncross = nant * (nant - 1) / 2;
  int j, k;
  if (bl >= ncross) {
    j = k = bl - ncross;
  } else {  // invert the fxkernel baseline order
    j = 0;
    int rem = bl;
    while (rem >= nant - 1 - j) { rem -= nant - 1 - j; j++; }
    k = j + 1 + rem;
  }
  int c = 0;
  for (int t = threadIdx.x; t < nfft; t += blockDim.x) {
    const int vj = geom[(size_t)j * nfft + t].valid;
    const int vk = geom[(size_t)k * nfft + t].valid;
    c += (vj && vk) ? 1 : 0;
    if (valid_flags && bl == 0) {
      // block 0 also exports every antenna's flags
      for (int a = 0; a < nant; a++) valid_flags[(size_t)a * nfft + t] = (uint8_t)geom[(size_t)a * nfft + t].valid;
    }
  }
  __shared__ int red[32];
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x < 32) {
    int v = (threadIdx.x < (int)(blockDim.x >> 5)) ? red[threadIdx.x] : 0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) counts[bl] = v;
  }
}

cudaError_t launch_counts(const Job &job, int autos, int32_t *counts, uint8_t *valid_flags, cudaStream_t s) {
  const int nbl = job.nant * (job.nant - 1) / 2 + (autos ? job.nant : 0);
  if (nbl == 0) return cudaSuccess;
  counts_kernel<<<nbl, 256, 0, s>>>(job.geom, job.nant, job.nfft, autos, counts, valid_flags);
  return cudaGetLastError();
}

// ----------------------------------------------------------------- twiddles
// tw[m] = exp(-2 pi i m / F), m < F, rounded once from double.  For F = 8192 the same
// allocation continues with the pass twiddles W_M^e (M = F/2) of the packed-pair kernel,
// laid out so that a warp reads consecutive entries:
//   pass 1, [r][k]  (256 entries):  e = 16 r k, k < 16
//   pass 2, [r][iv] (4096 entries): e = r iv,   iv < 256
cudaError_t make_twiddles(int F, float2 **out) {
  const size_t extra = F == 8192 ? (size_t)kPairTw1 + kPairTw2 : 0;
  std::vector<float2> h((size_t)F + extra);
  for (int m = 0; m < F; m++) {
    const double ang = -2.0 * 3.14159265358979323846 * (double)m / (double)F;
    h[(size_t)m] = make_float2((float)cos(ang), (float)sin(ang));
  }
  if (extra) {
    auto wm = [&](int e) { return h[(size_t)((2 * (long long)e) % F)]; };  // W_M^e = W_F^(2e)
    for (int r = 0; r < 16; r++)
      for (int k = 0; k < 16; k++) h[(size_t)F + (size_t)r * 16 + k] = wm(16 * r * k);
    for (int r = 0; r < 16; r++)
      for (int iv = 0; iv < 256; iv++) h[(size_t)F + kPairTw1 + (size_t)r * 256 + iv] = wm(r * iv);
  }
  cudaError_t e = cudaMalloc((void **)out, sizeof(float2) * h.size());
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*out, h.data(), sizeof(float2) * h.size(), cudaMemcpyHostToDevice);
}

int fstage_supported(int F) { return F >= 256 && F <= 32768 && (F & (F - 1)) == 0; }

cudaError_t launch_fstage(const Job &job, const float2 *twiddles, int t0, int nt, int T, void *chan, int chan_type,
                          float out_scale, cudaStream_t s, const float *cscale) {
  if (nt <= 0) return cudaSuccess;
  const FParams prm = fstage_params(job, twiddles, t0, T, chan, out_scale, nullptr, cscale);
  if (chan_type == CHAN_F32) {
    return job.is_complex ? launch_fstage_l<float2, true>(prm, nt, s) : launch_fstage_l<float2, false>(prm, nt, s);
  }
  if (chan_type == CHAN_F8) {
    return job.is_complex ? launch_fstage_l<__nv_fp8x2_e4m3, true>(prm, nt, s)
                          : launch_fstage_l<__nv_fp8x2_e4m3, false>(prm, nt, s);
  }
  return job.is_complex ? launch_fstage_l<__half2, true>(prm, nt, s) : launch_fstage_l<__half2, false>(prm, nt, s);
}

}  // namespace gxc
