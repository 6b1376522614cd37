// Channelising kernels of the F-stage (unpack -> fringe rotation -> FFT ->
// fractional-sample-delay correction -> cast -> write in the X-stage layout) and
// their templated launchers, shared by the production launcher (fstage.cu) and
// the decode probe (fstage_probe.cu).
//
// Every kernel template takes DBG (default false).  DBG kernels also write each
// decoded input sample, before the fringe rotation, to FParams::probe
// ([antenna][pol][FFT][sample] complex float); the production launcher never
// instantiates them.
//
// Reference path restated: fxkernel/src/fxkernel.cpp:443-487 unpack, :498-567
// fringerotate, :569-580 dofft, :595-634 fracSampleCorrect.
#pragma once

#include <cooperative_groups.h>
#include <math.h>
#include <type_traits>

#include "gxc_internal.h"

namespace gxc {

// ------------------------------------------------------------ FFT helpers
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// Complex add and subtract as one packed FP32-pair instruction each (add/sub.rn.f32x2,
// sm_100 and later): IEEE round-to-nearest per component, as the scalar adds, in half
// the issue slots.
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  float2 r;
  asm("{.reg .b64 pa, pb, pd;\n\t"
      "mov.b64 pa, {%2, %3};\n\t"
      "mov.b64 pb, {%4, %5};\n\t"
      "add.rn.f32x2 pd, pa, pb;\n\t"
      "mov.b64 {%0, %1}, pd;}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
  float2 r;
  asm("{.reg .b64 pa, pb, pd;\n\t"
      "mov.b64 pa, {%2, %3};\n\t"
      "mov.b64 pb, {%4, %5};\n\t"
      "sub.rn.f32x2 pd, pa, pb;\n\t"
      "mov.b64 {%0, %1}, pd;}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
// -i * a
__device__ __forceinline__ float2 cmul_mi(float2 a) { return make_float2(a.y, -a.x); }

// Forward DFTs (W = exp(-2 pi i / R)) on registers, natural order in and out.
__device__ __forceinline__ void dft2(float2 &a, float2 &b) {
  const float2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}
__device__ __forceinline__ void dft4(float2 &x0, float2 &x1, float2 &x2, float2 &x3) {
  const float2 s02 = cadd(x0, x2), d02 = csub(x0, x2);
  const float2 s13 = cadd(x1, x3), d13 = cmul_mi(csub(x1, x3));
  x0 = cadd(s02, s13);
  x2 = csub(s02, s13);
  x1 = cadd(d02, d13);
  x3 = csub(d02, d13);
}
template <int R> __device__ __forceinline__ void dft(float2 *u);
template <> __device__ __forceinline__ void dft<2>(float2 *u) { dft2(u[0], u[1]); }
template <> __device__ __forceinline__ void dft<4>(float2 *u) { dft4(u[0], u[1], u[2], u[3]); }
// 8 = 4 (n1) x 2 (n2): n = 2 n1 + n2, k = k1 + 4 k2.
template <> __device__ __forceinline__ void dft<8>(float2 *u) {
  const float r = 0.70710678118654752440f;
  dft4(u[0], u[2], u[4], u[6]);
  dft4(u[1], u[3], u[5], u[7]);
  // twiddle W8^(k1) on the n2 = 1 branch
  u[3] = cmul(u[3], make_float2(r, -r));
  u[5] = cmul_mi(u[5]);
  u[7] = cmul(u[7], make_float2(-r, -r));
  float2 y[8];
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++) {
    float2 a = u[2 * k1], b = u[2 * k1 + 1];
    dft2(a, b);
    y[k1] = a;
    y[k1 + 4] = b;
  }
#pragma unroll
  for (int q = 0; q < 8; q++) u[q] = y[q];
}
// 16 = 4 (n1) x 4 (n2): n = 4 n1 + n2, k = k1 + 4 k2.
template <> __device__ __forceinline__ void dft<16>(float2 *u) {
  const float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f, r = 0.70710678118654752440f;
#pragma unroll
  for (int n2 = 0; n2 < 4; n2++) dft4(u[n2], u[n2 + 4], u[n2 + 8], u[n2 + 12]);
  // after this, u[n2 + 4 k1] holds Y[n2][k1]; twiddle by W16^(n2 k1)
  u[5] = cmul(u[5], make_float2(c1, -s1));    // n2=1,k1=1: W^1
  u[9] = cmul(u[9], make_float2(r, -r));      // n2=1,k1=2: W^2
  u[13] = cmul(u[13], make_float2(s1, -c1));  // n2=1,k1=3: W^3
  u[6] = cmul(u[6], make_float2(r, -r));      // n2=2,k1=1: W^2
  u[10] = cmul_mi(u[10]);                     // n2=2,k1=2: W^4
  u[14] = cmul(u[14], make_float2(-r, -r));   // n2=2,k1=3: W^6
  u[7] = cmul(u[7], make_float2(s1, -c1));    // n2=3,k1=1: W^3
  u[11] = cmul(u[11], make_float2(-r, -r));   // n2=3,k1=2: W^6
  u[15] = cmul(u[15], make_float2(-c1, s1));  // n2=3,k1=3: W^9
  float2 y[16];
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++) {
    float2 a = u[4 * k1], b = u[4 * k1 + 1], c = u[4 * k1 + 2], d = u[4 * k1 + 3];
    dft4(a, b, c, d);  // over n2
    y[k1] = a;
    y[k1 + 4] = b;
    y[k1 + 8] = c;
    y[k1 + 12] = d;
  }
#pragma unroll
  for (int q = 0; q < 16; q++) u[q] = y[q];
}

__device__ __forceinline__ float level2bit(int code) {
  // fxkernel.cpp:17-18: {-HiMag, -1, 1, HiMag}, HiMag = 3.3359
  const float mag = (code == 0 || code == 3) ? 3.3359f : 1.0f;
  return (code & 2) ? mag : -mag;
}

template <typename OutT> __device__ __forceinline__ OutT to_out(float2 v, float scale);
template <> __device__ __forceinline__ float2 to_out<float2>(float2 v, float scale) {
  return make_float2(v.x * scale, v.y * scale);
}
template <> __device__ __forceinline__ __half2 to_out<__half2>(float2 v, float scale) {
  return __floats2half2_rn(v.x * scale, v.y * scale);
}
// E4M3 pair, round to nearest, saturating at +-448 (re in the low byte)
template <> __device__ __forceinline__ __nv_fp8x2_e4m3 to_out<__nv_fp8x2_e4m3>(float2 v, float scale) {
  return __nv_fp8x2_e4m3(make_float2(v.x * scale, v.y * scale));
}

struct FParams {
  Job job;
  const float2 *tw;    // W_F^m, m < F
  const float2 *twp1;  // F = 8192: pass-1 twiddles of the packed-pair kernel (make_twiddles), else null
  const float2 *twp2;  // F = 8192: pass-2 twiddles of the packed-pair kernel, else null
  int t0, T;
  void *chan;
  float out_scale;
  int sub_shift, sub_mask;    // substride = 1 << sub_shift
  int fsub_shift, fsub_mask;  // fsub = 1 << fsub_shift
  float2 *probe;              // DBG kernels: decoded samples [nant][2][nfft][F] before rotation
  const float *cscale;        // FP8 output: per-channel scale [nchan] (replaces out_scale), or null
};

// Output scale of channel c: FP8 output with per-channel scales uses cscale[c] (the caller then
// passes base = 1, or the kernel's own exact internal factor), every other case base.
template <typename OutT>
__device__ __forceinline__ float chan_scale(const float *cscale, int c, float base) {
  if constexpr (std::is_same<OutT, __nv_fp8x2_e4m3>::value) {
    if (cscale) return base * __ldg(&cscale[c]);
  }
  return base;
}

// float2 entries that follow the F-point twiddle table when F = 8192 (make_twiddles).
constexpr int kPairTw1 = 16 * 16, kPairTw2 = 16 * 256;

inline int fparams_ilog2(int x) {
  int l = 0;
  while ((1 << (l + 1)) <= x) l++;
  return l;
}

// Launch parameters of FFTs [t0, t0 + nt) of a block of T (twiddles from make_twiddles).
inline FParams fstage_params(const Job &job, const float2 *twiddles, int t0, int T, void *chan, float out_scale,
                             float2 *probe, const float *cscale = nullptr) {
  FParams prm;
  prm.job = job;
  prm.tw = twiddles;
  prm.twp1 = job.F == 8192 ? twiddles + job.F : nullptr;
  prm.twp2 = job.F == 8192 ? twiddles + job.F + kPairTw1 : nullptr;
  prm.t0 = t0;
  prm.T = T;
  prm.chan = chan;
  prm.out_scale = out_scale;
  prm.sub_shift = fparams_ilog2(job.substride);
  prm.sub_mask = job.substride - 1;
  prm.fsub_shift = fparams_ilog2(job.fsub);
  prm.fsub_mask = job.fsub - 1;
  prm.probe = probe;
  prm.cscale = cscale;
  return prm;
}

// DBG kernels: the decoded sample n of (ant, pol, FFT t), before the fringe rotation.
__device__ __forceinline__ void probe_store(const FParams &prm, int ant, int pol, int t, int n, float2 v) {
  const Job &job = prm.job;
  prm.probe[(((size_t)ant * 2 + pol) * job.nfft + t) * job.F + n] = v;
}

// W32^k = exp(-2 pi i k / 32), k < 16
__device__ constexpr float kC32[16] = {1.0f, 0.98078528040323044913f, 0.92387953251128675613f,
                                       0.83146961230254523708f, 0.70710678118654752440f, 0.55557023301960222474f,
                                       0.38268343236508977173f, 0.19509032201612826785f, 0.0f,
                                       -0.19509032201612826785f, -0.38268343236508977173f, -0.55557023301960222474f,
                                       -0.70710678118654752440f, -0.83146961230254523708f, -0.92387953251128675613f,
                                       -0.98078528040323044913f};
__device__ constexpr float kS32[16] = {0.0f, 0.19509032201612826785f, 0.38268343236508977173f,
                                       0.55557023301960222474f, 0.70710678118654752440f, 0.83146961230254523708f,
                                       0.92387953251128675613f, 0.98078528040323044913f, 1.0f,
                                       0.98078528040323044913f, 0.92387953251128675613f, 0.83146961230254523708f,
                                       0.70710678118654752440f, 0.55557023301960222474f, 0.38268343236508977173f,
                                       0.19509032201612826785f};
// 32 = 16 (n1) x 2 (n2): n = 2 n1 + n2, k = k1 + 16 k2.
template <> __device__ __forceinline__ void dft<32>(float2 *u) {
  float2 a[16], b[16];
#pragma unroll
  for (int i = 0; i < 16; i++) {
    a[i] = u[2 * i];
    b[i] = u[2 * i + 1];
  }
  dft<16>(a);
  dft<16>(b);
#pragma unroll
  for (int k = 1; k < 16; k++) b[k] = cmul(b[k], make_float2(kC32[k], -kS32[k]));
#pragma unroll
  for (int k = 0; k < 16; k++) {
    u[k] = cadd(a[k], b[k]);
    u[k + 16] = csub(a[k], b[k]);
  }
}

constexpr int hibit(int r) { return r >= 16 ? 16 : r >= 8 ? 8 : r >= 4 ? 4 : r >= 2 ? 2 : 1; }
constexpr int log2c(int x) { return x <= 1 ? 0 : 1 + log2c(x / 2); }

// Radix schedule and compile-time table splits for FFT length 2^L.
// A CTA transforms one pol of one FFT window; each of its F/32 threads holds
// 32 complex values per pass (2 or 3 passes, radices <= 32); two CTAs share an SM.
template <int L, bool CPLX>
struct FPlan {
  static constexpr int N = 1 << L;
  static constexpr int NTW = N / 32;                  // threads with FFT work
  static constexpr int NT = NTW < 32 ? 32 : NTW;      // threads launched
  static constexpr int R0 = L == 8 ? 16 : L == 9 ? 32 : L == 10 ? 32 : L == 11 ? 8 : L == 12 ? 16 : L == 13 ? 32 : 16;
  static constexpr int R1 = L == 8 ? 16 : L == 9 ? 16 : L == 10 ? 32 : L == 14 ? 32 : 16;
  static constexpr int R2 = L <= 10 ? 1 : (L == 14 ? 32 : 16);
  static constexpr int RL = R2 > 1 ? R2 : R1;         // radix of the last pass
  static constexpr int PAD = R0;                      // one smem slot of padding per R0 (conflict-free strided stores)
  static constexpr int PADN = N + N / R0;
  static constexpr int MINB = (L >= 14) ? 1 : 2;      // CTAs per SM (F = 16384 fills the shared memory)
  // table splits, fxkernel.cpp:57-64 (stride = sqrt(nchan) for square nchan; 2^floor(log2(nchan)/2) otherwise)
  static constexpr int NCHAN = CPLX ? N : N / 2;
  static constexpr int STRIDE = 1 << (log2c(NCHAN) / 2);
  static constexpr int SUB = N / STRIDE;              // fringe sub-table (substride)
  static constexpr int FSUB = NCHAN / STRIDE;         // frac-delay sub-table
  static_assert(R0 * R1 * R2 == N, "radix schedule");
};

// u[q*R + r] *= W_N^{r*k*S}, S = N/(P*R): exact table loads at powers of two,
// the rest as products of at most four of them.
template <int N, int R, int P>
__device__ __forceinline__ void twiddle(float2 *u, int k, const float2 *__restrict__ tw) {
  constexpr int S = N / (P * R);
  float2 w[R < 16 ? R : 16];
#pragma unroll
  for (int r = 1; r < R && r < 16; r++) {
    if ((r & (r - 1)) == 0) w[r] = __ldg(&tw[r * k * S]);
    else w[r] = cmul(w[hibit(r)], w[r - hibit(r)]);
    u[r] = cmul(u[r], w[r]);
  }
  if constexpr (R == 32) {
    const float2 w16 = __ldg(&tw[16 * k * S]);
    u[16] = cmul(u[16], w16);
#pragma unroll
    for (int r = 17; r < 32; r++) u[r] = cmul(u[r], cmul(w16, w[r - 16]));
  }
}

// 16-byte asynchronous global -> shared copy (LDGSTS, bypassing L1); completion
// is awaited with cp.async.wait_all before the barrier that publishes the data.
__device__ __forceinline__ void cp_async16(void *dst_smem, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst_smem)),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

template <int L, typename OutT, bool CPLX, bool DBG = false>
__global__ void __launch_bounds__(FPlan<L, CPLX>::NT, FPlan<L, CPLX>::MINB) fstage_kernel(FParams prm) {
  using Pl = FPlan<L, CPLX>;
  constexpr int N = Pl::N, NT = Pl::NT, NTW = Pl::NTW;
  constexpr int R0 = Pl::R0, R1 = Pl::R1, R2 = Pl::R2, RL = Pl::RL, PAD = Pl::PAD;
  constexpr int SUB = Pl::SUB, STRIDE = Pl::STRIDE, FSUB = Pl::FSUB, NCHAN = Pl::NCHAN;
  const Job &job = prm.job;
  extern __shared__ float2 smem[];
  float2 *buf = smem;                     // N + N/R0 (padded)
  float2 *tsub = buf + Pl::PADN;          // fringe rotator, fine part  [SUB]
  float2 *tstep = tsub + SUB;             // fringe rotator, coarse part [STRIDE]
  float2 *fsubt = tstep + STRIDE;         // frac-delay, fine part [FSUB]
  float2 *fstept = fsubt + FSUB;          // frac-delay, coarse part [STRIDE]
  unsigned char *stage = reinterpret_cast<unsigned char *>(fstept + STRIDE);  // packed input window

  // grid x = pol + 2 * FFT: the two pols of one window run side by side (the second
  // read of the packed window hits L2) and write neighbouring streams
  const int pol = blockIdx.x & 1;  // the pol this CTA transforms
  const int tl = blockIdx.x >> 1;
  const int ant = blockIdx.y;
  const int t = prm.t0 + tl;
  const int tid = threadIdx.x;
  const int nstreams = 2 * job.nant;
  const int s = 2 * ant + pol;
  OutT *chan = reinterpret_cast<OutT *>(prm.chan);
  // every thread reads the 32-byte record (one broadcast load): no barrier needed
  const Geom g = job.geom[(size_t)ant * job.nfft + t];

  // channelised layout [ctile][t][stream][16]: element (c, s) of this FFT
  OutT *out0 = chan + ((size_t)tl * nstreams + s) * CW;
  const size_t ctile_stride = (size_t)prm.T * nstreams * CW;

  if (!g.valid) {
    // flagged: the X-stage sums zeros, the baseline counts exclude this FFT
    const OutT z = to_out<OutT>(make_float2(0.f, 0.f), 1.f);
    for (int c = tid; c < NCHAN; c += NT) out0[(size_t)(c >> 4) * ctile_stride + (c & 15)] = z;
    return;
  }

  const long long stage_base = (CPLX ? 4LL * g.offset : ((long long)g.offset >> 1)) & ~15LL;
  {
    // stage the packed window with 16-byte loads (bounds: the buffer holds
    // (nfft+1)*F samples and offset <= (nfft-1)*F, so the window plus the
    // 16-byte rounding stays inside it)
    const uint4 *src = reinterpret_cast<const uint4 *>(job.inputs[ant] + stage_base);
    const long long last = CPLX ? 4LL * (g.offset + N) : (((long long)g.offset + N + 1) >> 1);
    const int nvec = (int)((last - stage_base + 15) >> 4);
    uint4 *dst = reinterpret_cast<uint4 *>(stage);
    for (int i = tid; i < nvec; i += NT) dst[i] = __ldg(&src[i]);
    const float c0 = g.c0, c1 = g.c1, cstep = g.cstep, cf = g.cf;
    for (int k = tid; k < SUB; k += NT) {
      float sn, cs;
      sincospif(-2.0f * fmaf((float)k, c1, c0), &sn, &cs);
      tsub[k] = make_float2(cs, sn);
    }
    for (int i = tid; i < STRIDE; i += NT) {
      float sn, cs;
      sincospif(-2.0f * ((float)i * cstep), &sn, &cs);
      tstep[i] = make_float2(cs, sn);
      sincospif(2.0f * ((float)(i * FSUB) * cf), &sn, &cs);
      fstept[i] = make_float2(cs, sn);
    }
    for (int k = tid; k < FSUB; k += NT) {
      float sn, cs;
      sincospif(2.0f * ((float)k * cf), &sn, &cs);
      fsubt[k] = make_float2(cs, sn);
    }
  }
  __syncthreads();

  const bool active = tid < NTW;
  const int off = g.offset;
  float2 u[32];
  // ---- pass 0 (span 1): decode + fringe-rotate from the staged window
  if (active) {
    constexpr int NB = N / R0;
    const int sbase = (int)(CPLX ? (4LL * off - stage_base) : (((long long)off >> 1) - stage_base));
#pragma unroll
    for (int q = 0; q < 32 / R0; q++) {
      const int iv = tid + q * NTW;
      float2 *v = &u[q * R0];
      // this thread's samples n = iv + r*NB: fine rotator index fixed, coarse index strided
      const float2 rs = tsub[iv & (SUB - 1)];
      const int p0 = (off & 1) + iv;  // 2-bit: sample index relative to byte off/2
      const int shift = 2 * (2 * (p0 & 1) + pol);
#pragma unroll
      for (int r = 0; r < R0; r++) {
        const int n = iv + r * NB;
        float2 rot;
        if constexpr (NB % SUB == 0) rot = cmul(rs, tstep[(iv / SUB) + r * (NB / SUB)]);
        else rot = cmul(tsub[n & (SUB - 1)], tstep[n / SUB]);
        if constexpr (CPLX) {
          // int8 (A.re, A.im, B.re, B.im) per time sample
          const char2 x = *reinterpret_cast<const char2 *>(stage + sbase + 4 * iv + 2 * pol + r * (4 * NB));
          if constexpr (DBG) probe_store(prm, ant, pol, t, n, make_float2((float)x.x, (float)x.y));
          v[r] = cmul(make_float2((float)x.x, (float)x.y), rot);
        } else {
          // 2-bit: byte m/2 holds A_m', B_m', A_m'+1, B_m'+1 (fxkernel.cpp:443-476)
          const int byte = stage[sbase + (p0 >> 1) + r * (NB / 2)];
          const float lv = level2bit((byte >> shift) & 3);
          if constexpr (DBG) probe_store(prm, ant, pol, t, n, make_float2(lv, 0.0f));
          v[r] = make_float2(lv * rot.x, lv * rot.y);
        }
      }
      dft<R0>(v);
    }
  }
  // store pass 0: element j + r with j = iv*R0, padded index iv*(R0+1) + r (buf is
  // not read before the next barrier)
  if (active) {
#pragma unroll
    for (int q = 0; q < 32 / R0; q++) {
      const int iv = tid + q * NTW;
      float2 *b = buf + iv * (R0 + 1);
#pragma unroll
      for (int r = 0; r < R0; r++) b[r] = u[q * R0 + r];
    }
  }
  __syncthreads();
  // ---- middle pass (3-pass schedules): radix R1, span R0
  if constexpr (R2 > 1) {
    constexpr int NB = N / R1;
    static_assert(NB % PAD == 0, "padding");
    if (active) {
#pragma unroll
      for (int q = 0; q < 32 / R1; q++) {
        const int iv = tid + q * NTW;
        const float2 *b = buf + iv + iv / PAD;
#pragma unroll
        for (int r = 0; r < R1; r++) u[q * R1 + r] = b[r * (NB + NB / PAD)];
        twiddle<N, R1, R0>(&u[q * R1], iv & (R0 - 1), prm.tw);
        dft<R1>(&u[q * R1]);
      }
    }
    __syncthreads();
    if (active) {
#pragma unroll
      for (int q = 0; q < 32 / R1; q++) {
        const int iv = tid + q * NTW;
        const int k = iv & (R0 - 1);
        const int j = (iv - k) * R1 + k;
        float2 *b = buf + j + j / PAD;
#pragma unroll
        for (int r = 0; r < R1; r++) b[r * (R0 + R0 / PAD)] = u[q * R1 + r];
      }
    }
    __syncthreads();
  }
  // ---- last pass: radix RL, span PL = N/RL (32/RL butterflies per thread);
  //      outputs c = iv + r*NB go straight to global
  if (active) {
    constexpr int PL = N / RL, NB = N / RL;
    static_assert(NB % PAD == 0 && NB % 16 == 0, "padding / channel tiles");
    constexpr int RKEEP = CPLX ? RL : RL / 2;  // real data keeps channels c < N/2
#pragma unroll
    for (int q = 0; q < 32 / RL; q++) {
      const int iv = tid + q * NTW;
      float2 *v = &u[q * RL];
      const float2 *b = buf + iv + iv / PAD;
#pragma unroll
      for (int r = 0; r < RL; r++) v[r] = b[r * (NB + NB / PAD)];
      twiddle<N, RL, PL>(v, iv, prm.tw);
      dft<RL>(v);
      const float2 fs = fsubt[iv & (FSUB - 1)];
      OutT *o = out0 + (size_t)(iv >> 4) * ctile_stride + (iv & 15);
#pragma unroll
      for (int r = 0; r < RKEEP; r++) {
        const int c = iv + r * NB;
        float2 fr;
        if constexpr (NB % FSUB == 0) fr = cmul(fs, fstept[(iv / FSUB) + r * (NB / FSUB)]);
        else fr = cmul(fsubt[c & (FSUB - 1)], fstept[c / FSUB]);
        o[(size_t)r * (NB / 16) * ctile_stride] = to_out<OutT>(cmul(v[r], fr), chan_scale<OutT>(prm.cscale, c, prm.out_scale));
      }
    }
  }
}

// -------------------------------------- 8192-point windows in packed FP32 pairs
// One radix-2 decimation-in-frequency step splits the N-point FFT into two
// M = N/2-point FFTs with the same structure and the same twiddles:
//   A[k] = X[2k]   = DFT_M( x[n] + x[n+M] )
//   B[k] = X[2k+1] = DFT_M( (x[n] - x[n+M]) W_N^n ),   n < M.
// A and B travel as the two lanes of packed FP32-pair registers, re = (A.re, B.re)
// and im = (A.im, B.im), so every add, subtract and twiddle multiply of both
// sub-FFTs is one packed instruction (add/sub/mul/fma.rn.f32x2: IEEE round to
// nearest per lane, half the issue slots of scalar code).  The sub-FFTs use the
// radix 16 x 16 x 16 Stockham schedule of the 4096-point kernel; bins 2k and
// 2k+1 are neighbouring channels and leave in one vector store.

struct P2 {
  float2 re, im;  // (A, B) lanes
};

__device__ __forceinline__ float2 pmul(float2 a, float2 b) {
  float2 r;
  asm("{.reg .b64 pa, pb, pd;\n\t"
      "mov.b64 pa, {%2, %3};\n\t"
      "mov.b64 pb, {%4, %5};\n\t"
      "mul.rn.f32x2 pd, pa, pb;\n\t"
      "mov.b64 {%0, %1}, pd;}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
// a * b + c per lane, one rounding
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) {
  float2 r;
  asm("{.reg .b64 pa, pb, pc, pd;\n\t"
      "mov.b64 pa, {%2, %3};\n\t"
      "mov.b64 pb, {%4, %5};\n\t"
      "mov.b64 pc, {%6, %7};\n\t"
      "fma.rn.f32x2 pd, pa, pb, pc;\n\t"
      "mov.b64 {%0, %1}, pd;}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return r;
}
// sign flip on the integer pipe (the FMA pipe is the kernel's busiest)
__device__ __forceinline__ float negi(float x) { return __int_as_float(__float_as_int(x) ^ (int)0x80000000); }
// both lanes times w = (wr, wi): four packed FMA-pipe instructions, as many pipe cycles as
// two scalar complex products
__device__ __forceinline__ void pcmul(P2 &u, float wr, float wi) {
  const float nwi = negi(wi);
  const float2 WR = make_float2(wr, wr), WI = make_float2(wi, wi), NWI = make_float2(nwi, nwi);
  const float2 re = pfma(u.re, WR, pmul(u.im, NWI));
  u.im = pfma(u.re, WI, pmul(u.im, WR));
  u.re = re;
}
// both lanes times the constant (cr, ci)
__device__ __forceinline__ void pcmul_c(P2 &u, float cr, float ci) {
  const float2 CR = make_float2(cr, cr), CI = make_float2(ci, ci), NCI = make_float2(-ci, -ci);
  const float2 re = pfma(u.re, CR, pmul(u.im, NCI));
  u.im = pfma(u.re, CI, pmul(u.im, CR));
  u.re = re;
}

// 4-point DFT of both lanes.  X2MI: the x2 operand holds z with x2 = -i z (the W16^4
// twiddle folded in).  KEEP2: only X0 and X1 are needed.
template <bool X2MI, bool KEEP2>
__device__ __forceinline__ void dft4p(P2 &x0, P2 &x1, P2 &x2, P2 &x3) {
  float2 s02r, s02i, d02r, d02i;
  if constexpr (X2MI) {  // x2 = (z.im, -z.re)
    s02r = cadd(x0.re, x2.im);
    s02i = csub(x0.im, x2.re);
    d02r = csub(x0.re, x2.im);
    d02i = cadd(x0.im, x2.re);
  } else {
    s02r = cadd(x0.re, x2.re);
    s02i = cadd(x0.im, x2.im);
    d02r = csub(x0.re, x2.re);
    d02i = csub(x0.im, x2.im);
  }
  const float2 s13r = cadd(x1.re, x3.re), s13i = cadd(x1.im, x3.im);
  const float2 tr = csub(x1.re, x3.re), ti = csub(x1.im, x3.im);
  x0.re = cadd(s02r, s13r);
  x0.im = cadd(s02i, s13i);
  // X1 = d02 - i t, X3 = d02 + i t
  x1.re = cadd(d02r, ti);
  x1.im = csub(d02i, tr);
  if constexpr (!KEEP2) {
    x2.re = csub(s02r, s13r);
    x2.im = csub(s02i, s13i);
    x3.re = csub(d02r, ti);
    x3.im = cadd(d02i, tr);
  }
}

// 16-point DFT of both lanes, the 4 x 4 factorisation of dft<16>.  KEEP8: only
// outputs k < 8 are needed (real data keeps the lower half of the band).
template <bool KEEP8>
__device__ __forceinline__ void dft16p(P2 *u) {
  const float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f, r = 0.70710678118654752440f;
#pragma unroll
  for (int n2 = 0; n2 < 4; n2++) dft4p<false, false>(u[n2], u[n2 + 4], u[n2 + 8], u[n2 + 12]);
  // u[n2 + 4 k1] = Y[n2][k1]; twiddle by W16^(n2 k1) (W^4 = -i is folded into the k1 = 2 DFT)
  pcmul_c(u[5], c1, -s1);
  pcmul_c(u[9], r, -r);
  pcmul_c(u[13], s1, -c1);
  pcmul_c(u[6], r, -r);
  pcmul_c(u[14], -r, -r);
  pcmul_c(u[7], s1, -c1);
  pcmul_c(u[11], -r, -r);
  pcmul_c(u[15], -c1, s1);
  P2 y[16];
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++) {
    P2 a = u[4 * k1], b = u[4 * k1 + 1], c = u[4 * k1 + 2], d = u[4 * k1 + 3];
    if (k1 == 2) dft4p<true, KEEP8>(a, b, c, d);
    else dft4p<false, KEEP8>(a, b, c, d);
    y[k1] = a;
    y[k1 + 4] = b;
    y[k1 + 8] = c;
    y[k1 + 12] = d;
  }
#pragma unroll
  for (int q = 0; q < 16; q++) u[q] = y[q];
}

// channels c and c+1 (c even) of one stream: one 16-, 8- or 4-byte store
template <typename OutT> __device__ __forceinline__ void store_pair(OutT *p, float2 a, float2 b);
template <> __device__ __forceinline__ void store_pair<float2>(float2 *p, float2 a, float2 b) {
  *reinterpret_cast<float4 *>(p) = make_float4(a.x, a.y, b.x, b.y);
}
template <> __device__ __forceinline__ void store_pair<__half2>(__half2 *p, float2 a, float2 b) {
  const __half2 ha = __floats2half2_rn(a.x, a.y), hb = __floats2half2_rn(b.x, b.y);
  *reinterpret_cast<uint2 *>(p) =
      make_uint2(*reinterpret_cast<const uint32_t *>(&ha), *reinterpret_cast<const uint32_t *>(&hb));
}
template <>
__device__ __forceinline__ void store_pair<__nv_fp8x2_e4m3>(__nv_fp8x2_e4m3 *p, float2 a, float2 b) {
  const __nv_fp8x2_e4m3 ea(a), eb(b);
  *reinterpret_cast<uint32_t *>(p) = (uint32_t)ea.__x | ((uint32_t)eb.__x << 16);
}

template <typename OutT, bool CPLX, bool DBG = false>
__global__ void __launch_bounds__(256, 2) fstage_pair_kernel(FParams prm) {
  using Pl = FPlan<13, CPLX>;  // window, rotator and frac-delay tables of the 8192-point FFT
  constexpr int N = Pl::N, M = N / 2, NT = 256, R = 16, PAD = 16;
  constexpr int NB = M / R;         // 256: butterflies per radix-16 pass (one per thread)
  constexpr int NB0 = N / 32;       // 256: pass 0 takes the samples n = iv + r*NB0, r < 32
  constexpr int PADM = M + M / PAD;
  constexpr int SUB = Pl::SUB, STRIDE = Pl::STRIDE, FSUB = Pl::FSUB, NCHAN = Pl::NCHAN;
  static_assert(NB == NT && NB0 % SUB == 0 && (2 * NB) % FSUB == 0 && NB % PAD == 0, "pair plan");
  const Job &job = prm.job;
  extern __shared__ float4 smem4[];
  float4 *buf = smem4;  // [PADM] pair elements {A.re, B.re, A.im, B.im}
  float2 *tsub = reinterpret_cast<float2 *>(buf + PADM);
  float2 *tstep = tsub + SUB;
  float2 *fsubt = tstep + STRIDE;
  float2 *fstept = fsubt + FSUB;
  unsigned char *stage = reinterpret_cast<unsigned char *>(fstept + STRIDE);

  const int pol = blockIdx.x & 1;
  const int tl = blockIdx.x >> 1;
  const int ant = blockIdx.y;
  const int t = prm.t0 + tl;
  const int iv = threadIdx.x;
  const int nstreams = 2 * job.nant;
  const int s = 2 * ant + pol;
  OutT *chan = reinterpret_cast<OutT *>(prm.chan);
  const Geom g = job.geom[(size_t)ant * job.nfft + t];
  OutT *out0 = chan + ((size_t)tl * nstreams + s) * CW;
  const size_t ctile_stride = (size_t)prm.T * nstreams * CW;

  if (!g.valid) {
    const OutT z = to_out<OutT>(make_float2(0.f, 0.f), 1.f);
    for (int c = iv; c < NCHAN; c += NT) out0[(size_t)(c >> 4) * ctile_stride + (c & 15)] = z;
    return;
  }

  const long long stage_base = (CPLX ? 4LL * g.offset : ((long long)g.offset >> 1)) & ~15LL;
  {
    // the packed window, 16-byte asynchronous copies (the buffer holds (nfft+1)*F samples and
    // offset <= (nfft-1)*F, so the window plus the 16-byte rounding stays inside it); the
    // rotator and frac-delay tables are evaluated while the copies are in flight
    const uint4 *src = reinterpret_cast<const uint4 *>(job.inputs[ant] + stage_base);
    const long long last = CPLX ? 4LL * (g.offset + N) : (((long long)g.offset + N + 1) >> 1);
    const int nvec = (int)((last - stage_base + 15) >> 4);
    uint4 *dst = reinterpret_cast<uint4 *>(stage);
    for (int i = iv; i < nvec; i += NT) cp_async16(dst + i, src + i);
    const float c0 = g.c0, c1 = g.c1, cstep = g.cstep, cf = g.cf;
    for (int k = iv; k < SUB; k += NT) {
      float sn, cs;
      sincospif(-2.0f * fmaf((float)k, c1, c0), &sn, &cs);
      tsub[k] = make_float2(cs, sn);
    }
    for (int i = iv; i < STRIDE; i += NT) {
      float sn, cs;
      sincospif(-2.0f * ((float)i * cstep), &sn, &cs);
      tstep[i] = make_float2(cs, sn);
      sincospif(2.0f * ((float)(i * FSUB) * cf), &sn, &cs);
      fstept[i] = make_float2(cs, sn);
    }
    for (int k = iv; k < FSUB; k += NT) {
      float sn, cs;
      sincospif(2.0f * ((float)k * cf), &sn, &cs);
      fsubt[k] = make_float2(cs, sn);
    }
    cp_async_wait_all();
  }
  __syncthreads();

  P2 u[R];
  // ---- pass 0: decode + fringe-rotate x[n] and x[n+M], n = iv + r*NB0 (r < 16), form the
  //      lanes A = x[n] + x[n+M], B = (x[n] - x[n+M]) W_N^n, then radix 16 over r
  {
    const int off = g.offset;
    const int sbase = (int)(CPLX ? (4LL * off - stage_base) : (((long long)off >> 1) - stage_base));
    const float2 rs = tsub[iv & (SUB - 1)];
    const int p0 = (off & 1) + iv;
    const int shift = 2 * (2 * (p0 & 1) + pol);
    auto sample = [&](int r) -> float2 {
      const float2 rot = cmul(rs, tstep[(iv / SUB) + r * (NB0 / SUB)]);
      if constexpr (CPLX) {
        const char2 x = *reinterpret_cast<const char2 *>(stage + sbase + 4 * iv + 2 * pol + r * (4 * NB0));
        if constexpr (DBG) probe_store(prm, ant, pol, t, iv + r * NB0, make_float2((float)x.x, (float)x.y));
        return cmul(make_float2((float)x.x, (float)x.y), rot);
      } else {
        const int byte = stage[sbase + (p0 >> 1) + r * (NB0 / 2)];
        const float lv = level2bit((byte >> shift) & 3);
        if constexpr (DBG) probe_store(prm, ant, pol, t, iv + r * NB0, make_float2(lv, 0.0f));
        return make_float2(lv * rot.x, lv * rot.y);
      }
    };
    const float2 wiv = __ldg(&prm.tw[iv]);  // W_N^n = W_N^iv W_32^r
#pragma unroll
    for (int r = 0; r < R; r++) {
      const float2 x0 = sample(r), x1 = sample(r + R);
      const float2 w = __ldg(&prm.tw[iv + NB0 * r]);
      const float2 b = cmul(make_float2(x0.x - x1.x, x0.y - x1.y), w);
      u[r].re = make_float2(x0.x + x1.x, b.x);
      u[r].im = make_float2(x0.y + x1.y, b.y);
    }
    dft16p<false>(u);
    float4 *bp = buf + iv * (R + 1);
#pragma unroll
    for (int r = 0; r < R; r++) bp[r] = make_float4(u[r].re.x, u[r].re.y, u[r].im.x, u[r].im.y);
  }
  __syncthreads();
  // ---- pass 1: radix 16, span 16 (in place)
  {
    const float4 *bp = buf + iv + iv / PAD;
#pragma unroll
    for (int r = 0; r < R; r++) {
      const float4 v = bp[r * (NB + NB / PAD)];
      u[r].re = make_float2(v.x, v.y);
      u[r].im = make_float2(v.z, v.w);
    }
    const int k = iv & (R - 1);
#pragma unroll
    for (int r = 1; r < R; r++) {  // W_M^(16 r k)
      const float2 w = __ldg(&prm.twp1[16 * r + k]);
      pcmul(u[r], w.x, w.y);
    }
    dft16p<false>(u);
  }
  __syncthreads();
  {
    const int k = iv & (R - 1);
    const int j = (iv - k) * R + k;
    float4 *bp = buf + j + j / PAD;
#pragma unroll
    for (int r = 0; r < R; r++) bp[r * (R + R / PAD)] = make_float4(u[r].re.x, u[r].re.y, u[r].im.x, u[r].im.y);
  }
  __syncthreads();
  // ---- pass 2: radix 16, span 256; sub-FFT bin kk = iv + r*NB is channel 2 kk (A) and 2 kk + 1 (B)
  {
    const float4 *bp = buf + iv + iv / PAD;
#pragma unroll
    for (int r = 0; r < R; r++) {
      const float4 v = bp[r * (NB + NB / PAD)];
      u[r].re = make_float2(v.x, v.y);
      u[r].im = make_float2(v.z, v.w);
    }
#pragma unroll
    for (int r = 1; r < R; r++) {  // W_M^(r iv)
      const float2 w = __ldg(&prm.twp2[NB * r + iv]);
      pcmul(u[r], w.x, w.y);
    }
    dft16p<!CPLX>(u);
    constexpr int RKEEP = CPLX ? R : R / 2;  // real data keeps channels c < N/2
    // frac-delay: fine part fixed per thread (FSUB divides 2*NB), output scale (a power of two) folded in
    const float sc = prm.out_scale;
    const float2 fa = fsubt[(2 * iv) & (FSUB - 1)], fb = fsubt[(2 * iv + 1) & (FSUB - 1)];
    const float2 fsA = make_float2(fa.x * sc, fa.y * sc), fsB = make_float2(fb.x * sc, fb.y * sc);
    OutT *o = out0 + (size_t)((2 * iv) >> 4) * ctile_stride + ((2 * iv) & 15);
#pragma unroll
    for (int r = 0; r < RKEEP; r++) {
      const float2 fst = fstept[(2 * iv) / FSUB + r * (2 * NB / FSUB)];
      float2 a = cmul(make_float2(u[r].re.x, u[r].im.x), cmul(fsA, fst));
      float2 b = cmul(make_float2(u[r].re.y, u[r].im.y), cmul(fsB, fst));
      if constexpr (std::is_same<OutT, __nv_fp8x2_e4m3>::value) {
        if (prm.cscale) {  // channels 2 iv + 2 NB r and the next one
          const int c = 2 * iv + r * 2 * NB;
          const float sa = __ldg(&prm.cscale[c]), sb = __ldg(&prm.cscale[c + 1]);
          a = make_float2(a.x * sa, a.y * sa);
          b = make_float2(b.x * sb, b.y * sb);
        }
      }
      store_pair<OutT>(o + (size_t)r * (2 * NB / 16) * ctile_stride, a, b);
    }
  }
}

template <typename OutT, bool CPLX, bool DBG = false>
static cudaError_t launch_fstage_pair(const FParams &prm, int nt, cudaStream_t s) {
  using Pl = FPlan<13, CPLX>;
  const Job &job = prm.job;
  if (job.substride != Pl::SUB || job.stride != Pl::STRIDE || job.fsub != Pl::FSUB || job.fstride != Pl::STRIDE ||
      job.nchan != Pl::NCHAN)
    return cudaErrorInvalidValue;
  constexpr int M = Pl::N / 2;
  const size_t stage_bytes = CPLX ? 4 * (size_t)Pl::N + 32 : (size_t)Pl::N / 2 + 32;
  const size_t smem = sizeof(float4) * ((size_t)M + M / 16) +
                      sizeof(float2) * ((size_t)Pl::SUB + 2 * Pl::STRIDE + Pl::FSUB) +
                      ((stage_bytes + 15) & ~(size_t)15);
  auto kern = fstage_pair_kernel<OutT, CPLX, DBG>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid(2u * (unsigned)nt, (unsigned)job.nant, 1u);
  kern<<<grid, 256, smem, s>>>(prm);
  return cudaGetLastError();
}

template <int L, typename OutT, bool CPLX, bool DBG = false>
static cudaError_t launch_fstage_t(const FParams &prm, int nt, cudaStream_t s) {
  using Pl = FPlan<L, CPLX>;
  const Job &job = prm.job;
  if (job.substride != Pl::SUB || job.stride != Pl::STRIDE || job.fsub != Pl::FSUB || job.fstride != Pl::STRIDE ||
      job.nchan != Pl::NCHAN)
    return cudaErrorInvalidValue;
  const size_t stage_bytes = CPLX ? 4 * (size_t)Pl::N + 32 : (size_t)Pl::N / 2 + 32;
  const size_t smem = sizeof(float2) * ((size_t)Pl::PADN + Pl::SUB + 2 * Pl::STRIDE + Pl::FSUB) +
                      ((stage_bytes + 15) & ~(size_t)15);
  auto kern = fstage_kernel<L, OutT, CPLX, DBG>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid(2u * (unsigned)nt, (unsigned)job.nant, 1u);
  kern<<<grid, Pl::NT, smem, s>>>(prm);
  return cudaGetLastError();
}

// ------------------------------------------------- 32768-point FFT windows
// One pol of one window is 256 KiB in FP32, more than a CTA's shared memory,
// so a cluster of two CTAs shares it (four-step factorisation N = 128 x 256):
//   step 1: CTA r takes columns n2 in [128r, 128r+128): 128-point FFTs over n1
//           of x[256 n1 + n2] (radix 32 then 4), decoded and fringe-rotated
//           from a staged copy of its 128 rows of the packed window, times the
//           twiddle W_N^(n2 k1);
//   step 2: after a cluster barrier, CTA r reads rows k1 in [64r, 64r+64) of
//           both CTAs' [k1][n2] buffers (half through distributed shared memory);
//   step 3: after a second cluster barrier, 256-point FFTs over n2 (radix 16 x 16)
//           give X[k1 + 128 k2], multiplied by the frac-delay phase and stored.
// Every twiddle is W_N^e = Thi[e >> 7] * Tlo[e & 127] from two shared tables
// (Thi[h] = W_N^(128 h), Tlo[l] = W_N^l), so no pass gathers from the N-entry table.
// Grid x = rank + 2 * (pol + 2 * FFT): the two pols of one window are neighbouring
// clusters (the second read of the window hits L2) and write neighbouring streams.
// The flagged-window path returns before any cluster barrier, in both CTAs alike.
constexpr int F15 = 32768;
constexpr int F15_STRIDE = 128;                 // fringe/frac table split (2^floor(log2 nchan / 2))
constexpr int F15_SUB = F15 / F15_STRIDE;       // 256
// complex slots of the shared buffer, reused by the passes: [n2][n1] columns 128 x 129,
// [k1][n2] rows 128 x 132, [k1][k2] rows 64 x 280.  Passes C and D give each row 8 lanes
// (8 consecutive elements) and 4 rows per warp; a row stride of 280 complex (16 banks mod 32)
// puts rows 0/2 and 1/3 in opposite bank halves, the minimum of 2 wavefronts per access.
constexpr int F15_RS = 280;
constexpr int F15_BUF = 64 * F15_RS;
// staged rows: 128 samples of one row n1 (4 bytes each for 8-bit complex, 2 bits per
// pol for 2-bit real) plus the 16-byte rounding of the row start
template <bool CPLX> struct F15Stage {
  static constexpr int ROW = CPLX ? 512 + 16 : 64 + 16;  // bytes per staged row (16-byte multiple)
  static constexpr int CHUNKS = ROW / 16;
  static constexpr int BYTES = 128 * ROW;
};

template <typename OutT, bool CPLX, bool DBG = false>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(512, 1) fstage_cluster_kernel(FParams prm) {
  namespace cg = cooperative_groups;
  using St = F15Stage<CPLX>;
  constexpr int NCHAN = CPLX ? F15 : F15 / 2;
  constexpr int FSUB = NCHAN / F15_STRIDE;
  const Job &job = prm.job;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ float2 smem[];
  float2 *buf = smem;                       // column, [k1][n2] and row buffers (reused)
  float2 *tsub = buf + F15_BUF;             // [F15_SUB]
  float2 *tstep = tsub + F15_SUB;           // [F15_STRIDE]
  float2 *fsubt = tstep + F15_STRIDE;       // [FSUB]
  float2 *fstept = fsubt + FSUB;            // [F15_STRIDE]
  float2 *thi = fstept + F15_STRIDE;        // [256] W_N^(128 h)
  float2 *tlo = thi + 256;                  // [128] W_N^l
  unsigned char *stage = reinterpret_cast<unsigned char *>(tlo + 128);  // [128][St::ROW]
  __shared__ Geom g;

  const int rk = (int)cluster.block_rank();
  const int pol = (blockIdx.x >> 1) & 1;
  const int tl = blockIdx.x >> 2;
  const int ant = blockIdx.y;
  const int t = prm.t0 + tl;
  const int tid = threadIdx.x;
  const int nstreams = 2 * job.nant;
  const int s = 2 * ant + pol;
  OutT *chan = reinterpret_cast<OutT *>(prm.chan);
  OutT *out0 = chan + ((size_t)tl * nstreams + s) * CW;
  const size_t ctile_stride = (size_t)prm.T * nstreams * CW;
  const float2 *__restrict__ tw = prm.tw;

  if (tid == 0) g = job.geom[(size_t)ant * job.nfft + t];
  __syncthreads();
  if (!g.valid) {  // both CTAs of the cluster see the same record
    const OutT z = to_out<OutT>(make_float2(0.f, 0.f), 1.f);
    for (int c = rk * (NCHAN / 2) + tid; c < (rk + 1) * (NCHAN / 2); c += 512)
      out0[(size_t)(c >> 4) * ctile_stride + (c & 15)] = z;
    return;
  }
  const long long off = g.offset;
  // stage rows n1 = 0..127 of this CTA's columns: samples off + 256 n1 + 128 rk + [0, 128)
  // (bounds: offset <= (nfft-1)*F and the buffer holds (nfft+1)*F samples, so the row
  // ends, rounded up to 16 bytes, stay inside it)
  const long long row0 = CPLX ? 4 * (off + 128 * rk) : ((off + 128 * rk) >> 1);
  const long long rbase = row0 & ~15LL;   // row n1 starts at rbase + n1 * (1024 or 128) bytes
  const int mis = (int)(row0 - rbase);
  {
    const unsigned char *src = job.inputs[ant] + rbase;
    constexpr long long RSTEP = CPLX ? 1024 : 128;
    for (int j = tid; j < 128 * St::CHUNKS; j += 512) {
      const int n1 = j / St::CHUNKS, c = j - n1 * St::CHUNKS;
      cp_async16(stage + n1 * St::ROW + 16 * c, src + n1 * RSTEP + 16 * c);
    }
  }
  {
    const float c0 = g.c0, c1 = g.c1, cstep = g.cstep, cf = g.cf;
    for (int k = tid; k < F15_SUB; k += 512) {
      float sn, cs;
      sincospif(-2.0f * fmaf((float)k, c1, c0), &sn, &cs);
      tsub[k] = make_float2(cs, sn);
    }
    for (int i = tid; i < F15_STRIDE; i += 512) {
      float sn, cs;
      sincospif(-2.0f * ((float)i * cstep), &sn, &cs);
      tstep[i] = make_float2(cs, sn);
      sincospif(2.0f * ((float)(i * FSUB) * cf), &sn, &cs);
      fstept[i] = make_float2(cs, sn);
    }
    for (int k = tid; k < FSUB; k += 512) {
      float sn, cs;
      sincospif(2.0f * ((float)k * cf), &sn, &cs);
      fsubt[k] = make_float2(cs, sn);
    }
    if (tid < 256) thi[tid] = __ldg(&tw[128 * tid]);
    else if (tid < 384) tlo[tid - 256] = __ldg(&tw[tid - 256]);
  }
  cp_async_wait_all();
  __syncthreads();

  float2 u[32];
  // ---- step 1, pass A: radix 32 over n1 = iv + 4 r (sample n = 256 n1 + n2)
  const int col = tid & 127, iv = tid >> 7;
  const int n2 = 128 * rk + col;
  {
    const float2 rs = tsub[n2];  // n mod 256 = n2
    // 2-bit: sample off + 256 n1 + n2 sits in byte (that >> 1) = rbase + 128 n1 + mis + (p >> 1)
    const int p = (int)(off & 1) + col;
    const int shift = 2 * (2 * (p & 1) + pol);
#pragma unroll
    for (int r = 0; r < 32; r++) {
      const int n1 = iv + 4 * r;
      const float2 rot = cmul(rs, tstep[n1]);
      const unsigned char *row = stage + n1 * St::ROW + mis;
      if constexpr (CPLX) {
        const char2 x = *reinterpret_cast<const char2 *>(row + 4 * col + 2 * pol);
        if constexpr (DBG) probe_store(prm, ant, pol, t, 256 * n1 + n2, make_float2((float)x.x, (float)x.y));
        u[r] = cmul(make_float2((float)x.x, (float)x.y), rot);
      } else {
        const int byte = row[p >> 1];
        const float lv = level2bit((byte >> shift) & 3);
        if constexpr (DBG) probe_store(prm, ant, pol, t, 256 * n1 + n2, make_float2(lv, 0.0f));
        u[r] = make_float2(lv * rot.x, lv * rot.y);
      }
    }
    dft<32>(u);
#pragma unroll
    for (int r = 0; r < 32; r++) buf[col * 129 + iv * 32 + r] = u[r];
  }
  __syncthreads();
  // ---- step 1, pass B: radix 4 (span 32), then the four-step twiddle W_N^(n2 k1)
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const int ivb = iv * 8 + q;
    float2 *v = &u[4 * q];
#pragma unroll
    for (int r = 0; r < 4; r++) v[r] = buf[col * 129 + ivb + 32 * r];
#pragma unroll
    for (int r = 1; r < 4; r++) v[r] = cmul(v[r], thi[2 * r * ivb]);  // W_N^(256 r ivb)
    dft<4>(v);
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int e = n2 * (ivb + 32 * r);  // < 256 * 128
      v[r] = cmul(v[r], cmul(thi[e >> 7], tlo[e & 127]));
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 8; q++)
#pragma unroll
    for (int r = 0; r < 4; r++) buf[(iv * 8 + q + 32 * r) * 132 + col] = u[4 * q + r];
  cluster.sync();  // both CTAs hold their [k1][n2] halves
  // ---- step 3, pass C: radix 16 over n2 for rows k1 of this CTA (half the columns remote)
  const int kr = tid >> 3, t8 = tid & 7;
  const int k1 = 64 * rk + kr;
  {
    const float2 *Y0 = cluster.map_shared_rank(buf, 0);
    const float2 *Y1 = cluster.map_shared_rank(buf, 1);
#pragma unroll
    for (int q = 0; q < 2; q++) {
      const int ivc = t8 + 8 * q;
#pragma unroll
      for (int r = 0; r < 16; r++) {
        const int nn = ivc + 16 * r;
        u[16 * q + r] = (r < 8) ? Y0[k1 * 132 + nn] : Y1[k1 * 132 + (nn - 128)];
      }
      dft<16>(&u[16 * q]);
    }
  }
  cluster.sync();  // every remote read of this CTA's buffer is done
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const int ivc = t8 + 8 * q;
#pragma unroll
    for (int r = 0; r < 16; r++) buf[kr * F15_RS + ivc * 17 + r] = u[16 * q + r];
  }
  __syncthreads();
  // ---- step 3, pass D: radix 16 (span 16); X[k1 + 128 k2], k2 = ivd + 16 r
  constexpr int RKEEP = CPLX ? 16 : 8;  // real data keeps channels c < N/2
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const int ivd = t8 + 8 * q;
    float2 *v = &u[16 * q];
#pragma unroll
    for (int r = 0; r < 16; r++) v[r] = buf[kr * F15_RS + ivd + 17 * r];
#pragma unroll
    for (int r = 1; r < 16; r++) v[r] = cmul(v[r], thi[r * ivd]);  // W_N^(128 r ivd)
    dft<16>(v);
#pragma unroll
    for (int r = 0; r < RKEEP; r++) {
      const int c = k1 + 128 * (ivd + 16 * r);
      const float2 fr = cmul(fsubt[c & (FSUB - 1)], fstept[c / FSUB]);
      out0[(size_t)(c >> 4) * ctile_stride + (c & 15)] =
          to_out<OutT>(cmul(v[r], fr), chan_scale<OutT>(prm.cscale, c, prm.out_scale));
    }
  }
}

template <typename OutT, bool CPLX, bool DBG = false>
static cudaError_t launch_fstage_cluster(const FParams &prm, int nt, cudaStream_t s) {
  const Job &job = prm.job;
  constexpr int NCHAN = CPLX ? F15 : F15 / 2;
  if (job.F != F15 || job.nchan != NCHAN || job.stride != F15_STRIDE || job.substride != F15_SUB ||
      job.fsub != NCHAN / F15_STRIDE)
    return cudaErrorInvalidValue;
  const size_t smem = sizeof(float2) * ((size_t)F15_BUF + F15_SUB + 2 * F15_STRIDE + NCHAN / F15_STRIDE + 256 + 128) +
                      F15Stage<CPLX>::BYTES;
  auto kern = fstage_cluster_kernel<OutT, CPLX, DBG>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid(4u * (unsigned)nt, (unsigned)job.nant, 1u);
  kern<<<grid, 512, smem, s>>>(prm);
  return cudaGetLastError();
}

// ------------------------ 16384- and 32768-point windows, FP16 / FP8 channelised output
// One CTA per (pol, FFT) with N/64 threads; passes of radix 32, 32 and N/1024 over
// n = iv + (N/R) r, each thread owning two 32-point groups in the first two passes (and
// two or four butterflies in the last).  The intermediate spectrum lives in shared memory
// as FP16 (N*4 bytes instead of N*8: one CTA holds a 32768-point window without a cluster,
// and two 16384-point CTAs share an SM), scaled by 2^-5 after each of the first two passes:
// for any input (|x| <= 127*sqrt(2)) the stored values stay below 6000, far inside FP16's
// range, and the two extra roundings (2^-11 relative) sit below the FP16 / FP8 output
// rounding.  The scale is undone exactly in the final cast.  In the in-place middle pass
// every thread keeps its first group's results as half2 registers until the barrier that
// ends all reads.
// rotator / frac-delay table split for FFT length 2^L (fxkernel.cpp:57-64 for square nchan)
template <int L, bool CPLX>
struct TPlan {
  static constexpr int N = 1 << L;
  static constexpr int NCHAN = CPLX ? N : N / 2;
  static constexpr int STRIDE = 1 << (log2c(NCHAN) / 2);
  static constexpr int SUB = N / STRIDE;
  static constexpr int FSUB = NCHAN / STRIDE;
};

template <int L>
struct HPlan {
  static constexpr int N = 1 << L;
  static constexpr int NT = N / 64;                  // threads: two 32-point groups each
  static constexpr int R = 32, RL = N / (32 * 32);   // radix of passes 0, 1 and of the last pass
  static constexpr int NB = N / R, NBL = N / RL;
  static constexpr int PADN = N + N / R;
  static constexpr int GL = NBL / NT;                // last-pass butterflies per thread
  static constexpr int MINB = L >= 15 ? 1 : 2;
};

template <int L, typename OutT, bool CPLX, bool DBG = false>
__global__ void __launch_bounds__(HPlan<L>::NT, HPlan<L>::MINB) fstage_h_kernel(FParams prm) {
  using H = HPlan<L>;
  using Pl = TPlan<L, CPLX>;
  constexpr int N = H::N, NT = H::NT, R = H::R, RL = H::RL, NB = H::NB, NBL = H::NBL, PADN = H::PADN;
  constexpr int NCHAN = Pl::NCHAN, STRIDE = Pl::STRIDE, SUB = Pl::SUB, FSUB = Pl::FSUB;
  static_assert(NB % SUB == 0 && NBL % FSUB == 0 && NBL % 16 == 0, "table splits / channel tiles");
  constexpr float SC = 1.0f / 32.0f;
  const Job &job = prm.job;
  extern __shared__ float2 smem[];
  float2 *tsub = smem;                 // [SUB]
  float2 *tstep = tsub + SUB;          // [STRIDE]
  float2 *fsubt = tstep + STRIDE;      // [FSUB]
  float2 *fstept = fsubt + FSUB;       // [STRIDE]
  __half2 *buf = reinterpret_cast<__half2 *>(fstept + STRIDE);          // [PADN]
  unsigned char *stage = reinterpret_cast<unsigned char *>(buf + PADN);  // 2-bit windows only

  const int s = blockIdx.x;  // grid x = stream (pol + 2 * antenna), y = FFT
  const int pol = s & 1;
  const int ant = s >> 1;
  const int tl = blockIdx.y;
  const int t = prm.t0 + tl;
  const int tid = threadIdx.x;
  const int nstreams = 2 * job.nant;
  OutT *chan = reinterpret_cast<OutT *>(prm.chan);
  const Geom g = job.geom[(size_t)ant * job.nfft + t];
  OutT *out0 = chan + ((size_t)tl * nstreams + s) * CW;
  const size_t ctile_stride = (size_t)prm.T * nstreams * CW;
  if (!g.valid) {
    const OutT z = to_out<OutT>(make_float2(0.f, 0.f), 1.f);
    for (int c = tid; c < NCHAN; c += NT) out0[(size_t)(c >> 4) * ctile_stride + (c & 15)] = z;
    return;
  }
  const long long off = g.offset;
  long long stage_base = 0;
  if constexpr (!CPLX) {
    // 2-bit: stage the packed window with 16-byte loads (the buffer holds (nfft+1)*F samples
    // and offset <= (nfft-1)*F, so the window plus the 16-byte rounding stays inside it)
    stage_base = (off >> 1) & ~15LL;
    const uint4 *src = reinterpret_cast<const uint4 *>(job.inputs[ant] + stage_base);
    const long long last = (off + N + 1) >> 1;
    const int nvec = (int)((last - stage_base + 15) >> 4);
    uint4 *dst = reinterpret_cast<uint4 *>(stage);
    for (int i = tid; i < nvec; i += NT) dst[i] = __ldg(&src[i]);
  }
  for (int k = tid; k < SUB; k += NT) {
    float sn, cs;
    sincospif(-2.0f * fmaf((float)k, g.c1, g.c0), &sn, &cs);
    tsub[k] = make_float2(cs, sn);
  }
  for (int i = tid; i < STRIDE; i += NT) {
    float sn, cs;
    sincospif(-2.0f * ((float)i * g.cstep), &sn, &cs);
    tstep[i] = make_float2(cs, sn);
    sincospif(2.0f * ((float)(i * FSUB) * g.cf), &sn, &cs);
    fstept[i] = make_float2(cs, sn);
  }
  for (int k = tid; k < FSUB; k += NT) {
    float sn, cs;
    sincospif(2.0f * ((float)k * g.cf), &sn, &cs);
    fsubt[k] = make_float2(cs, sn);
  }
  __syncthreads();

  // ---- pass 0 (span 1): decode + fringe-rotate, radix 32 over n = iv + NB r
#pragma unroll 1
  for (int q = 0; q < 2; q++) {
    const int iv = tid + NT * q;
    float2 u[32];
    const float2 rs = tsub[iv & (SUB - 1)];  // n mod SUB = iv mod SUB
    if constexpr (CPLX) {
      const uint8_t *in = job.inputs[ant] + 4 * (off + iv) + 2 * pol;
#pragma unroll
      for (int r = 0; r < 32; r++) {
        const char2 x = __ldg(reinterpret_cast<const char2 *>(in + 4LL * NB * r));
        if constexpr (DBG) probe_store(prm, ant, pol, t, iv + NB * r, make_float2((float)x.x, (float)x.y));
        u[r] = cmul(make_float2((float)x.x, (float)x.y), cmul(rs, tstep[(iv / SUB) + r * (NB / SUB)]));
      }
    } else {
      const int sbase = (int)((off >> 1) - stage_base);
      const int p0 = (int)(off & 1) + iv;
      const int shift = 2 * (2 * (p0 & 1) + pol);
#pragma unroll
      for (int r = 0; r < 32; r++) {
        const float2 rot = cmul(rs, tstep[(iv / SUB) + r * (NB / SUB)]);
        const int byte = stage[sbase + (p0 >> 1) + r * (NB / 2)];
        const float lv = level2bit((byte >> shift) & 3);
        if constexpr (DBG) probe_store(prm, ant, pol, t, iv + NB * r, make_float2(lv, 0.0f));
        u[r] = make_float2(lv * rot.x, lv * rot.y);
      }
    }
    dft<32>(u);
    __half2 *b = buf + iv * (R + 1);
#pragma unroll
    for (int r = 0; r < 32; r++) b[r] = __floats2half2_rn(u[r].x * SC, u[r].y * SC);
  }
  __syncthreads();
  // ---- pass 1: radix 32, span 32 (in place: both groups read before any write)
  {
    __half2 h[2][32];
#pragma unroll
    for (int q = 0; q < 2; q++) {
      const int iv = tid + NT * q;
      float2 u[32];
      const __half2 *b = buf + iv + iv / R;
#pragma unroll
      for (int r = 0; r < 32; r++) u[r] = __half22float2(b[r * (NB + NB / R)]);
      twiddle<N, R, R>(u, iv & (R - 1), prm.tw);
      dft<32>(u);
#pragma unroll
      for (int r = 0; r < 32; r++) h[q][r] = __floats2half2_rn(u[r].x * SC, u[r].y * SC);
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 2; q++) {
      const int iv = tid + NT * q;
      const int k = iv & (R - 1);
      const int j = (iv - k) * R + k;
      __half2 *b = buf + j + j / R;
#pragma unroll
      for (int r = 0; r < 32; r++) b[r * (R + 1)] = h[q][r];
    }
  }
  __syncthreads();
  // ---- last pass: radix RL, span NBL; outputs c = iv + NBL r go straight to global
  constexpr int RKEEP = CPLX ? RL : RL / 2;       // real data keeps channels c < N/2
  const float oscale = prm.out_scale * 1024.0f;  // undoes the two 2^-5 scalings exactly
#pragma unroll 1
  for (int q = 0; q < H::GL; q++) {
    const int iv = tid + NT * q;
    float2 v[RL];
    const __half2 *b = buf + iv + iv / R;
#pragma unroll
    for (int r = 0; r < RL; r++) v[r] = __half22float2(b[r * (NBL + NBL / R)]);
    twiddle<N, RL, NBL>(v, iv, prm.tw);
    dft<RL>(v);
    const float2 fs = fsubt[iv & (FSUB - 1)];
    OutT *o = out0 + (size_t)(iv >> 4) * ctile_stride + (iv & 15);
#pragma unroll
    for (int r = 0; r < RKEEP; r++) {
      const float2 fr = cmul(fs, fstept[(iv / FSUB) + r * (NBL / FSUB)]);
      o[(size_t)r * (NBL / 16) * ctile_stride] =
          to_out<OutT>(cmul(v[r], fr), chan_scale<OutT>(prm.cscale, iv + r * NBL, oscale));
    }
  }
}

template <int L, typename OutT, bool CPLX, bool DBG = false>
static cudaError_t launch_fstage_h(const FParams &prm, int nt, cudaStream_t s) {
  using H = HPlan<L>;
  using Pl = TPlan<L, CPLX>;
  const Job &job = prm.job;
  if (job.F != H::N || job.nchan != Pl::NCHAN || job.stride != Pl::STRIDE || job.substride != Pl::SUB ||
      job.fsub != Pl::FSUB || job.fstride != Pl::STRIDE)
    return cudaErrorInvalidValue;
  const size_t smem = sizeof(float2) * ((size_t)Pl::SUB + 2 * Pl::STRIDE + Pl::FSUB) +
                      sizeof(__half2) * (size_t)H::PADN + (CPLX ? 0 : (size_t)H::N / 2 + 48);
  auto kern = fstage_h_kernel<L, OutT, CPLX, DBG>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (nt > 65535) return cudaErrorInvalidValue;
  dim3 grid(2u * (unsigned)job.nant, (unsigned)nt, 1u);
  kern<<<grid, H::NT, smem, s>>>(prm);
  return cudaGetLastError();
}

template <typename OutT, bool CPLX, bool DBG = false>
static cudaError_t launch_fstage_l(const FParams &prm, int nt, cudaStream_t s) {
  switch (prm.job.log2F) {
    case 8: return launch_fstage_t<8, OutT, CPLX, DBG>(prm, nt, s);
    case 9: return launch_fstage_t<9, OutT, CPLX, DBG>(prm, nt, s);
    case 10: return launch_fstage_t<10, OutT, CPLX, DBG>(prm, nt, s);
    case 11: return launch_fstage_t<11, OutT, CPLX, DBG>(prm, nt, s);
    case 12: return launch_fstage_t<12, OutT, CPLX, DBG>(prm, nt, s);
    case 13: return launch_fstage_pair<OutT, CPLX, DBG>(prm, nt, s);  // packed FP32 pairs
    case 14:  // FP32 output: FP32 shared buffer; FP16 / FP8 output: FP16 buffer, two CTAs per SM
      if constexpr (std::is_same<OutT, float2>::value) return launch_fstage_t<14, OutT, CPLX, DBG>(prm, nt, s);
      else return launch_fstage_h<14, OutT, CPLX, DBG>(prm, nt, s);
    case 15:  // FP32 output: the 2-CTA cluster kernel; FP16 / FP8 output: one CTA with an FP16 buffer
      if constexpr (std::is_same<OutT, float2>::value) return launch_fstage_cluster<OutT, CPLX, DBG>(prm, nt, s);
      else return launch_fstage_h<15, OutT, CPLX, DBG>(prm, nt, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace gxc
