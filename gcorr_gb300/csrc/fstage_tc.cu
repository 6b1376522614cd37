// Tensor-core F-stage: 8192-point windows of 2-bit real data with FP16 or FP8
// channelised output, the FFT as two dense DFT products on tcgen05.
//
// Four-step factorisation N = 8192 = N1 x N2, N1 = 64, N2 = 128, n = n2 + 128 n1,
// k = k1 + 64 k2 (fxkernel's dofft, fxkernel/src/fxkernel.cpp:569-580, is the
// plain unnormalised forward DFT this restates):
//   X[k1 + 64 k2] = sum_n2 W128^(n2 k2) [ W8192^(n2 k1) sum_n1 W64^(n1 k1) x[n2 + 128 n1] ].
// Step 1 is a real GEMM per polarisation, D1 (128 x 128) = B1 (128 x 128) A1^T,
// with A1 the real form of DFT64 (row 2 k1 gives Re Y, row 2 k1 + 1 gives Im Y;
// K = [Re x over n1 | Im x over n1]) and B1 the decoded, fringe-rotated window
// (row n2, K as for A1): tensor-memory lane n2 holds Re and Im of Y[k1][n2] in
// adjacent columns.  The twiddle W8192^(n2 k1) and the fine part of the
// fractional-sample-delay correction, fsubt[k1], are applied on the CUDA cores
// while the result moves from tensor memory to shared memory as the A operand of
// step 2; both are geometric in k1, so one thread per (pol, n2) advances their
// product by one complex multiply per k1.  Step 2 is D3 (128 x 128) = A3 (128 x
// 256) B3^T: rows of A3 are (pol, k1), K = [Re Y' over n2 | Im Y' over n2], and
// B3 is the real form of the first 64 rows of DFT128 (row 2 k2 gives Re X,
// 2 k2 + 1 gives Im X; real data keeps channels k < 4096, i.e. k2 < 64).  The
// coarse frac-delay factor fstept[k2], the output scale and the cast are applied
// as D3 leaves tensor memory.
//
// Operands are FP16 (kind::f16) with FP32 accumulation in tensor memory.  The
// FFT then carries four FP16 roundings (the rotated samples, both DFT matrices and
// the twiddled intermediate) on top of the FP16 / FP8 output rounding; it serves
// the FP16 and FP8 channelised paths only (the FP32 path keeps the CUDA-core FFT).
//
// The rotator and frac-delay tables of the fxkernel layout fall on the four-step
// indices: with stride 64 and substride 128 (fxkernel.cpp:57-64), sample n has
// rotator tsub[n2] * tstep[n1] and channel k frac-delay fsubt[k1] * fstept[k2].
// tstep[n1] is folded into a per-window A1 (Re / Im of W64^(n1 k1) tstep[n1]), so
// B1 holds the real 2-bit levels and step 1 has K = 64; tsub[n2] joins the
// twiddle recurrence.
//
// One persistent CTA of 512 threads per SM (about 190 KB of shared memory) loops
// over the windows of the block, both polarisations of a window at a time (they
// share the geometry, the staged packed bytes, the rotator and the frac-delay
// tables, and fill the 128 rows of step 2).  The next window's packed bytes,
// geometry and tables load into a second staging buffer while the current
// window's step-1 MMAs run, and it is decoded into B1 and A1 while the step-2
// MMAs run.  Every mbarrier wait is bounded; on expiry the kernel sets an error
// flag (read by gxc_sync as GXC_ERR_TIMEOUT), lets issued MMAs drain, frees
// tensor memory and returns.
#include "fstage_kernels.cuh"
#include "gxc_internal.h"
#include "tcgen05_util.cuh"

#include <math.h>
#include <vector>

namespace gxc {

namespace ftc {

constexpr int N1 = 64, N2 = 128, F = N1 * N2, NCHAN = F / 2;
constexpr int SUB = 128, STRIDE = 64, FSUB = 64;  // rotator / frac-delay table split of nchan 4096
constexpr int NT = 512;                             // 16 warps: 4 groups of the 4 TMEM lane quarters
constexpr int NWG = NT / 128;
constexpr int KB = 128 * 128;                       // one 128-row SW128 K-block (64 FP16 K-elements)
// shared-memory image (byte offsets from a 1024-aligned base)
constexpr int OFF_A1 = 0;                  // the window's A1 (DFT64 times tstep), 1 K-block
constexpr int OFF_B3 = OFF_A1 + KB;        // DFT128 rows k2 < 64, 4 K-blocks (constant)
constexpr int OFF_BUF = OFF_B3 + 4 * KB;   // A3 (4 K-blocks)
constexpr int OFF_B1 = OFF_BUF + 4 * KB;   // B1 of pol 0 (1 K-block), B1 of pol 1 (1)
constexpr int CONST_BYTES = 4 * KB;        // the part copied from the table image (B3)
constexpr int OFF_W64 = OFF_B1 + 2 * KB;   // W64^j = exp(-2 pi i j / 64), j < 64 (float2)
// two staging buffers (window w and the next one): tables tsub[128], tstep[64], fsubt[64],
// fstept[64]; the packed window (2 pols, 2 bits) + 16-byte rounding; the geometry records
constexpr int TAB_BYTES = (SUB + STRIDE + FSUB + STRIDE) * 8;
constexpr int OFF_TAB = OFF_W64 + 64 * 8;
constexpr int STAGE_BYTES = F / 2 + 64;
constexpr int OFF_STAGE = OFF_TAB + 2 * TAB_BYTES;
constexpr int OFF_GEOM = OFF_STAGE + 2 * STAGE_BYTES;
constexpr int SMEM_BYTES = OFF_GEOM + 2 * (int)sizeof(Geom) + 1024;  // + alignment slack
// global table image: B3 in its swizzled shared-memory layout
constexpr int TABLE_BYTES = CONST_BYTES;
static_assert(OFF_BUF - OFF_B3 == 4 * KB && CONST_BYTES % 16 == 0, "layout");
static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");

struct Params {
  Job job;
  const uint4 *tables;  // TABLE_BYTES image (make_fstage_tc_tables)
  int t0, nt, T;
  void *chan;
  float out_scale;
  const float *cscale;  // FP8 output: per-channel scale [nchan] (replaces out_scale), or null
  float2 *probe;        // decode probe (DBG kernels): [nant][2][nfft][F] decoded samples
  int *err;
};

__device__ int g_ftc_err;

// byte offset of FP16 element (row, k) in a SW128 K-major tile of 128-byte rows
__host__ __device__ inline int sw128_off(int row, int k) {
  return row * 128 + ((((k >> 3) ^ (row & 7)) & 7) << 4) + (k & 7) * 2;
}

__device__ __forceinline__ uint32_t pack_h2(float a, float b) {
  const __half2 h = __floats2half2_rn(a, b);
  return *reinterpret_cast<const uint32_t *>(&h);
}

// FP16 levels of two 2-bit codes, packed (a low, b high): the level table of fxkernel.cpp:17-18
// {-HiMag, -1, 1, HiMag} as FP16 bit patterns, code c at bytes 2c, 2c+1 of {kHi:kLo}, picked by
// one byte permute.  HiMag = 3.3359 is 3.3359375 in FP16, the nearest half.
__device__ __forceinline__ uint32_t level_pair_h2(int a, int b) {
  constexpr uint32_t kLo = 0xBC00C2ACu, kHi = 0x42AC3C00u;  // codes 1, 0 | codes 3, 2
  const uint32_t sel = (uint32_t)(a * 0x22 + 0x10) | ((uint32_t)(b * 0x22 + 0x10) << 8);
  return tc::prmt(kLo, kHi, sel);
}

// Stages window w into buffer b: its geometry record, the packed bytes (asynchronous 16-byte
// copies; the buffer holds (nfft+1)*F samples and offset <= (nfft-1)*F, so the window plus the
// 16-byte rounding stays inside it) and the rotator / frac-delay tables.  A flagged window
// stages nothing but its record.
__device__ __forceinline__ void stage_window(const Params &p, int w, unsigned char *smem, int b) {
  const Job &job = p.job;
  const int tid = threadIdx.x;
  const int ant = w % job.nant, t = p.t0 + w / job.nant;
  const Geom g = job.geom[(size_t)ant * job.nfft + t];
  if (tid == 0) reinterpret_cast<Geom *>(smem + OFF_GEOM)[b] = g;
  if (!g.valid) return;
  unsigned char *stage = smem + OFF_STAGE + b * STAGE_BYTES;
  float2 *tsub = reinterpret_cast<float2 *>(smem + OFF_TAB + b * TAB_BYTES);
  float2 *tstep = tsub + SUB, *fsubt = tstep + STRIDE, *fstept = fsubt + FSUB;
  const long long stage_base = ((long long)g.offset >> 1) & ~15LL;
  const uint4 *src = reinterpret_cast<const uint4 *>(job.inputs[ant] + stage_base);
  const long long last = ((long long)g.offset + F + 1) >> 1;
  const int nvec = (int)((last - stage_base + 15) >> 4);
  for (int i = tid; i < nvec; i += NT) cp_async16(stage + 16 * i, src + i);
  float sn, cs;
  if (tid < SUB) {
    sincospif(-2.0f * fmaf((float)tid, g.c1, g.c0), &sn, &cs);
    tsub[tid] = make_float2(cs, sn);
  } else if (tid < SUB + STRIDE) {
    const int i = tid - SUB;
    sincospif(-2.0f * ((float)i * g.cstep), &sn, &cs);
    tstep[i] = make_float2(cs, sn);
    sincospif(2.0f * ((float)(i * FSUB) * g.cf), &sn, &cs);
    fstept[i] = make_float2(cs, sn);
  } else if (tid < SUB + STRIDE + FSUB) {
    const int k = tid - SUB - STRIDE;
    sincospif(2.0f * ((float)k * g.cf), &sn, &cs);
    fsubt[k] = make_float2(cs, sn);
  }
}

// DBG = true (decode probe): every decoded sample is also written to p.probe before the rotation.
template <typename OutT, bool DBG = false>
__global__ void __launch_bounds__(NT, 1) fstage_tc_kernel(Params p) {
  using namespace tc;
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar_mma1, bar_mma3;
  __shared__ uint32_t tmem_base_sh;
  unsigned char *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  const uint32_t sbase = smem_u32(smem);
  const Job &job = p.job;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nstreams = 2 * job.nant;
  const size_t ctile_stride = (size_t)p.T * nstreams * CW;
  OutT *chan = reinterpret_cast<OutT *>(p.chan);

  // constant operand B3 and the DFT64 roots, once per CTA
  {
    uint4 *dst = reinterpret_cast<uint4 *>(smem + OFF_B3);
    for (int i = tid; i < CONST_BYTES / 16; i += NT) dst[i] = __ldg(&p.tables[i]);
    if (tid < 64) {
      float sn, cs;
      sincospif(-(float)tid / 32.0f, &sn, &cs);
      reinterpret_cast<float2 *>(smem + OFF_W64)[tid] = make_float2(cs, sn);
    }
  }
  const float2 *w64 = reinterpret_cast<const float2 *>(smem + OFF_W64);
  if (tid == 0) {
    mbar_init(smem_u32(&bar_mma1), 1);
    mbar_init(smem_u32(&bar_mma3), 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(smem_u32(&tmem_base_sh), 512);
    tmem_relinquish();
  }
  const int nwin = p.nt * job.nant;
  const int G = (int)gridDim.x;
  if ((int)blockIdx.x < nwin) stage_window(p, blockIdx.x, smem, 0);
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_sh;

  // twiddle-epilogue role of this thread: TMEM lane quarter q1 (n2 = 32 q1 + lane), warp group
  // wg1 = (half of the k1 range) * 2 + pol; W8192^n2 and W8192^(32 half n2), once per CTA
  const int q1 = warp & 3, wg1 = warp >> 2, tn2 = 32 * q1 + lane;
  float2 tw_step, tw_base;
  {
    float sn, cs;
    sincospif(-(float)tn2 / 4096.0f, &sn, &cs);
    tw_step = make_float2(cs, sn);
    sincospif(-(float)((wg1 >> 1) * tn2) / 128.0f, &sn, &cs);
    tw_base = make_float2(cs, sn);
  }
  static_assert(NWG == 4, "four warp groups: two pols x two halves of k1");

  int phase = 0;    // windows correlated so far: the mbarriers' phase parity
  int pending = 0;  // 1: MMA1 issued and not yet waited for; 3: MMA3
  bool ok = true;
  // Decodes window wn, staged in buffer bn, into B1 and A1 (nothing for a flagged window).
  auto decode = [&](int wn, int bn) {
    const Geom g = reinterpret_cast<const Geom *>(smem + OFF_GEOM)[bn];
    if (!g.valid) return;
    const int ant = wn % job.nant, tl = wn / job.nant;
    const unsigned char *stage = smem + OFF_STAGE + bn * STAGE_BYTES;
    const float2 *tstep = reinterpret_cast<const float2 *>(smem + OFF_TAB + bn * TAB_BYTES) + SUB;
    const int off = g.offset;
    // ---- decode into B1 of both pols and build the window's A1.  The rotator of sample
    //      n = n2 + 128 n1 is tsub[n2] tstep[n1]: tstep[n1] goes into A1 (row 2 k1 + part, column
    //      n1: Re / Im of W64^(n1 k1) tstep[n1], one FP16 rounding), tsub[n2] into the twiddle
    //      epilogue, so B1 holds the real levels (B1_pol[n2][n1], K = n1) and step 1 needs K = 64.
    {
      const int sbase = (int)(((long long)off >> 1) - (((long long)off >> 1) & ~15LL));
#pragma unroll 1
      for (int task = tid; task < N2 * 8; task += NT) {  // (n2, o): n1 = 8o .. 8o+7
        const int n2 = task & (N2 - 1), o = task >> 7;
        const int p0 = (off & 1) + n2;  // sample index relative to byte off/2
        const unsigned char *bp = stage + sbase + (p0 >> 1) + 64 * (8 * o);
        const int sh0 = 2 * (2 * (p0 & 1)), sh1 = sh0 + 2;
        uint32_t h0[4], h1[4];
#pragma unroll
        for (int i = 0; i < 8; i += 2) {
          const int ba = bp[64 * i], bb = bp[64 * (i + 1)];
          const int ca0 = (ba >> sh0) & 3, cb0 = (bb >> sh0) & 3, ca1 = (ba >> sh1) & 3, cb1 = (bb >> sh1) & 3;
          h0[i >> 1] = level_pair_h2(ca0, cb0);
          h1[i >> 1] = level_pair_h2(ca1, cb1);
          if constexpr (DBG) {
            const float la0 = level2bit(ca0), lb0 = level2bit(cb0), la1 = level2bit(ca1), lb1 = level2bit(cb1);
            const size_t pi = (((size_t)ant * 2) * job.nfft + (p.t0 + tl)) * F + n2 + 128 * (8 * o + i);
            const size_t pp = (size_t)job.nfft * F;  // pol 1
            p.probe[pi] = make_float2(la0, 0.f);
            p.probe[pi + 128] = make_float2(lb0, 0.f);
            p.probe[pi + pp] = make_float2(la1, 0.f);
            p.probe[pi + pp + 128] = make_float2(lb1, 0.f);
          }
        }
        const int so = n2 * 128 + ((o ^ (n2 & 7)) << 4);
        *reinterpret_cast<uint4 *>(smem + OFF_B1 + 0 * KB + so) = make_uint4(h0[0], h0[1], h0[2], h0[3]);
        *reinterpret_cast<uint4 *>(smem + OFF_B1 + 1 * KB + so) = make_uint4(h1[0], h1[1], h1[2], h1[3]);
      }
      // A1: thread (k1, c), k1 = tid % 64 (a warp reads one tstep entry and consecutive roots),
      // writes columns n1 = 8c .. 8c+7 of rows 2 k1 (Re) and 2 k1 + 1 (Im).  tstep is geometric
      // (tstep[n1] = tstep[1]^n1), so along n1 the entry advances by the factor tstep[1] W64^k1.
      {
        const int k1 = tid & 63, c = tid >> 6;
        const float2 st = cmul(tstep[1], w64[k1]);
        float2 a = cmul(tstep[8 * c], w64[(8 * c * k1) & 63]);
        uint32_t hr[4], hi[4];
#pragma unroll
        for (int e = 0; e < 8; e += 2) {
          const float2 a1 = cmul(a, st);
          hr[e >> 1] = pack_h2(a.x, a1.x);
          hi[e >> 1] = pack_h2(a.y, a1.y);
          a = cmul(a1, st);
        }
        const int r0 = 2 * k1, r1 = r0 + 1;
        *reinterpret_cast<uint4 *>(smem + OFF_A1 + r0 * 128 + ((c ^ (r0 & 7)) << 4)) =
            make_uint4(hr[0], hr[1], hr[2], hr[3]);
        *reinterpret_cast<uint4 *>(smem + OFF_A1 + r1 * 128 + ((c ^ (r1 & 7)) << 4)) =
            make_uint4(hi[0], hi[1], hi[2], hi[3]);
      }
    }
  };
  if ((int)blockIdx.x < nwin) {  // the first window, staged above
    cp_async_wait_all();
    __syncthreads();
    decode(blockIdx.x, 0);
  }
  // Pipeline: B1 and A1 are free once step 1 of window w is done, so the next window (staged
  // during step 1) is decoded while step 2's MMAs run.
  int b = 0;        // staging buffer of window w
  for (int w = blockIdx.x; w < nwin; w += G, b ^= 1) {
    // B1 and A1 hold window w (decoded during the previous window's step 2, or above)
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const Geom g = reinterpret_cast<const Geom *>(smem + OFF_GEOM)[b];
    const int ant = w % job.nant, tl = w / job.nant;
    OutT *out0 = chan + ((size_t)tl * nstreams + 2 * ant) * CW;  // pol 0; pol 1 is CW further
    const bool more = w + G < nwin;
    if (!g.valid) {
      // flagged: the X-stage sums zeros, the baseline counts exclude this FFT
      if (more) {
        stage_window(p, w + G, smem, b ^ 1);
        cp_async_wait_all();
        __syncthreads();
        decode(w + G, b ^ 1);
      }
      const OutT z = to_out<OutT>(make_float2(0.f, 0.f), 1.f);
      for (int i = tid; i < 2 * NCHAN; i += NT) {
        const int pol = i / NCHAN, c = i - pol * NCHAN;
        out0[(size_t)pol * CW + (size_t)(c >> 4) * ctile_stride + (c & 15)] = z;
      }
      continue;
    }
    const float2 *tsub = reinterpret_cast<const float2 *>(smem + OFF_TAB + b * TAB_BYTES);
    const float2 *fsubt = tsub + SUB + STRIDE, *fstept = fsubt + FSUB;
    // ---- step 1: D1_pol (TMEM columns 128 pol ..) = B1_pol A1^T, K = 64: lane n2, column
    //      2 k1 + part, so a thread holds Re and Im of Y[k1][n2] / tsub[n2] for its n2 in
    //      adjacent columns
    if (tid == 0) {
      tc_fence_after();
#pragma unroll
      for (int pol = 0; pol < 2; pol++)
#pragma unroll
        for (int kk = 0; kk < 4; kk++)
          mma_f16(tmem + 128 * pol, desc_sw128(sbase + OFF_B1 + pol * KB + kk * 32),
                  desc_sw128(sbase + OFF_A1 + kk * 32), IDESC, kk > 0 ? 1u : 0u);
      mma_commit(smem_u32(&bar_mma1));
    }
    pending = 1;
    // the next window's bytes and tables load while the MMAs run (its buffer's last reader, the
    // previous window's epilogue, finished before the barrier at the top of this iteration)
    if (more) stage_window(p, w + G, smem, b ^ 1);
    ok = mbar_wait(smem_u32(&bar_mma1), phase & 1, p.err);
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    pending = 0;
    tc_fence_after();
    // ---- twiddle and fine frac-delay, FP16, into A3 (rows pol*64 + k1, K = [Re Y' n2 0..127 |
    //      Im Y' n2 0..127]).  Thread (pol, n2, half) takes k1 = 32 half .. 32 half + 31 of its row:
    //      Y'[k1][n2] = Y[k1][n2] W8192^(n2 k1) fsubt[k1] = Y[k1][n2] w0 r^(k1 - 32 half), with
    //      r = W8192^n2 e^(2 pi i cf) (fsubt is geometric in k1), so the factor advances by one
    //      complex multiply per k1 (over 32 steps its rounding grows to ~3e-6, far below FP16's).
    //      Multiplying row k1 by fsubt[k1] before step 2 scales X[k1 + 64 k2] by it for every k2.
    {
      const int pol = wg1 & 1, half = wg1 >> 1;
      const float2 fs1 = fsubt[1], fs0 = fsubt[32 * half];
      float2 r = cmul(tw_step, fs1), wk = cmul(cmul(tw_base, fs0), tsub[tn2]);  // tsub: the rotator's n2 part
      // byte offsets of the K positions n2 (Re) and 128 + n2 (Im) in row m = pol*64 + k1, for
      // the eight k1 & 7: rows of one 8-row group differ in the swizzle of their chunk index
      const int kc = tn2 & 63, kbase = OFF_BUF + (tn2 >> 6) * KB + (kc & 7) * 2;
      uint32_t xo[8];
#pragma unroll
      for (int e = 0; e < 8; e++) xo[e] = (uint32_t)(kbase + e * 128 + ((((kc >> 3) ^ e) & 7) << 4));
#pragma unroll 1
      for (int jj = 0; jj < 4; jj++) {
        const int k10 = 32 * half + 8 * jj;  // first k1 of the chunk (a multiple of 8)
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(32 * q1) << 16) + (uint32_t)(128 * pol + 2 * k10), v);
        unsigned char *row0 = smem + (pol * 64 + k10) * 128;
#pragma unroll
        for (int e = 0; e < 8; e++) {
          const float2 y = cmul(make_float2(v[2 * e], v[2 * e + 1]), wk);
          wk = cmul(wk, r);
          const uint32_t h = pack_h2(y.x, y.y);
          *reinterpret_cast<uint16_t *>(row0 + xo[e]) = (uint16_t)(h & 0xFFFFu);
          *reinterpret_cast<uint16_t *>(row0 + xo[e] + 2 * KB) = (uint16_t)(h >> 16);
        }
      }
    }
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    // ---- step 2: D3 (TMEM columns 256..383) = A3 B3^T, K = 256
    if (tid == 0) {
      tc_fence_after();
#pragma unroll
      for (int kk = 0; kk < 16; kk++) {
        const uint32_t o = (uint32_t)((kk >> 2) * KB + (kk & 3) * 32);
        mma_f16(tmem + 256, desc_sw128(sbase + OFF_BUF + o), desc_sw128(sbase + OFF_B3 + o), IDESC,
                kk > 0 ? 1u : 0u);
      }
      mma_commit(smem_u32(&bar_mma3));
    }
    pending = 3;
    if (more) {  // the next window's decode, while step 2 runs
      cp_async_wait_all();
      __syncthreads();
      decode(w + G, b ^ 1);
    }
    ok = mbar_wait(smem_u32(&bar_mma3), phase & 1, p.err);
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    pending = 0;
    tc_fence_after();
    // ---- frac-delay correction, scale, cast, store: row m = (pol, k1), columns (k2, re/im);
    //      warp group wg takes columns [128 wg / NWG, 128 (wg + 1) / NWG)
    {
      const int q = warp & 3, wg = warp >> 2;
      const int m = 32 * q + lane, pol = m >> 6, k1 = m & 63;
      const float sc = p.out_scale;
      OutT *o = out0 + (size_t)pol * CW + (k1 & 15);
      constexpr int CPER = 128 / NWG;
#pragma unroll 1
      for (int jj = 0; jj < CPER / 16; jj++) {
        const int col0 = wg * CPER + 16 * jj;
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(256 + col0), v);
#pragma unroll
        for (int e = 0; e < 8; e++) {
          const int k2 = (col0 >> 1) + e, k = k1 + 64 * k2;
          const float2 z = cmul(make_float2(v[2 * e], v[2 * e + 1]), fstept[k2]);  // fsubt[k1] is in A3
          o[(size_t)(k >> 4) * ctile_stride] = to_out<OutT>(z, chan_scale<OutT>(p.cscale, k, sc));
        }
      }
    }
    phase++;
  }
  // copies still in flight (a staged window the loop did not reach) and issued MMAs land before
  // the CTA exits and tensor memory is freed
  cp_async_wait_all();
  if (!ok && tid == 0 && pending) mbar_wait_drain(smem_u32(pending == 1 ? &bar_mma1 : &bar_mma3), phase & 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, 512);
}

}  // namespace ftc

int fstage_tc_supported(const Job &job, int chan_type) {
  return chan_type != CHAN_F32 && !job.is_complex && job.F == ftc::F && job.nchan == ftc::NCHAN &&
         job.stride == ftc::STRIDE && job.substride == ftc::SUB && job.fsub == ftc::FSUB &&
         job.fstride == ftc::STRIDE;
}

// Table image: A1 = real form of DFT64 and B3 = real form of DFT128 rows k2 < 64, each FP16
// rounded once from double and stored in its swizzled shared-memory layout; then the twiddle
// factors W8192^(16 j k1) and W8192^(i k1) as float2.
cudaError_t make_fstage_tc_tables(void **out) {
  using namespace ftc;
  std::vector<unsigned char> img((size_t)TABLE_BYTES, 0);
  const double pi = 3.14159265358979323846;
  auto put = [&](int base, int kb, int row, int k, double v) {
    const __half h = __double2half(v);
    memcpy(&img[(size_t)base + (size_t)kb * KB + (size_t)sw128_off(row, k)], &h, 2);
  };
  // B3[c3][K]: c3 = 2 k2 + part (k2 < 64); K-blocks 0,1: Re Y' n2 0..63, 64..127; 2,3: Im Y'
  for (int k2 = 0; k2 < N2 / 2; k2++)
    for (int n2 = 0; n2 < N2; n2++) {
      const double ps = 2.0 * pi * (double)((n2 * k2) % N2) / (double)N2;
      const double cs = cos(ps), sn = sin(ps);
      const int kb = n2 >> 6, k = n2 & 63;
      put(0, kb, 2 * k2, k, cs);
      put(0, kb + 2, 2 * k2, k, sn);
      put(0, kb, 2 * k2 + 1, k, -sn);
      put(0, kb + 2, 2 * k2 + 1, k, cs);
    }
  cudaError_t e = cudaMalloc(out, img.size());
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*out, img.data(), img.size(), cudaMemcpyHostToDevice);
}

cudaError_t launch_fstage_tc(const Job &job, const void *tables, int t0, int nt, int T, void *chan, int chan_type,
                             float out_scale, cudaStream_t s, const float *cscale, float2 *probe) {
  using namespace ftc;
  if (nt <= 0) return cudaSuccess;
  if (!fstage_tc_supported(job, chan_type) || !tables) return cudaErrorInvalidValue;
  Params p;
  p.job = job;
  p.tables = reinterpret_cast<const uint4 *>(tables);
  p.t0 = t0;
  p.nt = nt;
  p.T = T;
  p.chan = chan;
  p.out_scale = out_scale;
  p.cscale = cscale;
  p.probe = probe;
  cudaError_t e = cudaGetSymbolAddress((void **)&p.err, g_ftc_err);
  if (e != cudaSuccess) return e;
  int dev = 0, nsm = 0;
  e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const long long nwin = (long long)nt * job.nant;
  const unsigned grid = (unsigned)(nwin < nsm ? nwin : nsm);
  auto launch = [&](auto kern) -> cudaError_t {
    cudaError_t e2 = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e2 != cudaSuccess) return e2;
    kern<<<grid, NT, SMEM_BYTES, s>>>(p);
    return cudaGetLastError();
  };
  if (chan_type == CHAN_F8)
    return probe ? launch(fstage_tc_kernel<__nv_fp8x2_e4m3, true>) : launch(fstage_tc_kernel<__nv_fp8x2_e4m3>);
  return probe ? launch(fstage_tc_kernel<__half2, true>) : launch(fstage_tc_kernel<__half2>);
}

// Reads and clears the error flag of the tensor-core F-stage (a bounded wait expired).
cudaError_t fstage_tc_take_error(int *flag) {
  int zero = 0;
  cudaError_t e = cudaMemcpyFromSymbol(flag, ftc::g_ftc_err, sizeof(int));
  if (e == cudaSuccess && *flag) e = cudaMemcpyToSymbol(ftc::g_ftc_err, &zero, sizeof(int));
  return e;
}

}  // namespace gxc
