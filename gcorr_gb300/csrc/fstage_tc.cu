// Tensor-core F-stage: 8192-point windows of 2-bit real data with FP16 or FP8
// channelised output, the FFT as two dense DFT products on tcgen05.
//
// Four-step factorisation N = 8192 = N1 x N2, N1 = 64, N2 = 128, n = n2 + 128 n1,
// k = k1 + 64 k2 (fxkernel's dofft, fxkernel/src/fxkernel.cpp:569-580, is the
// plain unnormalised forward DFT this restates):
//   X[k1 + 64 k2] = sum_n2 W128^(n2 k2) [ W8192^(n2 k1) sum_n1 W64^(n1 k1) x[n2 + 128 n1] ].
// Step 1 is a real GEMM per polarisation, D1 (128 x 128) = A1 (128 x 128) B1^T,
// with A1 the real form of DFT64 (row 2 k1 gives Re Y, row 2 k1 + 1 gives Im Y;
// K = [Re x over n1 | Im x over n1]) and B1 the decoded, fringe-rotated window
// (row n2, K as for A1).  The twiddle W8192^(n2 k1) is applied on the CUDA cores
// while the result moves from tensor memory to shared memory as the A operand of
// step 2, D3 (128 x 128) = A3 (128 x 256) B3^T: rows of A3 are (pol, k1), K =
// [Re Y' over n2 | Im Y' over n2], and B3 is the real form of the first 64 rows
// of DFT128 (row 2 k2 gives Re X, 2 k2 + 1 gives Im X; real data keeps channels
// k < 4096, i.e. k2 < 64).  The fractional-sample-delay correction, the output
// scale and the cast are applied as D3 leaves tensor memory.
//
// Operands are FP16 (kind::f16) with FP32 accumulation in tensor memory.  The
// FFT then carries four FP16 roundings (the rotated samples, both DFT matrices and
// the twiddled intermediate) on top of the FP16 / FP8 output rounding; it serves
// the FP16 and FP8 channelised paths only (the FP32 path keeps the CUDA-core FFT).
//
// The rotator and frac-delay tables of the fxkernel layout fall on the four-step
// indices: with stride 64 and substride 128 (fxkernel.cpp:57-64), sample n has
// rotator tsub[n2] * tstep[n1] and channel k frac-delay fsubt[k1] * fstept[k2].
//
// One persistent CTA of 512 threads per SM (186 KB of shared memory) loops over the windows of
// the block, both polarisations of a window at a time (they share the geometry,
// the staged packed bytes, the rotator and the frac-delay tables, and fill the
// 128 rows of step 2).  The next window's packed bytes, geometry and tables load
// into a second staging buffer while the current window's step-1 MMAs run.  Every mbarrier wait is bounded; on expiry the kernel sets
// an error flag (read by gxc_sync as GXC_ERR_TIMEOUT), lets issued MMAs drain,
// frees tensor memory and returns.
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
constexpr int OFF_A1 = 0;                  // DFT64, 2 K-blocks
constexpr int OFF_B3 = OFF_A1 + 2 * KB;    // DFT128 rows k2 < 64, 4 K-blocks
constexpr int OFF_BUF = OFF_B3 + 4 * KB;   // B1 of pol 0 (2 K-blocks), B1 of pol 1 (2); later A3 (4)
constexpr int OFF_THI = OFF_BUF + 4 * KB;  // W8192^(16 j k1), [j < 8][k1]
constexpr int OFF_TLO = OFF_THI + 64 * 8 * 8;    // W8192^(i k1), [i < 16][k1]
constexpr int CONST_BYTES = OFF_TLO + 64 * 16 * 8 - OFF_A1;  // the part copied from the table image
// two staging buffers (window w and the next one): tables tsub[128], tstep[64], fsubt[64],
// fstept[64]; the packed window (2 pols, 2 bits) + 16-byte rounding; the geometry records
constexpr int TAB_BYTES = (SUB + STRIDE + FSUB + STRIDE) * 8;
constexpr int OFF_TAB = OFF_TLO + 64 * 16 * 8;
constexpr int STAGE_BYTES = F / 2 + 64;
constexpr int OFF_STAGE = OFF_TAB + 2 * TAB_BYTES;
constexpr int OFF_GEOM = OFF_STAGE + 2 * STAGE_BYTES;
constexpr int SMEM_BYTES = OFF_GEOM + 2 * (int)sizeof(Geom) + 1024;  // + alignment slack
// global table image: A1 and B3 in their swizzled shared-memory layout, then THI and TLO
constexpr int TABLE_BYTES = CONST_BYTES;
static_assert(OFF_BUF - OFF_B3 == 4 * KB && (OFF_THI - OFF_A1) % 16 == 0 && CONST_BYTES % 16 == 0, "layout");
static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");

struct Params {
  Job job;
  const uint4 *tables;  // TABLE_BYTES image (make_fstage_tc_tables)
  int t0, nt, T;
  void *chan;
  float out_scale;
  const float *cscale;  // FP8 output: per-channel scale [nchan] (replaces out_scale), or null
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

template <typename OutT>
__global__ void __launch_bounds__(NT, 1) fstage_tc_kernel(Params p) {
  using namespace tc;
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar_mma1, bar_mma3;
  __shared__ uint32_t tmem_base_sh;
  unsigned char *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  const uint32_t sbase = smem_u32(smem);
  const Job &job = p.job;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float2 *thi = reinterpret_cast<const float2 *>(smem + OFF_THI);
  const float2 *tlo = reinterpret_cast<const float2 *>(smem + OFF_TLO);
  const int nstreams = 2 * job.nant;
  const size_t ctile_stride = (size_t)p.T * nstreams * CW;
  OutT *chan = reinterpret_cast<OutT *>(p.chan);

  // constant operands and twiddles, once per CTA
  {
    uint4 *dst = reinterpret_cast<uint4 *>(smem + OFF_A1);
    for (int i = tid; i < CONST_BYTES / 16; i += NT) dst[i] = __ldg(&p.tables[i]);
  }
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

  int phase = 0;    // windows correlated so far: the mbarriers' phase parity
  int pending = 0;  // 1: MMA1 issued and not yet waited for; 3: MMA3
  bool ok = true;
  int b = 0;        // staging buffer of window w
  for (int w = blockIdx.x; w < nwin; w += G, b ^= 1) {
    // window w was staged into buffer b during the previous window (or above)
    cp_async_wait_all();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const Geom g = reinterpret_cast<const Geom *>(smem + OFF_GEOM)[b];
    const int ant = w % job.nant, tl = w / job.nant;
    OutT *out0 = chan + ((size_t)tl * nstreams + 2 * ant) * CW;  // pol 0; pol 1 is CW further
    if (!g.valid) {
      // flagged: the X-stage sums zeros, the baseline counts exclude this FFT
      if (w + G < nwin) stage_window(p, w + G, smem, b ^ 1);
      const OutT z = to_out<OutT>(make_float2(0.f, 0.f), 1.f);
      for (int i = tid; i < 2 * NCHAN; i += NT) {
        const int pol = i / NCHAN, c = i - pol * NCHAN;
        out0[(size_t)pol * CW + (size_t)(c >> 4) * ctile_stride + (c & 15)] = z;
      }
      continue;
    }
    const unsigned char *stage = smem + OFF_STAGE + b * STAGE_BYTES;
    const float2 *tsub = reinterpret_cast<const float2 *>(smem + OFF_TAB + b * TAB_BYTES);
    const float2 *tstep = tsub + SUB, *fsubt = tstep + STRIDE, *fstept = fsubt + FSUB;
    const int off = g.offset;
    // ---- decode + fringe-rotate into B1 of both pols: task (n2, o) covers n1 = 8o..8o+7
    {
      const int sbase = (int)(((long long)off >> 1) - (((long long)off >> 1) & ~15LL));
#pragma unroll 1
      for (int task = tid; task < N2 * 8; task += NT) {
        const int n2 = task & (N2 - 1), o = task >> 7;
        const int p0 = (off & 1) + n2;  // sample index relative to byte off/2
        const unsigned char *bp = stage + sbase + (p0 >> 1) + 64 * (8 * o);
        const int sh0 = 2 * (2 * (p0 & 1)), sh1 = sh0 + 2;
        const float2 rs = tsub[n2];
        uint32_t re0[4], im0[4], re1[4], im1[4];
#pragma unroll
        for (int i = 0; i < 8; i += 2) {
          float2 x0[2], x1[2];
#pragma unroll
          for (int u = 0; u < 2; u++) {
            const int n1 = 8 * o + i + u;
            const int byte = bp[64 * (i + u)];
            const float2 rot = cmul(rs, tstep[n1]);
            const float l0 = level2bit((byte >> sh0) & 3), l1 = level2bit((byte >> sh1) & 3);
            x0[u] = make_float2(l0 * rot.x, l0 * rot.y);
            x1[u] = make_float2(l1 * rot.x, l1 * rot.y);
          }
          re0[i >> 1] = pack_h2(x0[0].x, x0[1].x);
          im0[i >> 1] = pack_h2(x0[0].y, x0[1].y);
          re1[i >> 1] = pack_h2(x1[0].x, x1[1].x);
          im1[i >> 1] = pack_h2(x1[0].y, x1[1].y);
        }
        const int so = n2 * 128 + ((o ^ (n2 & 7)) << 4);
        *reinterpret_cast<uint4 *>(smem + OFF_BUF + 0 * KB + so) = make_uint4(re0[0], re0[1], re0[2], re0[3]);
        *reinterpret_cast<uint4 *>(smem + OFF_BUF + 1 * KB + so) = make_uint4(im0[0], im0[1], im0[2], im0[3]);
        *reinterpret_cast<uint4 *>(smem + OFF_BUF + 2 * KB + so) = make_uint4(re1[0], re1[1], re1[2], re1[3]);
        *reinterpret_cast<uint4 *>(smem + OFF_BUF + 3 * KB + so) = make_uint4(im1[0], im1[1], im1[2], im1[3]);
      }
    }
    fence_proxy_async_smem();
    __syncthreads();
    // ---- step 1: D1_pol (TMEM columns 128 pol ..) = A1 B1_pol^T, K = 128
    if (tid == 0) {
      tc_fence_after();
#pragma unroll
      for (int pol = 0; pol < 2; pol++)
#pragma unroll
        for (int kk = 0; kk < 8; kk++) {
          const uint32_t o = (uint32_t)((kk >> 2) * KB + (kk & 3) * 32);
          mma_f16(tmem + 128 * pol, desc_sw128(sbase + OFF_A1 + o),
                  desc_sw128(sbase + OFF_BUF + pol * 2 * KB + o), IDESC, kk > 0 ? 1u : 0u);
        }
      mma_commit(smem_u32(&bar_mma1));
    }
    pending = 1;
    // the next window's bytes and tables load while the MMAs run (its buffer's last reader, the
    // previous window's epilogue, finished before the barrier at the top of this iteration)
    if (w + G < nwin) stage_window(p, w + G, smem, b ^ 1);
    ok = mbar_wait(smem_u32(&bar_mma1), phase & 1, p.err);
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    pending = 0;
    tc_fence_after();
    // ---- twiddle, FP16, into A3 (rows pol*64 + k1, K = [Re Y' n2 0..127 | Im Y' n2 0..127]);
    //      warp group wg takes pol wg & 1 and half wg >> 1 of the n2 columns
    {
      const int q = warp & 3, wg = warp >> 2, pol = wg & 1;
      const int c = 32 * q + lane, k1 = c >> 1, part = c & 1;
      const int m = pol * 64 + k1;
      constexpr int JPER = 8 / (NWG / 2);
#pragma unroll 1
      for (int j = (wg >> 1) * JPER; j < (wg >> 1) * JPER + JPER; j++) {
        float v[16], pv[16];
        tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(128 * pol + 16 * j), v);
#pragma unroll
        for (int i = 0; i < 16; i++) pv[i] = __shfl_xor_sync(0xffffffffu, v[i], 1);
        const float2 wh = thi[j * 64 + k1];
        uint32_t h[8];
#pragma unroll
        for (int i = 0; i < 16; i += 2) {
          float y[2];
#pragma unroll
          for (int u = 0; u < 2; u++) {
            const float2 tw = cmul(wh, tlo[(i + u) * 64 + k1]);
            const float yr = part ? pv[i + u] : v[i + u], yi = part ? v[i + u] : pv[i + u];
            y[u] = part ? fmaf(yr, tw.y, yi * tw.x) : fmaf(yr, tw.x, -(yi * tw.y));
          }
          h[i >> 1] = pack_h2(y[0], y[1]);
        }
        // the two threads of a row store to the same positions of different K-blocks: they
        // write their two chunks in opposite orders so the 8-thread store phases see 8 banks
        const int kb = part * 2 + (j >> 2), o0 = 2 * (j & 3);
        unsigned char *row = smem + OFF_BUF + kb * KB + m * 128;
        const uint4 c0 = make_uint4(h[0], h[1], h[2], h[3]), c1 = make_uint4(h[4], h[5], h[6], h[7]);
        const int oa = o0 + part, ob = o0 + 1 - part;
        *reinterpret_cast<uint4 *>(row + ((oa ^ (m & 7)) << 4)) = part ? c1 : c0;
        *reinterpret_cast<uint4 *>(row + ((ob ^ (m & 7)) << 4)) = part ? c0 : c1;
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
      const float2 fs = fsubt[k1];
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
          const float2 fr = cmul(fs, fstept[k2]);
          const float2 z = cmul(make_float2(v[2 * e], v[2 * e + 1]), fr);
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
  // A1[c][K]: c = 2 k1 + part; K-block 0 multiplies Re x[n1], K-block 1 Im x[n1]
  for (int k1 = 0; k1 < N1; k1++)
    for (int n1 = 0; n1 < N1; n1++) {
      const double th = 2.0 * pi * (double)((n1 * k1) % N1) / (double)N1;
      const double cs = cos(th), sn = sin(th);
      put(OFF_A1, 0, 2 * k1, n1, cs);
      put(OFF_A1, 1, 2 * k1, n1, sn);
      put(OFF_A1, 0, 2 * k1 + 1, n1, -sn);
      put(OFF_A1, 1, 2 * k1 + 1, n1, cs);
    }
  // B3[c3][K]: c3 = 2 k2 + part (k2 < 64); K-blocks 0,1: Re Y' n2 0..63, 64..127; 2,3: Im Y'
  for (int k2 = 0; k2 < N2 / 2; k2++)
    for (int n2 = 0; n2 < N2; n2++) {
      const double ps = 2.0 * pi * (double)((n2 * k2) % N2) / (double)N2;
      const double cs = cos(ps), sn = sin(ps);
      const int kb = n2 >> 6, k = n2 & 63;
      put(OFF_B3, kb, 2 * k2, k, cs);
      put(OFF_B3, kb + 2, 2 * k2, k, sn);
      put(OFF_B3, kb, 2 * k2 + 1, k, -sn);
      put(OFF_B3, kb + 2, 2 * k2 + 1, k, cs);
    }
  float2 *th = reinterpret_cast<float2 *>(&img[(size_t)OFF_THI]);
  float2 *tl = reinterpret_cast<float2 *>(&img[(size_t)OFF_TLO]);
  for (int k1 = 0; k1 < N1; k1++) {
    for (int j = 0; j < 8; j++) {
      const double a = -2.0 * pi * (double)((16 * j * k1) % F) / (double)F;
      th[j * 64 + k1] = make_float2((float)cos(a), (float)sin(a));
    }
    for (int i = 0; i < 16; i++) {
      const double a = -2.0 * pi * (double)((i * k1) % F) / (double)F;
      tl[i * 64 + k1] = make_float2((float)cos(a), (float)sin(a));
    }
  }
  cudaError_t e = cudaMalloc(out, img.size());
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*out, img.data(), img.size(), cudaMemcpyHostToDevice);
}

cudaError_t launch_fstage_tc(const Job &job, const void *tables, int t0, int nt, int T, void *chan, int chan_type,
                             float out_scale, cudaStream_t s, const float *cscale) {
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
  cudaError_t e = cudaGetSymbolAddress((void **)&p.err, g_ftc_err);
  if (e != cudaSuccess) return e;
  int dev = 0, nsm = 0;
  e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const long long nwin = (long long)nt * job.nant;
  const unsigned grid = (unsigned)(nwin < nsm ? nwin : nsm);
  if (chan_type == CHAN_F8) {
    auto kern = fstage_tc_kernel<__nv_fp8x2_e4m3>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    kern<<<grid, NT, SMEM_BYTES, s>>>(p);
  } else {
    auto kern = fstage_tc_kernel<__half2>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    kern<<<grid, NT, SMEM_BYTES, s>>>(p);
  }
  return cudaGetLastError();
}

// Reads and clears the error flag of the tensor-core F-stage (a bounded wait expired).
cudaError_t fstage_tc_take_error(int *flag) {
  int zero = 0;
  cudaError_t e = cudaMemcpyFromSymbol(flag, ftc::g_ftc_err, sizeof(int));
  if (e == cudaSuccess && *flag) e = cudaMemcpyToSymbol(ftc::g_ftc_err, &zero, sizeof(int));
  return e;
}

}  // namespace gxc
