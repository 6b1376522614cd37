// tcgen05 tensor-core X-stage: per-channel visibility matrix V_c = X_c X_c^H
// over all streams (antenna x pol) and the FFTs of one block, FP16 inputs,
// FP32 accumulation in tensor memory (TMEM).
//
// Restates the baseline CMAC of FxKernel::process (fxkernel/src/fxkernel.cpp:328-355)
// as a real Gram matrix: with P_c = [Re X_c ; Im X_c] interleaved by row
// (row 2s = Re X_s, row 2s+1 = Im X_s, s = 2*ant + pol) and K = time,
//   G = P_c P_c^T,  Re V[s1][s2] = G[2s1][2s2] + G[2s1+1][2s2+1],
//                   Im V[s1][s2] = G[2s1+1][2s2] - G[2s1][2s2+1].
// One M=N=128, K=16 MMA (kind::f16, A and B the same K-major SW128 smem tile)
// covers g = 128/R channels stacked block-diagonally (R = rows per channel,
// padded to a power of two >= 16); four such groups fill the 512 TMEM columns,
// so a CTA owns CS = 4g channels for the whole FFT block.
//
// Roles (288 threads): producer thread 0 streams the channelised block
// ([ctile][t][stream][16] as the F-stage wrote it) into a 3-stage raw ring with
// TMA tile loads (cp.async.bulk.tensor, completion counted on mbarriers); warps
// 0-7 corner-turn each raw tile from shared memory into K-contiguous rows and
// store them swizzled (SW128) into a 2-stage operand ring; warp 8 allocates TMEM
// and one lane issues the MMAs and commits to the stage-release barriers; warps
// 0-3 then read TMEM (tcgen05.ld) and fold the Gram entries into the compensated
// visibility accumulators.  The 33-64 antenna kernel loads with plain gathers.
// Every mbarrier wait is bounded (iteration cap and %globaltimer); on expiry
// the kernel raises an error flag, lets issued MMAs drain, frees TMEM and exits.
#include <cuda.h>
#include <stdint.h>

#include <type_traits>

#include "gxc_internal.h"
#include "tcgen05_util.cuh"

namespace gxc {

namespace tc {

constexpr int STAGES = 2;                        // operand (SW128) stages
// Raw ring of the TMA-fed kernels: each stage holds one TMA tile of the channelised
// block, [t][stream][channels of this CTA] as stored, at most 32 KiB.
constexpr int RSTAGES = 3;
constexpr int RAW_BYTES = 32768;
constexpr int TILE_BYTES = 128 * 128;            // 128 rows x 128 bytes (one SW128 K-major tile)
constexpr int NPROD_WARPS = 8;
constexpr int NPROD = NPROD_WARPS * 32;
constexpr int NTHREADS = NPROD + 32;             // 33-64 antenna kernel: producers + MMA warp
constexpr int NTHREADS_TC = NPROD + 64;          // TMA-fed kernel: producers + MMA warp + TMA warp
constexpr int TMA_WARP = NPROD_WARPS + 1;

// FP16 path: one FP16 tile per group, K = 64 FFTs per stage, 4 groups (512 TMEM columns).
// SPLIT path (FP32 data): each value x is split into hi = TF32(x) (low 13 mantissa
// bits cleared) and lo = x - hi (exact); hi.hi^T + lo.hi^T + hi.lo^T is accumulated
// in FP32 with kind::tf32 MMAs (every product exact, relative error ~2^-20).
// Two tiles (hi, lo) per group, K = 32 FFTs per stage, 2 groups (256 TMEM columns).
template <bool SPLIT>
struct Cfg {
  static constexpr int KC = SPLIT ? 32 : 64;
  static constexpr int NG = SPLIT ? 2 : 4;
  static constexpr int TILES = SPLIT ? 2 : 1;
  static constexpr int KSTEP = SPLIT ? 8 : 16;
  static constexpr int GROUP_BYTES = TILES * TILE_BYTES;
  static constexpr int STAGE_BYTES = NG * GROUP_BYTES;  // 64 KiB
  static constexpr int TMEM_COLS = NG * 128;
};

struct Params {
  const void *chan;     // [ctile][T][n][16] half2 (FP16 path) or float2 (SPLIT path)
  int nant, nstream, nchan, T, nt, autos;
  int R, g, CS;         // rows per channel block, channels per MMA group, channels per CTA
  float2 *vsum, *vcomp;
  int *err;
  // TMA raw tiles (small-N kernels): box = rbx channels x nstream x rkc FFTs, rnbox boxes
  // (channel tiles) per raw chunk, rbox_bytes each
  int rbx, rnbox, rkc, rbox_bytes;
  // FP16 hi/lo split (FP32 data of known scale): values are multiplied by split_sc (a power of
  // two) before the split, and the Gram sums by split_unsc (its inverse squared) at the end
  float split_sc, split_unsc;
  // split of the block's FFTs across CTAs (FP16 / FP8 kernel): CTA b covers channel group
  // b mod (grid/kparts) and FFTs [kspan*part, kspan*(part+1)) of the block, part = b / (grid/kparts),
  // accumulating into plane `part` of vsum/vcomp (planes `plane` elements apart)
  int kparts, kspan;
  size_t plane;
  // FP16 / FP8 kernel: persist = 1 runs one CTA per SM over equal shares of all (group, chunk)
  // units; ngrp = channel groups of the launch
  int persist, ngrp;
};

// Adds val[i] into the compensated accumulators (vsum, vcomp) at off[i], for every i < N with
// use[i].  All loads of the batch are issued before its first store, so their latencies overlap
// (one load-add-store at a time waited a full memory round trip per output: in the FP16
// X-stage that was about a quarter of each CTA's time).
template <int N>
__device__ __forceinline__ void rmw_batch(float2 *vsum, float2 *vcomp, const size_t (&off)[N],
                                          const float2 (&val)[N], const bool (&use)[N]) {
  float2 sm[N], e[N];
#pragma unroll
  for (int i = 0; i < N; i++)
    if (use[i]) {
      sm[i] = vsum[off[i]];
      e[i] = vcomp[off[i]];
    }
#pragma unroll
  for (int i = 0; i < N; i++)
    if (use[i]) {
      two_sum_add(sm[i].x, e[i].x, val[i].x);
      two_sum_add(sm[i].y, e[i].y, val[i].y);
      vsum[off[i]] = sm[i];
      vcomp[off[i]] = e[i];
    }
}

// FP16 and FP8 paths: one accumulation over each segment of the FFT block (its TMEM rounding
// bias, ~1e-5 over 2048 FFTs, is far below the FP16 / FP8 quantisation error).
// A 128-byte SW128 row holds 64 FFTs of FP16 or 128 FFTs of FP8 (E4M3) values;
// either way one MMA consumes 32 bytes of every row (K = 16 or 32).
//
// Work is a list of segments per CTA, each a run of K chunks [k0, k1) (KC FFTs each) of one
// channel group g: the block's TMEM accumulation of that run, then its epilogue.  A segment that
// starts at chunk 0 adds into accumulator plane 0, one that starts later into plane 1;
// finalisation adds the planes.
//   persist = 0: grid = groups x kparts; CTA b covers group b mod groups, the chunks of its part.
//   persist = 1: grid = the SM count G, groups >= G.  CTA b takes whole groups b, b + G, ... for
//     the full rounds, so the CTAs running together work on neighbouring groups (two groups share
//     every 64-byte row of a 16-channel tile, read from DRAM once); the groups of the last,
//     partial round are halved in K and shared by pairs of CTAs when they are at most half the
//     CTAs, so fewer SMs wait out a last partial wave.  Each group is split at most once.
// Returns false past the CTA's last segment (an empty half is skipped, not returned).
__device__ __forceinline__ bool xstage_seg(const Params &p, int nck, int KC, int i, int *g, int *k0, int *k1) {
  if (!p.persist) {
    if (i > 0) return false;
    const int kpart = (int)blockIdx.x / p.ngrp;
    const int kck = (p.kspan + KC - 1) / KC;  // chunks of one part (kspan = nt when unsplit)
    *g = (int)blockIdx.x - kpart * p.ngrp;
    *k0 = kpart * kck;
    *k1 = *k0 + kck < nck ? *k0 + kck : nck;
    return *k1 > *k0;
  }
  const int G = (int)gridDim.x, b = (int)blockIdx.x;
  const int rounds = p.ngrp / G, rem = p.ngrp - rounds * G;
  if (i < rounds) {
    *g = i * G + b;
    *k0 = 0;
    *k1 = nck;
    return true;
  }
  if (i > rounds) return false;
  if (2 * rem > G) {  // too many leftover groups to halve: whole groups, one per CTA
    if (b >= rem) return false;
    *g = rounds * G + b;
    *k0 = 0;
    *k1 = nck;
    return true;
  }
  if (b >= 2 * rem) return false;
  const int kh = (nck + 1) / 2;
  *g = rounds * G + b / 2;
  *k0 = (b & 1) ? kh : 0;
  *k1 = (b & 1) ? nck : kh;
  return *k1 > *k0;
}

template <bool F8>
__global__ void __launch_bounds__(NTHREADS_TC, 1) xstage_tc_kernel(Params p, const __grid_constant__ CUtensorMap tmap) {
  using C = Cfg<false>;
  constexpr int KC = F8 ? 128 : C::KC, KSTEP = F8 ? 32 : C::KSTEP;
  constexpr int NG = C::NG, GROUP_BYTES = C::GROUP_BYTES, STAGE_BYTES = C::STAGE_BYTES;
  constexpr int TMEM_COLS = C::TMEM_COLS;
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar_full[STAGES], bar_empty[STAGES], raw_full[RSTAGES], raw_empty[RSTAGES],
      bar_done, bar_tfree, bar_final, bar_stg[2];
  __shared__ uint32_t tmem_base_sh;
  // 128-byte swizzle atoms need 1024-byte alignment of the shared-window address
  unsigned char *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  const uint32_t sbase = smem_u32(smem);
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int n = p.nstream;
  const int nck = (p.nt + KC - 1) / KC;  // K chunks of a group

  // zero the padding rows (2n..R-1 of each channel block) of the ring; producers never write
  // them (done here once, and again after each segment epilogue, which stages its results in
  // the idle ring)
  auto zero_padding = [&](int t0, int nthr) {
    if (2 * n >= p.R) return;
    const int pad = p.R - 2 * n;
    const int per_stage = NG * p.g * pad * 8;  // 16-byte words
    for (int i = t0; i < STAGES * per_stage; i += nthr) {
      const int st = i / per_stage, r0 = i - st * per_stage;
      const int w = r0 & 7, rr = r0 >> 3;
      const int G = rr / (p.g * pad), rem = rr - G * p.g * pad;
      const int gi = rem / pad, row = gi * p.R + 2 * n + (rem - gi * pad);
      *reinterpret_cast<uint4 *>(smem + (size_t)st * STAGE_BYTES + G * GROUP_BYTES + row * 128 + w * 16) =
          make_uint4(0, 0, 0, 0);
    }
  };
  zero_padding(tid, NTHREADS_TC);
  if (tid == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(smem_u32(&bar_full[s]), NPROD);
      mbar_init(smem_u32(&bar_empty[s]), 1);
    }
    for (int s = 0; s < RSTAGES; s++) {
      mbar_init(smem_u32(&raw_full[s]), 1);
      mbar_init(smem_u32(&raw_empty[s]), NPROD_WARPS);
    }
    mbar_init(smem_u32(&bar_done), 1);
    mbar_init(smem_u32(&bar_tfree), NPROD_WARPS);  // every producer warp has read its share of a segment's TMEM
    mbar_init(smem_u32(&bar_final), 1);
    mbar_init(smem_u32(&bar_stg[0]), NPROD);  // the producers have staged a segment's results
    mbar_init(smem_u32(&bar_stg[1]), NPROD);  // ... and added them into the accumulators
    fence_mbar_init();
  }
  if (warp == NPROD_WARPS) {
    tmem_alloc(smem_u32(&tmem_base_sh), TMEM_COLS);
    tmem_relinquish();
  }
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_sh;

  constexpr int TK = F8 ? 16 : 8;             // FFTs per 16-byte K chunk of a row
  constexpr int ESZ = F8 ? 2 : 4;             // bytes per complex value
  const int KCR = p.rkc;                      // FFTs per raw chunk (divides KC)
  const int RPO = KC / KCR;                   // raw chunks per operand stage
  if (warp == TMA_WARP) {
    // ------------------------------------------------------------ TMA producer
    // One lane streams every segment's chunks through the raw ring: one box per channel tile,
    // [t][stream][rbx channels] as stored, rows past the block's FFT count zero-filled.
    if (lane == 0) {
      const uint32_t raw_s = sbase + STAGES * STAGE_BYTES;
      int rc = 0;  // raw chunks issued by this CTA
      bool ok = true;
      int g, k0, k1;
      for (int i = 0; ok && xstage_seg(p, nck, KC, i, &g, &k0, &k1); i++) {
        const int cb = g * p.CS;
        const int x0 = p.rnbox == 1 ? ((cb & 15) & ~(p.rbx - 1)) : 0;
        for (int k = k0; k < k1 && ok; k++)
          for (int r = 0; r < RPO; r++, rc++) {
            const int rs = rc % RSTAGES;
            if (rc >= RSTAGES && !mbar_wait(smem_u32(&raw_empty[rs]), ((rc / RSTAGES) - 1) & 1, p.err)) {
              ok = false;
              break;
            }
            const uint32_t bar = smem_u32(&raw_full[rs]);
            mbar_expect_tx(bar, (uint32_t)(p.rbox_bytes * p.rnbox));
            for (int j = 0; j < p.rnbox; j++)
              tma_load_4d(raw_s + rs * RAW_BYTES + j * p.rbox_bytes, &tmap, x0, 0, k * KC + r * KCR, (cb >> 4) + j,
                          bar);
          }
      }
      // every copy issued lands before the CTA can exit (the last RSTAGES are the only
      // ones possibly unconsumed, and no later phase of their stages was started)
      for (int c = rc > RSTAGES ? rc - RSTAGES : 0; c < rc; c++)
        mbar_wait_drain(smem_u32(&raw_full[c % RSTAGES]), (c / RSTAGES) & 1);
    }
  } else if (warp < NPROD_WARPS) {
    // ------------------------------------------------------------ producers (+ epilogue: warps 0-3)
    // Corner-turn each raw chunk into K-contiguous SW128 rows of the operand stage;
    // every warp releases the raw stage on its own (raw_empty counts warps).  After a
    // segment's last chunk warps 0-3 fold its TMEM sums into the accumulators.
    const int BX = p.rbx, boxb = p.rbox_bytes;
    const unsigned char *raw0 = smem + STAGES * STAGE_BYTES;
    const int nq = p.CS / 4;                  // channel quads (CS >= 4)
    const int kq = KCR / TK;                  // K chunks per raw chunk
    const int ntask = kq * n * nq;            // (channel quad, stream, K chunk) per raw chunk
    const size_t tstride = (size_t)n * BX * ESZ;  // bytes between FFT rows of a box
    // A thread's tasks are the same in every raw chunk: tid and tid + NPROD (the launcher
    // keeps ntask <= 2 NPROD).  Decoded once here, packed as q | s << 8 | o << 16, so the
    // chunk loop does no integer division; g and R are powers of two.
    auto decode = [&](int task) {
      const int rest = task / nq, o = rest / n;
      return (task - rest * nq) | ((rest - o * n) << 8) | (o << 16);
    };
    const int tpk0 = decode(tid), tpk1 = decode(tid + NPROD);
    const int lg = 31 - __clz(p.g), lr = 31 - __clz(p.R);
    const int lcs = 31 - __clz(p.CS);  // CS is a power of two
    const int nbl = p.nant * (p.nant - 1) / 2 + (p.autos ? p.nant : 0);
    const int nent = nbl * 4 * p.CS;   // staged values of a segment (fits the operand ring)
    bool ok = true;
    int ch = 0;  // operand chunks produced by this CTA
    int sg = 0;  // segments finished
    int g, k0, k1;
    for (int i = 0; ok && xstage_seg(p, nck, KC, i, &g, &k0, &k1); i++) {
      const int cb = g * p.CS;  // first channel of the segment
      const int x0 = p.rnbox == 1 ? ((cb & 15) & ~(BX - 1)) : 0;
      const int cofs = p.rnbox == 1 ? (cb & 15) - x0 : 0;  // box index of the segment's first channel
      for (int k = k0; k < k1 && ok; k++, ch++) {
        const int st = ch % STAGES;
        if (ch >= STAGES && !mbar_wait(smem_u32(&bar_empty[st]), ((ch / STAGES) - 1) & 1, p.err)) {
          ok = false;
          break;
        }
        unsigned char *stage = smem + (size_t)st * STAGE_BYTES;
        for (int r = 0; r < RPO; r++) {
          const int rc = ch * RPO + r;
          const int rs = rc % RSTAGES;
          if (!mbar_wait(smem_u32(&raw_full[rs]), (rc / RSTAGES) & 1, p.err)) {
            ok = false;
            break;
          }
          const unsigned char *raw = raw0 + rs * RAW_BYTES;
            // task = (channel quad q, stream s, K chunk o), q then s fastest across lanes:
            // a warp reads consecutive 16-byte (or 8-byte) pieces of one FFT row
            {
    #pragma unroll 1
              for (int u2 = 0; u2 < 2; u2++) {
                const int task = tid + u2 * NPROD;
                if (task >= ntask) break;
                const int pk = u2 ? tpk1 : tpk0;
                const int q = pk & 255, s = (pk >> 8) & 255, o = pk >> 16;
                const int oo = r * kq + o;      // K chunk within the 128-byte row
                const int cc0 = cofs + 4 * q;   // first channel of the quad, counted in the boxes
                // which of the pair (re row, im row) this lane stores first: among 8 lanes the
                // first stores then cover all 8 swizzle positions (no bank conflicts)
                const int sw = nq == 1 ? ((s >> 2) & 1) : (q & 1);
                const unsigned char *src =
                    raw + (cc0 >> 4) * boxb + ((size_t)(o * TK) * n + s) * BX * ESZ + (cc0 & 15) * ESZ;
                if constexpr (F8) {
                  // 16 FFTs x 4 channels of E4M3 pairs (8 bytes per FFT) -> 8 rows (4 channels x re/im)
                  // of 16 FFT bytes: two prmt gather one channel's (re, im) bytes of 2 FFTs each, a
                  // third and fourth split them into 4 re bytes and 4 im bytes
                  uint2 v[16];
    #pragma unroll
                  for (int i = 0; i < 16; i++) v[i] = *reinterpret_cast<const uint2 *>(src + i * tstride);
    #pragma unroll
                  for (int ci = 0; ci < 4; ci++) {
                    const int cc = 4 * q + ci;
                    const int G = cc >> lg, gi = cc & (p.g - 1);
                    const int row = (gi << lr) + 2 * s;
                    const uint32_t sel = (ci & 1) ? 0x7362u : 0x5140u;
                    uint32_t re[4], im[4];
    #pragma unroll
                    for (int k = 0; k < 4; k++) {
                      const uint32_t a0 = (ci < 2) ? v[4 * k].x : v[4 * k].y;
                      const uint32_t a1 = (ci < 2) ? v[4 * k + 1].x : v[4 * k + 1].y;
                      const uint32_t a2 = (ci < 2) ? v[4 * k + 2].x : v[4 * k + 2].y;
                      const uint32_t a3 = (ci < 2) ? v[4 * k + 3].x : v[4 * k + 3].y;
                      const uint32_t t0 = prmt(a0, a1, sel), t1 = prmt(a2, a3, sel);
                      re[k] = prmt(t0, t1, 0x5410);
                      im[k] = prmt(t0, t1, 0x7632);
                    }
                    const uint4 vre = make_uint4(re[0], re[1], re[2], re[3]);
                    const uint4 vim = make_uint4(im[0], im[1], im[2], im[3]);
                    const int ra = row + sw, rb = row + 1 - sw;
                    unsigned char *gbase = stage + G * GROUP_BYTES;
                    *reinterpret_cast<uint4 *>(gbase + ra * 128 + ((oo ^ (ra & 7)) << 4)) = sw ? vim : vre;
                    *reinterpret_cast<uint4 *>(gbase + rb * 128 + ((oo ^ (rb & 7)) << 4)) = sw ? vre : vim;
                  }
                } else {
                  // 8 FFTs x 4 channels of FP16 complex -> 8 rows (4 channels x re/im) of 8 FFTs
                  uint4 v[8];
    #pragma unroll
                  for (int i = 0; i < 8; i++) v[i] = *reinterpret_cast<const uint4 *>(src + i * tstride);
    #pragma unroll
                  for (int ci = 0; ci < 4; ci++) {
                    const int cc = 4 * q + ci;
                    const int G = cc >> lg, gi = cc & (p.g - 1);
                    const int row = (gi << lr) + 2 * s;
                    uint32_t w[8];
    #pragma unroll
                    for (int i = 0; i < 8; i++)
                      w[i] = (ci == 0) ? v[i].x : (ci == 1) ? v[i].y : (ci == 2) ? v[i].z : v[i].w;
                    const uint4 vre = make_uint4(prmt(w[0], w[1], 0x5410), prmt(w[2], w[3], 0x5410),
                                                 prmt(w[4], w[5], 0x5410), prmt(w[6], w[7], 0x5410));
                    const uint4 vim = make_uint4(prmt(w[0], w[1], 0x7632), prmt(w[2], w[3], 0x7632),
                                                 prmt(w[4], w[5], 0x7632), prmt(w[6], w[7], 0x7632));
                    const int ra = row + sw, rb = row + 1 - sw;
                    unsigned char *gbase = stage + G * GROUP_BYTES;
                    *reinterpret_cast<uint4 *>(gbase + ra * 128 + ((oo ^ (ra & 7)) << 4)) = sw ? vim : vre;
                    *reinterpret_cast<uint4 *>(gbase + rb * 128 + ((oo ^ (rb & 7)) << 4)) = sw ? vre : vim;
                  }
                }
              }
            }
          __syncwarp();  // this warp's reads of the raw stage are done (their values are stored)
          if (lane == 0) mbar_arrive(smem_u32(&raw_empty[rs]));
        }
        if (!ok) break;
        fence_proxy_async_smem();
        mbar_arrive(smem_u32(&bar_full[st]));
      }
      if (!ok) break;
      // ------------------------------------------------------------ epilogue of the segment
      // The segment's MMAs are done, so the operand ring is idle until the producers start the
      // next segment: the eight producer warps stage the segment's visibilities there, as
      // [baseline x product][CS channels], and release tensor memory; then all of them add the
      // staged values into the accumulators, CS consecutive channels of a (baseline, product)
      // contiguous in memory, so a warp's loads and stores touch 8 sectors instead of 32.
      // Warp w reads TMEM lane quarter w % 4 (the lanes a warp may access) of the groups
      // G = w / 4, w / 4 + 2.  The two producer-wide syncs are mbarriers with bounded waits.
      {
        float2 *const stg = reinterpret_cast<float2 *>(smem);
        ok = mbar_wait(smem_u32(&bar_done), sg & 1, p.err);
        tc_fence_after();
        if (ok) {
          const int wq = warp & 3;  // TMEM lane quarter
          const int row = 32 * wq + lane;
          const int my_gi = row / p.R;
          const int r = row - my_gi * p.R;
          const int s1 = r >> 1, part1 = r & 1;
          const int gi0 = (32 * wq) / p.R;
          const int col0 = gi0 * p.R;
          const int clen = p.R > 32 ? p.R : 32;
          const int j = s1 >> 1, l = s1 & 1;
          for (int G = warp >> 2; G < NG; G += 2) {
            const int cl = G * p.g + my_gi;  // channel within the CTA's CS
            for (int pc = 0; pc < clen; pc += 16) {
              __syncwarp();  // tcgen05.ld is warp-collective: reconverge after the divergent skip below
              const int col = col0 + pc;
              float v[16], pv[16];
              tmem_ld16(tmem + ((uint32_t)(32 * wq) << 16) + (uint32_t)(G * 128 + col), v);
#pragma unroll
              for (int q = 0; q < 16; q++) pv[q] = __shfl_xor_sync(0xffffffffu, v[q], 1);
              if (col < my_gi * p.R || col >= (my_gi + 1) * p.R || s1 >= n) continue;
              const int s2b = (col - my_gi * p.R) >> 1;
#pragma unroll
              for (int qq = 0; qq < 4; qq++) {
                const int q = qq + 4 * part1;
                const int s2 = s2b + q;
                if (s2 >= n) continue;
                const int k = s2 >> 1, m = s2 & 1;
                if (j > k || (j == k && !p.autos)) continue;
                float re, im;
                if (part1 == 0) {
                  re = v[2 * q] + pv[2 * q + 1];
                  im = pv[2 * q] - v[2 * q + 1];
                } else {
                  re = pv[2 * q] + v[2 * q + 1];
                  im = v[2 * q] - pv[2 * q + 1];
                }
                const int bl = baseline_index(j, k, p.nant);
                stg[((bl * 4 + 2 * l + m) << lcs) + cl] = make_float2(re, im);
              }
            }
          }
        }
        // this warp's TMEM reads of the segment are done: the MMAs of the next segment may
        // overwrite the accumulators
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&bar_tfree));
        mbar_arrive(smem_u32(&bar_stg[0]));
        ok = ok && mbar_wait(smem_u32(&bar_stg[0]), sg & 1, p.err);
        if (ok) {
          float2 *const vsum = p.vsum + (k0 > 0 ? p.plane : 0);
          float2 *const vcomp = p.vcomp + (k0 > 0 ? p.plane : 0);
          for (int e0 = tid; e0 < nent; e0 += 8 * NPROD) {
            size_t off[8];
            float2 val[8];
            bool use[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
              const int e = e0 + u * NPROD;
              use[u] = e < nent;
              off[u] = (size_t)(e >> lcs) * p.nchan + cb + (e & (p.CS - 1));
              val[u] = use[u] ? stg[e] : make_float2(0.f, 0.f);
            }
            rmw_batch<8>(vsum, vcomp, off, val, use);
          }
        }
        mbar_arrive(smem_u32(&bar_stg[1]));
        ok = ok && mbar_wait(smem_u32(&bar_stg[1]), sg & 1, p.err);
        zero_padding(tid, NPROD);  // the staging overwrote them; the next stage's fence covers these writes
      }
      sg++;
    }
  } else if (lane == 0) {
    // ------------------------------------------------------------ MMA issuer
    int ch = 0, sg = 0;
    bool ok = true;
    int g, k0, k1;
    for (int i = 0; ok && xstage_seg(p, nck, KC, i, &g, &k0, &k1); i++) {
      // the previous segment's epilogue has read the accumulators this one starts afresh
      if (sg > 0 && !mbar_wait(smem_u32(&bar_tfree), (sg - 1) & 1, p.err)) break;
      tc_fence_after();
      for (int k = k0; k < k1; k++, ch++) {
        const int st = ch % STAGES;
        if (!mbar_wait(smem_u32(&bar_full[st]), (ch / STAGES) & 1, p.err)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t sa = sbase + st * STAGE_BYTES;
#pragma unroll
        for (int G = 0; G < NG; G++) {
#pragma unroll
          for (int kk = 0; kk < KC / KSTEP; kk++) {
            const uint32_t acc = (k > k0 || kk > 0) ? 1u : 0u;
            const uint64_t dh = desc_sw128(sa + G * GROUP_BYTES + kk * 32);
            if constexpr (F8) mma_f8(tmem + G * 128, dh, dh, IDESC, acc);
            else mma_f16(tmem + G * 128, dh, dh, IDESC, acc);
          }
        }
        mma_commit(smem_u32(&bar_empty[st]));
      }
      if (!ok) break;
      mma_commit(smem_u32(&bar_done));
      sg++;
    }
    mma_commit(smem_u32(&bar_final));
    mbar_wait(smem_u32(&bar_final), 0, p.err);  // issued MMAs drained before TMEM is freed
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == NPROD_WARPS) tmem_dealloc(tmem, TMEM_COLS);
}


// SPLIT path with periodic drains.  TMEM accumulation rounds towards zero, so
// its relative bias grows with the number of MMAs accumulated; here the MMA
// issuer alternates between two accumulator sets every DP stages (DP*KC = 128
// FFTs) and four dedicated epilogue warps fold each finished set into
// per-thread FP32 register sums (round-to-nearest) while the other set fills.
// R (rows per channel block) is a template parameter so the register sums are
// indexed at compile time.
constexpr int NEPI_WARPS = 4;
constexpr int NTHREADS_SPLIT = NPROD + 32 + NEPI_WARPS * 32 + 32;  // + TMA warp (the last)
// 14 warps put 4 on one of the SM's four 16K-register sub-partitions: at most 128 registers
// per thread (the R = 128 epilogue's 128 register sums then spill a little)
constexpr int TMA_WARP_SPLIT = NPROD_WARPS + 1 + NEPI_WARPS;

// H16 = false: TF32 hi (top 11 significand bits) and lo halves, kind::tf32, 32 FFTs per stage.
// H16 = true: FP16 hi and lo halves of the scaled value (the same 22 significand bits for
// values in FP16's normal range; a subnormal lo only adds an absolute error near 2^-25),
// kind::f16 at twice the tf32 rate and half the shared-memory bytes, 64 FFTs per stage.  Used
// where the data's scale is known (the F-stage's output): FP16's exponent range must hold it.
template <int R, bool H16>
__global__ void __launch_bounds__(NTHREADS_SPLIT, 1) xstage_tc_split_kernel(Params p,
                                                                            const __grid_constant__ CUtensorMap tmap) {
  using C = Cfg<true>;
  constexpr int KC = H16 ? 64 : C::KC, KSTEP = H16 ? 16 : C::KSTEP;
  constexpr int TKC = H16 ? 8 : 4;       // FFTs per 16-byte chunk of an operand row
  constexpr int NG = C::NG, GROUP_BYTES = C::GROUP_BYTES, STAGE_BYTES = C::STAGE_BYTES;
  constexpr int NSET = 2, SET_COLS = NG * 128, TMEM_COLS = NSET * SET_COLS;  // 512
  constexpr int DP = 128 / KC;           // stages per drain period (128 FFTs)
  constexpr int GCH = 128 / R;           // channels per MMA group
  constexpr int WP = (R > 32 ? R : 32) / 16;  // 16-column pieces a warp reads per group
  constexpr int PP = R / 16;             // pieces in one channel block
  static_assert(TMEM_COLS == 512, "TMEM budget");
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar_full[STAGES], bar_empty[STAGES], raw_full[RSTAGES], raw_empty[RSTAGES],
      bar_ready[NSET], bar_drained[NSET], bar_done;
  __shared__ uint32_t tmem_base_sh;
  unsigned char *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  const uint32_t sbase = smem_u32(smem);
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int cb = blockIdx.x * p.CS;
  const int n = p.nstream;
  const int nchunks = (p.nt + KC - 1) / KC;
  const int nper = (nchunks + DP - 1) / DP;

  if (2 * n < R) {  // zero the padding rows of both tiles (hi, lo) of every group of every stage
    const int pad = R - 2 * n;
    const int per_stage = NG * GCH * pad * 8 * 2;
    for (int i = tid; i < STAGES * per_stage; i += NTHREADS_SPLIT) {
      const int st = i / per_stage, r0 = i - st * per_stage;
      const int w = r0 & 7, rr = (r0 >> 3) >> 1, tile = (r0 >> 3) & 1;
      const int G = rr / (GCH * pad), rem = rr - G * GCH * pad;
      const int gi = rem / pad, row = gi * R + 2 * n + (rem - gi * pad);
      *reinterpret_cast<uint4 *>(smem + (size_t)st * STAGE_BYTES + G * GROUP_BYTES + tile * TILE_BYTES + row * 128 +
                                 w * 16) = make_uint4(0, 0, 0, 0);
    }
  }
  if (tid == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(smem_u32(&bar_full[s]), NPROD);
      mbar_init(smem_u32(&bar_empty[s]), 1);
    }
    for (int s = 0; s < RSTAGES; s++) {
      mbar_init(smem_u32(&raw_full[s]), 1);
      mbar_init(smem_u32(&raw_empty[s]), NPROD_WARPS);
    }
    for (int b = 0; b < NSET; b++) {
      mbar_init(smem_u32(&bar_ready[b]), 1);
      mbar_init(smem_u32(&bar_drained[b]), NEPI_WARPS * 32);
    }
    mbar_init(smem_u32(&bar_done), 1);
    fence_mbar_init();
  }
  if (warp == NPROD_WARPS) {
    tmem_alloc(smem_u32(&tmem_base_sh), TMEM_COLS);
    tmem_relinquish();
  }
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_sh;

  const int KCR = p.rkc;      // FFTs per raw chunk (divides KC)
  const int RPO = KC / KCR;   // raw chunks per operand stage
  const int nraw = nchunks * RPO;
  if (warp == TMA_WARP_SPLIT) {
    // ------------------------------------------------------------ TMA producer
    // One lane streams the block through the raw ring (raw chunks of KCR FFTs, one box per
    // channel tile, rows past the block zero-filled).
    if (lane == 0) {
      const int x0 = p.rnbox == 1 ? ((cb & 15) & ~(p.rbx - 1)) : 0;
      const uint32_t raw_s = sbase + STAGES * STAGE_BYTES;
      int issued = 0;
      for (int rc = 0; rc < nraw; rc++) {
        const int rs = rc % RSTAGES;
        if (rc >= RSTAGES && !mbar_wait(smem_u32(&raw_empty[rs]), ((rc / RSTAGES) - 1) & 1, p.err)) break;
        const uint32_t bar = smem_u32(&raw_full[rs]);
        mbar_expect_tx(bar, (uint32_t)(p.rbox_bytes * p.rnbox));
        for (int j = 0; j < p.rnbox; j++)
          tma_load_4d(raw_s + rs * RAW_BYTES + j * p.rbox_bytes, &tmap, x0, 0, rc * KCR, (cb >> 4) + j, bar);
        issued = rc + 1;
      }
      for (int rc = issued > RSTAGES ? issued - RSTAGES : 0; rc < issued; rc++)
        mbar_wait_drain(smem_u32(&raw_full[rc % RSTAGES]), (rc / RSTAGES) & 1);
    }
  } else if (warp < NPROD_WARPS) {
    // ------------------------------------------------------------ producers
    // Split each FP32 value of a raw chunk into hi and lo and store both tiles; every warp
    // releases the raw stage on its own (raw_empty counts warps).
    const int BX = p.rbx, boxb = p.rbox_bytes;
    const int x0 = p.rnbox == 1 ? ((cb & 15) & ~(BX - 1)) : 0;
    const int cofs = p.rnbox == 1 ? (cb & 15) - x0 : 0;
    const unsigned char *raw0 = smem + STAGES * STAGE_BYTES;
    const int nq = p.CS / 2;           // channel pairs
    const int kq = KCR / TKC;          // 16-byte K chunks per raw chunk
    const int ntask = kq * n * nq;     // (pair, stream, K chunk) per raw chunk
    const size_t tstride = (size_t)n * BX * 8;  // bytes between FFT rows of a box
    const float sc = p.split_sc;
    // A thread's tasks are the same in every raw chunk: tid and tid + NPROD (the launcher
    // keeps ntask <= 2 NPROD), decoded once here so the chunk loop does no integer division.
    int tq[2], ts[2], to[2];
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const int task = tid + j * NPROD;
      const int rest = task / nq;
      tq[j] = task - rest * nq;
      to[j] = rest / n;
      ts[j] = rest - to[j] * n;
    }
    bool ok = true;
    for (int ch = 0; ch < nchunks && ok; ch++) {
      const int st = ch % STAGES;
      if (ch >= STAGES && !mbar_wait(smem_u32(&bar_empty[st]), ((ch / STAGES) - 1) & 1, p.err)) break;
      unsigned char *stage = smem + (size_t)st * STAGE_BYTES;
      for (int rr = 0; rr < RPO; rr++) {
        const int rc = ch * RPO + rr;
        const int rs = rc % RSTAGES;
        if (!mbar_wait(smem_u32(&raw_full[rs]), (rc / RSTAGES) & 1, p.err)) {
          ok = false;
          break;
        }
        const unsigned char *raw = raw0 + rs * RAW_BYTES;
        // task = (pair q, stream s, 16-byte K chunk o), q then s fastest across lanes: a warp
        // reads consecutive 16-byte pieces of one FFT row (conflict-free)
        constexpr int UT = H16 ? 1 : 2;  // tasks per thread in flight (TKC float4 loads each)
#pragma unroll
        for (int j0 = 0; j0 < 2; j0 += UT) {
          if (tid + j0 * NPROD >= ntask) break;
          float4 v[UT][TKC];
#pragma unroll
          for (int u2 = 0; u2 < UT; u2++) {
            const int task = tid + (j0 + u2) * NPROD;
            const int q = tq[j0 + u2], s = ts[j0 + u2], o = to[j0 + u2];
            const int cc0 = cofs + 2 * q;
            const unsigned char *src =
                raw + (cc0 >> 4) * boxb + ((size_t)(TKC * o) * n + s) * BX * 8 + (cc0 & 15) * 8;
#pragma unroll
            for (int i = 0; i < TKC; i++)
              v[u2][i] = task < ntask ? *reinterpret_cast<const float4 *>(src + i * tstride)
                                      : make_float4(0.f, 0.f, 0.f, 0.f);
          }
#pragma unroll
          for (int u2 = 0; u2 < UT; u2++) {
            const int task = tid + (j0 + u2) * NPROD;
            if (task >= ntask) break;
            const int q = tq[j0 + u2], s = ts[j0 + u2], o = to[j0 + u2];
            const int oo = rr * kq + o;  // K chunk within the 128-byte row
            // which part (re, im) this lane stores first: among 8 lanes the first stores
            // then cover all 8 swizzle positions (no bank conflicts)
            const int sw = nq == 1 ? ((s >> 2) & 1) : (q & 1);
#pragma unroll
            for (int ci = 0; ci < 2; ci++) {
              const int cc = 2 * q + ci;
              const int G = cc / GCH, gi = cc - G * GCH;
#pragma unroll
              for (int pp = 0; pp < 2; pp++) {
                const int part = pp ^ sw;
                const int row = gi * R + 2 * s + part;
                uint32_t hi[4], lo[4];
                if constexpr (H16) {
#pragma unroll
                  for (int i = 0; i < 4; i++) {
                    const float4 &f0 = v[u2][2 * i], &f1 = v[u2][2 * i + 1];
                    const float x0v = sc * (ci ? (part ? f0.w : f0.z) : (part ? f0.y : f0.x));
                    const float x1v = sc * (ci ? (part ? f1.w : f1.z) : (part ? f1.y : f1.x));
                    // packed conversions (cvt.rn.f16x2.f32): the same round-to-nearest halves,
                    // two values and their packing per instruction
                    const __half2 h = __floats2half2_rn(x0v, x1v);
                    const float2 hb = __half22float2(h);
                    const __half2 lw = __floats2half2_rn(x0v - hb.x, x1v - hb.y);
                    hi[i] = reinterpret_cast<const uint32_t &>(h);
                    lo[i] = reinterpret_cast<const uint32_t &>(lw);
                  }
                } else {
#pragma unroll
                  for (int i = 0; i < 4; i++) {
                    const float4 &f = v[u2][i];
                    const float x = ci ? (part ? f.w : f.z) : (part ? f.y : f.x);
                    hi[i] = __float_as_uint(x) & 0xFFFFE000u;
                    lo[i] = __float_as_uint(x - __uint_as_float(hi[i]));
                  }
                }
                unsigned char *gbase = stage + G * GROUP_BYTES;
                const int swz = (oo ^ (row & 7)) << 4;
                *reinterpret_cast<uint4 *>(gbase + row * 128 + swz) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
                *reinterpret_cast<uint4 *>(gbase + TILE_BYTES + row * 128 + swz) =
                    make_uint4(lo[0], lo[1], lo[2], lo[3]);
              }
            }
          }
        }
        __syncwarp();  // this warp's reads of the raw stage are done (their values are stored)
        if (lane == 0) mbar_arrive(smem_u32(&raw_empty[rs]));
      }
      if (!ok) break;
      fence_proxy_async_smem();
      mbar_arrive(smem_u32(&bar_full[st]));
    }
  } else if (warp == NPROD_WARPS) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      bool ok = true;
      for (int ch = 0; ch < nchunks && ok; ch++) {
        const int st = ch % STAGES;
        const int pd = ch / DP, b = pd & 1;
        const bool first = (ch % DP) == 0;
        if (first && pd >= 2 && !mbar_wait(smem_u32(&bar_drained[b]), ((pd >> 1) - 1) & 1, p.err)) break;
        if (!mbar_wait(smem_u32(&bar_full[st]), (ch / STAGES) & 1, p.err)) break;
        tc_fence_after();
        const uint32_t sa = sbase + st * STAGE_BYTES;
#pragma unroll
        for (int G = 0; G < NG; G++) {
          const uint32_t d = tmem + b * SET_COLS + G * 128;
#pragma unroll
          for (int kk = 0; kk < KC / KSTEP; kk++) {
            const uint64_t dh = desc_sw128(sa + G * GROUP_BYTES + kk * 32);
            const uint64_t dl = desc_sw128(sa + G * GROUP_BYTES + TILE_BYTES + kk * 32);
            if constexpr (H16) {
              mma_f16(d, dh, dh, IDESC, (first && kk == 0) ? 0u : 1u);
              mma_f16(d, dl, dh, IDESC, 1u);
              mma_f16(d, dh, dl, IDESC, 1u);
            } else {
              mma_tf32(d, dh, dh, IDESC_TF32, (first && kk == 0) ? 0u : 1u);
              mma_tf32(d, dl, dh, IDESC_TF32, 1u);
              mma_tf32(d, dh, dl, IDESC_TF32, 1u);
            }
          }
        }
        mma_commit(smem_u32(&bar_empty[st]));
        if ((ch % DP) == DP - 1 || ch == nchunks - 1) mma_commit(smem_u32(&bar_ready[b]));
      }
      mma_commit(smem_u32(&bar_done));
      mbar_wait(smem_u32(&bar_done), 0, p.err);  // every issued MMA has finished before TMEM is freed
    }
  } else {
    // ------------------------------------------------------------ epilogue warps
    const int qd = warp & 3;  // TMEM lane quadrant this warp may access
    const int row = 32 * qd + lane;
    const int my_gi = row / R;
    const int r = row - my_gi * R;
    const int s1 = r >> 1, part1 = r & 1;
    const int gi0 = (32 * qd) / R;
    float2 acc[NG][PP][4];
#pragma unroll
    for (int G = 0; G < NG; G++)
#pragma unroll
      for (int a = 0; a < PP; a++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[G][a][q] = make_float2(0.f, 0.f);
    bool ok = true;
    for (int pd = 0; pd < nper; pd++) {
      const int b = pd & 1;
      if (!mbar_wait(smem_u32(&bar_ready[b]), (pd >> 1) & 1, p.err)) {
        ok = false;
        break;
      }
      tc_fence_after();
#pragma unroll
      for (int G = 0; G < NG; G++) {
#pragma unroll
        for (int pw = 0; pw < WP; pw++) {
          const int col = gi0 * R + 16 * pw;
          float v[16], pv[16];
          tmem_ld16(tmem + ((uint32_t)(32 * qd) << 16) + (uint32_t)(b * SET_COLS + G * 128 + col), v);
#pragma unroll
          for (int q = 0; q < 16; q++) pv[q] = __shfl_xor_sync(0xffffffffu, v[q], 1);
          // piece pw covers block gi0 + (16*pw)/R, piece index within the block (16*pw % R)/16
          const bool mine = (gi0 + (16 * pw) / R) == my_gi;
          const int a = ((16 * pw) % R) / 16;
#pragma unroll
          for (int qq = 0; qq < 4; qq++) {
            const int q = qq + 4 * part1;
            float re, im;
            if (part1 == 0) {
              re = v[2 * q] + pv[2 * q + 1];
              im = pv[2 * q] - v[2 * q + 1];
            } else {
              re = pv[2 * q] + v[2 * q + 1];
              im = v[2 * q] - pv[2 * q + 1];
            }
#pragma unroll
            for (int aa = 0; aa < PP; aa++) {
              if (mine && aa == a) {
                acc[G][aa][qq].x += re;
                acc[G][aa][qq].y += im;
              }
            }
          }
        }
      }
      tc_fence_before();
      mbar_arrive(smem_u32(&bar_drained[b]));
    }
    // Stage the block's visibilities, [baseline x product][CS channels], in the operand ring (idle
    // once the last drain is done: every MMA has finished); all threads then add them into the
    // accumulators below, CS consecutive channels of a (baseline, product) contiguous in memory.
    if (ok && s1 < n) {
      const int j = s1 >> 1, l = s1 & 1;
#pragma unroll
      for (int G = 0; G < NG; G++) {
        const int cl = G * GCH + my_gi;  // channel within the CTA's CS
#pragma unroll
        for (int a = 0; a < PP; a++) {
#pragma unroll
          for (int qq = 0; qq < 4; qq++) {
            const int s2 = 8 * a + qq + 4 * part1;
            if (s2 >= n) continue;
            const int k = s2 >> 1, m = s2 & 1;
            if (j > k || (j == k && !p.autos)) continue;
            const int bl = baseline_index(j, k, p.nant);
            // the Gram sums times split_unsc: exact, a power of two
            reinterpret_cast<float2 *>(smem)[(bl * 4 + 2 * l + m) * p.CS + cl] =
                make_float2(acc[G][a][qq].x * p.split_unsc, acc[G][a][qq].y * p.split_unsc);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (!*(volatile int *)p.err) {  // a timed-out role may have left the staging incomplete
    const int nbl = p.nant * (p.nant - 1) / 2 + (p.autos ? p.nant : 0);
    const int nent = nbl * 4 * p.CS;
    const int lcs = 31 - __clz(p.CS);  // CS is a power of two
    const float2 *stg = reinterpret_cast<const float2 *>(smem);
    for (int e0 = tid; e0 < nent; e0 += 8 * NTHREADS_SPLIT) {
      size_t off[8];
      float2 val[8];
      bool use[8];
#pragma unroll
      for (int u = 0; u < 8; u++) {
        const int e = e0 + u * NTHREADS_SPLIT;
        use[u] = e < nent;
        off[u] = (size_t)(e >> lcs) * p.nchan + cb + (e & (p.CS - 1));
        val[u] = use[u] ? stg[e] : make_float2(0.f, 0.f);
      }
      rmw_batch<8>(p.vsum, p.vcomp, off, val, use);
    }
  }
  if (warp == NPROD_WARPS) tmem_dealloc(tmem, TMEM_COLS);
}


// FP16 path for 33..64 antennas (R = 256 rows per channel, one channel per CTA).
// The Gram matrix is split into M-halves: D_top = P[0:128] P^T (N = 256) and
// D_bot = P[128:256] P[128:256]^T (N = 128); the lower-left block is the
// transpose of D_top's right half and is not needed (only j <= k is output).
// 384 of the 512 TMEM columns; one 32 KiB stage per 64 FFTs (4 stages).
constexpr int BIG_STAGES = 4;
constexpr int BIG_STAGE_BYTES = 256 * 128;
constexpr uint32_t IDESC_N256 = (1u << 4) | ((256u >> 3) << 17) | ((128u >> 4) << 24);

template <bool F8>
__global__ void __launch_bounds__(NTHREADS, 1) xstage_tc_big_kernel(Params p) {
  constexpr int KC = F8 ? 128 : 64, KSTEP = F8 ? 32 : 16;
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar_full[BIG_STAGES], bar_empty[BIG_STAGES], bar_done;
  __shared__ uint32_t tmem_base_sh;
  unsigned char *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  const uint32_t sbase = smem_u32(smem);
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int c = blockIdx.x;  // the one channel of this CTA
  const int n = p.nstream;
  const int nchunks = (p.nt + KC - 1) / KC;

  if (2 * n < 256) {  // zero the padding rows 2n..255 of every stage
    const int per_stage = (256 - 2 * n) * 8;
    for (int i = tid; i < BIG_STAGES * per_stage; i += NTHREADS) {
      const int st = i / per_stage, r0 = i - st * per_stage;
      *reinterpret_cast<uint4 *>(smem + (size_t)st * BIG_STAGE_BYTES + (2 * n + (r0 >> 3)) * 128 + (r0 & 7) * 16) =
          make_uint4(0, 0, 0, 0);
    }
  }
  if (tid == 0) {
    for (int s = 0; s < BIG_STAGES; s++) {
      mbar_init(smem_u32(&bar_full[s]), NPROD);
      mbar_init(smem_u32(&bar_empty[s]), 1);
    }
    mbar_init(smem_u32(&bar_done), 1);
    fence_mbar_init();
  }
  if (warp == NPROD_WARPS) {
    tmem_alloc(smem_u32(&tmem_base_sh), 512);
    tmem_relinquish();
  }
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_sh;

  if (warp < NPROD_WARPS) {
    // task = (stream s, 16-byte K chunk o): 8 FFTs (FP16) or 16 FFTs (FP8) of one stream of this channel
    const int ntask = 8 * n;
    const size_t esz = F8 ? 2 : 4;
    const unsigned char *src = (const unsigned char *)p.chan + (((size_t)(c >> 4) * p.T * n) * CW + (c & 15)) * esz;
    for (int ch = 0; ch < nchunks; ch++) {
      const int st = ch % BIG_STAGES;
      if (ch >= BIG_STAGES && !mbar_wait(smem_u32(&bar_empty[st]), ((ch / BIG_STAGES) - 1) & 1, p.err)) break;
      unsigned char *stage = smem + (size_t)st * BIG_STAGE_BYTES;
      const int tb = ch * KC;
      // four tasks per thread in flight: all their loads are issued before the first
      // corner-turn (the loads are 2- or 4-byte gathers, so latency, not bandwidth, rules)
      constexpr int U = 4;
      constexpr int NL = F8 ? 16 : 8;  // loads per task
      for (int task0 = tid; task0 < ntask; task0 += U * NPROD) {
        uint32_t w[U][NL];
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int task = task0 + u * NPROD;
          const int s = task % n;
          const int o = task / n;
#pragma unroll
          for (int i = 0; i < NL; i++) {
            const int t = tb + NL * o + i;
            if (task < ntask && t < p.nt) {
              const unsigned char *a = src + ((size_t)t * n + s) * CW * esz;
              w[u][i] = F8 ? (uint32_t)__ldg(reinterpret_cast<const unsigned short *>(a))
                           : __ldg(reinterpret_cast<const uint32_t *>(a));
            } else {
              w[u][i] = 0u;
            }
          }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int task = task0 + u * NPROD;
          if (task >= ntask) break;
          const int s = task % n;
          const int o = task / n;
          uint4 re, im;
          if constexpr (F8) {
            // 16 E4M3 pairs (re low byte, im high byte) -> 16 re bytes and 16 im bytes
            uint32_t x[8];
#pragma unroll
            for (int i = 0; i < 8; i++) x[i] = w[u][2 * i] | (w[u][2 * i + 1] << 16);  // re, im, re', im'
            re = make_uint4(prmt(x[0], x[1], 0x6420), prmt(x[2], x[3], 0x6420), prmt(x[4], x[5], 0x6420),
                            prmt(x[6], x[7], 0x6420));
            im = make_uint4(prmt(x[0], x[1], 0x7531), prmt(x[2], x[3], 0x7531), prmt(x[4], x[5], 0x7531),
                            prmt(x[6], x[7], 0x7531));
          } else {
            const uint32_t *x = w[u];
            re = make_uint4(prmt(x[0], x[1], 0x5410), prmt(x[2], x[3], 0x5410), prmt(x[4], x[5], 0x5410),
                            prmt(x[6], x[7], 0x5410));
            im = make_uint4(prmt(x[0], x[1], 0x7632), prmt(x[2], x[3], 0x7632), prmt(x[4], x[5], 0x7632),
                            prmt(x[6], x[7], 0x7632));
          }
          const int row = 2 * s;
          *reinterpret_cast<uint4 *>(stage + row * 128 + ((o ^ (row & 7)) << 4)) = re;
          *reinterpret_cast<uint4 *>(stage + (row + 1) * 128 + ((o ^ ((row + 1) & 7)) << 4)) = im;
        }
      }
      fence_proxy_async_smem();
      mbar_arrive(smem_u32(&bar_full[st]));
    }
  } else if (lane == 0) {
    for (int ch = 0; ch < nchunks; ch++) {
      const int st = ch % BIG_STAGES;
      if (!mbar_wait(smem_u32(&bar_full[st]), (ch / BIG_STAGES) & 1, p.err)) break;
      tc_fence_after();
      const uint32_t sa = sbase + st * BIG_STAGE_BYTES;
#pragma unroll
      for (int kk = 0; kk < KC / KSTEP; kk++) {
        const uint32_t acc = (ch > 0 || kk > 0) ? 1u : 0u;
        const uint64_t dall = desc_sw128(sa + kk * 32);            // rows 0..255 (also the top half's A)
        const uint64_t dbot = desc_sw128(sa + 128 * 128 + kk * 32);  // rows 128..255
        if constexpr (F8) {
          mma_f8(tmem, dall, dall, IDESC_N256, acc);
          mma_f8(tmem + 256, dbot, dbot, IDESC, acc);
        } else {
          mma_f16(tmem, dall, dall, IDESC_N256, acc);                // D_top: rows 0..127 x cols 0..255
          mma_f16(tmem + 256, dbot, dbot, IDESC, acc);               // D_bot: rows 128..255 x cols 128..255
        }
      }
      mma_commit(smem_u32(&bar_empty[st]));
    }
    mma_commit(smem_u32(&bar_done));
    mbar_wait(smem_u32(&bar_done), 0, p.err);
  }

  if (warp < 4) {
    const bool ok = mbar_wait(smem_u32(&bar_done), 0, p.err);
    tc_fence_after();
    if (ok) {
      // half 0: TMEM lane = row a (0..127), columns 0..255;  half 1: lane = row 128 + a, columns 128..255
      for (int half = 0; half < 2; half++) {
        const int arow = 128 * half + 32 * warp + lane;
        const int s1 = arow >> 1, part1 = arow & 1;
        const int j = s1 >> 1, l = s1 & 1;
        const int npc = half ? 8 : 16;
        for (int pc = 0; pc < npc; pc++) {
          __syncwarp();
          float v[16], pv[16];
          const uint32_t col = half ? (256u + 16u * pc) : (16u * pc);
          tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + col, v);
#pragma unroll
          for (int q = 0; q < 16; q++) pv[q] = __shfl_xor_sync(0xffffffffu, v[q], 1);
          if (s1 >= n) continue;
          const int s2b = (half ? 64 : 0) + 8 * pc;
#pragma unroll
          for (int qq = 0; qq < 4; qq++) {
            const int q = qq + 4 * part1;
            const int s2 = s2b + q;
            if (s2 >= n) continue;
            const int k = s2 >> 1, m = s2 & 1;
            if (j > k || (j == k && !p.autos)) continue;
            float re, im;
            if (part1 == 0) {
              re = v[2 * q] + pv[2 * q + 1];
              im = pv[2 * q] - v[2 * q + 1];
            } else {
              re = pv[2 * q] + v[2 * q + 1];
              im = v[2 * q] - pv[2 * q + 1];
            }
            const int bl = baseline_index(j, k, p.nant);
            const size_t o = ((size_t)bl * 4 + 2 * l + m) * p.nchan + c;
            float2 sm = p.vsum[o], e = p.vcomp[o];
            two_sum_add(sm.x, e.x, re);
            two_sum_add(sm.y, e.y, im);
            p.vsum[o] = sm;
            p.vcomp[o] = e;
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == NPROD_WARPS) tmem_dealloc(tmem, 512);
}

// FP16 / FP8 path for 33..64 antennas with two CTA types in one launch; the Gram matrix
// P P^T of a channel (256 rows: re/im of every stream) is split into D_top = P[0:128] P^T
// (N = 256) and D_bot = P[128:256] P[128:256]^T (N = 128), as in the kernel above, but the two
// parts are computed by different CTAs so each CTA covers more channels in its 512 TMEM columns:
//   top CTAs (2 of every 3 blocks): 2 channels, D_top of each (256 columns each), loading
//     all streams of both channels (8-byte FP16 / 4-byte FP8 gathers);
//   bottom CTAs (every third block): 4 channels, D_bot of each (128 columns each), loading the bottom 64
//     streams of the four channels (16-byte FP16 / 8-byte FP8 gathers).
// A 32-byte sector read from L2 then carries 2 or 4 useful channels instead of 1: 2.5 KB of
// sectors per channel and FFT instead of 4 KB.
constexpr int B2_STAGES = 3;
constexpr int B2_STAGE_BYTES = 65536;  // top: 2 channels x 256 rows; bottom: 4 channels x 128 rows (128 B each)

// Producer body: NCH channels from c0 (within one 16-channel tile), streams [s_lo, n), operand
// rows of channel ci at ci*ROWS + 2*(s - s_lo) (re) and +1 (im).
template <bool F8, int NCH, int ROWS>
__device__ __forceinline__ void big2_produce(const Params &p, unsigned char *stage, int c0, int s_lo, int tb,
                                             int tid) {
  constexpr int NL = F8 ? 16 : 8;  // loads (FFTs) per task
  constexpr int U = NCH == 2 ? 4 : 2;  // tasks per thread with all their gathers in flight (8 gave 5-17 % less)
  using V = typename std::conditional<F8, typename std::conditional<NCH == 2, uint32_t, uint2>::type,
                                      typename std::conditional<NCH == 2, uint2, uint4>::type>::type;
  const int n = p.nstream;
  const int ns = n - s_lo;
  const int ntask = 8 * ns;  // (stream, 16-byte K chunk of a row)
  const size_t esz = F8 ? 2 : 4;
  const unsigned char *src = (const unsigned char *)p.chan + (((size_t)(c0 >> 4) * p.T * n) * CW + (c0 & 15)) * esz;
  for (int task0 = tid; task0 < ntask; task0 += U * NPROD) {
    V w[U][NL];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int task = task0 + u * NPROD;
      const int s = s_lo + task % ns;
      const int o = task / ns;
#pragma unroll
      for (int i = 0; i < NL; i++) {
        const int t = tb + NL * o + i;
        if (task < ntask && t < p.nt) {
          w[u][i] = __ldg(reinterpret_cast<const V *>(src + ((size_t)t * n + s) * CW * esz));
        } else {
          w[u][i] = V{};
        }
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int task = task0 + u * NPROD;
      if (task >= ntask) break;
      const int s = s_lo + task % ns;
      const int o = task / ns;
      const int sr = s - s_lo;
      const int sw = (sr >> 2) & 1;  // lanes s..s+7 store their first row at 8 swizzle positions
#pragma unroll
      for (int ci = 0; ci < NCH; ci++) {
        uint4 re, im;
        if constexpr (F8) {
          // channel ci's (re, im) byte pair of FFT i, two FFTs per word: re(2i), im(2i), re(2i+1), im(2i+1)
          uint32_t x[8];
#pragma unroll
          for (int i = 0; i < 8; i++) {
            uint32_t a, b2;
            if constexpr (NCH == 2) {
              a = w[u][2 * i];
              b2 = w[u][2 * i + 1];
            } else {
              a = ci < 2 ? w[u][2 * i].x : w[u][2 * i].y;
              b2 = ci < 2 ? w[u][2 * i + 1].x : w[u][2 * i + 1].y;
            }
            x[i] = prmt(a, b2, (ci & 1) ? 0x7632u : 0x5410u);
          }
          re = make_uint4(prmt(x[0], x[1], 0x6420), prmt(x[2], x[3], 0x6420), prmt(x[4], x[5], 0x6420),
                          prmt(x[6], x[7], 0x6420));
          im = make_uint4(prmt(x[0], x[1], 0x7531), prmt(x[2], x[3], 0x7531), prmt(x[4], x[5], 0x7531),
                          prmt(x[6], x[7], 0x7531));
        } else {
          uint32_t x[8];
#pragma unroll
          for (int i = 0; i < 8; i++) {
            if constexpr (NCH == 2) x[i] = ci ? w[u][i].y : w[u][i].x;
            else x[i] = ci == 0 ? w[u][i].x : ci == 1 ? w[u][i].y : ci == 2 ? w[u][i].z : w[u][i].w;
          }
          re = make_uint4(prmt(x[0], x[1], 0x5410), prmt(x[2], x[3], 0x5410), prmt(x[4], x[5], 0x5410),
                          prmt(x[6], x[7], 0x5410));
          im = make_uint4(prmt(x[0], x[1], 0x7632), prmt(x[2], x[3], 0x7632), prmt(x[4], x[5], 0x7632),
                          prmt(x[6], x[7], 0x7632));
        }
        const int ra = ci * ROWS + 2 * sr + sw, rb = ci * ROWS + 2 * sr + 1 - sw;
        *reinterpret_cast<uint4 *>(stage + ra * 128 + ((o ^ (ra & 7)) << 4)) = sw ? im : re;
        *reinterpret_cast<uint4 *>(stage + rb * 128 + ((o ^ (rb & 7)) << 4)) = sw ? re : im;
      }
    }
  }
}

// Epilogue of one channel's TMEM block: rows (TMEM lanes) are streams s_lo + row/2 (re/im by
// row parity), columns npc*16 starting at col0 are streams s2_lo + col/2.
// The CTA's outputs as a compact index: its antennas [ja, jb) own the cross baselines (j, k), j in
// [ja, jb), k > j (contiguous in the j-major baseline order, from cross_start) and, with autos,
// the autos of [ja, jb) after them.
struct Big2Span {
  int ja, cross_start, ncr, nloc;
  __device__ Big2Span(const Params &p, int ja_, int jb) : ja(ja_) {
    const int m = p.nant - 1;
    cross_start = ja * m - ja * (ja - 1) / 2;
    ncr = jb * m - jb * (jb - 1) / 2 - cross_start;
    nloc = ncr + (p.autos ? jb - ja : 0);
  }
};

// Stages the channel's Gram entries of this warp's TMEM lanes as complex visibilities at
// stg[(loc * 4 + product) * nch + ci] (loc: the baseline's compact index, Big2Span).
__device__ __forceinline__ void big2_epilogue(const Params &p, uint32_t tmem, int warp, int lane, int s_lo,
                                              int s2_lo, uint32_t col0, int npc, float2 *stg, int ci, int nch,
                                              const Big2Span &sp) {
  const int n = p.nstream;
  const int arow = 32 * warp + lane;
  const int s1 = s_lo + (arow >> 1), part1 = arow & 1;
  const int j = s1 >> 1, l = s1 & 1;
  for (int pc0 = 0; pc0 < npc; pc0++) {
#pragma unroll
    for (int u = 0; u < 1; u++) {
      const int pc = pc0 + u;
      __syncwarp();  // tcgen05.ld is warp-collective: reconverge after the divergent skips below
      float v[16], pv[16];
      tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + col0 + 16u * pc, v);
#pragma unroll
      for (int q = 0; q < 16; q++) pv[q] = __shfl_xor_sync(0xffffffffu, v[q], 1);
      if (s1 >= n) continue;
      const int s2b = s2_lo + 8 * pc;
#pragma unroll
      for (int qq = 0; qq < 4; qq++) {
        const int q = qq + 4 * part1;
        const int s2 = s2b + q;
        if (s2 >= n) continue;
        const int k = s2 >> 1, m = s2 & 1;
        if (j > k || (j == k && !p.autos)) continue;
        float re, im;
        if (part1 == 0) {
          re = v[2 * q] + pv[2 * q + 1];
          im = pv[2 * q] - v[2 * q + 1];
        } else {
          re = pv[2 * q] + v[2 * q + 1];
          im = v[2 * q] - pv[2 * q + 1];
        }
        const int loc = j < k ? baseline_index(j, k, p.nant) - sp.cross_start : sp.ncr + (j - sp.ja);
        stg[(loc * 4 + 2 * l + m) * nch + ci] = make_float2(re, im);
      }
    }
  }
}

template <bool F8>
__global__ void __launch_bounds__(NTHREADS, 1) xstage_tc_big2_kernel(Params p) {
  constexpr int KC = F8 ? 128 : 64, KSTEP = F8 ? 32 : 16;
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar_full[B2_STAGES], bar_empty[B2_STAGES], bar_done;
  __shared__ uint32_t tmem_base_sh;
  unsigned char *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  const uint32_t sbase = smem_u32(smem);
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int n = p.nstream;
  const int nchunks = (p.nt + KC - 1) / KC;
  // blocks 3g, 3g+1: top CTAs of channels 4g..4g+1 and 4g+2..4g+3; block 3g+2: the bottom CTA of
  // channels 4g..4g+3.  The three run together and share the group's sectors in L2 (the bottom
  // streams are read by both kinds)
  const int grp = (int)blockIdx.x / 3, kind = (int)blockIdx.x - 3 * grp;
  const bool top = kind < 2;
  const int nch = top ? 2 : 4;
  const int c0 = 4 * grp + (top ? 2 * kind : 0);
  const int rows = top ? 256 : 128;  // operand rows per channel
  const int s_lo = top ? 0 : 64;      // first stream of the loaded rows

  {  // zero the padding rows (streams n..) of every channel block of every stage
    const int used = 2 * (n - s_lo), pad = rows - used;
    if (pad > 0) {
      const int per_stage = nch * pad * 8;  // 16-byte words
      for (int i = tid; i < B2_STAGES * per_stage; i += NTHREADS) {
        const int st = i / per_stage, r0 = i - st * per_stage;
        const int w = r0 & 7, rr = r0 >> 3;
        const int ci = rr / pad, row = ci * rows + used + (rr - ci * pad);
        *reinterpret_cast<uint4 *>(smem + (size_t)st * B2_STAGE_BYTES + row * 128 + w * 16) = make_uint4(0, 0, 0, 0);
      }
    }
  }
  if (tid == 0) {
    for (int s = 0; s < B2_STAGES; s++) {
      mbar_init(smem_u32(&bar_full[s]), NPROD);
      mbar_init(smem_u32(&bar_empty[s]), 1);
    }
    mbar_init(smem_u32(&bar_done), 1);
    fence_mbar_init();
  }
  if (warp == NPROD_WARPS) {
    tmem_alloc(smem_u32(&tmem_base_sh), 512);
    tmem_relinquish();
  }
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_sh;

  if (warp < NPROD_WARPS) {
    for (int ch = 0; ch < nchunks; ch++) {
      const int st = ch % B2_STAGES;
      if (ch >= B2_STAGES && !mbar_wait(smem_u32(&bar_empty[st]), ((ch / B2_STAGES) - 1) & 1, p.err)) break;
      unsigned char *stage = smem + (size_t)st * B2_STAGE_BYTES;
      if (top) big2_produce<F8, 2, 256>(p, stage, c0, 0, ch * KC, tid);
      else big2_produce<F8, 4, 128>(p, stage, c0, 64, ch * KC, tid);
      fence_proxy_async_smem();
      mbar_arrive(smem_u32(&bar_full[st]));
    }
  } else if (lane == 0) {
    // ------------------------------------------------------------ MMA issuer
    for (int ch = 0; ch < nchunks; ch++) {
      const int st = ch % B2_STAGES;
      if (!mbar_wait(smem_u32(&bar_full[st]), (ch / B2_STAGES) & 1, p.err)) break;
      tc_fence_after();
      const uint32_t sa = sbase + st * B2_STAGE_BYTES;
#pragma unroll
      for (int kk = 0; kk < KC / KSTEP; kk++) {
        const uint32_t acc = (ch > 0 || kk > 0) ? 1u : 0u;
        for (int ci = 0; ci < nch; ci++) {
          const uint64_t d = desc_sw128(sa + ci * rows * 128 + kk * 32);
          if (top) {  // rows 0..127 of the channel's 256 against all 256: D_top, 256 columns
            if constexpr (F8) mma_f8(tmem + ci * 256, d, d, IDESC_N256, acc);
            else mma_f16(tmem + ci * 256, d, d, IDESC_N256, acc);
          } else {    // the channel's 128 bottom rows against themselves: D_bot, 128 columns
            if constexpr (F8) mma_f8(tmem + ci * 128, d, d, IDESC, acc);
            else mma_f16(tmem + ci * 128, d, d, IDESC, acc);
          }
        }
      }
      mma_commit(smem_u32(&bar_empty[st]));
    }
    mma_commit(smem_u32(&bar_done));
    mbar_wait(smem_u32(&bar_done), 0, p.err);  // issued MMAs drained before TMEM is read or freed
  }

  // Epilogue: warps 0-3 (the TMEM lane quarters) stage the CTA's visibilities in the operand
  // stages, idle once every MMA is done; then all warps add them into the accumulators, the nch
  // channels of a (baseline, product) contiguous there (per-output gathers touched one sector
  // per lane).
  const Big2Span sp(p, top ? 0 : 32, top ? (p.nant < 32 ? p.nant : 32) : p.nant);
  float2 *const stg = reinterpret_cast<float2 *>(smem);
  if (warp < 4) {
    const bool ok = mbar_wait(smem_u32(&bar_done), 0, p.err);
    tc_fence_after();
    if (ok) {
      for (int ci = 0; ci < nch; ci++) {
        if (top) big2_epilogue(p, tmem, warp, lane, 0, 0, (uint32_t)(ci * 256), 16, stg, ci, nch, sp);
        else big2_epilogue(p, tmem, warp, lane, 64, 64, (uint32_t)(ci * 128), 8, stg, ci, nch, sp);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (!*(volatile int *)p.err) {  // a timed-out role may have left the staging incomplete
    const int lnch = top ? 1 : 2;  // log2(nch)
    const int nent = sp.nloc * 4 * nch;
    const int ncross = p.nant * (p.nant - 1) / 2;
    for (int e0 = tid; e0 < nent; e0 += 4 * NTHREADS) {
      size_t off[4];
      float2 val[4];
      bool use[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int e = e0 + u * NTHREADS;
        use[u] = e < nent;
        const int loc = e >> (lnch + 2), prod = (e >> lnch) & 3, ci = e & (nch - 1);
        const int bl = loc < sp.ncr ? sp.cross_start + loc : ncross + sp.ja + (loc - sp.ncr);
        off[u] = ((size_t)bl * 4 + prod) * p.nchan + c0 + ci;
        val[u] = use[u] ? stg[e] : make_float2(0.f, 0.f);
      }
      rmw_batch<4>(p.vsum, p.vcomp, off, val, use);
    }
  }
  if (warp == NPROD_WARPS) tmem_dealloc(tmem, 512);
}

}  // namespace tc

// two rows (re, im) per stream, two streams per antenna: up to 32 antennas fill one
// M = 128 tile per channel; 33..64 antennas use the split-M kernel (FP16 or FP8)
int xstage_tensor_supported(int nant) { return nant >= 1 && 4 * nant <= 256; }

static int g_err_dev = -1;
static int *g_err = nullptr;

cudaError_t xstage_tensor_error_flag(int **flag) {
  int dev = 0;
  cudaGetDevice(&dev);
  if (!g_err || g_err_dev != dev) {
    cudaError_t e = cudaMalloc(&g_err, sizeof(int));
    if (e != cudaSuccess) return e;
    e = cudaMemset(g_err, 0, sizeof(int));
    if (e != cudaSuccess) return e;
    g_err_dev = dev;
  }
  *flag = g_err;
  return cudaSuccess;
}

// Reads and clears the device-side timeout flag of the tensor-core X-stage (1 = a wait expired).
cudaError_t xstage_tensor_take_error(int *flag) {
  *flag = 0;
  if (!g_err) return cudaSuccess;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != g_err_dev) return cudaSuccess;
  cudaError_t e = cudaMemcpy(flag, g_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && *flag) e = cudaMemset(g_err, 0, sizeof(int));
  return e;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link dependency).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(ptr);
  }
  return fn;
}

// Tensor map of the channelised block [ctile][T][n][16] (esz bytes per complex value) for the
// raw TMA tiles of the small-N tensor kernels: dims (channel in tile, stream, FFT, tile), the
// FFT extent cut at nt so rows of later FFTs read as zeros; box (bx, n, kc, 1).
static cudaError_t raw_tensor_map(CUtensorMap *m, const void *chan, int esz, int n, int nt, int T, int nchan, int bx,
                                  int kc) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn) return cudaErrorNotSupported;
  const CUtensorMapDataType dt = esz == 8   ? CU_TENSOR_MAP_DATA_TYPE_INT64
                                 : esz == 4 ? CU_TENSOR_MAP_DATA_TYPE_UINT32
                                            : CU_TENSOR_MAP_DATA_TYPE_UINT16;
  const cuuint64_t dims[4] = {(cuuint64_t)CW, (cuuint64_t)n, (cuuint64_t)nt, (cuuint64_t)(nchan / CW)};
  const cuuint64_t strides[3] = {(cuuint64_t)CW * esz, (cuuint64_t)CW * n * esz, (cuuint64_t)CW * n * T * esz};
  const cuuint32_t box[4] = {(cuuint32_t)bx, (cuuint32_t)n, (cuuint32_t)kc, 1u};
  const cuuint32_t estr[4] = {1u, 1u, 1u, 1u};
  const CUresult r = fn(m, dt, 4, const_cast<void *>(chan), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// Channels per CTA of the tensor-core X-stage for nant antennas (the channel count must divide by it).
int xstage_tensor_channels_per_cta(int nant, int chan_type) {
  if (4 * nant > 128) return chan_type == CHAN_F32 ? 0 : 1;  // split-M kernel: one channel, FP16 or FP8
  int R = 16;
  while (R < 4 * nant) R <<= 1;  // 2 rows (re, im) per stream, 2 streams per antenna
  return (chan_type == CHAN_F32 ? tc::Cfg<true>::NG : tc::Cfg<false>::NG) * (128 / R);
}

// True when the tensor-core X-stage can run this shape.
int xstage_tensor_fits(int nant, int nchan, int chan_type) {
  if (!xstage_tensor_supported(nant)) return 0;
  const int cs = xstage_tensor_channels_per_cta(nant, chan_type);
  return cs > 0 && nchan % cs == 0;
}

cudaError_t launch_xstage_tensor(const void *chan, int chan_type, int nant, int nchan, int T, int nt, int autos,
                                 float2 *vsum, float2 *vcomp, cudaStream_t s, int split_e, int kparts_max,
                                 size_t plane) {
  if (nt <= 0) return cudaSuccess;
  if (!xstage_tensor_supported(nant)) return cudaErrorInvalidValue;
  tc::Params p;
  p.chan = chan;
  p.nant = nant;
  p.nstream = 2 * nant;
  p.nchan = nchan;
  p.T = T;
  p.nt = nt;
  p.autos = autos;
  int R = 16;
  while (R < 2 * p.nstream) R <<= 1;  // 2 rows (re, im) per stream
  p.R = R;
  p.g = R <= 128 ? 128 / R : 1;
  p.CS = xstage_tensor_channels_per_cta(nant, chan_type);
  if (p.CS <= 0 || nchan % p.CS) return cudaErrorInvalidValue;
  p.vsum = vsum;
  p.vcomp = vcomp;
  p.kparts = 1;
  p.persist = 0;
  p.ngrp = 0;
  p.kspan = nt;
  p.plane = plane;
  // FP32 data: FP16 hi/lo split of values scaled by 2^-split_e when split_e >= 0, else TF32 split
  const bool h16 = chan_type == CHAN_F32 && split_e >= 0;
  p.split_sc = h16 ? ldexpf(1.0f, -split_e) : 1.0f;
  p.split_unsc = h16 ? ldexpf(1.0f, 2 * split_e) : 1.0f;
  cudaError_t e = xstage_tensor_error_flag(&p.err);
  if (e != cudaSuccess) return e;
  if (R > 128) {
    const size_t bsmem = (size_t)tc::BIG_STAGES * tc::BIG_STAGE_BYTES + 1024;
    // big2's staged epilogue: at most (1520 + 32) baselines x 4 products x 2 channels (top CTAs,
    // 64 antennas) = 99 KB, inside its 3 x 64 KiB operand stages
    static_assert((1520 + 32) * 4 * 2 * 8 <= tc::B2_STAGES * tc::B2_STAGE_BYTES &&
                      (496 + 32) * 4 * 4 * 8 <= tc::B2_STAGES * tc::B2_STAGE_BYTES,
                  "big2 epilogue staging");
    if (nchan % 4 == 0) {
      // per group of 4 channels: two top CTAs (2 channels, D_top) and one bottom CTA (4 channels, D_bot)
      const size_t b2smem = (size_t)tc::B2_STAGES * tc::B2_STAGE_BYTES + 1024;
      auto kern2 = chan_type == CHAN_F8 ? tc::xstage_tc_big2_kernel<true> : tc::xstage_tc_big2_kernel<false>;
      e = cudaFuncSetAttribute(kern2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b2smem);
      if (e != cudaSuccess) return e;
      kern2<<<nchan / 2 + nchan / 4, tc::NTHREADS, b2smem, s>>>(p);
      return cudaGetLastError();
    }
    auto kern = chan_type == CHAN_F8 ? tc::xstage_tc_big_kernel<true> : tc::xstage_tc_big_kernel<false>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bsmem);
    if (e != cudaSuccess) return e;
    kern<<<nchan, tc::NTHREADS, bsmem, s>>>(p);
    return cudaGetLastError();
  }
  // small-N kernels: raw TMA tiles of rbx channels (at least 16 bytes: FP8 with 4 channels per
  // CTA loads 8, of which the CTA uses its 4) x all streams x rkc FFTs, one box per channel tile
  const int esz = (int)chan_elem_bytes(chan_type);
  const int KC = chan_type == CHAN_F32 ? (h16 ? 64 : tc::Cfg<true>::KC) : chan_type == CHAN_F8 ? 128 : tc::Cfg<false>::KC;
  p.rnbox = p.CS > CW ? p.CS / CW : 1;
  p.rbx = p.CS > CW ? CW : (p.CS * esz >= 16 ? p.CS : 16 / esz);
  if (p.rbx * esz < 16 || p.rbx > CW || (p.CS > CW && p.CS % CW)) return cudaErrorInvalidValue;
  int kc = KC;
  while (kc > 8 && (size_t)p.rnbox * p.rbx * p.nstream * kc * esz > (size_t)tc::RAW_BYTES) kc >>= 1;
  p.rkc = kc;
  p.rbox_bytes = p.rbx * p.nstream * kc * esz;
  // producer tasks per raw chunk, (channel quad or pair, stream, 16-byte K chunk): at most two
  // per producer thread, which the kernels decode once
  const int tk = chan_type == CHAN_F32 ? (h16 ? 8 : 4) : chan_type == CHAN_F8 ? 16 : 8;
  const int per_task = chan_type == CHAN_F32 ? 2 : 4;
  if ((kc / tk) * p.nstream * (p.CS / per_task) > 2 * tc::NPROD) return cudaErrorInvalidValue;
  if ((size_t)p.rnbox * p.rbox_bytes > (size_t)tc::RAW_BYTES || KC % kc ||
      kc % (chan_type == CHAN_F8 ? 16 : 8))
    return cudaErrorInvalidValue;
  CUtensorMap tmap;
  e = raw_tensor_map(&tmap, chan, esz, p.nstream, nt, T, nchan, p.rbx, kc);
  if (e != cudaSuccess) return e;
  const size_t smem = (size_t)tc::STAGES * 65536 + (size_t)tc::RSTAGES * tc::RAW_BYTES + 1024;
  static_assert(tc::Cfg<true>::STAGE_BYTES == 65536 && tc::Cfg<false>::STAGE_BYTES == 65536, "stage size");
  if (chan_type == CHAN_F32) {
    // the block's visibilities are staged as [baseline x product][CS] in the operand ring
    const size_t nbl = (size_t)nant * (nant - 1) / 2 + (autos ? nant : 0);
    if (nbl * 4 * p.CS * sizeof(float2) > (size_t)tc::STAGES * tc::Cfg<true>::STAGE_BYTES || (p.CS & (p.CS - 1)))
      return cudaErrorInvalidValue;
    auto launch = [&](auto kern) -> cudaError_t {
      cudaError_t e2 = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e2 != cudaSuccess) return e2;
      kern<<<nchan / p.CS, tc::NTHREADS_SPLIT, smem, s>>>(p, tmap);
      return cudaSuccess;
    };
    switch (R * 2 + (h16 ? 1 : 0)) {
      case 32: e = launch(tc::xstage_tc_split_kernel<16, false>); break;
      case 33: e = launch(tc::xstage_tc_split_kernel<16, true>); break;
      case 64: e = launch(tc::xstage_tc_split_kernel<32, false>); break;
      case 65: e = launch(tc::xstage_tc_split_kernel<32, true>); break;
      case 128: e = launch(tc::xstage_tc_split_kernel<64, false>); break;
      case 129: e = launch(tc::xstage_tc_split_kernel<64, true>); break;
      case 256: e = launch(tc::xstage_tc_split_kernel<128, false>); break;
      case 257: e = launch(tc::xstage_tc_split_kernel<128, true>); break;
      default: return cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
  } else {
    // one CTA per SM (its shared memory): when the channel groups leave SMs idle (fewer groups
    // than SMs), split the block's FFTs in two halves, each into its own accumulator plane (with
    // nt >= 4 KC both halves hold more than KC FFTs, so no CTA accumulates nothing).  Measured:
    // 6 antennas (64 groups) FP16 0.49 -> 0.30 ms; with 512 groups (3.4 waves) the split was
    // slower (9.0 -> 10.3 ms), its halved CTAs paying their pipeline fill and drain twice.
    const int ngrp = nchan / p.CS;
    // each segment epilogue stages [baseline x product][CS] visibilities in the operand ring
    const size_t nbl = (size_t)nant * (nant - 1) / 2 + (autos ? nant : 0);
    if (nbl * 4 * p.CS * sizeof(float2) > (size_t)tc::STAGES * tc::Cfg<false>::STAGE_BYTES ||
        (p.CS & (p.CS - 1)))
      return cudaErrorInvalidValue;
    int dev = 0, nsm = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    p.ngrp = ngrp;
    p.persist = 0;
    if (kparts_max >= 2 && plane > 0 && nt >= 4 * KC && (ngrp < nsm || kparts_max >= 3)) {
      p.kparts = 2;
      p.kspan = (nt / 2 + KC - 1) / KC * KC;
    } else if (kparts_max == 2 && plane > 0 && ngrp >= nsm) {
      // at least as many groups as SMs: one CTA per SM, each an equal share of all (group, K
      // chunk) units, so no SM idles in a last partial wave (512 groups are 3.37 waves)
      p.persist = 1;
    }
    auto kern = chan_type == CHAN_F8 ? tc::xstage_tc_kernel<true> : tc::xstage_tc_kernel<false>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<p.persist ? nsm : ngrp * p.kparts, tc::NTHREADS_TC, smem, s>>>(p, tmap);
  }
  return cudaGetLastError();
}

}  // namespace gxc
