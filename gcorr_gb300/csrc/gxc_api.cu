// C ABI of libgxcorr (declared in include/gxc.h): the FxKernel-shaped
// boundary, argument validation with status codes, device buffers, and the
// per-sub-integration launch sequence.
//
// Reference boundary: fxkernel/src/fxkernel.h:29-64 (FxKernel ctor, setInputData,
// setDelays, process, accumulate); reference call sequence of a GPU
// sub-integration: gcorr/src/testgpukernel.cu:462-534.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "gxc_internal.h"

using namespace gxc;

struct gxc_handle {
  gxc_config cfg;
  Job job;
  int device = 0;
  int F = 0, log2F = 0, nbl = 0, T = 0, nblocks = 0;
  int T0 = 0;  // FFTs in the first block when the inputs are copied from the host (<= T)
  std::vector<std::pair<int, int>> blk;  // blocks of the last process(): (first FFT, FFT count)
  int chan_type = CHAN_F32;
  int xeng = GXC_XENGINE_CUDA_CORE;
  bool tc_fstage = false;  // tensor-core F-stage (fstage_tc.cu)
  void *d_tc_tables = nullptr;
  float out_scale = 1.f;   // applied to channelised values before the cast
  float vis_scale = 1.f;   // 1/out_scale^2, applied at finalisation
  // FP8 per-channel scales (GXC_FP8_SCALE_CHANNEL): calibration block of cal_T FFTs in FP32,
  // per-channel output scale and its inverse square
  int cal_T = 0;
  float2 *d_cal = nullptr;
  float *d_cscale = nullptr, *d_cvscale = nullptr;
  size_t bytes_per_ant = 0;

  // inputs
  std::vector<const uint8_t *> user_ptrs;
  bool input_on_host = false;
  bool have_input = false, have_delays = false;
  uint8_t *d_inbuf = nullptr;          // staging for host inputs [nant][bytes_per_ant]
  // host inputs are copied on copy_stream in time-ordered chunks (in_chunk_ev[j]: every antenna's
  // bytes [0, in_chunk_end[j]) are on the device); each F-stage block waits for its chunk
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_fork = nullptr;
  std::vector<cudaEvent_t> in_chunk_ev;
  std::vector<long long> in_chunk_end;
  const uint8_t **d_inptrs = nullptr;  // device array of per-antenna device pointers
  double *d_poly = nullptr, *d_fso = nullptr;
  // frame validity (gxc_set_frame_validity): user device pointers, uploaded per process()
  std::vector<const uint8_t *> user_fvalid;
  const uint8_t **d_fvalid = nullptr;
  std::vector<double> poly, fso;

  // state
  Geom *d_geom = nullptr;
  int32_t *d_counts = nullptr;
  uint8_t *d_valid = nullptr;
  float2 *d_tw = nullptr;
  int2 *d_pairs = nullptr;  // tile pairs of the CUDA-core X-stage
  void *d_chan = nullptr;
  float2 *d_vsum = nullptr, *d_vcomp = nullptr, *d_vis = nullptr;
  cudaStream_t last_stream = nullptr;
  cudaEvent_t ev_done = nullptr;
  bool processed = false;
  int launches = 0;

  bool stage_timing = false;
  std::vector<cudaEvent_t> ev_stage;  // per block: F start, F end (= X start), X end
  cudaEvent_t ev_begin = nullptr, ev_end = nullptr;

  std::string err;
};

namespace {

// time-ordered input chunks of host-input handles (each at least kMinInChunkBytes per antenna)
constexpr int kInChunks = 8;
constexpr size_t kMinInChunkBytes = 1 << 20;

gxc_status fail(gxc_handle *h, gxc_status s, const std::string &msg) {
  if (h) h->err = msg;
  return s;
}

gxc_status cuda_fail(gxc_handle *h, cudaError_t e, const char *what) {
  std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  return fail(h, e == cudaErrorMemoryAllocation ? GXC_ERR_OUT_OF_MEMORY : GXC_ERR_CUDA, m);
}

#define GXC_CUDA(h, call, what)                          \
  do {                                                   \
    cudaError_t e__ = (call);                            \
    if (e__ != cudaSuccess) return cuda_fail(h, e__, what); \
  } while (0)

int ilog2i(int x) {
  int l = 0;
  while ((1 << (l + 1)) <= x) l++;
  return l;
}

bool is_pow2(long long x) { return x > 0 && (x & (x - 1)) == 0; }

int fft_len(const gxc_config *c) { return c->is_complex ? c->nchan : 2 * c->nchan; }

std::string validate(const gxc_config *c, gxc_status *st) {
  *st = GXC_ERR_INVALID_ARGUMENT;
  if (!c) return "null config";
  if (c->nant < 1) return "nant must be >= 1";
  if (c->nfft < 1) return "nfft must be >= 1";
  if (c->nchan < 16) return "nchan must be >= 16";
  if (!(c->nbit == 2 || c->nbit == 8)) return "nbit must be 2 or 8";  // fxkernel.cpp:46-55
  if (!(c->bw_hz > 0.0) || !isfinite(c->bw_hz)) return "bandwidth must be positive";
  if (!isfinite(c->lo_hz)) return "LO must be finite";
  if (c->precision < GXC_PRECISION_FP32 || c->precision > GXC_PRECISION_FP8) return "bad precision";
  if (c->rotator != GXC_ROTATOR_EXACT && c->rotator != GXC_ROTATOR_FXKERNEL) return "bad rotator";
  if (c->x_engine < GXC_XENGINE_AUTO || c->x_engine > GXC_XENGINE_TENSOR) return "bad x_engine";
  if (c->fft_block < 0) return "fft_block must be >= 0";
  if (c->fft_engine < GXC_FFT_AUTO || c->fft_engine > GXC_FFT_TENSOR) return "bad fft_engine";
  if (c->x_split < GXC_XSPLIT_AUTO || c->x_split > GXC_XSPLIT_ON) return "bad x_split";
  if (c->fp8_scaling < GXC_FP8_SCALE_CHANNEL || c->fp8_scaling > GXC_FP8_SCALE_HANDLE) return "bad fp8_scaling";
  const long long F = fft_len(c);
  if (!is_pow2(F)) return "FFT length (2*nchan real, nchan complex) must be a power of two";
  if (c->rotator == GXC_ROTATOR_FXKERNEL) {
    const int s = (int)sqrt((double)c->nchan);
    if (s * s != c->nchan) return "the fxkernel rotator needs a square nchan (fxkernel.cpp:58-63)";
  }
  if ((long long)c->nfft * F > 2147483647LL) return "nfft*F exceeds the 32-bit sample index of the input format";
  *st = GXC_ERR_UNSUPPORTED;
  if (!((c->nbit == 2 && !c->is_complex) || (c->nbit == 8 && c->is_complex)))
    return "supported input formats: 2-bit real, 8-bit complex";
  if (!fstage_supported((int)F)) return "FFT length outside 256..32768";
  if (c->fft_engine == GXC_FFT_TENSOR && !(F == 8192 && !c->is_complex && c->precision != GXC_PRECISION_FP32))
    return "tensor-core FFT: needs 8192-point windows of 2-bit real data (nchan 4096) and FP16 or FP8 output";
  if (c->x_engine == GXC_XENGINE_TENSOR) {
    if (!xstage_tensor_fits(c->nant, c->nchan, chan_type_of(c->precision)))
      return "tensor-core X-stage: needs nant <= 64 (FP16), <= 32 (FP32, FP8) and nchan a multiple of its channel "
             "tile";
  }
  *st = GXC_OK;
  return "";
}

size_t input_bytes(const gxc_config *c) {
  const size_t F = (size_t)fft_len(c);
  const size_t comps = c->is_complex ? 2 : 1;
  return (size_t)(c->nfft + 1) * F * 2u * comps * (size_t)c->nbit / 8u;
}

}  // namespace

extern "C" {

void gxc_config_init(gxc_config *c) {
  if (!c) return;
  memset(c, 0, sizeof(*c));
  c->nbit = 2;
  c->precision = GXC_PRECISION_FP32;
  c->rotator = GXC_ROTATOR_EXACT;
  c->autos = 1;
  c->x_engine = GXC_XENGINE_AUTO;
  c->device = -1;
}

gxc_status gxc_validate_config(const gxc_config *c) {
  gxc_status st;
  validate(c, &st);
  return st;
}

size_t gxc_input_bytes_per_antenna(const gxc_config *c) { return c ? input_bytes(c) : 0; }

// geometry_kernel: off(i) = i F - nd(i), nd(i) = int_rz((mean(i) - fso)/Ts + 0.5), where mean(i) is the
// mean of the delay polynomial at i, i + 1/2 and i + 1 (FFT units), so it lies between the
// polynomial's extremes on [t0, t0+nt].  Two samples of margin cover the rounding and the +-1
// fix-ups; windows past maxoffset are flagged and read nothing.  The staging reads whole 16-byte
// blocks.
long long gxc_input_bytes_for_ffts(const gxc_config *c, const double *poly, const double *fso, int t0, int nt) {
  if (!c || !poly || !fso || c->nant < 1 || c->nchan < 1 || c->nfft < 1 || c->bw_hz <= 0.0 || t0 < 0 || nt < 1 ||
      (long long)t0 + nt > c->nfft)
    return 0;
  const long long total = (long long)input_bytes(c);
  const long long F = fft_len(c);
  const double Ts = c->is_complex ? 1.0 / c->bw_hz : 1.0 / (2.0 * c->bw_hz);
  const long long maxoffset = (long long)(c->nfft - 1) * F;
  const double x0 = (double)t0, x1 = (double)t0 + (double)nt;
  long long need = 0;
  for (int a = 0; a < c->nant; a++) {
    const double p0 = poly[3 * a], p1 = poly[3 * a + 1], p2 = poly[3 * a + 2];
    auto d = [&](double x) { return p0 * x * x + p1 * x + p2; };
    double dmin = fmin(d(x0), d(x1)), dmax = fmax(d(x0), d(x1));
    if (p0 != 0.0) {
      const double xv = -p1 / (2.0 * p0);
      if (xv > x0 && xv < x1) {
        dmin = fmin(dmin, d(xv));
        dmax = fmax(dmax, d(xv));
      }
    }
    const double ndf_lo = (dmin - fso[a]) / Ts, ndf_hi = (dmax - fso[a]) / Ts;
    if (!(fabs(ndf_lo) < 1.0e9) || !(fabs(ndf_hi) < 1.0e9)) return total;  // not finite: the whole buffer
    const long long nd_min = (long long)floor(ndf_lo) - 2, nd_max = (long long)ceil(ndf_hi) + 2;
    if ((long long)t0 * F - nd_max > maxoffset) continue;  // every window past the end: flagged
    long long off = (long long)(t0 + nt - 1) * F - nd_min;
    if (off > maxoffset) off = maxoffset;
    if (off < 0) continue;  // every window before the start: flagged
    const long long end = off + F + 1;  // samples
    long long bytes = c->is_complex ? 4 * end : (end + 1) / 2;
    bytes = (bytes + 15) / 16 * 16 + 16;
    if (bytes > need) need = bytes;
  }
  return need < total ? need : total;
}

int gxc_num_baselines(const gxc_config *c) {
  if (!c || c->nant < 1) return 0;
  return c->nant * (c->nant - 1) / 2 + (c->autos ? c->nant : 0);
}

const char *gxc_status_string(gxc_status s) {
  switch (s) {
    case GXC_OK: return "ok";
    case GXC_ERR_INVALID_ARGUMENT: return "invalid argument";
    case GXC_ERR_UNSUPPORTED: return "unsupported";
    case GXC_ERR_CUDA: return "CUDA error";
    case GXC_ERR_OUT_OF_MEMORY: return "out of memory";
    case GXC_ERR_STATE: return "bad call order";
    case GXC_ERR_TIMEOUT: return "device wait timed out";
    case GXC_END_OF_DATA: return "end of data";
  }
  return "unknown status";
}

const char *gxc_last_error(const gxc_handle *h) { return h ? h->err.c_str() : "null handle"; }
int gxc_last_launch_count(const gxc_handle *h) { return h ? h->launches : 0; }
int gxc_fft_block(const gxc_handle *h) { return h ? h->T : 0; }
int gxc_num_blocks(const gxc_handle *h) { return h ? h->nblocks : 0; }
int gxc_fft_engine(const gxc_handle *h) { return h && h->tc_fstage ? GXC_FFT_TENSOR : GXC_FFT_CUDA_CORE; }
const float *gxc_device_visibilities(const gxc_handle *h) { return h ? (const float *)h->d_vis : nullptr; }

static void release(gxc_handle *h) {
  cudaFree(h->d_inbuf);
  cudaFree((void *)h->d_inptrs);
  cudaFree(h->d_poly);
  cudaFree(h->d_fso);
  cudaFree((void *)h->d_fvalid);
  cudaFree(h->d_geom);
  cudaFree(h->d_counts);
  cudaFree(h->d_valid);
  cudaFree(h->d_tw);
  cudaFree(h->d_tc_tables);
  cudaFree(h->d_cal);
  cudaFree(h->d_cscale);
  cudaFree(h->d_cvscale);
  cudaFree(h->d_pairs);
  cudaFree(h->d_chan);
  cudaFree(h->d_vsum);
  cudaFree(h->d_vcomp);
  cudaFree(h->d_vis);
  if (h->ev_done) cudaEventDestroy(h->ev_done);
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  for (cudaEvent_t e : h->in_chunk_ev) cudaEventDestroy(e);
  if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
  for (cudaEvent_t e : h->ev_stage) cudaEventDestroy(e);
  if (h->ev_begin) cudaEventDestroy(h->ev_begin);
  if (h->ev_end) cudaEventDestroy(h->ev_end);
}

gxc_status gxc_create(const gxc_config *cfg, gxc_handle **out) {
  if (!out) return GXC_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  gxc_status st;
  std::string msg = validate(cfg, &st);
  if (st != GXC_OK) {
    fprintf(stderr, "gxc_create: %s\n", msg.c_str());
    return st;
  }
  gxc_handle *h = new gxc_handle();
  h->cfg = *cfg;
  if (cfg->device >= 0) {
    cudaError_t e = cudaSetDevice(cfg->device);
    if (e != cudaSuccess) {
      fprintf(stderr, "gxc_create: cudaSetDevice(%d): %s\n", cfg->device, cudaGetErrorString(e));
      delete h;
      return GXC_ERR_CUDA;
    }
  }
  cudaGetDevice(&h->device);
  const int nant = cfg->nant;
  h->F = fft_len(cfg);
  h->log2F = ilog2i(h->F);
  h->nbl = gxc_num_baselines(cfg);
  h->bytes_per_ant = input_bytes(cfg);
  h->chan_type = chan_type_of(cfg->precision);
  h->xeng = cfg->x_engine;
  // AUTO: tensor cores whenever the antenna count and channel tile fit.  FP32 data
  // uses the TF32 hi/lo split, whose TMEM accumulators are drained every 128
  // FFTs (TMEM accumulation rounds towards zero; the drains bound that bias at
  // about 3e-6 relative, inside the FP32 tolerance, whatever the integration length).
  if (h->xeng == GXC_XENGINE_AUTO)
    h->xeng = xstage_tensor_fits(nant, cfg->nchan, h->chan_type) ? GXC_XENGINE_TENSOR : GXC_XENGINE_CUDA_CORE;
  // FP16 storage keeps |X| near the sample rms: scale by 2^-floor(log2(F)/2),
  // an exact power of two undone exactly at finalisation.
  // FP8 (E4M3, largest finite 448) uses the same scale, and 2^-4 more for 8-bit data
  // (sigma ~20 per component): the spectra then sit near rms 2..4, far from saturation.
  if (h->chan_type != CHAN_F32) {
    const int e = h->log2F / 2 + ((h->chan_type == CHAN_F8 && cfg->is_complex) ? 4 : 0);
    h->out_scale = ldexpf(1.0f, -e);
    h->vis_scale = ldexpf(1.0f, 2 * e);
  }
  // FFT block T (FFTs per F/X pass).  Every block adds its partial sums into the
  // compensated accumulators (read + write of sum and comp) and pays each X-stage CTA's
  // pipeline fill and epilogue once, so T is chosen large: enough that the accumulator
  // traffic stays under ~6% of the channelised data of a block, at least 4096 FFTs, up to
  // 16384 while the channelised block stays within 16 GiB (measured, 16 antennas x 4096
  // channels: 4096 -> 16384 FFTs took the FP16 X-stage from 6.3 to 5.5 ms and the FP32 one
  // from 13.7 to 12.8 ms per second of data), and small enough for the device memory budget
  // (40% of the free memory, leaving room for inputs and the caller).
  const size_t esz = chan_elem_bytes(h->chan_type);
  const size_t per_fft = (size_t)cfg->nchan * 2 * nant * esz;
  int T = cfg->fft_block;
  if (T <= 0) {
    const size_t nvis_b = (size_t)(h->nbl > 0 ? h->nbl : 1) * 4 * cfg->nchan * sizeof(float2) * 4;
    size_t want = (16 * nvis_b + per_fft - 1) / per_fft;
    size_t big = ((size_t)16 << 30) / per_fft;
    if (big > 16384) big = 16384;
    if (want < big) want = big;
    if (want < 4096) want = 4096;  // fewer, longer X passes amortise each CTA's set-up and epilogue
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      cudaGetLastError();
      free_b = (size_t)8 << 30;
    }
    size_t cap = (size_t)(0.4 * (double)free_b) / per_fft;
    if (cap < 64) cap = 64;
    size_t tt = want < cap ? want : cap;
    if (tt > (size_t)cfg->nfft) tt = (size_t)cfg->nfft;
    T = (int)tt;
    if (T > 64 && T < cfg->nfft) T -= T % 64;
  }
  if (T > cfg->nfft) T = cfg->nfft;
  h->T = T;
  h->nblocks = (cfg->nfft + T - 1) / T;
  // host inputs: the first F-stage waits for the copy of its block's samples, so a chosen T
  // starts with a 4096-FFT block and doubles up to T (each block then needs samples that were
  // copied while the previous one ran, for copies at least half as fast as the correlation)
  h->T0 = (cfg->fft_block <= 0 && T > 4096) ? 4096 : T;

  // rotator/frac table split (fxkernel.cpp:57-64; power-of-two split for non-square nchan)
  int stride = (int)sqrt((double)cfg->nchan);
  if (stride * stride != cfg->nchan) stride = 1 << (ilog2i(cfg->nchan) / 2);
  Job &j = h->job;
  j.nant = nant;
  j.nchan = cfg->nchan;
  j.nfft = cfg->nfft;
  j.F = h->F;
  j.log2F = h->log2F;
  j.is_complex = cfg->is_complex;
  j.rotator = cfg->rotator;
  j.stride = stride;
  j.substride = h->F / stride;
  j.fstride = stride;
  j.fsub = cfg->nchan / stride;
  j.fractional_lo = (cfg->lo_hz - (double)(long long)cfg->lo_hz) > 0.00000000001;
  j.lo_hz = cfg->lo_hz;
  j.bw_hz = cfg->bw_hz;
  j.Ts = cfg->is_complex ? 1.0 / cfg->bw_hz : 1.0 / (2.0 * cfg->bw_hz);
  j.maxoffset = (long long)(cfg->nfft - 1) * h->F;
  j.fvalid = nullptr;
  j.samples_per_frame = 0;

  cudaError_t e = cudaSuccess;
  auto A = [&](void **p, size_t n) {
    if (e == cudaSuccess) e = cudaMalloc(p, n);
  };
  A((void **)&h->d_inptrs, sizeof(uint8_t *) * nant);
  A((void **)&h->d_poly, sizeof(double) * 3 * nant);
  A((void **)&h->d_fso, sizeof(double) * nant);
  A((void **)&h->d_fvalid, sizeof(uint8_t *) * nant);
  A((void **)&h->d_geom, sizeof(Geom) * (size_t)nant * cfg->nfft);
  A((void **)&h->d_counts, sizeof(int32_t) * (h->nbl > 0 ? h->nbl : 1));
  A((void **)&h->d_valid, (size_t)nant * cfg->nfft);
  A(&h->d_chan, per_fft * (size_t)T);
  const size_t nvis = (size_t)(h->nbl > 0 ? h->nbl : 1) * 4 * cfg->nchan;
  // two accumulator planes: the tensor X-stage may split a block's FFTs across two CTAs per
  // channel group (launch_xstage_tensor); finalisation sums the planes
  A((void **)&h->d_vsum, sizeof(float2) * nvis * 2);
  A((void **)&h->d_vcomp, sizeof(float2) * nvis * 2);
  A((void **)&h->d_vis, sizeof(float2) * nvis);
  if (e == cudaSuccess) e = make_twiddles(h->F, &h->d_tw);
  if (e == cudaSuccess) e = make_tile_pairs(nant, &h->d_pairs);
  // the tensor-core F-stage runs when asked for; AUTO keeps the CUDA-core FFT, which measured
  // faster (16 antennas, nchan 4096, FP16: F-stage 41.1 ms against 44.4 ms per sub-integration)
  // AUTO takes the tensor-core F-stage where it runs (8192-point 2-bit real windows, FP16 or
  // FP8 channelised data): 36.2 ms against 40.1 ms for the CUDA-core FFT per second of the
  // 16-antenna, 512 Ms/s workload at FP16
  h->tc_fstage = cfg->fft_engine != GXC_FFT_CUDA_CORE && fstage_tc_supported(j, h->chan_type);
  if (e == cudaSuccess && h->tc_fstage) e = make_fstage_tc_tables(&h->d_tc_tables);
  if (h->chan_type == CHAN_F8 && cfg->fp8_scaling == GXC_FP8_SCALE_CHANNEL) {
    // calibration block: up to 64 FFTs, at most 256 MB of FP32 channelised data (at least 4 FFTs)
    const size_t per_fft32 = (size_t)cfg->nchan * 2 * nant * sizeof(float2);
    size_t ct = ((size_t)256 << 20) / per_fft32;
    if (ct > 64) ct = 64;
    if (ct < 4) ct = 4;
    if (ct > (size_t)cfg->nfft) ct = (size_t)cfg->nfft;
    h->cal_T = (int)ct;
    A((void **)&h->d_cal, per_fft32 * ct);
    A((void **)&h->d_cscale, sizeof(float) * cfg->nchan);
    A((void **)&h->d_cvscale, sizeof(float) * cfg->nchan);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMemset(h->d_vis, 0, sizeof(float2) * nvis);
  if (e != cudaSuccess) {
    fprintf(stderr, "gxc_create: %s\n", cudaGetErrorString(e));
    release(h);
    delete h;
    return e == cudaErrorMemoryAllocation ? GXC_ERR_OUT_OF_MEMORY : GXC_ERR_CUDA;
  }
  j.inputs = h->d_inptrs;
  j.poly = h->d_poly;
  j.fso = h->d_fso;
  j.geom = h->d_geom;
  h->poly.assign(3 * (size_t)nant, 0.0);
  h->fso.assign((size_t)nant, 0.0);
  *out = h;
  return GXC_OK;
}

gxc_status gxc_destroy(gxc_handle *h) {
  if (!h) return GXC_ERR_INVALID_ARGUMENT;
  cudaSetDevice(h->device);
  if (h->ev_done && h->processed) cudaEventSynchronize(h->ev_done);
  release(h);
  delete h;
  return GXC_OK;
}

gxc_status gxc_set_input(gxc_handle *h, const uint8_t *const *per_ant, size_t bytes_per_ant) {
  if (!h) return GXC_ERR_INVALID_ARGUMENT;
  if (!per_ant) return fail(h, GXC_ERR_INVALID_ARGUMENT, "null input pointer array");
  if (bytes_per_ant < h->bytes_per_ant)
    return fail(h, GXC_ERR_INVALID_ARGUMENT,
                "input buffers too small: need " + std::to_string(h->bytes_per_ant) + " bytes per antenna");
  cudaSetDevice(h->device);
  int n_dev = 0, n_host = 0;
  for (int a = 0; a < h->cfg.nant; a++) {
    if (!per_ant[a]) return fail(h, GXC_ERR_INVALID_ARGUMENT, "null input buffer for antenna " + std::to_string(a));
    cudaPointerAttributes attr;
    cudaError_t e = cudaPointerGetAttributes(&attr, per_ant[a]);
    if (e != cudaSuccess) {
      cudaGetLastError();
      n_host++;
      continue;
    }
    if (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged) {
      // the F-stage stages each FFT window with 16-byte vector loads
      if ((uintptr_t)per_ant[a] & 15u)
        return fail(h, GXC_ERR_INVALID_ARGUMENT, "device input buffers must be 16-byte aligned");
      n_dev++;
    } else {
      n_host++;
    }
  }
  if (n_dev && n_host) return fail(h, GXC_ERR_INVALID_ARGUMENT, "inputs must be all host or all device buffers");
  h->input_on_host = n_host > 0;
  h->user_ptrs.assign(per_ant, per_ant + h->cfg.nant);
  if (h->input_on_host && !h->d_inbuf) {
    cudaError_t e = cudaMalloc((void **)&h->d_inbuf, h->bytes_per_ant * (size_t)h->cfg.nant);
    if (e != cudaSuccess) return cuda_fail(h, e, "allocating the device input buffer");
  }
  if (h->input_on_host && h->in_chunk_ev.empty()) {
    // the copy stream and chunk events (created once; a failure leaves the handle without host
    // input until a later call succeeds)
    const int nch = h->bytes_per_ant >= (size_t)kInChunks * kMinInChunkBytes ? kInChunks : 1;
    cudaError_t e = cudaSuccess;
    if (!h->copy_stream) e = cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess && !h->ev_fork) e = cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming);
    std::vector<cudaEvent_t> evs;
    for (int j = 0; e == cudaSuccess && j < nch; j++) {
      cudaEvent_t c = nullptr;
      e = cudaEventCreateWithFlags(&c, cudaEventDisableTiming);
      if (e == cudaSuccess) evs.push_back(c);
    }
    if (e != cudaSuccess) {
      for (cudaEvent_t c : evs) cudaEventDestroy(c);
      h->have_input = false;
      return cuda_fail(h, e, "creating the input copy stream");
    }
    h->in_chunk_ev = evs;
    h->in_chunk_end.assign((size_t)nch, 0);
  }
  h->have_input = true;
  return GXC_OK;
}

gxc_status gxc_set_frame_validity(gxc_handle *h, const uint8_t *const *valid, size_t nframes,
                                  int64_t samples_per_frame) {
  if (!h) return GXC_ERR_INVALID_ARGUMENT;
  if (!valid) {
    h->user_fvalid.clear();
    h->job.fvalid = nullptr;
    h->job.samples_per_frame = 0;
    return GXC_OK;
  }
  if (samples_per_frame < 1) return fail(h, GXC_ERR_INVALID_ARGUMENT, "samples_per_frame must be >= 1");
  const long long need = (long long)(h->cfg.nfft + 1) * h->F;  // every sample of the input buffer
  if ((long long)nframes * samples_per_frame < need)
    return fail(h, GXC_ERR_INVALID_ARGUMENT,
                "frame validity covers " + std::to_string((long long)nframes * samples_per_frame) + " samples, need " +
                    std::to_string(need));
  cudaSetDevice(h->device);
  for (int a = 0; a < h->cfg.nant; a++) {
    if (!valid[a]) continue;
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, valid[a]) != cudaSuccess ||
        (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged)) {
      cudaGetLastError();
      return fail(h, GXC_ERR_INVALID_ARGUMENT, "frame validity must be device memory");
    }
  }
  h->user_fvalid.assign(valid, valid + h->cfg.nant);
  h->job.fvalid = h->d_fvalid;
  h->job.samples_per_frame = samples_per_frame;
  return GXC_OK;
}

gxc_status gxc_set_delays(gxc_handle *h, const double *poly, const double *fso) {
  if (!h) return GXC_ERR_INVALID_ARGUMENT;
  if (!poly || !fso) return fail(h, GXC_ERR_INVALID_ARGUMENT, "null delay arrays");
  memcpy(h->poly.data(), poly, sizeof(double) * 3 * h->cfg.nant);
  memcpy(h->fso.data(), fso, sizeof(double) * h->cfg.nant);
  h->have_delays = true;
  return GXC_OK;
}

// FP8 per-channel scales from the calibration block cal [ctile][t < nt][stream][16] (FP32 spectra):
// one CTA per 16-channel tile; channel c's RMS over the nonzero values of all FFTs and streams
// (flagged FFTs hold zeros), scale 2^e with e = floor(log2(4 / rms)) so the RMS lands in [2, 4),
// clamped to [-60, 60]; a channel with no data keeps the handle's exponent def_e.  vscale = 2^-2e.
__global__ void chan_scales_kernel(const float2 *__restrict__ cal, int nstream, int nchan, int nt, int def_e,
                                   float *__restrict__ cscale, float *__restrict__ cvscale) {
  const int tile = blockIdx.x, ci = threadIdx.x & 15, j = threadIdx.x >> 4;  // 16 x 16 threads
  const int n = nt * nstream;
  const float2 *base = cal + (size_t)tile * n * 16;
  double acc = 0.0;
  int cnt = 0;
  for (int i = j; i < n; i += 16) {
    const float2 v = base[(size_t)i * 16 + ci];
    const double p = (double)v.x * v.x + (double)v.y * v.y;
    acc += p;
    cnt += p > 0.0 ? 1 : 0;
  }
  __shared__ double sacc[16][17];
  __shared__ int scnt[16][17];
  sacc[j][ci] = acc;
  scnt[j][ci] = cnt;
  __syncthreads();
  if (j == 0) {
    for (int k = 1; k < 16; k++) {
      acc += sacc[k][ci];
      cnt += scnt[k][ci];
    }
    int e = def_e;
    if (cnt > 0 && acc > 0.0 && isfinite(acc)) {
      const double rms = sqrt(acc / cnt);
      e = (int)floor(log2(4.0 / rms));
      e = e < -60 ? -60 : e > 60 ? 60 : e;
    }
    const int c = tile * 16 + ci;
    if (c < nchan) {
      cscale[c] = ldexpf(1.0f, e);
      cvscale[c] = ldexpf(1.0f, -2 * e);
    }
  }
}

static cudaError_t launch_chan_scales(const float2 *cal, int nstream, int nchan, int nt, int def_e, float *cscale,
                                      float *cvscale, cudaStream_t s) {
  chan_scales_kernel<<<(unsigned)((nchan + 15) / 16), 256, 0, s>>>(cal, nstream, nchan, nt, def_e, cscale, cvscale);
  return cudaGetLastError();
}

// finalisation: vis = (sum + comp) * scale / count (fxkernel.cpp:358-367)
// Sums the two accumulator planes (i and i + n) with a compensated add; a plane no launch wrote
// is zero and leaves the result bit-identical to the first plane's.
__global__ void finalize_kernel(const float2 *__restrict__ vsum, const float2 *__restrict__ vcomp,
                                const int32_t *__restrict__ counts, int nchan, size_t n, float scale,
                                const float *__restrict__ chan_vscale,
                                float2 *__restrict__ vis) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int bl = (int)(i / ((size_t)4 * nchan));
  const int cnt = counts[bl];
  const float2 s0 = vsum[i], c0 = vcomp[i], s1 = vsum[i + n], c1 = vcomp[i + n];
  float sx = s0.x, ex = c0.x, sy = s0.y, ey = c0.y;
  two_sum_add(sx, ex, s1.x);
  two_sum_add(sy, ey, s1.y);
  const float sc = chan_vscale ? chan_vscale[i % nchan] : scale;
  float re = (sx + (ex + c1.x)) * sc, im = (sy + (ey + c1.y)) * sc;
  if (cnt > 0) {
    re /= (float)cnt;
    im /= (float)cnt;
  }
  vis[i] = make_float2(re, im);
}

// Per-call parameters of up to kAnt antennas (about 10 KB: kernel parameters of up to
// 32 KB are allowed on this architecture).
struct UploadChunk {
  static constexpr int kAnt = 256;
  int a0, n;
  const uint8_t *ptrs[kAnt];
  const uint8_t *fvalid[kAnt];
  double poly[3 * kAnt];
  double fso[kAnt];
};

__global__ void upload_kernel(const __grid_constant__ UploadChunk u, const uint8_t **d_ptrs, double *d_poly,
                              double *d_fso, const uint8_t **d_fvalid) {
  for (int i = threadIdx.x; i < u.n; i += blockDim.x) {
    d_ptrs[u.a0 + i] = u.ptrs[i];
    d_fvalid[u.a0 + i] = u.fvalid[i];
    d_fso[u.a0 + i] = u.fso[i];
    for (int j = 0; j < 3; j++) d_poly[3 * (u.a0 + i) + j] = u.poly[3 * i + j];
  }
}

__global__ void add_kernel(float *__restrict__ dst, const float *__restrict__ src, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] += src[i];
}

gxc_status gxc_process(gxc_handle *h, void *stream) { return gxc::process_chained(h, stream, nullptr, nullptr); }

// process() with its host->device input copies ordered behind copy_wait (when given) and
// followed by a record of copy_done (when given); batches use it to chain the jobs' copies.
extern "C++" gxc_status gxc::process_chained(gxc_handle *h, void *stream, cudaEvent_t copy_wait,
                                             cudaEvent_t copy_done, int nchunk, const cudaEvent_t *chunk_ev,
                                             const long long *chunk_end) {
  if (!h) return GXC_ERR_INVALID_ARGUMENT;
  if (!h->have_input) return fail(h, GXC_ERR_STATE, "process() before set_input()");
  if (!h->have_delays) return fail(h, GXC_ERR_STATE, "process() before set_delays()");
  if (h->input_on_host && h->in_chunk_ev.empty()) return fail(h, GXC_ERR_STATE, "host input without a copy stream");
  cudaSetDevice(h->device);
  cudaStream_t s = (cudaStream_t)stream;
  const gxc_config &c = h->cfg;
  const int nant = c.nant;
  int launches = 0;

  // input pointers and the delay model travel as kernel parameters of a one-block upload
  // kernel (no host->device memcpy on the stream: small copies would queue on the copy
  // engine behind bulk input copies of other streams, and need no host wait here)
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  GXC_CUDA(h, cudaStreamIsCapturing(s, &cap), "querying stream capture");
  const bool capturing = cap != cudaStreamCaptureStatusNone;
  // inside a capture the handle's events become graph nodes that record on every replay,
  // so sync() and the getters wait for the latest graph launch; stage timing is off there
  const unsigned rec_flags = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
  const bool timing = h->stage_timing && !capturing;
  for (int a0 = 0; a0 < nant; a0 += UploadChunk::kAnt) {
    UploadChunk u;
    u.a0 = a0;
    u.n = nant - a0 < UploadChunk::kAnt ? nant - a0 : UploadChunk::kAnt;
    for (int i = 0; i < u.n; i++) {
      const int a = a0 + i;
      u.ptrs[i] = h->input_on_host ? h->d_inbuf + (size_t)a * h->bytes_per_ant : h->user_ptrs[a];
      for (int j = 0; j < 3; j++) u.poly[3 * i + j] = h->poly[3 * (size_t)a + j];
      u.fso[i] = h->fso[a];
      u.fvalid[i] = h->user_fvalid.empty() ? nullptr : h->user_fvalid[a];
    }
    upload_kernel<<<1, 128, 0, s>>>(u, h->d_inptrs, h->d_poly, h->d_fso, h->d_fvalid);
    GXC_CUDA(h, cudaGetLastError(), "upload kernel");
    launches++;
  }
  if (h->input_on_host) {
    // host inputs: copied on the handle's copy stream (forked from s) in time-ordered chunks, so
    // the F-stage blocks below start while later samples still load
    GXC_CUDA(h, cudaEventRecord(h->ev_fork, s), "forking the input copies");
    GXC_CUDA(h, cudaStreamWaitEvent(h->copy_stream, h->ev_fork, 0), "forking the input copies");
    if (copy_wait) GXC_CUDA(h, cudaStreamWaitEvent(h->copy_stream, copy_wait, 0), "ordering the input copies");
    // inside a capture (batch graphs) one chunk: many small memcpy nodes cost the graph more than
    // the overlap gains
    const int nch = capturing ? 1 : (int)h->in_chunk_ev.size();
    const long long bpa = (long long)h->bytes_per_ant;
    long long c0 = 0;
    for (int j = 0; j < nch; j++) {
      long long c1 = bpa;
      if (j < nch - 1) c1 = std::min(bpa, (bpa * (j + 1) / nch + 4095) / 4096 * 4096);
      for (int a = 0; c1 > c0 && a < nant; a++)
        GXC_CUDA(h,
                 cudaMemcpyAsync(h->d_inbuf + (size_t)a * h->bytes_per_ant + c0, h->user_ptrs[a] + c0,
                                 (size_t)(c1 - c0), cudaMemcpyHostToDevice, h->copy_stream),
                 "copying input to the device");
      // copy_done before the last chunk's event, so that the join on that event (below) also
      // covers it inside a stream capture
      if (j == nch - 1 && copy_done)
        GXC_CUDA(h, cudaEventRecordWithFlags(copy_done, h->copy_stream, rec_flags), "recording the input copies");
      GXC_CUDA(h, cudaEventRecord(h->in_chunk_ev[j], h->copy_stream), "recording an input chunk");
      h->in_chunk_end[j] = c1;
      if (c1 > c0) c0 = c1;
    }
    nchunk = nch;
    chunk_ev = h->in_chunk_ev.data();
    chunk_end = h->in_chunk_end.data();
  } else if (copy_done) {
    GXC_CUDA(h, cudaEventRecordWithFlags(copy_done, s, rec_flags), "recording the input copies");
  }
  if (timing) GXC_CUDA(h, cudaEventRecord(h->ev_begin, s), "timing event");

  GXC_CUDA(h, launch_geometry(h->job, s), "geometry kernel");
  launches++;
  if (h->nbl > 0) {
    GXC_CUDA(h, launch_counts(h->job, c.autos, h->d_counts, h->d_valid, s), "counts kernel");
    launches++;
  }
  const size_t nvis = (size_t)h->nbl * 4 * c.nchan;
  GXC_CUDA(h, cudaMemsetAsync(h->d_vsum, 0, sizeof(float2) * nvis * 2, s), "clearing accumulators");
  GXC_CUDA(h, cudaMemsetAsync(h->d_vcomp, 0, sizeof(float2) * nvis * 2, s), "clearing accumulators");

  // blocks: T FFTs each; with host inputs T0, 2 T0, 4 T0, ... up to T
  h->blk.clear();
  for (int t0 = 0, bt = h->input_on_host ? h->T0 : h->T; t0 < c.nfft;) {
    const int nt = (c.nfft - t0) < bt ? (c.nfft - t0) : bt;
    h->blk.emplace_back(t0, nt);
    t0 += nt;
    bt = 2 * bt < h->T ? 2 * bt : h->T;
  }
  h->nblocks = (int)h->blk.size();
  if (timing && h->ev_stage.size() != (size_t)3 * h->nblocks) {
    for (cudaEvent_t e : h->ev_stage) cudaEventDestroy(e);
    h->ev_stage.assign((size_t)3 * h->nblocks, nullptr);
    for (auto &e : h->ev_stage) GXC_CUDA(h, cudaEventCreate(&e), "timing event");
  }
  int waited = -1;  // input chunks already waited for
  for (int b = 0; b < h->nblocks; b++) {
    const int t0 = h->blk[(size_t)b].first, nt = h->blk[(size_t)b].second;
    if (nchunk > 0) {
      // the first input chunk that holds every window of this block
      const long long need = gxc_input_bytes_for_ffts(&c, h->poly.data(), h->fso.data(), t0, nt);
      int j = 0;
      while (j < nchunk - 1 && chunk_end[j] < need) j++;
      if (j > waited) {
        GXC_CUDA(h, cudaStreamWaitEvent(s, chunk_ev[j], 0), "ordering the input chunks");
        waited = j;
      }
    }
    if (b == 0 && h->d_cscale) {
      // FP8 per-channel scales: the first cal_T FFTs channelised in FP32, each channel's RMS over
      // them and all streams, a power of two per channel
      GXC_CUDA(h, launch_fstage(h->job, h->d_tw, 0, h->cal_T, h->cal_T, h->d_cal, CHAN_F32, 1.0f, s),
               "F-stage calibration kernel");
      GXC_CUDA(h, launch_chan_scales(h->d_cal, 2 * nant, c.nchan, h->cal_T, -ilog2i(h->F) / 2 - (c.is_complex ? 4 : 0),
                                     h->d_cscale, h->d_cvscale, s),
               "channel scale kernel");
      launches += 2;
    }
    // with per-channel FP8 scales the channel's scale replaces the handle's
    const float osc = h->d_cscale ? 1.0f : h->out_scale;
    if (timing) GXC_CUDA(h, cudaEventRecord(h->ev_stage[3 * b], s), "timing event");
    if (h->tc_fstage)
      GXC_CUDA(h, launch_fstage_tc(h->job, h->d_tc_tables, t0, nt, h->T, h->d_chan, h->chan_type, osc, s,
                                   h->d_cscale),
               "tensor-core F-stage kernel");
    else
      GXC_CUDA(h, launch_fstage(h->job, h->d_tw, t0, nt, h->T, h->d_chan, h->chan_type, osc, s, h->d_cscale),
               "F-stage kernel");
    launches++;
    if (timing) GXC_CUDA(h, cudaEventRecord(h->ev_stage[3 * b + 1], s), "timing event");
    if (h->nbl > 0) {
      if (h->xeng == GXC_XENGINE_TENSOR) {
        // FP32 spectra go through the FP16 hi/lo split scaled by 2^-(log2F/2): a spectrum value is
        // at most F * 128*sqrt(2) (8-bit complex; 2-bit real is below that), which after the scale
        // is <= 2^ceil(log2F/2) * 182 <= 46592 < 65504, the FP16 maximum, for every F <= 32768.
        GXC_CUDA(h,
                 launch_xstage_tensor(h->d_chan, h->chan_type, nant, c.nchan, h->T, nt, c.autos, h->d_vsum,
                                      h->d_vcomp, s, h->log2F / 2,
                                      c.x_split == GXC_XSPLIT_OFF ? 1 : c.x_split == GXC_XSPLIT_ON ? 3 : 2, nvis),
                 "tensor-core X-stage kernel");
      } else {
        GXC_CUDA(h,
                 launch_xstage_cuda_core(h->d_chan, h->chan_type, nant, c.nchan, h->T, nt, c.autos, h->d_pairs,
                                         h->d_vsum, h->d_vcomp, s),
                 "X-stage kernel");
      }
      launches++;
    }
    if (timing) GXC_CUDA(h, cudaEventRecord(h->ev_stage[3 * b + 2], s), "timing event");
  }
  // join the input copies (the last blocks may not need the last chunk)
  if (nchunk > 0) GXC_CUDA(h, cudaStreamWaitEvent(s, chunk_ev[nchunk - 1], 0), "joining the input copies");
  if (nvis > 0) {
    const int th = 256;
    finalize_kernel<<<(unsigned)((nvis + th - 1) / th), th, 0, s>>>(h->d_vsum, h->d_vcomp, h->d_counts, c.nchan,
                                                                     nvis, h->vis_scale, h->d_cvscale, h->d_vis);
    GXC_CUDA(h, cudaGetLastError(), "finalize kernel");
    launches++;
  }
  if (timing) GXC_CUDA(h, cudaEventRecord(h->ev_end, s), "timing event");
  GXC_CUDA(h, cudaEventRecordWithFlags(h->ev_done, s, rec_flags), "recording the completion event");
  if (!capturing) h->last_stream = s;
  h->processed = true;
  h->launches = launches;
  return GXC_OK;
}

gxc_status gxc_probe_unpack(gxc_handle *h, float *decoded) {
  if (!h) return GXC_ERR_INVALID_ARGUMENT;
  if (!decoded) return fail(h, GXC_ERR_INVALID_ARGUMENT, "null output");
  if (h->have_input && h->input_on_host)
    return fail(h, GXC_ERR_UNSUPPORTED, "the decode probe takes device inputs");
  gxc_status st = gxc_process(h, nullptr);  // uploads pointers and delays, computes the geometry
  if (st == GXC_OK) st = gxc_sync(h);
  if (st != GXC_OK) return st;
  const gxc_config &c = h->cfg;
  const size_t n = (size_t)c.nant * 2 * c.nfft * h->F;
  float2 *probe = nullptr;
  void *chan = nullptr;
  cudaError_t e = cudaMalloc((void **)&probe, n * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&chan, (size_t)h->T * c.nchan * 2 * c.nant * sizeof(float2));
  if (e == cudaSuccess) e = cudaMemset(probe, 0xFF, n * sizeof(float2));  // NaN
  for (int b = 0; e == cudaSuccess && b < h->nblocks; b++) {
    const int t0 = b * h->T;
    const int nt = (c.nfft - t0) < h->T ? (c.nfft - t0) : h->T;
    // the probe runs the handle's own F-stage kernel family
    e = h->tc_fstage ? launch_fstage_tc(h->job, h->d_tc_tables, t0, nt, h->T, chan, h->chan_type, h->out_scale,
                                        nullptr, nullptr, probe)
                     : launch_fstage_probe(h->job, h->d_tw, t0, nt, h->T, chan, h->chan_type, h->out_scale, probe,
                                           nullptr);
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(decoded, probe, n * sizeof(float2), cudaMemcpyDefault);
  cudaFree(probe);
  cudaFree(chan);
  if (e != cudaSuccess) return cuda_fail(h, e, "decode probe");
  return GXC_OK;
}

gxc_status gxc_sync(gxc_handle *h) {
  if (!h) return GXC_ERR_INVALID_ARGUMENT;
  if (!h->processed) return GXC_OK;
  cudaSetDevice(h->device);
  GXC_CUDA(h, cudaEventSynchronize(h->ev_done), "synchronising");
  GXC_CUDA(h, cudaGetLastError(), "device error");
  if (h->xeng == GXC_XENGINE_TENSOR) {
    int flag = 0;
    GXC_CUDA(h, xstage_tensor_take_error(&flag), "reading the X-stage status");
    if (flag) return fail(h, GXC_ERR_TIMEOUT, "tensor-core X-stage: a bounded device wait expired");
  }
  if (h->tc_fstage) {
    int flag = 0;
    GXC_CUDA(h, fstage_tc_take_error(&flag), "reading the F-stage status");
    if (flag) return fail(h, GXC_ERR_TIMEOUT, "tensor-core F-stage: a bounded device wait expired");
  }
  return GXC_OK;
}

static bool is_device_ptr(const void *p) {
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

gxc_status gxc_get_visibilities(gxc_handle *h, float *out) {
  if (!h) return GXC_ERR_INVALID_ARGUMENT;
  if (!out) return fail(h, GXC_ERR_INVALID_ARGUMENT, "null output");
  if (!h->processed) return fail(h, GXC_ERR_STATE, "no processed sub-integration");
  gxc_status st = gxc_sync(h);
  if (st != GXC_OK) return st;
  const size_t n = (size_t)h->nbl * 4 * h->cfg.nchan * 2;
  GXC_CUDA(h, cudaMemcpy(out, h->d_vis, n * sizeof(float), cudaMemcpyDefault), "copying visibilities");
  return GXC_OK;
}

gxc_status gxc_accumulate(gxc_handle *h, float *odata) {
  if (!h) return GXC_ERR_INVALID_ARGUMENT;
  if (!odata) return fail(h, GXC_ERR_INVALID_ARGUMENT, "null output");
  if (!h->processed) return fail(h, GXC_ERR_STATE, "no processed sub-integration");
  gxc_status st = gxc_sync(h);
  if (st != GXC_OK) return st;
  const size_t n = (size_t)h->nbl * 4 * h->cfg.nchan * 2;
  if (is_device_ptr(odata)) {
    const int th = 256;
    add_kernel<<<(unsigned)((n + th - 1) / th), th, 0, h->last_stream>>>(odata, (const float *)h->d_vis, n);
    GXC_CUDA(h, cudaGetLastError(), "accumulate kernel");
    GXC_CUDA(h, cudaStreamSynchronize(h->last_stream), "accumulate");
  } else {
    std::vector<float> tmp(n);
    GXC_CUDA(h, cudaMemcpy(tmp.data(), h->d_vis, n * sizeof(float), cudaMemcpyDeviceToHost), "copying visibilities");
    for (size_t i = 0; i < n; i++) odata[i] += tmp[i];
  }
  return GXC_OK;
}

gxc_status gxc_get_baseline_counts(gxc_handle *h, int32_t *counts) {
  if (!h) return GXC_ERR_INVALID_ARGUMENT;
  if (!counts) return fail(h, GXC_ERR_INVALID_ARGUMENT, "null output");
  if (!h->processed) return fail(h, GXC_ERR_STATE, "no processed sub-integration");
  gxc_status st = gxc_sync(h);
  if (st != GXC_OK) return st;
  if (h->nbl > 0)
    GXC_CUDA(h, cudaMemcpy(counts, h->d_counts, sizeof(int32_t) * h->nbl, cudaMemcpyDeviceToHost), "copying counts");
  return GXC_OK;
}

gxc_status gxc_get_valid_flags(gxc_handle *h, uint8_t *flags) {
  if (!h) return GXC_ERR_INVALID_ARGUMENT;
  if (!flags) return fail(h, GXC_ERR_INVALID_ARGUMENT, "null output");
  if (!h->processed) return fail(h, GXC_ERR_STATE, "no processed sub-integration");
  if (h->nbl == 0) return fail(h, GXC_ERR_STATE, "no baselines: flags are not exported");
  gxc_status st = gxc_sync(h);
  if (st != GXC_OK) return st;
  GXC_CUDA(h, cudaMemcpy(flags, h->d_valid, (size_t)h->cfg.nant * h->cfg.nfft, cudaMemcpyDeviceToHost),
           "copying flags");
  return GXC_OK;
}

gxc_status gxc_enable_stage_timing(gxc_handle *h, int enable) {
  if (!h) return GXC_ERR_INVALID_ARGUMENT;
  cudaSetDevice(h->device);
  h->stage_timing = enable != 0;
  if (h->stage_timing && !h->ev_begin) {
    GXC_CUDA(h, cudaEventCreate(&h->ev_begin), "timing event");
    GXC_CUDA(h, cudaEventCreate(&h->ev_end), "timing event");
  }
  return GXC_OK;
}

gxc_status gxc_stage_times(gxc_handle *h, float *f_ms, float *x_ms, float *total_ms) {
  if (!h) return GXC_ERR_INVALID_ARGUMENT;
  if (!h->stage_timing || !h->processed) return fail(h, GXC_ERR_STATE, "stage timing not enabled/recorded");
  gxc_status st = gxc_sync(h);
  if (st != GXC_OK) return st;
  float fs = 0.f, xs = 0.f, tot = 0.f;
  for (int b = 0; b < h->nblocks; b++) {
    float a = 0.f, x = 0.f;
    GXC_CUDA(h, cudaEventElapsedTime(&a, h->ev_stage[3 * b], h->ev_stage[3 * b + 1]), "timing");
    GXC_CUDA(h, cudaEventElapsedTime(&x, h->ev_stage[3 * b + 1], h->ev_stage[3 * b + 2]), "timing");
    fs += a;
    xs += x;
  }
  GXC_CUDA(h, cudaEventElapsedTime(&tot, h->ev_begin, h->ev_end), "timing");
  if (f_ms) *f_ms = fs;
  if (x_ms) *x_ms = xs;
  if (total_ms) *total_ms = tot;
  return GXC_OK;
}

}  // extern "C"
