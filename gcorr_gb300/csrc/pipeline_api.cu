// Streaming ingest of consecutive sub-integrations from host memory, with a
// device-side long-integration accumulator and linear->circular polarisation
// conversion of the visibilities.
//
// The reference GPU driver copies each sub-integration's input and waits for
// the previous stream before reusing its buffer (gcorr/src/testgpukernel.cu:462-486);
// the CPU path calls process() then accumulate() per sub-integration
// (fxkernel/src/testfxkernel.cpp:81-108).  Here the input of sub-integration
// k+1 is copied on a copy stream into the second of `nslots` device input
// slots while sub-integration k is correlated on the compute stream, so the
// host->device traffic hides behind the F and X stages.  Per slot, events
// order the work: `consumed` (compute done, the slot may be overwritten and the
// visibilities were copied out) and one per input chunk: the copy runs in time
// order in kChunks pieces of every antenna, and each F-stage launch waits only
// for the piece that holds its FFT windows (gxc_input_bytes_for_ffts), so the
// correlation of a sub-integration starts while its later samples still load.
//
// Polarisation conversion follows the voltage-domain form of the reference's
// linear2circular kernels (examples/chris/bench/gpubench.cu:145-160): per
// antenna and channel, P1' = g1*P1 - g2*P2 and P2' = g1*P1 + g2*P2.  That is a
// 2x2 Jones matrix J = [[g1, -g2], [g1, g2]] on the voltages, so on the
// visibility matrix of a baseline (j,k), V = [[AA, AB], [BA, BB]], it is
// V' = J_j V J_k^H exactly; applying it to the nbl*4*nchan visibilities
// instead of the nant*2*nchan*nfft voltages is the same result for a fraction
// of the traffic.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "gxc_internal.h"

namespace {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {  // a * conj(b)
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

// Antennas (j,k) of baseline b: crosses in fxkernel order, then autos.
__device__ __forceinline__ void baseline_pair(int b, int nant, int *j, int *k) {
  const int ncross = nant * (nant - 1) / 2;
  if (b >= ncross) {
    *j = *k = b - ncross;
    return;
  }
  int a = 0;
  int row = nant - 1;
  while (b >= row) {
    b -= row;
    a++;
    row--;
  }
  *j = a;
  *k = a + 1 + b;
}

// One thread per (baseline, channel).  gains: [nant][2][nchan] complex, or
// null for ideal feeds (g1 = 1/sqrt2, g2 = i/sqrt2: P1' = (X - iY)/sqrt2,
// P2' = (X + iY)/sqrt2).
__global__ void lin2circ_kernel(float2 *vis, const float2 *gains, int nant, int nbl, int nchan) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)nbl * nchan) return;
  const int b = (int)(i / nchan);
  const int c = (int)(i % nchan);
  int j, k;
  baseline_pair(b, nant, &j, &k);
  const float r = 0.70710678118654752f;
  float2 gj1 = make_float2(r, 0.f), gj2 = make_float2(0.f, r), gk1 = gj1, gk2 = gj2;
  if (gains) {
    gj1 = gains[((size_t)j * 2 + 0) * nchan + c];
    gj2 = gains[((size_t)j * 2 + 1) * nchan + c];
    gk1 = gains[((size_t)k * 2 + 0) * nchan + c];
    gk2 = gains[((size_t)k * 2 + 1) * nchan + c];
  }
  float2 *v = vis + (size_t)b * 4 * nchan + c;
  const float2 aa = v[0], ab = v[nchan], ba = v[2 * nchan], bb = v[3 * nchan];
  // W = J_j V : rows of J_j are (g1, -g2) and (g1, g2)
  const float2 w00 = csub(cmul(gj1, aa), cmul(gj2, ba)), w01 = csub(cmul(gj1, ab), cmul(gj2, bb));
  const float2 w10 = cadd(cmul(gj1, aa), cmul(gj2, ba)), w11 = cadd(cmul(gj1, ab), cmul(gj2, bb));
  // V' = W J_k^H : columns of J_k^H are conj of rows of J_k
  v[0] = csub(cmulc(w00, gk1), cmulc(w01, gk2));
  v[nchan] = cadd(cmulc(w00, gk1), cmulc(w01, gk2));
  v[2 * nchan] = csub(cmulc(w10, gk1), cmulc(w11, gk2));
  v[3 * nchan] = cadd(cmulc(w10, gk1), cmulc(w11, gk2));
}

// Long integration: compensated (TwoSum) running sum of sub-integration visibilities.
__global__ void integrate_kernel(const float *vis, float *sum, float *comp, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    gxc::two_sum_add(sum[i], comp[i], vis[i]);
}

__global__ void integration_out_kernel(const float *sum, const float *comp, float *out, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = sum[i] + comp[i];
}

unsigned grid_for(size_t n, int th) {
  size_t g = (n + th - 1) / th;
  return (unsigned)(g < 4096 ? (g ? g : 1) : 4096);
}

// input chunks per sub-integration (each at least kMinChunkBytes per antenna)
constexpr int kChunks = 8;
constexpr size_t kMinChunkBytes = 1 << 20;

}  // namespace

struct gxc_pipeline {
  gxc_config cfg{};
  gxc_handle *h = nullptr;
  int device = 0;
  int nslots = 2;
  size_t bytes_per_ant = 0, ant_stride = 0;
  int nbl = 0;
  size_t nvis_floats = 0;
  std::vector<uint8_t *> slot_buf;
  std::vector<cudaEvent_t> loaded, consumed;
  int nchunk = 1;
  std::vector<cudaEvent_t> chunk_ev;  // [slot][nchunk]: input bytes [0, chunk_end[j]) loaded
  std::vector<int64_t> slot_seq;
  cudaStream_t copy = nullptr, compute = nullptr;
  int64_t next_seq = 0;
  // long integration
  float *isum = nullptr, *icomp = nullptr;
  int nintegrated = 0;
  // polarisation conversion
  bool lin2circ = false;
  float2 *d_gains = nullptr;
  std::string err;
};

namespace {

gxc_status pfail(gxc_pipeline *p, gxc_status st, const std::string &m) {
  if (p) p->err = m;
  return st;
}

#define PCUDA(p, call, what)                                                                 \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) return pfail(p, GXC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e_)); \
  } while (0)

void destroy_pipeline(gxc_pipeline *p) {
  if (p->compute) cudaStreamSynchronize(p->compute);
  if (p->copy) cudaStreamSynchronize(p->copy);
  for (uint8_t *b : p->slot_buf) cudaFree(b);
  for (cudaEvent_t e : p->loaded) cudaEventDestroy(e);
  for (cudaEvent_t e : p->consumed) cudaEventDestroy(e);
  for (cudaEvent_t e : p->chunk_ev) cudaEventDestroy(e);
  if (p->copy) cudaStreamDestroy(p->copy);
  if (p->compute) cudaStreamDestroy(p->compute);
  if (p->isum) cudaFree(p->isum);
  if (p->icomp) cudaFree(p->icomp);
  if (p->d_gains) cudaFree(p->d_gains);
  if (p->h) gxc_destroy(p->h);
  delete p;
}

}  // namespace

extern "C" {

gxc_status gxc_pipeline_create(const gxc_config *cfg, int nslots, int integrate, gxc_pipeline **out) {
  if (!cfg || !out || nslots < 1 || nslots > 8) return GXC_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  gxc_pipeline *p = new gxc_pipeline();
  p->cfg = *cfg;
  p->nslots = nslots;
  gxc_status st = gxc_create(cfg, &p->h);
  if (st != GXC_OK) {
    destroy_pipeline(p);
    return st;
  }
  cudaGetDevice(&p->device);
  p->bytes_per_ant = gxc_input_bytes_per_antenna(cfg);
  p->ant_stride = (p->bytes_per_ant + 255) / 256 * 256;
  p->nbl = gxc_num_baselines(cfg);
  p->nvis_floats = (size_t)p->nbl * 4 * cfg->nchan * 2;
  p->nchunk = p->bytes_per_ant >= (size_t)kChunks * kMinChunkBytes ? kChunks : 1;
  cudaError_t e = cudaStreamCreateWithFlags(&p->copy, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->compute, cudaStreamNonBlocking);
  for (int s = 0; e == cudaSuccess && s < nslots; s++) {
    uint8_t *buf = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    e = cudaMalloc(&buf, p->ant_stride * cfg->nant);
    if (e == cudaSuccess) p->slot_buf.push_back(buf);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&a, cudaEventDisableTiming);
    if (e == cudaSuccess) p->loaded.push_back(a);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b, cudaEventDisableTiming);
    if (e == cudaSuccess) p->consumed.push_back(b);
    for (int j = 0; e == cudaSuccess && j < p->nchunk; j++) {
      cudaEvent_t c = nullptr;
      e = cudaEventCreateWithFlags(&c, cudaEventDisableTiming);
      if (e == cudaSuccess) p->chunk_ev.push_back(c);
    }
    p->slot_seq.push_back(-1);
  }
  if (e == cudaSuccess && integrate && p->nvis_floats) {
    e = cudaMalloc(&p->isum, p->nvis_floats * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&p->icomp, p->nvis_floats * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(p->isum, 0, p->nvis_floats * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(p->icomp, 0, p->nvis_floats * sizeof(float));
  }
  if (e != cudaSuccess) {
    fprintf(stderr, "gxc_pipeline_create: %s\n", cudaGetErrorString(e));
    destroy_pipeline(p);
    return e == cudaErrorMemoryAllocation ? GXC_ERR_OUT_OF_MEMORY : GXC_ERR_CUDA;
  }
  *out = p;
  return GXC_OK;
}

gxc_status gxc_pipeline_set_lin2circ(gxc_pipeline *p, int enable, const float *gains) {
  if (!p) return GXC_ERR_INVALID_ARGUMENT;
  cudaSetDevice(p->device);
  PCUDA(p, cudaStreamSynchronize(p->compute), "waiting for the compute stream");
  p->lin2circ = enable != 0;
  if (p->d_gains) {
    cudaFree(p->d_gains);
    p->d_gains = nullptr;
  }
  if (enable && gains) {
    const size_t n = (size_t)p->cfg.nant * 2 * p->cfg.nchan;
    PCUDA(p, cudaMalloc(&p->d_gains, n * sizeof(float2)), "allocating gains");
    PCUDA(p, cudaMemcpy(p->d_gains, gains, n * sizeof(float2), cudaMemcpyDefault), "copying gains");
  }
  return GXC_OK;
}

gxc_status gxc_pipeline_submit(gxc_pipeline *p, const uint8_t *const *inputs, const double *poly, const double *fso,
                               float *vis_out, int64_t *seq_out) {
  if (!p || !inputs || !poly || !fso) return GXC_ERR_INVALID_ARGUMENT;
  for (int a = 0; a < p->cfg.nant; a++)
    if (!inputs[a]) return pfail(p, GXC_ERR_INVALID_ARGUMENT, "null input buffer");
  cudaSetDevice(p->device);
  const int64_t seq = p->next_seq;
  const int slot = (int)(seq % p->nslots);
  uint8_t *buf = p->slot_buf[slot];
  // copy stream: wait until the slot's previous sub-integration was correlated, then load it in
  // time order, chunk by chunk across the antennas
  PCUDA(p, cudaStreamWaitEvent(p->copy, p->consumed[slot], 0), "ordering the copy");
  const int nch = p->nchunk;
  cudaEvent_t *cev = p->chunk_ev.data() + (size_t)slot * nch;
  std::vector<long long> chunk_end(nch);
  long long c0 = 0;
  for (int j = 0; j < nch; j++) {
    long long c1 = (long long)p->bytes_per_ant;
    if (j < nch - 1) {
      c1 = ((long long)p->bytes_per_ant * (j + 1) / nch + 4095) / 4096 * 4096;
      if (c1 > (long long)p->bytes_per_ant) c1 = (long long)p->bytes_per_ant;
    }
    for (int a = 0; c1 > c0 && a < p->cfg.nant; a++)
      PCUDA(p, cudaMemcpyAsync(buf + (size_t)a * p->ant_stride + c0, inputs[a] + c0, (size_t)(c1 - c0), cudaMemcpyDefault,
                               p->copy),
            "copying input to the device");
    PCUDA(p, cudaEventRecord(cev[j], p->copy), "recording a load event");
    chunk_end[j] = c1;
    if (c1 > c0) c0 = c1;
  }
  PCUDA(p, cudaEventRecord(p->loaded[slot], p->copy), "recording the load event");
  // compute stream: correlate (each F-stage launch waits for its input chunk), post-process, copy out
  std::vector<const uint8_t *> ptrs(p->cfg.nant);
  for (int a = 0; a < p->cfg.nant; a++) ptrs[a] = buf + (size_t)a * p->ant_stride;
  gxc_status st = gxc_set_input(p->h, ptrs.data(), p->bytes_per_ant);
  if (st == GXC_OK) st = gxc_set_delays(p->h, poly, fso);
  if (st == GXC_OK) st = gxc::process_chained(p->h, p->compute, nullptr, nullptr, nch, cev, chunk_end.data());
  if (st != GXC_OK) return pfail(p, st, std::string("process: ") + gxc_last_error(p->h));
  float *d_vis = const_cast<float *>(gxc_device_visibilities(p->h));
  const int th = 256;
  if (p->lin2circ && p->nbl > 0) {
    const size_t n = (size_t)p->nbl * p->cfg.nchan;
    lin2circ_kernel<<<(unsigned)((n + th - 1) / th), th, 0, p->compute>>>((float2 *)d_vis, p->d_gains, p->cfg.nant,
                                                                         p->nbl, p->cfg.nchan);
    PCUDA(p, cudaGetLastError(), "polarisation conversion kernel");
  }
  if (p->isum) {
    integrate_kernel<<<grid_for(p->nvis_floats, th), th, 0, p->compute>>>(d_vis, p->isum, p->icomp, p->nvis_floats);
    PCUDA(p, cudaGetLastError(), "integration kernel");
    p->nintegrated++;
  }
  if (vis_out && p->nvis_floats)
    PCUDA(p, cudaMemcpyAsync(vis_out, d_vis, p->nvis_floats * sizeof(float), cudaMemcpyDefault, p->compute),
          "copying visibilities out");
  PCUDA(p, cudaEventRecord(p->consumed[slot], p->compute), "recording the completion event");
  p->slot_seq[slot] = seq;
  p->next_seq = seq + 1;
  if (seq_out) *seq_out = seq;
  return GXC_OK;
}

gxc_status gxc_pipeline_wait(gxc_pipeline *p, int64_t seq) {
  if (!p || seq < 0 || seq >= p->next_seq) return GXC_ERR_INVALID_ARGUMENT;
  cudaSetDevice(p->device);
  const int slot = (int)(seq % p->nslots);
  // the slot's event marks its latest sub-integration, which completes after `seq`
  PCUDA(p, cudaEventSynchronize(p->consumed[slot]), "waiting for a sub-integration");
  return GXC_OK;
}

gxc_status gxc_pipeline_sync(gxc_pipeline *p) {
  if (!p) return GXC_ERR_INVALID_ARGUMENT;
  cudaSetDevice(p->device);
  PCUDA(p, cudaStreamSynchronize(p->copy), "copy stream");
  PCUDA(p, cudaStreamSynchronize(p->compute), "compute stream");
  gxc_status st = gxc_sync(p->h);
  if (st != GXC_OK) return pfail(p, st, gxc_last_error(p->h));
  return GXC_OK;
}

gxc_status gxc_pipeline_integration(gxc_pipeline *p, float *out, int reset, int *nsub) {
  if (!p) return GXC_ERR_INVALID_ARGUMENT;
  if (!p->isum) return pfail(p, GXC_ERR_STATE, "pipeline created without integration");
  gxc_status st = gxc_pipeline_sync(p);
  if (st != GXC_OK) return st;
  if (nsub) *nsub = p->nintegrated;
  if (out && p->nvis_floats) {
    float *tmp = nullptr;
    PCUDA(p, cudaMalloc(&tmp, p->nvis_floats * sizeof(float)), "integration scratch");
    integration_out_kernel<<<grid_for(p->nvis_floats, 256), 256, 0, p->compute>>>(p->isum, p->icomp, tmp,
                                                                                  p->nvis_floats);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(out, tmp, p->nvis_floats * sizeof(float), cudaMemcpyDefault, p->compute);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->compute);
    cudaFree(tmp);
    if (e != cudaSuccess) return pfail(p, GXC_ERR_CUDA, std::string("integration read-out: ") + cudaGetErrorString(e));
  }
  if (reset) {
    PCUDA(p, cudaMemsetAsync(p->isum, 0, p->nvis_floats * sizeof(float), p->compute), "integration reset");
    PCUDA(p, cudaMemsetAsync(p->icomp, 0, p->nvis_floats * sizeof(float), p->compute), "integration reset");
    PCUDA(p, cudaStreamSynchronize(p->compute), "integration reset");
    p->nintegrated = 0;
  }
  return GXC_OK;
}

gxc_handle *gxc_pipeline_handle(gxc_pipeline *p) { return p ? p->h : nullptr; }

const char *gxc_pipeline_last_error(const gxc_pipeline *p) { return p ? p->err.c_str() : "null pipeline"; }

gxc_status gxc_pipeline_destroy(gxc_pipeline *p) {
  if (!p) return GXC_ERR_INVALID_ARGUMENT;
  cudaSetDevice(p->device);
  destroy_pipeline(p);
  return GXC_OK;
}

gxc_status gxc_lin2circ(float *vis, const float *gains, int nant, int nchan, int autos, void *stream) {
  if (!vis || nant < 1 || nchan < 1) return GXC_ERR_INVALID_ARGUMENT;
  const int nbl = nant * (nant - 1) / 2 + (autos ? nant : 0);
  if (nbl == 0) return GXC_OK;
  const size_t n = (size_t)nbl * nchan;
  const int th = 256;
  lin2circ_kernel<<<(unsigned)((n + th - 1) / th), th, 0, (cudaStream_t)stream>>>((float2 *)vis,
                                                                                   (const float2 *)gains, nant, nbl,
                                                                                   nchan);
  return cudaGetLastError() == cudaSuccess ? GXC_OK : GXC_ERR_CUDA;
}

}  // extern "C"
