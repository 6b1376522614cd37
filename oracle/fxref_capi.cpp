/*
 * fxref_capi.cpp — C entry points around the reference's own FxKernel class
 * (TEST INFRASTRUCTURE ONLY).
 *
 * Linked with the reference's unmodified fxkernel/src/fxkernel.cpp and the
 * IPP-compatible shim in oracle/ipp_shim/ into oracle/_ref/libfxref.so, so that
 * tests can run the reference process() (fxkernel/src/fxkernel.h:29-64) on the
 * same inputs as the GPU engine.  The FxKernel constructor exit()s on
 * configurations it rejects (fxkernel/src/fxkernel.cpp:46-63) and unpack()
 * only handles 2-bit data (:489-496), so those cases are refused here first.
 */
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>
#include "fxkernel.h"

extern "C" {

/* Runs one sub-integration through the reference and returns its normalised
 * visibilities, complex64 interleaved in [nant*(nant-1)/2][4][nchan] order.
 * Returns 0 on success, nonzero when the reference cannot run the case. */
int fxref_process(int nant, int nchan, int nfft, int nbit, double lo, double bw, int iscomplex,
                  const uint8_t *const *inputs, const double *poly /* [nant][3] */, const double *fso,
                  float *vis_out) {
  if (nbit != 2 || iscomplex) return 2;
  int s = (int)std::sqrt((double)nchan);
  if (s * s != nchan) return 3;
  if (nant < 2 || nfft < 1) return 4;

  FxKernel fx(nant, nchan, nfft, nbit, lo, bw, iscomplex != 0);
  u8 **idata = new u8 *[nant];
  double **delays = new double *[nant];
  double *offsets = new double[nant];
  for (int a = 0; a < nant; a++) {
    idata[a] = const_cast<u8 *>(inputs[a]);
    delays[a] = new double[3];
    for (int k = 0; k < 3; k++) delays[a][k] = poly[3 * a + k];
    offsets[a] = fso[a];
  }
  fx.setInputData(idata);
  fx.setDelays(delays, offsets);
  fx.process();

  const int nbl = nant * (nant - 1) / 2;
  cf32 ***odata = new cf32 **[nbl];
  for (int b = 0; b < nbl; b++) {
    odata[b] = new cf32 *[4];
    for (int p = 0; p < 4; p++) {
      odata[b][p] = reinterpret_cast<cf32 *>(vis_out + ((size_t)b * 4 + p) * 2 * (size_t)nchan);
      std::memset(odata[b][p], 0, sizeof(cf32) * (size_t)nchan);
    }
  }
  fx.accumulate(odata);
  for (int b = 0; b < nbl; b++) delete[] odata[b];
  delete[] odata;
  for (int a = 0; a < nant; a++) delete[] delays[a];
  delete[] delays;
  delete[] offsets;
  delete[] idata;
  return 0;
}

/* Writes the reference's text visibility dump (fxkernel.cpp:370-412) for one sub-integration. */
int fxref_save(int nant, int nchan, int nfft, int nbit, double lo, double bw, int iscomplex,
               const uint8_t *const *inputs, const double *poly, const double *fso, const char *path) {
  if (nbit != 2 || iscomplex) return 2;
  int s = (int)std::sqrt((double)nchan);
  if (s * s != nchan) return 3;
  FxKernel fx(nant, nchan, nfft, nbit, lo, bw, iscomplex != 0);
  u8 **idata = new u8 *[nant];
  double **delays = new double *[nant];
  double *offsets = new double[nant];
  for (int a = 0; a < nant; a++) {
    idata[a] = const_cast<u8 *>(inputs[a]);
    delays[a] = new double[3];
    for (int k = 0; k < 3; k++) delays[a][k] = poly[3 * a + k];
    offsets[a] = fso[a];
  }
  fx.setInputData(idata);
  fx.setDelays(delays, offsets);
  fx.process();
  fx.saveVisibilities(path);
  for (int a = 0; a < nant; a++) delete[] delays[a];
  delete[] delays;
  delete[] offsets;
  delete[] idata;
  return 0;
}

/* CPU baseline: the reference's thread replication (fxkernel/src/bench_fxkernel.cpp:93-139), one
 * FxKernel per thread, each constructed and given its delays before the clock starts.  Thread t
 * processes FFTs [fft0 + t*nfft/nthreads, fft0 + (t+1)*nfft/nthreads) of the sub-integration whose
 * buffers are `inputs` (each holding at least (fft0+nfft+1) FFT windows): its input pointers start
 * at the slice's first window and its delay polynomial is re-expanded about the slice's first FFT
 * (t -> t + start).  Returns the wall-clock seconds from the common start to the last thread's end
 * of process(), or a negative value when the reference cannot run the case. */
double fxref_bench(int nant, int nchan, int nbit, double lo, double bw, int iscomplex, const uint8_t *const *inputs,
                   const double *poly, const double *fso, int fft0, int nfft, int nthreads) {
  if (nbit != 2 || iscomplex) return -2.0;
  int s = (int)std::sqrt((double)nchan);
  if (s * s != nchan) return -3.0;
  if (nant < 2 || nfft < 1 || nthreads < 1 || fft0 < 0) return -4.0;
  if (nthreads > nfft) nthreads = nfft;
  const long long F = 2LL * nchan;
  const long long bytes_per_fft = F * 2 * nbit / 8;  // 2 pols of F real samples
  struct Slice {
    FxKernel *fx = nullptr;
    std::vector<u8 *> idata;
    std::vector<double *> dptr;
    std::vector<double> d, off;
  };
  std::vector<Slice> sl((size_t)nthreads);
  for (int t = 0; t < nthreads; t++) {
    const int b = fft0 + (int)((long long)nfft * t / nthreads), e = fft0 + (int)((long long)nfft * (t + 1) / nthreads);
    Slice &x = sl[(size_t)t];
    x.fx = new FxKernel(nant, nchan, e - b, nbit, lo, bw, false);
    x.idata.resize((size_t)nant);
    x.d.resize((size_t)nant * 3);
    x.dptr.resize((size_t)nant);
    x.off.assign(fso, fso + nant);
    const double sb = (double)b;
    for (int a = 0; a < nant; a++) {
      x.idata[(size_t)a] = const_cast<u8 *>(inputs[a]) + (long long)b * bytes_per_fft;
      const double p0 = poly[3 * a], p1 = poly[3 * a + 1], p2 = poly[3 * a + 2];
      x.d[3 * (size_t)a] = p0;
      x.d[3 * (size_t)a + 1] = p1 + 2.0 * p0 * sb;
      x.d[3 * (size_t)a + 2] = p2 + p1 * sb + p0 * sb * sb;
      x.dptr[(size_t)a] = &x.d[3 * (size_t)a];
    }
    x.fx->setDelays(x.dptr.data(), x.off.data());
    x.fx->setInputData(x.idata.data());
  }
  std::atomic<int> go(0);
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; t++)
    th.emplace_back([&, t] {
      while (!go.load(std::memory_order_acquire)) std::this_thread::yield();
      sl[(size_t)t].fx->process();
    });
  const auto t0 = std::chrono::steady_clock::now();
  go.store(1, std::memory_order_release);
  for (auto &x : th) x.join();
  const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  for (auto &x : sl) delete x.fx;
  return dt;
}

}  // extern "C"
