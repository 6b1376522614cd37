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
#include <cmath>
#include <cstdint>
#include <cstring>
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

}  // extern "C"
