/*
 * fxkernel_gxc.h — header-only C++ FxKernel with the reference's public
 * signatures (fxkernel/src/fxkernel.h:18-64), running on the GB300 engine
 * through the C ABI in gxc.h.  A driver written against the reference class
 * (fxkernel/src/testfxkernel.cpp:81-108, fxkernel/src/bench_fxkernel.cpp:110-128)
 * compiles against this header and links libgxcorr.so instead of fxkernel.cpp + IPP.
 *
 * Behaviour matches the reference by default: cross baselines only
 * (nant*(nant-1)/2, fxkernel.cpp:147), the reference's fringe-rotator table
 * when nchan is a perfect square (fxkernel.cpp:57-64,104-114; exact rotator
 * otherwise), FP32, and exit(1) with a message on a configuration the engine
 * rejects (fxkernel.cpp:46-63).  The extended constructor exposes the engine's
 * own options (precision, exact rotator, autocorrelations).
 *
 * Types: u8 and cf32 follow fxkernel/src/vectordefs.h:12-17 (IPP's Ipp8u and
 * Ipp32fc, a struct of float re, im); they are defined here unless the IPP
 * types are already visible (GXC_HAVE_IPP_TYPES).
 */
#ifndef FXKERNEL_GXC_H
#define FXKERNEL_GXC_H

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <vector>

#include "gxc.h"

#ifndef GXC_HAVE_IPP_TYPES
typedef uint8_t u8;
typedef struct { float re; float im; } cf32;
#endif

class FxKernel {
 public:
  struct Options {
    int precision = GXC_PRECISION_FP32;
    int rotator = -1;  /* -1: the reference's table when nchan is square, else exact */
    int autos = 0;
    int x_engine = GXC_XENGINE_AUTO;
    int device = -1;
    int fft_engine = GXC_FFT_AUTO;
    int x_split = GXC_XSPLIT_AUTO;
    int fp8_scaling = GXC_FP8_SCALE_CHANNEL;
  };

  /* fxkernel/src/fxkernel.h:29 */
  FxKernel(int nant, int nchan, int nfft, int nbit, double localosc, double bw, bool is_complex)
      : FxKernel(nant, nchan, nfft, nbit, localosc, bw, is_complex, Options()) {}

  FxKernel(int nant, int nchan, int nfft, int nbit, double localosc, double bw, bool is_complex,
           const Options &opt)
      : numantennas(nant), numchannels(nchan), bandwidth(bw) {
    gxc_config c;
    gxc_config_init(&c);
    c.nant = nant;
    c.nchan = nchan;
    c.nfft = nfft;
    c.nbit = nbit;
    c.is_complex = is_complex ? 1 : 0;
    c.lo_hz = localosc;
    c.bw_hz = bw;
    c.precision = opt.precision;
    int s = (int)std::sqrt((double)nchan);
    c.rotator = opt.rotator >= 0 ? opt.rotator : (s * s == nchan ? GXC_ROTATOR_FXKERNEL : GXC_ROTATOR_EXACT);
    c.autos = opt.autos;
    c.x_engine = opt.x_engine;
    c.device = opt.device;
    c.fft_engine = opt.fft_engine;
    c.x_split = opt.x_split;
    c.fp8_scaling = opt.fp8_scaling;
    cfg_ = c;
    gxc_status st = gxc_create(&c, &h);
    if (st != GXC_OK) {
      std::fprintf(stderr, "FxKernel: %s (configuration rejected or no GPU). Aborting\n", gxc_status_string(st));
      std::exit(1);
    }
    nbaselines = gxc_num_baselines(&c);
    vis.resize((size_t)nbaselines * 4 * nchan);
  }

  ~FxKernel() { gxc_destroy(h); }
  FxKernel(const FxKernel &) = delete;
  FxKernel &operator=(const FxKernel &) = delete;

  /* fxkernel/src/fxkernel.h:40 — one buffer per antenna, the whole sub-integration */
  void setInputData(u8 **idata) {
    check(gxc_set_input(h, (const uint8_t *const *)idata, gxc_input_bytes_per_antenna(&cfg_)), "setInputData");
  }

  /* fxkernel/src/fxkernel.h:47 — d[ant][3] polynomial, f[ant] file start offsets */
  void setDelays(double **d, double *f) {
    std::vector<double> poly((size_t)numantennas * 3);
    for (int a = 0; a < numantennas; a++)
      for (int k = 0; k < 3; k++) poly[(size_t)a * 3 + k] = d[a][k];
    check(gxc_set_delays(h, poly.data(), f), "setDelays");
  }

  /* fxkernel/src/fxkernel.h:52 — synchronous, like the reference */
  void process() {
    check(gxc_process(h, nullptr), "process");
    check(gxc_get_visibilities(h, reinterpret_cast<float *>(vis.data())), "process");
  }

  /* fxkernel/src/fxkernel.h:58 — odata[baseline][product][channel] += visibilities */
  void accumulate(cf32 ***odata) {
    for (int b = 0; b < nbaselines; b++)
      for (int p = 0; p < 4; p++) {
        const cf32 *v = &vis[((size_t)b * 4 + p) * numchannels];
        for (int c = 0; c < numchannels; c++) {
          odata[b][p][c].re += v[c].re;
          odata[b][p][c].im += v[c].im;
        }
      }
  }

  /* fxkernel/src/fxkernel.h:64 — text dump in the format of fxkernel.cpp:370-412 */
  void saveVisibilities(const char *outfile) {
    check(gxc_save_visibilities(outfile, reinterpret_cast<const float *>(vis.data()), nbaselines, numchannels,
                                bandwidth),
          "saveVisibilities");
  }

  int baselines() const { return nbaselines; }
  gxc_handle *handle() { return h; }
  const cf32 *visibilities() const { return vis.data(); }

 private:
  void check(gxc_status st, const char *what) {
    if (st != GXC_OK) {
      std::fprintf(stderr, "FxKernel::%s: %s: %s\n", what, gxc_status_string(st), gxc_last_error(h));
      std::exit(1);
    }
  }

  gxc_handle *h = nullptr;
  gxc_config cfg_;
  int numantennas, numchannels, nbaselines = 0;
  double bandwidth;
  std::vector<cf32> vis;
};

#endif /* FXKERNEL_GXC_H */
