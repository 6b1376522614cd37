/*
 * fxoracle.h — CPU restatement of the reference FX correlator path (TEST INFRASTRUCTURE ONLY).
 *
 * This is the checker for the GPU engine, not part of it: only tests/, the smoke
 * entry point and bench.py's CPU-baseline / reference arm may load it.
 *
 * Two restatements of FxKernel::process() (fxkernel/src/fxkernel.cpp:253-368):
 *   fxo_port_process   FP32, step for step the reference algorithm (LUT unpack,
 *                      sub/step-table fringe rotator, FP32 FFT, sub/step fractional
 *                      delay, conjugate-multiply-accumulate, normalise).  With
 *                      rotator = FXO_ROT_FXKERNEL it reproduces the reference's
 *                      half-rate real-data step table (fxkernel.cpp:112 vs :553-558).
 *                      Multi-threaded over FFT ranges like bench_fxkernel.cpp:93-139.
 *   fxo_exact_process  FP64 oracle: same geometry/rounding/flagging, exact linear
 *                      fringe rotator, FP64 FFT and accumulation, autos, any
 *                      power-of-two FFT length, 8-bit complex input.
 *
 * Output layout (both): complex [nbl][4][nchan] in fxkernel baseline order
 * (0,1),(0,2)..(nant-2,nant-1), products AA,AB,BA,BB; when autos are on, nant
 * auto "baselines" (0,0),(1,1).. follow in the same [4][nchan] form.
 */
#ifndef GXC_FXORACLE_H
#define GXC_FXORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { FXO_ROT_EXACT = 0, FXO_ROT_FXKERNEL = 1 };

typedef struct fxo_config {
  int nant;
  int nchan;
  int nfft;
  int nbit;       /* 2 (real) or 8 (complex) */
  int is_complex; /* 0 or 1 */
  double lo_hz;
  double bw_hz;
  int rotator;    /* FXO_ROT_* */
  int autos;      /* 0 or 1 */
} fxo_config;

/* Per-(antenna, FFT) geometry: fxkernel.cpp:288-309 with getStationDelay :425-440. */
typedef struct fxo_geom {
  int offset;       /* first sample of the FFT window in the antenna stream */
  int valid;        /* 0 when the window leaves the buffer (flagged) */
  double frac;      /* residual (fractional) delay in seconds */
  double a, b;      /* delay gradient across the FFT (s) and delay at its start (s) */
} fxo_geom;

int fxo_fft_length(const fxo_config *c);
double fxo_sample_time(const fxo_config *c);
size_t fxo_bytes_per_antenna(const fxo_config *c);
int fxo_num_baselines(const fxo_config *c); /* crosses (+ autos when enabled) */

void fxo_lut2bit(uint8_t byte, float out[4]);
void fxo_geometry(const fxo_config *c, const double *poly3, double fso, int fft, fxo_geom *g);
/* Unpack nsamp samples from sample `offset` into two complex (interleaved re,im) float arrays. */
void fxo_unpack(const fxo_config *c, const uint8_t *in, int offset, int nsamp, float *pol0, float *pol1);

/* Returns 0 on success, nonzero on bad arguments.  vis: complex64 interleaved,
 * counts: int32 per output baseline.  fft_begin/fft_end restrict the FFT range
 * (use 0, nfft for the whole sub-integration); normalise=0 leaves raw sums. */
int fxo_port_process(const fxo_config *c, const uint8_t *const *inputs, const double *poly /*[nant][3]*/,
                     const double *fso, int nthreads, float *vis, int32_t *counts);
int fxo_port_process_range(const fxo_config *c, const uint8_t *const *inputs, const double *poly,
                           const double *fso, int fft_begin, int fft_end, int normalise,
                           float *vis, int32_t *counts);
int fxo_exact_process(const fxo_config *c, const uint8_t *const *inputs, const double *poly,
                      const double *fso, double *vis /* complex128 */, int32_t *counts);
/* fxo_exact_process with extra per-(antenna, FFT) flags: mask [nant][nfft], 0 flags the
 * FFT of that antenna on top of the geometry (NULL = no extra flags). */
int fxo_exact_process_masked(const fxo_config *c, const uint8_t *const *inputs, const double *poly,
                             const double *fso, const uint8_t *mask, double *vis, int32_t *counts);

/* Channelised spectrum of one (antenna, FFT) after fringe rotation, FFT and
 * fractional-delay correction (before conjugation): 2 pols x nchan complex. */
int fxo_port_channelise(const fxo_config *c, const uint8_t *input, const double *poly3, double fso,
                        int fft, float *out /* [2][nchan] complex64 */);
int fxo_exact_channelise(const fxo_config *c, const uint8_t *input, const double *poly3, double fso,
                         int fft, double *out /* [2][nchan] complex128 */);

#ifdef __cplusplus
}
#endif

#endif
