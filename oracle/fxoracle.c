/*
 * fxoracle.c — CPU restatement of the reference FX correlator path.
 *
 * TEST INFRASTRUCTURE ONLY: this is the oracle that checks the GPU engine and
 * the timed CPU baseline; the product library never links or calls it.
 * Every step cites the reference source it restates (paths relative to the
 * gcorr project root).  Built with -ffp-contract=off so that x86 and aarch64
 * hosts round identically.
 */
#include "fxoracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define FXO_TWO_PI (2.0 * 3.14159265358979323846)

/* ------------------------------------------------------------ basic sizes */

/* fxkernel/src/fxkernel.cpp:31-43: fftchannels = 2*nchan (real) or nchan (complex). */
int fxo_fft_length(const fxo_config *c) { return c->is_complex ? c->nchan : 2 * c->nchan; }

/* fxkernel/src/fxkernel.cpp:31,38: sampletime = 1/(2 bw), doubled for complex data. */
double fxo_sample_time(const fxo_config *c) {
  double t = 1.0 / (2.0 * c->bw_hz);
  if (c->is_complex) t *= 2.0;
  return t;
}

/* Bytes of packed input per antenna: (nfft+1) FFT windows of F time samples,
 * 2 pols, nbit bits per real component (2 components when complex).
 * For 2-bit real this equals fxkernel/src/common.cpp:82; for 8-bit complex the
 * reference formula counts one component only (see the 8-bit note in fxo_unpack). */
size_t fxo_bytes_per_antenna(const fxo_config *c) {
  size_t F = (size_t)fxo_fft_length(c);
  size_t comps = c->is_complex ? 2 : 1;
  return (size_t)(c->nfft + 1) * F * 2u * comps * (size_t)c->nbit / 8u;
}

int fxo_num_baselines(const fxo_config *c) {
  return c->nant * (c->nant - 1) / 2 + (c->autos ? c->nant : 0);
}

static int is_pow2(int x) { return x > 0 && (x & (x - 1)) == 0; }

static int check_config(const fxo_config *c) {
  if (c->nant < 1 || c->nchan < 2 || c->nfft < 1) return 1;
  if (!((c->nbit == 2 && !c->is_complex) || (c->nbit == 8 && c->is_complex))) return 2;
  if (!is_pow2(fxo_fft_length(c))) return 3;
  if (!(c->bw_hz > 0.0)) return 4;
  if (c->rotator == FXO_ROT_FXKERNEL) {
    int s = (int)sqrt((double)c->nchan);
    if (s * s != c->nchan) return 5; /* fxkernel.cpp:58-63 */
  }
  return 0;
}

/* ---------------------------------------------------------- 2-bit levels */

/* fxkernel/src/fxkernel.cpp:15-28: level = lut4level[(b >> 2i) & 3], im = 0. */
void fxo_lut2bit(uint8_t byte, float out[4]) {
  static const float HiMag = 3.3359f;
  const float lv[4] = {-HiMag, -1.0f, 1.0f, HiMag};
  for (int i = 0; i < 4; i++) out[i] = lv[(byte >> (2 * i)) & 3];
}

/* ------------------------------------------------------------- geometry */

/* fxkernel/src/fxkernel.cpp:425-440 (getStationDelay) and :288-309 (offset,
 * integer rounding with int(x+0.5), +-1 edge fix-ups, validity flag). */
void fxo_geometry(const fxo_config *c, const double *p, double fso, int i, fxo_geom *g) {
  const int F = fxo_fft_length(c);
  const double Ts = fxo_sample_time(c);
  double fi = (double)i;
  double d0 = p[0] * fi * fi + p[1] * fi + p[2];
  double d1 = p[0] * (fi + 0.5) * (fi + 0.5) + p[1] * (fi + 0.5) + p[2];
  double d2 = p[0] * (fi + 1.0) * (fi + 1.0) + p[1] * (fi + 1.0) + p[2];
  double a = d2 - d0;
  double b = d0 + (d1 - (a * 0.5 + d0)) / 3.0;
  double mean = a * 0.5 + b;
  double ndf = (mean - fso) / Ts;
  g->a = a;
  g->b = b;
  g->valid = 0;
  g->offset = 0;
  g->frac = 0.0;
  /* Non-finite or absurd delays are flagged rather than fed to int(). */
  if (!(fabs(ndf) < 1.0e9)) return;
  int nd = (int)(ndf + 0.5);
  double frac = -(ndf - nd) * Ts;
  long long off = (long long)i * F - nd;
  long long maxoff = (long long)(c->nfft - 1) * F;
  if (off == -1) { off++; frac += Ts; }
  if (off == maxoff + 1) { off--; frac -= Ts; }
  g->frac = frac;
  if (off < 0 || off > maxoff) return;
  g->offset = (int)off;
  g->valid = 1;
}

/* ---------------------------------------------------------------- unpack */

/* 2-bit real: fxkernel/src/fxkernel.cpp:443-476.  Byte k holds time samples
 * 2k and 2k+1 of both pols as A_t, B_t, A_t+1, B_t+1 (2 bits each, LSB first);
 * the odd-offset head/tail handling there reduces to "sample offset+o".
 * 8-bit complex: fxkernel/src/fxkernel.cpp:478-487 reads (A.re, A.im, B.re, B.im)
 * int8 per time sample; the reference starts at byte offset*2 (a bug, it is
 * never dispatched: :489-496); this restatement starts at byte offset*4. */
void fxo_unpack(const fxo_config *c, const uint8_t *in, int offset, int nsamp, float *p0, float *p1) {
  if (c->nbit == 2) {
    float lv[4];
    for (int o = 0; o < nsamp; o++) {
      long long m = (long long)offset + o;
      fxo_lut2bit(in[m >> 1], lv);
      int h = (int)(m & 1) * 2;
      p0[2 * o] = lv[h];
      p0[2 * o + 1] = 0.0f;
      p1[2 * o] = lv[h + 1];
      p1[2 * o + 1] = 0.0f;
    }
  } else {
    const int8_t *s = (const int8_t *)in + (size_t)offset * 4u;
    for (int o = 0; o < nsamp; o++) {
      p0[2 * o] = (float)s[4 * o + 0];
      p0[2 * o + 1] = (float)s[4 * o + 1];
      p1[2 * o] = (float)s[4 * o + 2];
      p1[2 * o + 1] = (float)s[4 * o + 3];
    }
  }
}

/* ------------------------------------------------------------ FFT (port) */

/* Unnormalised forward DFT X[k] = sum x[n] e^{-2 pi i nk/N}, as
 * ippsFFTFwd_CToC_32fc with IPP_FFT_NODIV_BY_ANY (fxkernel.cpp:139-143,574).
 * Iterative radix-2 in single precision with double-rounded twiddles. */
typedef struct fft32 {
  int n, lg;
  int *rev;
  float *twr, *twi;
} fft32;

static int fft32_init(fft32 *f, int n) {
  f->n = n;
  f->lg = 0;
  while ((1 << f->lg) < n) f->lg++;
  f->rev = (int *)malloc(sizeof(int) * (size_t)n);
  f->twr = (float *)malloc(sizeof(float) * (size_t)(n / 2 + 1));
  f->twi = (float *)malloc(sizeof(float) * (size_t)(n / 2 + 1));
  if (!f->rev || !f->twr || !f->twi) return 1;
  for (int i = 0; i < n; i++) {
    unsigned r = 0, v = (unsigned)i;
    for (int b = 0; b < f->lg; b++) { r = (r << 1) | (v & 1u); v >>= 1; }
    f->rev[i] = (int)r;
  }
  for (int k = 0; k < n / 2; k++) {
    double ang = -FXO_TWO_PI * (double)k / (double)n;
    f->twr[k] = (float)cos(ang);
    f->twi[k] = (float)sin(ang);
  }
  return 0;
}

static void fft32_free(fft32 *f) {
  free(f->rev);
  free(f->twr);
  free(f->twi);
}

/* src and dst: interleaved complex, distinct buffers. */
static void fft32_fwd(const fft32 *f, const float *src, float *dst) {
  const int n = f->n;
  for (int i = 0; i < n; i++) {
    int r = f->rev[i];
    dst[2 * r] = src[2 * i];
    dst[2 * r + 1] = src[2 * i + 1];
  }
  for (int len = 2; len <= n; len <<= 1) {
    const int half = len >> 1, step = n / len;
    for (int i = 0; i < n; i += len) {
      float *u = dst + 2 * i, *v = dst + 2 * (i + half);
      for (int j = 0; j < half; j++) {
        float wr = f->twr[j * step], wi = f->twi[j * step];
        float xr = v[2 * j], xi = v[2 * j + 1];
        float tr = xr * wr - xi * wi, ti = xr * wi + xi * wr;
        float ur = u[2 * j], ui = u[2 * j + 1];
        u[2 * j] = ur + tr;
        u[2 * j + 1] = ui + ti;
        v[2 * j] = ur - tr;
        v[2 * j + 1] = ui - ti;
      }
    }
  }
}

/* ------------------------------------------------- port: per-thread state */

typedef struct port_ws {
  const fxo_config *c;
  int F, nchan, stride, substride, fstride, fsub;
  int fractional_lo;
  double Ts;
  fft32 fft;
  float *unp0, *unp1;           /* F complex */
  float *chan;                  /* [nant][2][F] complex */
  float *conj;                  /* [nant][2][nchan] complex */
  int *valid;                   /* [nant] */
  double *subxoff, *stepxoff;   /* fxkernel.cpp:105-114 */
  float *rot;                   /* F complex (complexrotator) */
  float *stepc;                 /* stride complex */
  float *subfreq, *stepfreq;    /* fxkernel.cpp:171-175 */
  float *fracrot, *fstepc;      /* nchan complex, fstride complex */
} port_ws;

static void port_ws_free(port_ws *w) {
  fft32_free(&w->fft);
  free(w->unp0); free(w->unp1); free(w->chan); free(w->conj); free(w->valid);
  free(w->subxoff); free(w->stepxoff); free(w->rot); free(w->stepc);
  free(w->subfreq); free(w->stepfreq); free(w->fracrot); free(w->fstepc);
}

static int ilog2i(int x) { int l = 0; while ((1 << (l + 1)) <= x) l++; return l; }

static int port_ws_init(port_ws *w, const fxo_config *c) {
  memset(w, 0, sizeof(*w));
  w->c = c;
  w->F = fxo_fft_length(c);
  w->nchan = c->nchan;
  w->Ts = fxo_sample_time(c);
  /* fxkernel.cpp:58-64: stride = sqrt(nchan) (square nchan), substride = (2/cfact)*stride.
   * For non-square power-of-two nchan (exact mode only) the same factorisation
   * is taken with stride = 2^floor(log2(nchan)/2). */
  int s = (int)sqrt((double)c->nchan);
  if (s * s != c->nchan) s = 1 << (ilog2i(c->nchan) / 2);
  w->stride = s;
  w->substride = w->F / s;
  w->fstride = s;
  w->fsub = c->nchan / s;
  /* fxkernel.cpp:67-71 */
  w->fractional_lo = (c->lo_hz - (double)(int)c->lo_hz) > 0.00000000001;
  if (fft32_init(&w->fft, w->F)) return 1;
  const int F = w->F, nc = w->nchan, na = c->nant;
  w->unp0 = (float *)malloc(sizeof(float) * 2 * (size_t)F);
  w->unp1 = (float *)malloc(sizeof(float) * 2 * (size_t)F);
  w->chan = (float *)malloc(sizeof(float) * 2 * (size_t)F * 2 * (size_t)na);
  w->conj = (float *)malloc(sizeof(float) * 2 * (size_t)nc * 2 * (size_t)na);
  w->valid = (int *)calloc((size_t)na, sizeof(int));
  w->subxoff = (double *)malloc(sizeof(double) * (size_t)w->substride);
  w->stepxoff = (double *)malloc(sizeof(double) * (size_t)w->stride);
  w->rot = (float *)malloc(sizeof(float) * 2 * (size_t)F);
  w->stepc = (float *)malloc(sizeof(float) * 2 * (size_t)w->stride);
  w->subfreq = (float *)malloc(sizeof(float) * (size_t)w->fsub);
  w->stepfreq = (float *)malloc(sizeof(float) * (size_t)w->fstride);
  w->fracrot = (float *)malloc(sizeof(float) * 2 * (size_t)nc);
  w->fstepc = (float *)malloc(sizeof(float) * 2 * (size_t)w->fstride);
  if (!w->unp0 || !w->unp1 || !w->chan || !w->conj || !w->valid || !w->subxoff || !w->stepxoff ||
      !w->rot || !w->stepc || !w->subfreq || !w->stepfreq || !w->fracrot || !w->fstepc)
    return 1;
  /* fxkernel.cpp:105-114.  FXKERNEL mode keeps the reference's step offset
   * i*stride/F (applied every substride samples); EXACT uses i*substride/F. */
  for (int i = 0; i < w->substride; i++) w->subxoff[i] = (double)i / (double)F;
  for (int i = 0; i < w->stride; i++) {
    int mult = (c->rotator == FXO_ROT_FXKERNEL) ? w->stride : w->substride;
    w->stepxoff[i] = (double)(i * mult) / (double)F;
  }
  /* fxkernel.cpp:171-175 */
  for (int i = 0; i < w->fsub; i++)
    w->subfreq[i] = (float)((FXO_TWO_PI * i * c->bw_hz) / (double)nc);
  for (int i = 0; i < w->fstride; i++)
    w->stepfreq[i] = (float)((FXO_TWO_PI * i * w->fsub * c->bw_hz) / (double)nc);
  return 0;
}

static inline void cmul(float ar, float ai, float br, float bi, float *cr, float *ci) {
  float r = ar * br - ai * bi;
  float i = ar * bi + ai * br;
  *cr = r;
  *ci = i;
}

/* fxkernel/src/fxkernel.cpp:498-567 (fringerotate), applied to both pols. */
static void port_fringerotate(port_ws *w, double a, double b) {
  const fxo_config *c = w->c;
  const int sub = w->substride, st = w->stride, F = w->F;
  int integerdelay = (int)b;
  b -= integerdelay;
  for (int k = 0; k < sub; k++) {
    double x = w->subxoff[k] * a + b;
    double ph = x * c->lo_hz;
    if (w->fractional_lo) ph += (c->lo_hz - (double)(int)c->lo_hz) * (double)integerdelay;
    float arg = (float)(-FXO_TWO_PI * (ph - (double)(int)ph));
    w->rot[2 * k] = cosf(arg);
    w->rot[2 * k + 1] = sinf(arg);
  }
  for (int i = 0; i < st; i++) {
    double ph = (w->stepxoff[i] * a) * c->lo_hz;
    float arg = (float)(-FXO_TWO_PI * (ph - (double)(int)ph));
    w->stepc[2 * i] = cosf(arg);
    w->stepc[2 * i + 1] = sinf(arg);
  }
  for (int i = 1; i < st; i++)
    for (int k = 0; k < sub; k++)
      cmul(w->rot[2 * k], w->rot[2 * k + 1], w->stepc[2 * i], w->stepc[2 * i + 1],
           &w->rot[2 * (i * sub + k)], &w->rot[2 * (i * sub + k) + 1]);
  for (int n = 0; n < F; n++) {
    cmul(w->unp0[2 * n], w->unp0[2 * n + 1], w->rot[2 * n], w->rot[2 * n + 1], &w->unp0[2 * n], &w->unp0[2 * n + 1]);
    cmul(w->unp1[2 * n], w->unp1[2 * n + 1], w->rot[2 * n], w->rot[2 * n + 1], &w->unp1[2 * n], &w->unp1[2 * n + 1]);
  }
}

/* fxkernel/src/fxkernel.cpp:595-634 (fracSampleCorrect) on one pol spectrum. */
static void port_fracrot_build(port_ws *w, double fracdelay) {
  const float fd = (float)fracdelay; /* ippsMulC_32f takes an Ipp32f constant */
  for (int k = 0; k < w->fsub; k++) {
    float arg = w->subfreq[k] * fd;
    w->fracrot[2 * k] = cosf(arg);
    w->fracrot[2 * k + 1] = sinf(arg);
  }
  for (int i = 0; i < w->fstride; i++) {
    float arg = w->stepfreq[i] * fd;
    w->fstepc[2 * i] = cosf(arg);
    w->fstepc[2 * i + 1] = sinf(arg);
  }
  for (int i = 1; i < w->fstride; i++)
    for (int k = 0; k < w->fsub; k++)
      cmul(w->fracrot[2 * k], w->fracrot[2 * k + 1], w->fstepc[2 * i], w->fstepc[2 * i + 1],
           &w->fracrot[2 * (i * w->fsub + k)], &w->fracrot[2 * (i * w->fsub + k) + 1]);
}

/* One antenna, one FFT: unpack, rotate, FFT, fractional delay (fxkernel.cpp:288-324).
 * Returns validity; the spectrum lands in w->chan[ant]. */
static int port_station(port_ws *w, const uint8_t *input, const double *poly3, double fso, int i, int ant) {
  fxo_geom g;
  fxo_geometry(w->c, poly3, fso, i, &g);
  if (!g.valid) return 0;
  const int F = w->F, nc = w->nchan;
  fxo_unpack(w->c, input, g.offset, F, w->unp0, w->unp1);
  port_fringerotate(w, g.a, g.b);
  float *c0 = w->chan + (size_t)(2 * ant) * 2 * F;
  float *c1 = c0 + 2 * (size_t)F;
  fft32_fwd(&w->fft, w->unp0, c0);
  fft32_fwd(&w->fft, w->unp1, c1);
  port_fracrot_build(w, g.frac);
  for (int ch = 0; ch < nc; ch++) {
    cmul(c0[2 * ch], c0[2 * ch + 1], w->fracrot[2 * ch], w->fracrot[2 * ch + 1], &c0[2 * ch], &c0[2 * ch + 1]);
    cmul(c1[2 * ch], c1[2 * ch + 1], w->fracrot[2 * ch], w->fracrot[2 * ch + 1], &c1[2 * ch], &c1[2 * ch + 1]);
  }
  return 1;
}

int fxo_port_channelise(const fxo_config *c, const uint8_t *input, const double *poly3, double fso, int fft,
                        float *out) {
  if (check_config(c)) return 1;
  fxo_config c1 = *c;
  c1.nant = 1;
  port_ws w;
  if (port_ws_init(&w, &c1)) { port_ws_free(&w); return 2; }
  int v = port_station(&w, input, poly3, fso, fft, 0);
  const int F = w.F, nc = w.nchan;
  for (int p = 0; p < 2; p++)
    for (int ch = 0; ch < nc; ch++) {
      out[2 * (p * nc + ch)] = v ? w.chan[2 * ((size_t)p * F + ch)] : 0.0f;
      out[2 * (p * nc + ch) + 1] = v ? w.chan[2 * ((size_t)p * F + ch) + 1] : 0.0f;
    }
  port_ws_free(&w);
  return 0;
}

/* FFT range [b, e) of process(): fxkernel.cpp:276-356 (station loop, conjugate,
 * baseline CMAC with ippsAddProduct_32fc, baseline counts).  Accumulates raw sums. */
static void port_range(port_ws *w, const uint8_t *const *inputs, const double *poly, const double *fso, int b, int e,
                       float *vis, int32_t *counts) {
  const fxo_config *c = w->c;
  const int na = c->nant, nc = w->nchan, F = w->F;
  const int ncross = na * (na - 1) / 2;
  for (int i = b; i < e; i++) {
    for (int j = 0; j < na; j++) {
      w->valid[j] = port_station(w, inputs[j], poly + 3 * j, fso[j], i, j);
      if (!w->valid[j]) continue;
      for (int p = 0; p < 2; p++) { /* conjChannels, fxkernel.cpp:582-593 */
        const float *src = w->chan + (size_t)(2 * j + p) * 2 * F;
        float *dst = w->conj + (size_t)(2 * j + p) * 2 * nc;
        for (int ch = 0; ch < nc; ch++) { dst[2 * ch] = src[2 * ch]; dst[2 * ch + 1] = -src[2 * ch + 1]; }
      }
    }
    int bl = 0;
    for (int j = 0; j < na - 1; j++) {
      if (!w->valid[j]) { bl += na - (j + 1); continue; }
      for (int k = j + 1; k < na; k++) {
        if (!w->valid[k]) { bl++; continue; }
        for (int l = 0; l < 2; l++)
          for (int m = 0; m < 2; m++) {
            const float *x = w->chan + (size_t)(2 * j + l) * 2 * F;
            const float *y = w->conj + (size_t)(2 * k + m) * 2 * nc;
            float *v = vis + ((size_t)bl * 4 + 2 * l + m) * 2 * nc;
            for (int ch = 0; ch < nc; ch++) {
              float re = x[2 * ch] * y[2 * ch] - x[2 * ch + 1] * y[2 * ch + 1];
              float im = x[2 * ch] * y[2 * ch + 1] + x[2 * ch + 1] * y[2 * ch];
              v[2 * ch] += re;
              v[2 * ch + 1] += im;
            }
          }
        counts[bl]++;
        bl++;
      }
    }
    if (c->autos) {
      for (int j = 0; j < na; j++) {
        if (!w->valid[j]) continue;
        int ab = ncross + j;
        for (int l = 0; l < 2; l++)
          for (int m = 0; m < 2; m++) {
            const float *x = w->chan + (size_t)(2 * j + l) * 2 * F;
            const float *y = w->conj + (size_t)(2 * j + m) * 2 * nc;
            float *v = vis + ((size_t)ab * 4 + 2 * l + m) * 2 * nc;
            for (int ch = 0; ch < nc; ch++) {
              float re = x[2 * ch] * y[2 * ch] - x[2 * ch + 1] * y[2 * ch + 1];
              float im = x[2 * ch] * y[2 * ch + 1] + x[2 * ch + 1] * y[2 * ch];
              v[2 * ch] += re;
              v[2 * ch + 1] += im;
            }
          }
        counts[ab]++;
      }
    }
  }
}

/* fxkernel.cpp:358-367: divide each baseline by its count (skipped when 0). */
static void port_normalise(const fxo_config *c, float *vis, const int32_t *counts) {
  const int nbl = fxo_num_baselines(c), nc = c->nchan;
  for (int bl = 0; bl < nbl; bl++) {
    if (counts[bl] == 0) continue;
    float n = (float)counts[bl];
    float *v = vis + (size_t)bl * 4 * 2 * nc;
    for (int x = 0; x < 4 * 2 * nc; x++) v[x] /= n;
  }
}

int fxo_port_process_range(const fxo_config *c, const uint8_t *const *inputs, const double *poly, const double *fso,
                           int fft_begin, int fft_end, int normalise, float *vis, int32_t *counts) {
  if (check_config(c)) return 1;
  if (fft_begin < 0 || fft_end > c->nfft || fft_begin > fft_end) return 1;
  const int nbl = fxo_num_baselines(c);
  memset(vis, 0, sizeof(float) * 2 * (size_t)nbl * 4 * (size_t)c->nchan);
  memset(counts, 0, sizeof(int32_t) * (size_t)nbl);
  port_ws w;
  if (port_ws_init(&w, c)) { port_ws_free(&w); return 2; }
  port_range(&w, inputs, poly, fso, fft_begin, fft_end, vis, counts);
  port_ws_free(&w);
  if (normalise) port_normalise(c, vis, counts);
  return 0;
}

typedef struct port_job {
  const fxo_config *c;
  const uint8_t *const *inputs;
  const double *poly, *fso;
  int b, e;
  float *vis;
  int32_t *counts;
  int rc;
} port_job;

static void *port_thread(void *arg) {
  port_job *j = (port_job *)arg;
  j->rc = fxo_port_process_range(j->c, j->inputs, j->poly, j->fso, j->b, j->e, 0, j->vis, j->counts);
  return NULL;
}

/* One worker per thread on a contiguous FFT slice, merged afterwards: the
 * thread replication of fxkernel/src/bench_fxkernel.cpp:93-139 applied to one
 * sub-integration, followed by the normalisation of fxkernel.cpp:358-367. */
int fxo_port_process(const fxo_config *c, const uint8_t *const *inputs, const double *poly, const double *fso,
                     int nthreads, float *vis, int32_t *counts) {
  if (check_config(c)) return 1;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > c->nfft) nthreads = c->nfft;
  const int nbl = fxo_num_baselines(c);
  const size_t nv = 2 * (size_t)nbl * 4 * (size_t)c->nchan;
  if (nthreads == 1) return fxo_port_process_range(c, inputs, poly, fso, 0, c->nfft, 1, vis, counts);
  port_job *jobs = (port_job *)calloc((size_t)nthreads, sizeof(port_job));
  pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
  float *bufs = (float *)malloc(sizeof(float) * nv * (size_t)nthreads);
  int32_t *cbufs = (int32_t *)malloc(sizeof(int32_t) * (size_t)nbl * (size_t)nthreads);
  if (!jobs || !th || !bufs || !cbufs) { free(jobs); free(th); free(bufs); free(cbufs); return 2; }
  for (int t = 0; t < nthreads; t++) {
    jobs[t].c = c; jobs[t].inputs = inputs; jobs[t].poly = poly; jobs[t].fso = fso;
    jobs[t].b = (int)((long long)c->nfft * t / nthreads);
    jobs[t].e = (int)((long long)c->nfft * (t + 1) / nthreads);
    jobs[t].vis = bufs + nv * (size_t)t;
    jobs[t].counts = cbufs + (size_t)nbl * (size_t)t;
    pthread_create(&th[t], NULL, port_thread, &jobs[t]);
  }
  int rc = 0;
  for (int t = 0; t < nthreads; t++) { pthread_join(th[t], NULL); rc |= jobs[t].rc; }
  memset(vis, 0, sizeof(float) * nv);
  memset(counts, 0, sizeof(int32_t) * (size_t)nbl);
  for (int t = 0; t < nthreads; t++) { /* accumulate(), fxkernel.cpp:414-423 */
    for (size_t x = 0; x < nv; x++) vis[x] += jobs[t].vis[x];
    for (int bl = 0; bl < nbl; bl++) counts[bl] += jobs[t].counts[bl];
  }
  port_normalise(c, vis, counts);
  free(jobs); free(th); free(bufs); free(cbufs);
  return rc;
}

/* --------------------------------------------------------- FP64 oracle */

static void fft64(double *re, double *im, int n) {
  int lg = 0;
  while ((1 << lg) < n) lg++;
  for (int i = 0; i < n; i++) {
    unsigned r = 0, v = (unsigned)i;
    for (int b = 0; b < lg; b++) { r = (r << 1) | (v & 1u); v >>= 1; }
    if ((int)r > i) {
      double t = re[i]; re[i] = re[r]; re[r] = t;
      t = im[i]; im[i] = im[r]; im[r] = t;
    }
  }
  for (int len = 2; len <= n; len <<= 1) {
    int half = len >> 1;
    for (int j = 0; j < half; j++) {
      double ang = -FXO_TWO_PI * (double)j / (double)len;
      double wr = cos(ang), wi = sin(ang);
      for (int i = 0; i < n; i += len) {
        double xr = re[i + j + half], xi = im[i + j + half];
        double tr = xr * wr - xi * wi, ti = xr * wi + xi * wr;
        double ur = re[i + j], ui = im[i + j];
        re[i + j] = ur + tr; im[i + j] = ui + ti;
        re[i + j + half] = ur - tr; im[i + j + half] = ui - ti;
      }
    }
  }
}

/* Fringe phase in turns of sample n of an FFT window with delay a*n/F + b
 * (fxkernel.cpp:498-535): the exact linear model, or, for FXO_ROT_FXKERNEL,
 * the reference's sub/step split with the half-rate step offset. */
static double exact_phase_turns(const fxo_config *c, int F, int stride, int substride, double a, double b, int n) {
  int integerdelay = (int)b;
  double br = b - integerdelay;
  double lofrac = c->lo_hz - (double)(int)c->lo_hz;
  double extra = (lofrac > 0.00000000001) ? lofrac * (double)integerdelay : 0.0;
  if (c->rotator == FXO_ROT_FXKERNEL) {
    int i = n / substride, k = n % substride;
    double ps = ((double)k / (double)F * a + br) * c->lo_hz + extra;
    double pt = ((double)(i * stride) / (double)F * a) * c->lo_hz;
    return (ps - floor(ps)) + (pt - floor(pt));
  }
  double ph = ((double)n / (double)F * a + br) * c->lo_hz + extra;
  return ph - floor(ph);
}

static int exact_station(const fxo_config *c, const uint8_t *input, const double *poly3, double fso, int i,
                         double *re0, double *im0, double *re1, double *im1, float *tmp0, float *tmp1) {
  const int F = fxo_fft_length(c), nc = c->nchan;
  fxo_geom g;
  fxo_geometry(c, poly3, fso, i, &g);
  if (!g.valid) return 0;
  fxo_unpack(c, input, g.offset, F, tmp0, tmp1);
  int s = (int)sqrt((double)nc);
  if (s * s != nc) s = 1 << (ilog2i(nc) / 2);
  int substride = F / s;
  for (int n = 0; n < F; n++) {
    double ph = exact_phase_turns(c, F, s, substride, g.a, g.b, n);
    double cr = cos(-FXO_TWO_PI * ph), ci = sin(-FXO_TWO_PI * ph);
    double xr = tmp0[2 * n], xi = tmp0[2 * n + 1];
    re0[n] = xr * cr - xi * ci; im0[n] = xr * ci + xi * cr;
    xr = tmp1[2 * n]; xi = tmp1[2 * n + 1];
    re1[n] = xr * cr - xi * ci; im1[n] = xr * ci + xi * cr;
  }
  fft64(re0, im0, F);
  fft64(re1, im1, F);
  /* fractional-sample correction X[c] *= exp(i 2 pi c bw/nchan frac) (fxkernel.cpp:171-175,595-634) */
  for (int ch = 0; ch < nc; ch++) {
    double ang = FXO_TWO_PI * (double)ch * c->bw_hz / (double)nc * g.frac;
    double cr = cos(ang), ci = sin(ang);
    double xr = re0[ch], xi = im0[ch];
    re0[ch] = xr * cr - xi * ci; im0[ch] = xr * ci + xi * cr;
    xr = re1[ch]; xi = im1[ch];
    re1[ch] = xr * cr - xi * ci; im1[ch] = xr * ci + xi * cr;
  }
  return 1;
}

int fxo_exact_channelise(const fxo_config *c, const uint8_t *input, const double *poly3, double fso, int fft,
                         double *out) {
  if (check_config(c)) return 1;
  const int F = fxo_fft_length(c), nc = c->nchan;
  double *buf = (double *)malloc(sizeof(double) * 4 * (size_t)F);
  float *tmp = (float *)malloc(sizeof(float) * 4 * (size_t)F);
  if (!buf || !tmp) { free(buf); free(tmp); return 2; }
  int v = exact_station(c, input, poly3, fso, fft, buf, buf + F, buf + 2 * F, buf + 3 * F, tmp, tmp + 2 * F);
  for (int p = 0; p < 2; p++)
    for (int ch = 0; ch < nc; ch++) {
      out[2 * (p * nc + ch)] = v ? buf[(2 * p) * F + ch] : 0.0;
      out[2 * (p * nc + ch) + 1] = v ? buf[(2 * p + 1) * F + ch] : 0.0;
    }
  free(buf); free(tmp);
  return 0;
}

int fxo_exact_process(const fxo_config *c, const uint8_t *const *inputs, const double *poly, const double *fso,
                      double *vis, int32_t *counts) {
  return fxo_exact_process_masked(c, inputs, poly, fso, NULL, vis, counts);
}

int fxo_exact_process_masked(const fxo_config *c, const uint8_t *const *inputs, const double *poly,
                             const double *fso, const uint8_t *mask, double *vis, int32_t *counts) {
  if (check_config(c)) return 1;
  const int na = c->nant, nc = c->nchan, F = fxo_fft_length(c);
  const int ncross = na * (na - 1) / 2, nbl = fxo_num_baselines(c);
  memset(vis, 0, sizeof(double) * 2 * (size_t)nbl * 4 * (size_t)nc);
  memset(counts, 0, sizeof(int32_t) * (size_t)nbl);
  double *X = (double *)malloc(sizeof(double) * 4 * (size_t)F * (size_t)na); /* [ant][re0,im0,re1,im1][F] */
  float *tmp = (float *)malloc(sizeof(float) * 4 * (size_t)F);
  int *valid = (int *)calloc((size_t)na, sizeof(int));
  if (!X || !tmp || !valid) { free(X); free(tmp); free(valid); return 2; }
  for (int i = 0; i < c->nfft; i++) {
    for (int j = 0; j < na; j++) {
      double *x = X + (size_t)j * 4 * F;
      valid[j] = exact_station(c, inputs[j], poly + 3 * j, fso[j], i, x, x + F, x + 2 * F, x + 3 * F, tmp, tmp + 2 * F);
      if (mask && !mask[(size_t)j * c->nfft + i]) valid[j] = 0;
    }
    for (int j = 0; j < na; j++) {
      if (!valid[j]) continue;
      for (int k = c->autos ? j : j + 1; k < na; k++) {
        if (!valid[k]) continue;
        int bl = (k == j) ? ncross + j : j * na - j * (j + 1) / 2 + (k - j - 1);
        for (int l = 0; l < 2; l++)
          for (int m = 0; m < 2; m++) {
            const double *xr = X + (size_t)j * 4 * F + (size_t)(2 * l) * F, *xi = xr + F;
            const double *yr = X + (size_t)k * 4 * F + (size_t)(2 * m) * F, *yi = yr + F;
            double *v = vis + ((size_t)bl * 4 + 2 * l + m) * 2 * nc;
            for (int ch = 0; ch < nc; ch++) { /* x * conj(y) */
              v[2 * ch] += xr[ch] * yr[ch] + xi[ch] * yi[ch];
              v[2 * ch + 1] += xi[ch] * yr[ch] - xr[ch] * yi[ch];
            }
          }
        counts[bl]++;
      }
    }
  }
  for (int bl = 0; bl < nbl; bl++) {
    if (counts[bl] == 0) continue;
    double *v = vis + (size_t)bl * 4 * 2 * nc;
    for (int x = 0; x < 4 * 2 * nc; x++) v[x] /= (double)counts[bl];
  }
  free(X); free(tmp); free(valid);
  return 0;
}
