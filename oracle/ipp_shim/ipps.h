/*
 * ipps.h — minimal Intel-IPP-compatible shim (TEST INFRASTRUCTURE ONLY).
 *
 * Intel IPP (version unpinned by the reference: fxkernel/configure.ac:19 asks
 * pkg-config for "ipp" with no version) is not available on either build host
 * (x86_64 container without IPP, aarch64 GPU host where IPP does not exist).
 * This header implements, from IPP's published semantics, exactly the
 * primitives the reference FX kernel calls through fxkernel/src/vectordefs.h:24-68
 * plus the FFT set-up calls in fxkernel/src/fxkernel.cpp:139-144, so that the
 * reference's own fxkernel.cpp compiles unmodified into oracle/_ref/.
 *
 * Semantics chosen (documented deviations from real IPP):
 *   - ippsFFTFwd_CToC_32fc: unnormalised forward DFT, X[k] = sum_n x[n] e^{-2 pi i kn/N},
 *     computed internally in double precision and rounded to float once
 *     (GXC_SHIM_FFT_F32 selects a float-internal radix-2 instead).
 *   - ippsSinCos_32f_A11: libm sinf/cosf (more accurate than IPP's 11-bit A11 flavour).
 *   - everything else is the obvious element-wise formula in single precision.
 *
 * Nothing here is used by the product library; only oracle/_ref links it.
 */
#ifndef GXC_IPP_SHIM_IPPS_H
#define GXC_IPP_SHIM_IPPS_H

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "ippcore.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- alloc */
static inline void *gxc_shim_alloc(size_t n) {
  void *p = NULL;
  if (n == 0) n = 64;
  if (posix_memalign(&p, 64, n) != 0) return NULL;
  return p;
}
static inline Ipp8u *ippsMalloc_8u(int len) { return (Ipp8u *)gxc_shim_alloc((size_t)len); }
static inline Ipp32f *ippsMalloc_32f(int len) { return (Ipp32f *)gxc_shim_alloc((size_t)len * sizeof(Ipp32f)); }
static inline Ipp64f *ippsMalloc_64f(int len) { return (Ipp64f *)gxc_shim_alloc((size_t)len * sizeof(Ipp64f)); }
static inline Ipp32fc *ippsMalloc_32fc(int len) { return (Ipp32fc *)gxc_shim_alloc((size_t)len * sizeof(Ipp32fc)); }
static inline Ipp64fc *ippsMalloc_64fc(int len) { return (Ipp64fc *)gxc_shim_alloc((size_t)len * sizeof(Ipp64fc)); }
static inline void ippsFree(void *p) { free(p); }

/* --------------------------------------------------------- element-wise */
static inline IppStatus ippsAdd_32fc_I(const Ipp32fc *src, Ipp32fc *srcdst, int len) {
  for (int i = 0; i < len; i++) { srcdst[i].re += src[i].re; srcdst[i].im += src[i].im; }
  return ippStsNoErr;
}
static inline IppStatus ippsAddC_64f_I(Ipp64f val, Ipp64f *srcdst, int len) {
  for (int i = 0; i < len; i++) srcdst[i] += val;
  return ippStsNoErr;
}
/* srcdst += src1 * src2 (complex product, no conjugation) */
static inline IppStatus ippsAddProduct_32fc(const Ipp32fc *src1, const Ipp32fc *src2, Ipp32fc *srcdst, int len) {
  for (int i = 0; i < len; i++) {
    Ipp32f re = src1[i].re * src2[i].re - src1[i].im * src2[i].im;
    Ipp32f im = src1[i].re * src2[i].im + src1[i].im * src2[i].re;
    srcdst[i].re += re;
    srcdst[i].im += im;
  }
  return ippStsNoErr;
}
static inline IppStatus ippsConj_32fc(const Ipp32fc *src, Ipp32fc *dst, int len) {
  for (int i = 0; i < len; i++) { dst[i].re = src[i].re; dst[i].im = -src[i].im; }
  return ippStsNoErr;
}
static inline IppStatus ippsDivC_32fc_I(Ipp32fc val, Ipp32fc *srcdst, int len) {
  if (val.im == 0.0f) {
    for (int i = 0; i < len; i++) { srcdst[i].re /= val.re; srcdst[i].im /= val.re; }
  } else {
    Ipp32f den = val.re * val.re + val.im * val.im;
    for (int i = 0; i < len; i++) {
      Ipp32f re = (srcdst[i].re * val.re + srcdst[i].im * val.im) / den;
      Ipp32f im = (srcdst[i].im * val.re - srcdst[i].re * val.im) / den;
      srcdst[i].re = re; srcdst[i].im = im;
    }
  }
  return ippStsNoErr;
}
static inline IppStatus ippsMagnitude_32fc(const Ipp32fc *src, Ipp32f *dst, int len) {
  for (int i = 0; i < len; i++) dst[i] = sqrtf(src[i].re * src[i].re + src[i].im * src[i].im);
  return ippStsNoErr;
}
static inline IppStatus ippsMul_32fc(const Ipp32fc *src1, const Ipp32fc *src2, Ipp32fc *dst, int len) {
  for (int i = 0; i < len; i++) {
    Ipp32f re = src1[i].re * src2[i].re - src1[i].im * src2[i].im;
    Ipp32f im = src1[i].re * src2[i].im + src1[i].im * src2[i].re;
    dst[i].re = re; dst[i].im = im;
  }
  return ippStsNoErr;
}
/* srcdst = srcdst * src */
static inline IppStatus ippsMul_32fc_I(const Ipp32fc *src, Ipp32fc *srcdst, int len) {
  for (int i = 0; i < len; i++) {
    Ipp32f re = srcdst[i].re * src[i].re - srcdst[i].im * src[i].im;
    Ipp32f im = srcdst[i].re * src[i].im + srcdst[i].im * src[i].re;
    srcdst[i].re = re; srcdst[i].im = im;
  }
  return ippStsNoErr;
}
static inline IppStatus ippsMulC_32f(const Ipp32f *src, Ipp32f val, Ipp32f *dst, int len) {
  for (int i = 0; i < len; i++) dst[i] = src[i] * val;
  return ippStsNoErr;
}
static inline IppStatus ippsMulC_32fc(const Ipp32fc *src, Ipp32fc val, Ipp32fc *dst, int len) {
  for (int i = 0; i < len; i++) {
    Ipp32f re = src[i].re * val.re - src[i].im * val.im;
    Ipp32f im = src[i].re * val.im + src[i].im * val.re;
    dst[i].re = re; dst[i].im = im;
  }
  return ippStsNoErr;
}
static inline IppStatus ippsMulC_32fc_I(Ipp32fc val, Ipp32fc *srcdst, int len) {
  return ippsMulC_32fc(srcdst, val, srcdst, len);
}
static inline IppStatus ippsMulC_64f(const Ipp64f *src, Ipp64f val, Ipp64f *dst, int len) {
  for (int i = 0; i < len; i++) dst[i] = src[i] * val;
  return ippStsNoErr;
}
static inline IppStatus ippsMulC_64f_I(Ipp64f val, Ipp64f *srcdst, int len) {
  for (int i = 0; i < len; i++) srcdst[i] *= val;
  return ippStsNoErr;
}
static inline IppStatus ippsPhase_32fc(const Ipp32fc *src, Ipp32f *dst, int len) {
  for (int i = 0; i < len; i++) dst[i] = atan2f(src[i].im, src[i].re);
  return ippStsNoErr;
}
static inline IppStatus ippsRealToCplx_32f(const Ipp32f *re, const Ipp32f *im, Ipp32fc *dst, int len) {
  for (int i = 0; i < len; i++) {
    dst[i].re = re ? re[i] : 0.0f;
    dst[i].im = im ? im[i] : 0.0f;
  }
  return ippStsNoErr;
}
static inline IppStatus ippsZero_32fc(Ipp32fc *dst, int len) {
  memset(dst, 0, (size_t)len * sizeof(Ipp32fc));
  return ippStsNoErr;
}

/* ---------------------------------------------------------------- copies */
static inline IppStatus ippsCopy_8u(const Ipp8u *src, Ipp8u *dst, int len) { memmove(dst, src, (size_t)len); return ippStsNoErr; }
static inline IppStatus ippsCopy_16s(const Ipp16s *src, Ipp16s *dst, int len) { memmove(dst, src, (size_t)len * 2); return ippStsNoErr; }
static inline IppStatus ippsCopy_32f(const Ipp32f *src, Ipp32f *dst, int len) { memmove(dst, src, (size_t)len * 4); return ippStsNoErr; }
static inline IppStatus ippsCopy_32fc(const Ipp32fc *src, Ipp32fc *dst, int len) { memmove(dst, src, (size_t)len * 8); return ippStsNoErr; }
static inline IppStatus ippsCopy_64f(const Ipp64f *src, Ipp64f *dst, int len) { memmove(dst, src, (size_t)len * 8); return ippStsNoErr; }

/* ------------------------------------------------------------------- FFT */
/* The spec lives inside the caller-provided spec buffer: header + twiddles. */
typedef struct IppsFFTSpec_C_32fc {
  int order;
  int n;
  int flag;
  double *tw_re; /* e^{-2 pi i k/n}, k < n/2 */
  double *tw_im;
  float *twf;    /* the same twiddles rounded to float, interleaved re, im */
  int *bitrev;   /* bit-reversed index of every i < n */
} IppsFFTSpec_C_32fc;

static inline IppStatus ippsFFTGetSize_C_32fc(int order, int flag, IppHintAlgorithm hint,
                                              int *pSpecSize, int *pSpecBufferSize, int *pBufferSize) {
  (void)flag; (void)hint;
  if (order < 0 || order > 27) return ippStsFftOrderErr;
  int n = 1 << order;
  *pSpecSize = (int)(sizeof(IppsFFTSpec_C_32fc) + 3 * 64 + (size_t)n * (sizeof(double) + sizeof(float) + sizeof(int)));
  *pSpecBufferSize = 0;
  /* work buffer: two complex-double arrays of n */
  *pBufferSize = (int)((size_t)n * 4 * sizeof(double) + 64);
  return ippStsNoErr;
}

static inline IppStatus ippsFFTInit_C_32fc(IppsFFTSpec_C_32fc **ppSpec, int order, int flag, IppHintAlgorithm hint,
                                           Ipp8u *pSpec, Ipp8u *pSpecBuffer) {
  (void)hint; (void)pSpecBuffer;
  if (order < 0 || order > 27) return ippStsFftOrderErr;
  IppsFFTSpec_C_32fc *s = (IppsFFTSpec_C_32fc *)pSpec;
  s->order = order;
  s->n = 1 << order;
  s->flag = flag;
  uintptr_t base = (uintptr_t)(pSpec + sizeof(IppsFFTSpec_C_32fc));
  base = (base + 63) & ~(uintptr_t)63;
  s->tw_re = (double *)base;
  s->tw_im = s->tw_re + (s->n / 2 > 0 ? s->n / 2 : 1);
  const int nh = s->n / 2 > 0 ? s->n / 2 : 1;
  s->twf = (float *)(((uintptr_t)(s->tw_im + nh) + 63) & ~(uintptr_t)63);
  s->bitrev = (int *)(((uintptr_t)(s->twf + 2 * nh) + 63) & ~(uintptr_t)63);
  for (int k = 0; k < s->n / 2; k++) {
    double ang = -2.0 * 3.14159265358979323846264338327950288 * (double)k / (double)s->n;
    s->tw_re[k] = cos(ang);
    s->tw_im[k] = sin(ang);
    s->twf[2 * k] = (float)s->tw_re[k];
    s->twf[2 * k + 1] = (float)s->tw_im[k];
  }
  for (int i = 0; i < s->n; i++) {
    unsigned r = 0, v = (unsigned)i;
    for (int b = 0; b < order; b++) { r = (r << 1) | (v & 1u); v >>= 1; }
    s->bitrev[i] = (int)r;
  }
  *ppSpec = s;
  return ippStsNoErr;
}

#ifdef GXC_SHIM_FFT_F32
/* Iterative radix-2 decimation-in-time FFT in single precision (float twiddles, float
 * butterflies): the CPU-baseline build, closer to IPP's own float arithmetic and speed than the
 * double-precision default below. */
static inline IppStatus ippsFFTFwd_CToC_32fc(const Ipp32fc *src, Ipp32fc *dst, const IppsFFTSpec_C_32fc *s,
                                             Ipp8u *buf) {
  const int n = s->n;
  float *x = (float *)(((uintptr_t)buf + 63) & ~(uintptr_t)63); /* interleaved re, im */
  for (int i = 0; i < n; i++) {
    const int r = s->bitrev[i];
    x[2 * r] = src[i].re;
    x[2 * r + 1] = src[i].im;
  }
  for (int len = 2; len <= n; len <<= 1) {
    const int half = len >> 1, step = n / len;
    for (int i = 0; i < n; i += len) {
      float *a = x + 2 * i, *b = x + 2 * (i + half);
      for (int j = 0; j < half; j++) {
        const float wr = s->twf[2 * j * step], wi = s->twf[2 * j * step + 1];
        const float xr = b[2 * j], xi = b[2 * j + 1];
        const float vr = xr * wr - xi * wi, vi = xr * wi + xi * wr;
        const float ur = a[2 * j], ui = a[2 * j + 1];
        a[2 * j] = ur + vr; a[2 * j + 1] = ui + vi;
        b[2 * j] = ur - vr; b[2 * j + 1] = ui - vi;
      }
    }
  }
  const float scale = s->flag == IPP_FFT_DIV_FWD_BY_N ? 1.0f / (float)n : 1.0f;
  for (int i = 0; i < n; i++) {
    dst[i].re = x[2 * i] * scale;
    dst[i].im = x[2 * i + 1] * scale;
  }
  return ippStsNoErr;
}
#else
/* Iterative radix-2 decimation-in-time FFT in double precision. */
static inline IppStatus ippsFFTFwd_CToC_32fc(const Ipp32fc *src, Ipp32fc *dst, const IppsFFTSpec_C_32fc *s,
                                             Ipp8u *buf) {
  int n = s->n;
  double *re = (double *)(((uintptr_t)buf + 63) & ~(uintptr_t)63);
  double *im = re + n;
  /* bit-reversed load */
  for (int i = 0; i < n; i++) {
    unsigned r = 0, v = (unsigned)i;
    for (int b = 0; b < s->order; b++) { r = (r << 1) | (v & 1u); v >>= 1; }
    re[r] = (double)src[i].re;
    im[r] = (double)src[i].im;
  }
  for (int len = 2; len <= n; len <<= 1) {
    int half = len >> 1;
    int step = n / len;
    for (int i = 0; i < n; i += len) {
      for (int j = 0; j < half; j++) {
        double wr = s->tw_re[j * step], wi = s->tw_im[j * step];
        double ur = re[i + j], ui = im[i + j];
        double xr = re[i + j + half], xi = im[i + j + half];
        double vr = xr * wr - xi * wi, vi = xr * wi + xi * wr;
        re[i + j] = ur + vr; im[i + j] = ui + vi;
        re[i + j + half] = ur - vr; im[i + j + half] = ui - vi;
      }
    }
  }
  double scale = 1.0;
  if (s->flag == IPP_FFT_DIV_FWD_BY_N) scale = 1.0 / (double)n;
  for (int i = 0; i < n; i++) {
    dst[i].re = (Ipp32f)(re[i] * scale);
    dst[i].im = (Ipp32f)(im[i] * scale);
  }
  return ippStsNoErr;
}
#endif

#ifdef __cplusplus
}
#endif

#endif
