/*
 * fxkernel.h (drop-in include directory) — what a driver that includes the
 * reference's fxkernel/src/fxkernel.h gets on the GB300 engine: the FxKernel
 * class with the reference's signatures (fxkernel_gxc.h, over the C ABI in
 * gxc.h), plus the handful of IPP calls the reference's benchmark driver makes
 * itself (fxkernel/src/bench_fxkernel.cpp:50-80: ippsRandGauss*_8u,
 * ippsMalloc_8u, ippsFree), which the reference's fxkernel.h brings in through
 * <ipps.h> (fxkernel/src/fxkernel.h:5).
 *
 * The reference's own drivers (fxkernel/src/testfxkernel.cpp,
 * fxkernel/src/bench_fxkernel.cpp) compile unchanged against this directory:
 *   g++ -std=c++17 -I include/fxkernel_dropin -I include driver.cpp \
 *       -L gcorr_gb300 -lgxcorr -pthread
 */
#ifndef GXC_DROPIN_FXKERNEL_H
#define GXC_DROPIN_FXKERNEL_H

#include <cmath>
#include <cstdint>
#include <cstdlib>

#include "fxkernel_gxc.h"
#include "vectordefs.h"

typedef uint8_t Ipp8u;
typedef int IppStatus;
#ifndef ippStsNoErr
#define ippStsNoErr 0
#endif

/* Gaussian byte generator with IPP's interface (mean and standard deviation in
 * byte units, results rounded and saturated to 0..255).  The numbers come from
 * splitmix64 and the Box-Muller transform, not from IPP's generator: the
 * benchmark driver only needs random input, not IPP's exact sequence. */
typedef struct IppsRandGaussState_8u {
  uint64_t s;
  double mean, sd;
  int have;
  double spare;
} IppsRandGaussState_8u;

static inline uint64_t gxc_dropin_splitmix64(uint64_t *s) {
  uint64_t z = (*s += 0x9e3779b97f4a7c15ULL);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

static inline IppStatus ippsRandGaussGetSize_8u(int *size) {
  *size = (int)sizeof(IppsRandGaussState_8u);
  return ippStsNoErr;
}

static inline Ipp8u *ippsMalloc_8u(int len) { return (Ipp8u *)std::malloc(len > 0 ? (size_t)len : 1); }
static inline void ippsFree(void *p) { std::free(p); }

static inline IppStatus ippsRandGaussInit_8u(IppsRandGaussState_8u *st, Ipp8u mean, Ipp8u sd, unsigned int seed) {
  st->s = seed;
  st->mean = mean;
  st->sd = sd;
  st->have = 0;
  st->spare = 0.0;
  return ippStsNoErr;
}

static inline IppStatus ippsRandGauss_8u(Ipp8u *dst, int len, IppsRandGaussState_8u *st) {
  const double two_pi = 6.283185307179586476925286766559;
  for (int i = 0; i < len; i++) {
    double g;
    if (st->have) {
      g = st->spare;
      st->have = 0;
    } else {
      /* two uniforms in (0, 1] from the top 53 bits */
      const double u1 = ((double)(gxc_dropin_splitmix64(&st->s) >> 11) + 1.0) * (1.0 / 9007199254740992.0);
      const double u2 = (double)(gxc_dropin_splitmix64(&st->s) >> 11) * (1.0 / 9007199254740992.0);
      const double r = std::sqrt(-2.0 * std::log(u1));
      g = r * std::cos(two_pi * u2);
      st->spare = r * std::sin(two_pi * u2);
      st->have = 1;
    }
    double v = std::nearbyint(st->mean + st->sd * g);
    dst[i] = (Ipp8u)(v < 0.0 ? 0.0 : v > 255.0 ? 255.0 : v);
  }
  return ippStsNoErr;
}

#endif /* GXC_DROPIN_FXKERNEL_H */
