/*
 * ippvm.h — vector-math part of the IPP-compatible shim (TEST INFRASTRUCTURE ONLY).
 * ippsSinCos_32f_A11 is served by libm sinf/cosf (more accurate than IPP's A11 flavour).
 */
#ifndef GXC_IPP_SHIM_IPPVM_H
#define GXC_IPP_SHIM_IPPVM_H

#include <math.h>
#include "ippcore.h"

#ifdef __cplusplus
extern "C" {
#endif

static inline IppStatus ippsSinCos_32f_A11(const Ipp32f *src, Ipp32f *dstSin, Ipp32f *dstCos, int len) {
  for (int i = 0; i < len; i++) {
    dstSin[i] = sinf(src[i]);
    dstCos[i] = cosf(src[i]);
  }
  return ippStsNoErr;
}

#ifdef __cplusplus
}
#endif

#endif
