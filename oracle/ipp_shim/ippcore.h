/*
 * ippcore.h — types and constants of the IPP-compatible shim (TEST INFRASTRUCTURE ONLY).
 * See ipps.h in this directory for what the shim is for and the semantics it follows.
 */
#ifndef GXC_IPP_SHIM_IPPCORE_H
#define GXC_IPP_SHIM_IPPCORE_H

#include <stdint.h>
#include <stdlib.h>

typedef uint8_t Ipp8u;
typedef int8_t Ipp8s;
typedef int16_t Ipp16s;
typedef float Ipp32f;
typedef double Ipp64f;
typedef struct { Ipp32f re; Ipp32f im; } Ipp32fc;
typedef struct { Ipp64f re; Ipp64f im; } Ipp64fc;

typedef int IppStatus;
#define ippStsNoErr 0
#define ippStsFftOrderErr (-15)

typedef enum { ippAlgHintNone = 0, ippAlgHintFast = 1, ippAlgHintAccurate = 2 } IppHintAlgorithm;

#define IPP_FFT_DIV_FWD_BY_N 1
#define IPP_FFT_DIV_INV_BY_N 2
#define IPP_FFT_DIV_BY_SQRTN 4
#define IPP_FFT_NODIV_BY_ANY 8

#define IPP_PI 3.14159265358979323846

static inline void ippFree(void *p) { free(p); }

#endif
