/*
 * vectordefs.h (drop-in include directory) — the vector helpers the
 * reference's drivers call directly (fxkernel/src/vectordefs.h:12-17,24,31,54:
 * the u8 / cf32 types, vectorAlloc_u8, vectorFree, vectorCopy_u8).  Buffers come
 * from pinned host memory (gxc_host_alloc), the kind the engine copies to the
 * GPU fastest, and vectorFree releases both these and the buffers of
 * allocDataHost (gxc_common.h), which are pinned the same way.
 */
#ifndef GXC_DROPIN_VECTORDEFS_H
#define GXC_DROPIN_VECTORDEFS_H

#include <cstring>

#include "fxkernel_gxc.h"

static inline u8 *gxc_dropin_alloc_u8(int length) {
  void *p = nullptr;
  if (gxc_host_alloc(length > 0 ? (size_t)length : 1, &p) != GXC_OK) return nullptr;
  return (u8 *)p;
}

#define vectorAlloc_u8(length) gxc_dropin_alloc_u8(length)
#define vectorFree(memptr) gxc_host_free((void *)(memptr))
#define vectorCopy_u8(src, dest, length) std::memcpy((dest), (src), (size_t)(length))

#endif /* GXC_DROPIN_VECTORDEFS_H */
