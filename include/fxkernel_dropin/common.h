/*
 * common.h (drop-in include directory) — the reference's harness helpers
 * (fxkernel/src/common.h:41-60: parseConfig, allocDataHost, readdata, and the
 * std names it brings into scope) on the GB300 engine's C ABI (gxc_common.h).
 * Like the reference's common.h in its CPU build, it also includes fxkernel.h.
 */
#ifndef GXC_DROPIN_COMMON_H
#define GXC_DROPIN_COMMON_H

#include <sstream>

#include "gxc_common.h"
#include "fxkernel.h"

#endif /* GXC_DROPIN_COMMON_H */
