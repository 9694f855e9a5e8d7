/* Stand-in for tg/src/platform/tg_platform.h (Win32 only): heap calls map to libc.
 * Test infrastructure for the parity oracle; not part of the product. */
#ifndef TG_PLATFORM_H
#define TG_PLATFORM_H
#include "tg_common.h"
#define TG_MAX_PATH 260
#define tgp_malloc(size) malloc(size)
#define tgp_free(p)      free(p)
#endif
