/* Stand-in for tg/src/graphics/tg_graphics.h: only the data-model header, no Vulkan.
 * Test infrastructure for the parity oracle. */
#ifndef TG_GRAPHICS_H
#define TG_GRAPHICS_H
#include "graphics/tg_graphics_core.h"
#endif
