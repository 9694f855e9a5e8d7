/* Stand-in for tg/src/memory/tg_memory.h: the reference's stack allocator
 * (tg_memory.c:267) becomes a LIFO of malloc'd blocks and the tracked heap
 * becomes plain calloc/free.  Test infrastructure for the parity oracle. */
#ifndef TG_MEMORY_H
#define TG_MEMORY_H
#include "tg_common.h"
void* tgref_stack_alloc(tg_size size);
void  tgref_stack_free(tg_size size);
#define TG_MALLOC(size)        calloc(1, (size))
#define TG_FREE(p)             free(p)
#define TG_MALLOC_STACK(size)  tgref_stack_alloc(size)
#define TG_FREE_STACK(size)    tgref_stack_free(size)
void tg_memory_nullify(tg_size size, void* p_memory);
#endif
