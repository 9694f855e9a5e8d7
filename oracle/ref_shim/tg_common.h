/*
 * Stand-in for tg's tg_common.h (tg/src/tg_common.h:1-120) used only when the
 * reference's CPU files are compiled on Linux for the parity oracle.  It
 * provides the same type names and constants without MSVC literal suffixes
 * (tg_common.h:67-79 uses i8/i16/i32/i64/ui* suffixes that gcc rejects).
 * TG_ASSERT reports through tgref_assert_fail instead of writing through a
 * null pointer (tg_common.h:33), so a violated reference precondition is
 * detected and reported rather than crashing or running on.
 * Test infrastructure only: nothing in the product includes this header.
 */
#ifndef TG_COMMON_H
#define TG_COMMON_H

#include <stdio.h>
#include <stdlib.h>

#define TG_CPU_x64

/* A failed reference precondition unwinds to the driver (ref_driver.c), which
 * reports the scene as one the reference cannot build, instead of crashing. */
void tgref_assert_fail(const char* condition, const char* file, int line);
#define TG_ASSERT(condition) \
    do { if (!(condition)) tgref_assert_fail(#condition, __FILE__, __LINE__); } while (0)
#define TG_DEBUG_PARAM(param)
#define TG_INVALID_CODEPATH()    abort()
#define TG_NOT_IMPLEMENTED()     abort()
#define TG_STATIC_ASSERT(condition) _Static_assert((condition), #condition)

#define TG_SIZEOF_MEMBER(type, member)  sizeof(((type*)0)->member)
#define TG_OFFSET_OF(type, member)      ((tg_size)&(((type*)0)->member))
#define TG_UNUSED(x)                    ((void)(x))
#define TG_INOUT
#define TG_OUT

#define TG_NULL   ((void*)0)
#define TG_TRUE   1
#define TG_FALSE  0

#define TG_F32_MAX            3.402823466e+38f
#define TG_F32_MIN            (-TG_F32_MAX)
#define TG_F32_MIN_POSITIVE   1.175494351e-38f
#define TG_F32_EPSILON        1.192092896e-07f
#define TG_F64_MAX_POSITIVE   1.7976931348623158e+308
#define TG_F64_MIN_POSITIVE   2.2250738585072014e-308
#define TG_F64_EPSILON        2.2204460492503131e-016

#define TG_I8_MIN   (-127 - 1)
#define TG_I16_MIN  (-32767 - 1)
#define TG_I32_MIN  (-2147483647 - 1)
#define TG_I64_MIN  (-9223372036854775807LL - 1)
#define TG_I8_MAX   127
#define TG_I16_MAX  32767
#define TG_I32_MAX  2147483647
#define TG_I64_MAX  9223372036854775807LL
#define TG_U8_MAX   0xffu
#define TG_U16_MAX  0xffffu
#define TG_U32_MAX  0xffffffffu
#define TG_U64_MAX  0xffffffffffffffffull

#define TG_IEEE_754_FLOAT_SIGN_BITS      1
#define TG_IEEE_754_FLOAT_EXPONENT_BITS  8
#define TG_IEEE_754_FLOAT_MANTISSA_BITS  23
#define TG_IEEE_754_FLOAT_SIGN_MASK      0x80000000
#define TG_IEEE_754_FLOAT_EXPONENT_MASK  0x7f800000
#define TG_IEEE_754_FLOAT_MANSISSA_MASK  0x007fffff

typedef int                 b32;
typedef float               f32;
typedef signed char         i8;
typedef short               i16;
typedef int                 i32;
typedef unsigned char       u8;
typedef unsigned short      u16;
typedef unsigned int        u32;
typedef double              f64;
typedef long long           i64;
typedef unsigned long long  u64;
typedef unsigned long long  tg_size;

#endif
