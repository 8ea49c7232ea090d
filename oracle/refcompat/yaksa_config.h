/*
 * Configuration header for compiling the reference's own test programs
 * (test/pack, test/dtpools, test/simple) against this project's libraries.
 * The reference generates this file with autoconf; the test programs only read
 * the ALIGNOF_* values (test/dtpools/src/dtpools_misc.c:14-120), which are the
 * C11 alignments of the named types on the compiling host.
 */
#ifndef YAKSA_GB300_REFCOMPAT_CONFIG_H
#define YAKSA_GB300_REFCOMPAT_CONFIG_H
#include <stdint.h>
#include <stddef.h>
#include <wchar.h>
#define HAVE_C11_ATOMICS 1
#define HAVE_GCC_ATTRIBUTE 1
#define ALIGNOF__BOOL _Alignof(_Bool)
#define ALIGNOF_CHAR _Alignof(char)
#define ALIGNOF_SIGNED_CHAR _Alignof(signed char)
#define ALIGNOF_UNSIGNED_CHAR _Alignof(unsigned char)
#define ALIGNOF_WCHAR_T _Alignof(wchar_t)
#define ALIGNOF_INT8_T _Alignof(int8_t)
#define ALIGNOF_INT16_T _Alignof(int16_t)
#define ALIGNOF_INT32_T _Alignof(int32_t)
#define ALIGNOF_INT64_T _Alignof(int64_t)
#define ALIGNOF_UINT8_T _Alignof(uint8_t)
#define ALIGNOF_UINT16_T _Alignof(uint16_t)
#define ALIGNOF_UINT32_T _Alignof(uint32_t)
#define ALIGNOF_UINT64_T _Alignof(uint64_t)
#define ALIGNOF_INT _Alignof(int)
#define ALIGNOF_UNSIGNED _Alignof(unsigned)
#define ALIGNOF_SHORT _Alignof(short)
#define ALIGNOF_UNSIGNED_SHORT _Alignof(unsigned short)
#define ALIGNOF_LONG _Alignof(long)
#define ALIGNOF_UNSIGNED_LONG _Alignof(unsigned long)
#define ALIGNOF_LONG_LONG _Alignof(long long)
#define ALIGNOF_UNSIGNED_LONG_LONG _Alignof(unsigned long long)
#define ALIGNOF_INT_FAST8_T _Alignof(int_fast8_t)
#define ALIGNOF_INT_FAST16_T _Alignof(int_fast16_t)
#define ALIGNOF_INT_FAST32_T _Alignof(int_fast32_t)
#define ALIGNOF_INT_FAST64_T _Alignof(int_fast64_t)
#define ALIGNOF_UINT_FAST8_T _Alignof(uint_fast8_t)
#define ALIGNOF_UINT_FAST16_T _Alignof(uint_fast16_t)
#define ALIGNOF_UINT_FAST32_T _Alignof(uint_fast32_t)
#define ALIGNOF_UINT_FAST64_T _Alignof(uint_fast64_t)
#define ALIGNOF_INT_LEAST8_T _Alignof(int_least8_t)
#define ALIGNOF_INT_LEAST16_T _Alignof(int_least16_t)
#define ALIGNOF_INT_LEAST32_T _Alignof(int_least32_t)
#define ALIGNOF_INT_LEAST64_T _Alignof(int_least64_t)
#define ALIGNOF_UINT_LEAST8_T _Alignof(uint_least8_t)
#define ALIGNOF_UINT_LEAST16_T _Alignof(uint_least16_t)
#define ALIGNOF_UINT_LEAST32_T _Alignof(uint_least32_t)
#define ALIGNOF_UINT_LEAST64_T _Alignof(uint_least64_t)
#define ALIGNOF_BYTE 1
#define ALIGNOF_INTMAX_T _Alignof(intmax_t)
#define ALIGNOF_UINTMAX_T _Alignof(uintmax_t)
#define ALIGNOF_SIZE_T _Alignof(size_t)
#define ALIGNOF_INTPTR_T _Alignof(intptr_t)
#define ALIGNOF_UINTPTR_T _Alignof(uintptr_t)
#define ALIGNOF_PTRDIFF_T _Alignof(ptrdiff_t)
#define ALIGNOF_FLOAT _Alignof(float)
#define ALIGNOF_DOUBLE _Alignof(double)
#define ALIGNOF_LONG_DOUBLE _Alignof(long double)
#endif
