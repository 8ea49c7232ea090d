/*
 * quad_harness.c -- test infrastructure: the binary128 routines of yk_quad.h next to
 * the C compiler's own _Float128 arithmetic (libgcc's soft-float on x86_64, and the
 * long double of aarch64), over the same arrays of 16-byte values.  The host test
 * (test_quad_cpu.py) compiles it with gcc and compares the two sides bit for bit.
 *
 * op: 0 a + b, 1 a * b, 2 a - b, 3 a < b (result 1 or 0 in the low byte); for
 * the complex form the elements are 32-byte (re, im) pairs and the op is a * b.
 */
#include <string.h>
#include "yk_quad.h"

static yk_u128 ld(const unsigned char *p)
{
    yk_u128 v;
    memcpy(&v, p, 16);
    return v;
}

static void st(unsigned char *p, yk_u128 v)
{
    memcpy(p, &v, 16);
}

void quad_ours(int op, const unsigned char *a, const unsigned char *b, unsigned char *out, long n)
{
    for (long i = 0; i < n; i++) {
        const yk_u128 x = ld(a + 16 * i), y = ld(b + 16 * i);
        yk_u128 r = 0;
        switch (op) {
            case 0: r = yk_q_add(x, y); break;
            case 1: r = yk_q_mul(x, y); break;
            case 2: r = yk_q_sub(x, y); break;
            default: r = (yk_u128) yk_q_lt(x, y); break;
        }
        st(out + 16 * i, r);
    }
}

void quad_gcc(int op, const unsigned char *a, const unsigned char *b, unsigned char *out, long n)
{
    for (long i = 0; i < n; i++) {
        _Float128 x, y, r;
        memcpy(&x, a + 16 * i, 16);
        memcpy(&y, b + 16 * i, 16);
        switch (op) {
            case 0: r = x + y; break;
            case 1: r = x * y; break;
            case 2: r = x - y; break;
            default: st(out + 16 * i, (yk_u128) (x < y)); continue;
        }
        memcpy(out + 16 * i, &r, 16);
    }
}

void cquad_ours(const unsigned char *a, const unsigned char *b, unsigned char *out, long n)
{
    for (long i = 0; i < n; i++) {
        yk_u128 x, y;
        yk_q_cmul(ld(a + 32 * i), ld(a + 32 * i + 16), ld(b + 32 * i), ld(b + 32 * i + 16), &x, &y);
        st(out + 32 * i, x);
        st(out + 32 * i + 16, y);
    }
}

void cquad_gcc(const unsigned char *a, const unsigned char *b, unsigned char *out, long n)
{
    for (long i = 0; i < n; i++) {
        _Complex _Float128 x, y, r;
        memcpy(&x, a + 32 * i, 32);
        memcpy(&y, b + 32 * i, 32);
        r = x * y;
        memcpy(out + 32 * i, &r, 32);
    }
}
