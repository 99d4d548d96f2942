// float-float arithmetic (two FP32 words, ~48-bit mantissa) for the mixed-precision
// kernels: error-free products by fmaf, Dekker/Knuth sums, power-of-two shifts on the
// bit patterns.  Shared by the q-sum and element kernels.
#pragma once
#include "common.cuh"

namespace capsgpu {

struct ff { float h, l; };
struct ffe { float h, l; int e, pad; }; // (h + l) * 2^e
// exponent carried by a zero table value, far below any nonzero one, so that a maximum over
// exponents needs no zero test and a zero aligned to it scales to 0
constexpr int FFE_ZERO_E = -(1 << 20);
CAPS_DEV ff ff_fast2(float a, float b) { const float s = a + b; return ff{s, b - (s - a)}; }
CAPS_DEV ff ff_mul(ff x, ff y)
{
    const float p = x.h * y.h;
    float e = fmaf(x.h, y.h, -p);
    e = fmaf(x.h, y.l, e);
    e = fmaf(x.l, y.h, e);
    return ff_fast2(p, e);
}
CAPS_DEV ff ff_add(ff x, ff y)
{
    const float s = x.h + y.h, bb = s - x.h;
    float e = (x.h - (s - bb)) + (y.h - bb);
    e += x.l + y.l;
    return ff_fast2(s, e);
}
CAPS_DEV ff ff_neg(ff x) { return ff{-x.h, -x.l}; }
CAPS_DEV int fexpo(float x) { return (int)((__float_as_uint(x) >> 23) & 0xff) - 127; }
// x * 2^k on the bit patterns; flushes to zero below 2^-120
CAPS_DEV float fshift(float x, int k)
{
    const unsigned b = __float_as_uint(x);
    const int ex = (int)((b >> 23) & 0xff);
    if (ex == 0 || ex + k <= 6) return 0.0f;
    return __uint_as_float(b + ((unsigned)k << 23));
}
CAPS_DEV ff ff_shift(ff x, int k) { return ff{fshift(x.h, k), fshift(x.l, k)}; }
CAPS_DEV ff ff_from_d(double x) { const float h = (float)x; return ff{h, (float)(x - (double)h)}; }
CAPS_DEV double ff_to_d(ff x) { return (double)x.h + (double)x.l; }
// exact int64 -> float-float (48 of the 63 bits kept) times 2^k
CAPS_DEV ff ff_from_ll(long long v, int k)
{
    const float h = (float)v;
    const long long r = v - (long long)h;
    return ff{fshift(h, k), fshift((float)r, k)};
}

} // namespace capsgpu
