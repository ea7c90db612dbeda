// The FP64 -> double-float split of the double-float contraction engine: a value becomes an
// unevaluated pair hi + lo of FP32 numbers (~48 significant bits), so products and sums run on the
// FP32 pipe, GB300's FP64 pipe being 1/60 of its FP32 rate.
#pragma once

#include <cstdint>

namespace ttgb {

// The split is built from the bits of x with integer operations: h is x rounded to 24 significant
// bits (the sign, exponent and top 23 stored mantissa bits, plus one unit when the first dropped
// bit is set - a carry into the exponent is the correct rounding), l is the signed remainder
// (|l| <= 2^-24 |h|) converted to FP32 and scaled by the exponent, so x = h + l to 2^-48 relative.
// The obvious form h = (float)x, l = (float)(x - h) runs two conversions and a subtraction on the
// FP64 pipe for every loaded element; on GB300 that pipe then bounds the kernel (ncu: FP64 pipe 51%
// active against 31% for the FP32 FMA pipe).
__device__ __forceinline__ void df_split(double x, float& h, float& l) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(u >> 32), lo = (unsigned)u;
  const unsigned sign = hi & 0x80000000u;
  const int fe = (int)((hi >> 20) & 0x7ffu) - 896;   // biased FP32 exponent of x (1023 - 127)
  if (fe >= 1 && fe <= 254) {
    const unsigned rb = (lo >> 28) & 1u;
    h = __uint_as_float((sign | ((unsigned)fe << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29)) + rb);
    // x - h in units of 2^(e - 1075): the 29 dropped bits, less 2^29 when h was rounded up
    const int rem = (int)(lo & 0x1fffffffu) - (int)(rb << 29);
    const float r = __int2float_rn(rem) * 0x1p-52f * __uint_as_float((unsigned)fe << 23);
    l = __uint_as_float(__float_as_uint(r) ^ sign);
  } else if (((hi & 0x7fffffffu) | lo) == 0u) {   // +-0 (also every masked load)
    h = __uint_as_float(sign);
    l = 0.f;
  } else {   // outside the FP32 range: the engine is only chosen when operands fit
    h = (float)x;
    l = 0.f;
  }
}


}  // namespace ttgb
