// Double-float arithmetic on the FP32 pipe: a value is an unevaluated pair hi + lo of FP32 numbers
// (~48 significant bits). Used where GB300's FP64 pipe (1/60 of its FP32 rate) would bound a kernel
// and ~1e-14 relative accuracy per operation suffices.
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


struct Df {
  float h, l;
};

__device__ __forceinline__ Df df_of(double x) {
  Df r;
  df_split(x, r.h, r.l);
  return r;
}

__device__ __forceinline__ double df_to_double(Df a) { return (double)a.h + (double)a.l; }

// error-free product a.h * b.h plus the cross terms: (p, e) with a b = p + e to ~2^-48
__device__ __forceinline__ void df_prod(Df a, Df b, float& p, float& e) {
  p = a.h * b.h;
  e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
}

// c - a b, renormalised
__device__ __forceinline__ Df df_fms(Df c, Df a, Df b) {
  float p, e;
  df_prod(a, b, p, e);
  const float s = c.h - p;
  const float bb = s - c.h;
  const float err = (c.h - (s - bb)) + (-p - bb);
  const float lo = (c.l - e) + err;
  Df r;
  r.h = s + lo;
  r.l = lo - (r.h - s);
  return r;
}

// a b, renormalised
__device__ __forceinline__ Df df_mul(Df a, Df b) {
  float p, e;
  df_prod(a, b, p, e);
  Df r;
  r.h = p + e;
  r.l = e - (r.h - p);
  return r;
}

// A double-float number with arithmetic operators, for templates written over a value type T
// (the cluster Jacobi): + - * and fma renormalise their result; comparisons and the conversion to
// double evaluate hi + lo in FP64.
struct DfN {
  float h, l;
  DfN() = default;
  __device__ __forceinline__ explicit DfN(double x) { df_split(x, h, l); }
  __device__ __forceinline__ explicit DfN(int x) : h((float)x), l(0.f) {}
  __device__ __forceinline__ static DfN make(float hi, float lo) {
    DfN r;
    r.h = hi;
    r.l = lo;
    return r;
  }
  __device__ __forceinline__ explicit operator double() const { return (double)h + (double)l; }
};

__device__ __forceinline__ DfN operator+(DfN a, DfN b) {
  const float s = a.h + b.h;
  const float bb = s - a.h;
  const float err = (a.h - (s - bb)) + (b.h - bb);
  const float lo = err + (a.l + b.l);
  const float h = s + lo;
  return DfN::make(h, lo - (h - s));
}
__device__ __forceinline__ DfN operator-(DfN a) { return DfN::make(-a.h, -a.l); }
__device__ __forceinline__ DfN operator-(DfN a, DfN b) { return a + (-b); }
__device__ __forceinline__ DfN operator*(DfN a, DfN b) {
  float p, e;
  df_prod(Df{a.h, a.l}, Df{b.h, b.l}, p, e);
  const float h = p + e;
  return DfN::make(h, e - (h - p));
}
// the FP64 and FP32 fma stay visible beside the double-float one inside this namespace
using ::fma;

// c + a b
__device__ __forceinline__ DfN fma(DfN a, DfN b, DfN c) {
  float p, e;
  df_prod(Df{a.h, a.l}, Df{b.h, b.l}, p, e);
  const float s = c.h + p;
  const float bb = s - c.h;
  const float err = (c.h - (s - bb)) + (p - bb);
  const float lo = (c.l + e) + err;
  const float h = s + lo;
  return DfN::make(h, lo - (h - s));
}
__device__ __forceinline__ bool operator>(DfN a, DfN b) { return (double)a > (double)b; }

}  // namespace ttgb
