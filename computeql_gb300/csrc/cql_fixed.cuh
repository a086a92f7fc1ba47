// Fixed-point decimals in integer arithmetic on the bits of a double (GB300's FP64 rate is a small
// fraction of its integer rate). Shared by the fixed-point scale search and every reduce that scales
// an argument by 10^s the way the reference's shaders do (floor(v * 10^s + 0.5)).
//
// With |v| = m * 2^-sh, W = floor(m*10^s / 2^sh + 1/2) is the nearest integer to |v|*10^s; the
// reference's test "whole / 10^s == v" holds exactly when W / 10^s rounds back to v, i.e. when
// W*2^sh - m*10^s lies inside v's rounding interval (half an ulp either side, a quarter below a power
// of two, ties to the even mantissa). For |v| < 2^31 and s <= 6 the reference's rounded product and
// the exact one give the same W whenever the test can pass.
#pragma once

#include <stdint.h>

#define FIXED_MAX_SCALE 6

static __constant__ unsigned long long c_fix_pow10[FIXED_MAX_SCALE + 1] = { 1ull, 10ull, 100ull, 1000ull, 10000ull, 100000ull, 1000000ull };

// |v| = m * 2^-sh; `big` when !(|v| < 2^31), which includes infinities and NaN
struct FixVal
{
  unsigned long long m;
  int sh;
  bool neg;
  bool big;
  unsigned long long mag_bits;   // |v| as f64 bits
};

__device__ __forceinline__ FixVal fix_decode_f64(unsigned long long bits)
{
  FixVal f;
  uint32_t e = (uint32_t)(bits >> 52) & 0x7ffu;
  unsigned long long frac = bits & 0xfffffffffffffull;
  f.neg = (bits >> 63) != 0;
  f.m = e ? (frac | (1ull << 52)) : frac;
  f.sh = e ? 1075 - (int)e : 1074;
  f.big = e >= 1023u + 31u;
  f.mag_bits = bits & 0x7fffffffffffffffull;
  return f;
}

// a float as the double it converts to exactly
__device__ __forceinline__ FixVal fix_decode_f32(uint32_t bits)
{
  FixVal f;
  uint32_t e = (bits >> 23) & 0xffu;
  uint32_t frac = bits & 0x7fffffu;
  f.neg = (bits >> 31) != 0;
  if (e)
  {
    f.m = ((unsigned long long)(frac | 0x800000u)) << 29;
    f.sh = 1075 - (int)(e + 896u);
    f.mag_bits = ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)frac << 29);
  }
  else
  {
    f.m = (unsigned long long)frac << 29;   // zero, or a subnormal float: |v| < 2^-126, never whole
    f.sh = 1075 - 896 + 29;
    f.mag_bits = 0;
  }
  f.big = e >= 127u + 31u;
  return f;
}

// The nearest integer W to |v| * 10^s; returns whether W / 10^s rounds back to |v|.
__device__ __forceinline__ bool fix_whole(const FixVal& f, int s, unsigned long long* out_w)
{
  unsigned long long p = c_fix_pow10[s];
  *out_w = 0;
  if (f.m == 0) return true;
  if (f.sh >= 75) return false;   // |v| * 10^s < 1/4 rounds to 0, which is not v
  if (f.sh <= 21) return false;   // |v| >= 2^31: outside the fixed-point range
  bool pow2 = f.m == (1ull << 52);
  bool even = (f.m & 1ull) == 0;
  if (s <= 3 && f.sh <= 63)
  {
    // m * p < 2^63: everything fits 64 bits
    unsigned long long P = f.m * p;
    unsigned long long W = (P + (1ull << (f.sh - 1))) >> f.sh;
    *out_w = W;
    if (W == 0) return false;
    unsigned long long Ws = W << f.sh;
    if (Ws >= P)
    {
      unsigned long long d2 = (Ws - P) << 1;
      return d2 < p || (d2 == p && even);
    }
    unsigned long long d = P - Ws;
    if (pow2) return (d << 2) <= p;
    return (d << 1) < p || ((d << 1) == p && even);
  }
  unsigned __int128 P = (unsigned __int128)f.m * p;
  unsigned __int128 W = (P + ((unsigned __int128)1 << (f.sh - 1))) >> f.sh;
  *out_w = (unsigned long long)W;
  if (W == 0) return false;
  unsigned __int128 Ws = W << f.sh;
  if (Ws >= P)
  {
    unsigned __int128 d2 = (Ws - P) << 1;
    return d2 < p || (d2 == p && even);
  }
  unsigned __int128 d = P - Ws;
  if (pow2) return (d << 2) <= p;
  return (d << 1) < p || ((d << 1) == p && even);
}

// floor(v * 10^s + 0.5) of a value known to be whole at scale s (|v| * 10^s < 2^31): the nearest
// integer to the exact product, which is that value's floor(v * 10^s + 0.5) in FP64 too
__device__ __forceinline__ int fix_scaled(const FixVal& f, int s)
{
  if (f.m == 0 || f.sh >= 75 || f.sh <= 21) return 0;
  unsigned long long p = c_fix_pow10[s], w;
  if (s <= 3 && f.sh <= 63) w = (f.m * p + (1ull << (f.sh - 1))) >> f.sh;
  else w = (unsigned long long)(((unsigned __int128)f.m * p + ((unsigned __int128)1 << (f.sh - 1))) >> f.sh);
  return f.neg ? -(int)w : (int)w;
}

