// df64.cuh -- double-float ("float pair") arithmetic for the FP64-accurate
// operator on the FP32 pipe.
//
// GB300 executes FP32 at about 60x its FP64 rate, while the FFT passes of the
// FP64 operator are bound by the FP64 pipe.  A df64 value is the unevaluated
// sum hi + lo of two floats with |lo| <= ulp(hi) / 2: 48 significant bits.
// The operations are the classical error-free transformations (Knuth's
// TwoSum, Dekker's FastTwoSum, the FMA-based exact product) combined as in
// the double-double literature (Hida, Li & Bailey, "Library for double-double
// and quad-double arithmetic", 2000; Joldes, Muller & Popescu, "Tight and
// rigorous error bounds for basic building blocks of double-word
// arithmetic", ACM TOMS 2017):
//   add: |err| <= 2^-47 (|a| + |b|)  (the "sloppy" sum: the bound is relative
//        to the operands, which is the bound the FFT error analysis uses);
//   mul: |err| <= 2^-46 |a b|.
// Every float operation is an explicitly rounded intrinsic (__fadd_rn,
// __fmul_rn, __fmaf_rn), so the compiler can neither contract nor reorder
// them.
//
// Exponent range: a value keeps its 48 bits while |lo| stays a normal float,
// i.e. for |x| >= 2^-102 (about 2e-31); smaller parts of a field lose bits
// gradually (norm-wise the error stays at the 2^-47 level of the field's
// largest entries).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fft.cuh"

namespace bri17gb {

struct __align__(8) df64 {
  float hi, lo;
  df64() = default;
  // Exact split of a double into hi + lo (host, and compile-time constants
  // in device code).
  __host__ __device__ constexpr df64(double d)
      : hi(static_cast<float>(d)),
        lo(static_cast<float>(d - static_cast<double>(static_cast<float>(d)))) {}
  __host__ __device__ constexpr df64(float h, float l) : hi(h), lo(l) {}
};

struct __align__(16) df64c {
  df64 x, y;
};

template <>
struct CplxOf<df64> {
  using type = df64c;
};

__device__ __forceinline__ df64 df_neg(df64 a) { return df64(-a.hi, -a.lo); }

__device__ __forceinline__ df64 df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fadd_rn(s, -a);
  const float e = __fadd_rn(__fadd_rn(a, -__fadd_rn(s, -bb)), __fadd_rn(b, -bb));
  return df64(s, e);
}

// |a| >= |b| (or a == 0).
__device__ __forceinline__ df64 df_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df64(s, __fadd_rn(b, -__fadd_rn(s, -a)));
}

__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  const df64 s = df_two_sum(a.hi, b.hi);
  const float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return df_fast_two_sum(s.hi, e);
}

__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }

__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }

__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df_fast_two_sum(p, e);
}

// a * b + c * d with both products kept exact to the end (hi product plus
// its FMA-computed error, and the cross terms) and a single error-free sum
// and renormalisation: 19 float operations against 25 for two products and
// a sum, with the same operand-relative bound as the sloppy sum,
// |err| <= about 2^-46 (|a b| + |c d|).
__device__ __forceinline__ df64 df_dot2(df64 a, df64 b, df64 c, df64 d) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float q = __fmul_rn(c.hi, d.hi);
  float e = __fadd_rn(__fmaf_rn(a.hi, b.hi, -p), __fmaf_rn(c.hi, d.hi, -q));
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  e = __fmaf_rn(c.hi, d.lo, e);
  e = __fmaf_rn(c.lo, d.hi, e);
  const df64 s = df_two_sum(p, q);
  return df_fast_two_sum(s.hi, __fadd_rn(s.lo, e));
}

// a * b + c * d + e * f the same way: three exact products, two error-free
// sums, one renormalisation (31 float operations against 43).
__device__ __forceinline__ df64 df_dot3(df64 a, df64 b, df64 c, df64 d, df64 e, df64 f) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float q = __fmul_rn(c.hi, d.hi);
  const float r = __fmul_rn(e.hi, f.hi);
  float err = __fadd_rn(__fadd_rn(__fmaf_rn(a.hi, b.hi, -p), __fmaf_rn(c.hi, d.hi, -q)),
                        __fmaf_rn(e.hi, f.hi, -r));
  err = __fmaf_rn(a.hi, b.lo, err);
  err = __fmaf_rn(a.lo, b.hi, err);
  err = __fmaf_rn(c.hi, d.lo, err);
  err = __fmaf_rn(c.lo, d.hi, err);
  err = __fmaf_rn(e.hi, f.lo, err);
  err = __fmaf_rn(e.lo, f.hi, err);
  const df64 s1 = df_two_sum(p, q);
  const df64 s2 = df_two_sum(s1.hi, r);
  return df_fast_two_sum(s2.hi, __fadd_rn(__fadd_rn(s1.lo, s2.lo), err));
}

// a * b + c: df64, and the single-rounding FMA for float and double (these
// overloads keep namespace-scope calls of fma(...) on the built-in FMA).
__device__ __forceinline__ df64 fma(df64 a, df64 b, df64 c) { return a * b + c; }
__device__ __forceinline__ float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma(double a, double b, double c) { return __fma_rn(a, b, c); }

// Loads of constant tables (read-only cache where the type allows).
template <typename T>
__device__ __forceinline__ T ldg_val(const T* p) {
  return __ldg(p);
}
template <>
__device__ __forceinline__ df64 ldg_val<df64>(const df64* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return df64(v.x, v.y);
}

// Real fields of a df64 operator are FP64 in memory.
template <typename T>
struct IoOf {
  using type = T;
};
template <>
struct IoOf<df64> {
  using type = double;
};

template <typename T>
__device__ __forceinline__ T from_io(typename IoOf<T>::type v) {
  return v;
}
template <typename T>
__device__ __forceinline__ typename IoOf<T>::type to_io(T v) {
  return v;
}

// double -> hi + lo without the FP64 pipe: the 53-bit significand is split
// by integer operations into its top 24 bits rounded to nearest even (hi)
// and the signed remainder (lo, rounded to 24 bits), each scaled by an
// exact power of two; integer operations only.  Zeros and subnormal doubles
// give a signed zero, infinities infinity, NaN a NaN, and magnitudes beyond
// the float range infinity.
__device__ __forceinline__ float df_pow2(int e) {
  // 2^e for e in [-149, 127] (subnormal range included), built exactly.
  if (e >= -126) return __int_as_float((e + 127) << 23);
  return __int_as_float(1 << (e + 149));
}

static __device__ __noinline__ df64 df_from_double_general(double v) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  const int ex = (int)((bits >> 52) & 0x7FF);
  const bool neg = (bits >> 63) != 0;
  const unsigned fsign = neg ? 0x80000000u : 0u;
  if (ex == 0) return df64(__uint_as_float(fsign), 0.f);
  if (ex == 0x7FF)  // infinity, or a quiet NaN
    return df64(__uint_as_float(fsign | 0x7F800000u | ((bits & ((1ull << 52) - 1)) ? 0x400000u : 0u)),
                0.f);
  const long long sig = (long long)((bits & ((1ull << 52) - 1)) | (1ull << 52));
  long long q = sig >> 29;              // top 24 bits
  long long r = sig & ((1ll << 29) - 1);  // low 29 bits
  if (r > (1ll << 28) || (r == (1ll << 28) && (q & 1))) {
    q += 1;
    r -= 1ll << 29;
  }
  // value = sig * 2^(ex - 1075) = q * 2^(ex - 1046) + r * 2^(ex - 1075)
  const int eh = ex - 1046, el = ex - 1075;
  float hi, lo;
  if (eh > 127 - 24) {
    hi = __uint_as_float(0x7F800000u);  // beyond the float range: infinity
    lo = 0.f;
  } else {
    // q <= 2^24 and |r| <= 2^28 convert to float (q exactly, r rounded);
    // the power-of-two scalings are exact unless they underflow.
    // (32-bit integer conversions: the 64-bit ones do not run on the FP32
    // side.)
    const float sh = eh >= -149 ? df_pow2(eh) : 0.f;
    hi = __fmul_rn(__int2float_rn((int)q), sh);
    // Split the scaling of lo so that neither factor underflows early.
    const int el1 = el < -126 ? -126 : el;
    lo = __fmul_rn(__fmul_rn(__int2float_rn((int)r), df_pow2(el1)),
                   el < -126 ? (el - el1 >= -149 ? df_pow2(el - el1) : 0.f) : 1.f);
  }
  return neg ? df64(-hi, -lo) : df64(hi, lo);
}

// hi + lo -> double by integer operations only (float-to-double conversions
// and the add would run on the FP64 pipe): hi's 24-bit significand goes to
// the top of 53 bits, lo's is added or subtracted at its offset (bits below
// the 53 are dropped: error below 2^-52 relative), then one normalisation.
// Zero or subnormal hi gives a signed zero; an infinite or NaN part gives
// infinity or NaN.
static __device__ __noinline__ double df_to_double_general(df64 v) {
  const unsigned hb = __float_as_uint(v.hi), lb = __float_as_uint(v.lo);
  const int eh = (int)((hb >> 23) & 0xFF), el = (int)((lb >> 23) & 0xFF);
  unsigned long long sign = (unsigned long long)(hb >> 31) << 63;
  if (eh == 0xFF || el == 0xFF) {
    const unsigned long long nan = (el == 0xFF && (lb & 0x7FFFFFu)) ? (1ull << 51) : 0;
    return __longlong_as_double((long long)(sign | (0x7FFull << 52) |
                                            ((unsigned long long)(hb & 0x7FFFFFu) << 29) | nan));
  }
  if (eh == 0) return __longlong_as_double((long long)sign);
  long long M = (long long)((hb & 0x7FFFFFu) | 0x800000u) << 29;
  const int shift = eh - el;
  if (el != 0) {
    long long L = (long long)((lb & 0x7FFFFFu) | 0x800000u);
    L = shift <= 29 ? (L << (29 - shift)) : (shift - 29 < 62 ? (L >> (shift - 29)) : 0);
    M = ((hb ^ lb) >> 31) == 0 ? M + L : M - L;
  }
  if (M == 0) return __longlong_as_double((long long)sign);
  if (M < 0) {
    M = -M;
    sign ^= 1ull << 63;
  }
  // Put the leading bit at position 52.
  const int lead = 63 - __clzll(M);
  int e = eh - 127 + 1023 + (lead - 52);
  M = lead >= 52 ? (M >> (lead - 52)) : (M << (52 - lead));
  if (e <= 0) return __longlong_as_double((long long)sign);
  if (e >= 0x7FF) return __longlong_as_double((long long)(sign | (0x7FFull << 52)));
  return __longlong_as_double(
      (long long)(sign | ((unsigned long long)e << 52) | ((unsigned long long)M & ((1ull << 52) - 1))));
}

// Fast paths of the conversions, 32-bit integer operations only (the
// general forms above work on 64-bit integers and normalise with variable
// shifts; on the FP64 operator's 128^3 fields they took about a tenth of the
// float-pair application).
//
// double -> hi + lo for biased exponents E in [949, 1149] (|v| in about
// [2^-74, 2^126]): hi's 23 fraction bits are the double's top 23, rounded to
// nearest even on the 29 below (the carry of the rounding increment runs
// into hi's exponent as it should); the signed remainder (|r| <= 2^28)
// converts to a float rounded to nearest and is scaled by 2^(E - 1075),
// a normal power of two in this range.  Same values as the general form.
template <>
__device__ __forceinline__ df64 from_io<df64>(double v) {
  const unsigned h = (unsigned)__double2hiint(v), l = (unsigned)__double2loint(v);
  const unsigned E = (h >> 20) & 0x7FFu;
  if (E < 949u || E > 1149u) return df_from_double_general(v);
  const unsigned sign = h & 0x80000000u;
  const unsigned frac = ((h & 0xFFFFFu) << 3) | (l >> 29);
  const unsigned r = l & 0x1FFFFFFFu;
  const unsigned up = (r > 0x10000000u || (r == 0x10000000u && (frac & 1u))) ? 1u : 0u;
  const float hi = __uint_as_float((sign | ((E - 896u) << 23) | frac) + up);
  const int rem = (int)r - (up ? 0x20000000 : 0);
  float lo = __fmul_rn(__int2float_rn(rem), __uint_as_float((E - 948u) << 23));
  if (sign) lo = -lo;
  return df64(hi, lo);
}

// hi + lo -> double for a normalised pair (|lo| <= ulp(hi)/2, so lo sits at
// least 24 binades below hi) of normal floats, or a zero lo.  With
// s = e_hi - e_lo, lo is m_lo 2^(29 - s) units of the double's last place
// in hi's binade: exact for s <= 29; for s >= 30 lo's bits below that place
// are dropped (|lo| truncated), as in the general form.  That many units
// are added to or taken from hi's double bit pattern, which stays in hi's
// binade unless hi is a power of two and lo has the other sign; that case,
// specials, subnormal parts and pairs that are not normalised go to the
// general form.  Same values as the general form.
template <>
__device__ __forceinline__ double to_io<df64>(df64 v) {
  const unsigned hb = __float_as_uint(v.hi), lb = __float_as_uint(v.lo);
  const unsigned eh = (hb >> 23) & 0xFFu, el = (lb >> 23) & 0xFFu;
  const unsigned s = eh - el;
  const bool lo_zero = (lb << 1) == 0u;
  const bool neg = ((hb ^ lb) >> 31) != 0u;
  // hi as a double: sign, exponent rebased by 1023 - 127 = 896, the 23
  // fraction bits at the top of the 52.
  const unsigned long long dh =
      ((unsigned long long)((hb & 0x80000000u) | (((hb & 0x7FFFFFFFu) >> 3) + (896u << 20)))
       << 32) |
      (unsigned long long)((hb & 7u) << 29);
  if (eh - 1u >= 254u) return df_to_double_general(v);
  if (lo_zero) return __longlong_as_double((long long)dh);
  if (el - 1u >= 254u || s < 24u || (neg && (hb & 0x7FFFFFu) == 0u))
    return df_to_double_general(v);
  const unsigned ml = (lb & 0x7FFFFFu) | 0x800000u;
  const unsigned L = s <= 29u ? ml << (29u - s) : ml >> (s - 29u < 31u ? s - 29u : 31u);
  return __longlong_as_double((long long)(neg ? dh - L : dh + L));
}

// Complex products of float pairs: each part is one df_dot2 (the generic
// forms would round each of the four products and the two sums).
template <>
__device__ __forceinline__ df64c cmul<df64>(df64c a, df64c b) {
  df64c r;
  r.x = df_dot2(a.x, b.x, df_neg(a.y), b.y);
  r.y = df_dot2(a.x, b.y, a.y, b.x);
  return r;
}

// a * conj(b)
template <>
__device__ __forceinline__ df64c cmulc<df64>(df64c a, df64c b) {
  df64c r;
  r.x = df_dot2(a.x, b.x, a.y, b.y);
  r.y = df_dot2(a.y, b.x, df_neg(a.x), b.y);
  return r;
}

// Sums inside a butterfly (fft.cuh badd / bsub / bnorm): the hi parts by
// TwoSum, the lo parts added to its error term, without the final
// renormalisation (8 float operations instead of 11); bnorm renormalises a
// butterfly's outputs.  A sum of such pairs stays within the sloppy sum's
// operand-relative bound to first order.
__device__ __forceinline__ df64 df_add_nr(df64 a, df64 b) {
  const df64 s = df_two_sum(a.hi, b.hi);
  return df64(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

template <>
__device__ __forceinline__ df64c badd<df64>(df64c a, df64c b) {
  df64c r;
  r.x = df_add_nr(a.x, b.x);
  r.y = df_add_nr(a.y, b.y);
  return r;
}

template <>
__device__ __forceinline__ df64c bsub<df64>(df64c a, df64c b) {
  df64c r;
  r.x = df_add_nr(a.x, df_neg(b.x));
  r.y = df_add_nr(a.y, df_neg(b.y));
  return r;
}

template <>
__device__ __forceinline__ df64c bnorm<df64>(df64c a) {
  df64c r;
  r.x = df_fast_two_sum(a.x.hi, a.x.lo);
  r.y = df_fast_two_sum(a.y.hi, a.y.lo);
  return r;
}

}  // namespace bri17gb
