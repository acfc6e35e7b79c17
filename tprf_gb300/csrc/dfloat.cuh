// Double-float ("df64") arithmetic: a real number is an unevaluated sum
// hi + lo of two FP32 values, |lo| <= ulp(hi), about 48 significant bits.
//
// GB300 executes FP32 at ~70x its FP64 rate, so the FFT stages of this path
// run their butterflies in this representation on the FP32 pipe. The
// operations are the classical error-free transformations: Knuth's TwoSum,
// Dekker's Fast2Sum (quick_two_sum) and the FMA-based TwoProduct, combined as
// in the published double-double algorithms (Hida, Li & Bailey, "Algorithms
// for quad-double precision floating point arithmetic", 2001), applied to two
// floats instead of two doubles. Additions use the "sloppy" variant (one
// TwoSum plus a Fast2Sum): its error is bounded relative to |a| + |b|, which
// is what an FFT needs. Every float operation uses a _rn intrinsic so the
// compiler can neither contract nor reassociate it.
//
// Conversions from FP64 use integer bit operations only (the FP64 pipe's
// conversion instructions are slower on GB300); conversions to FP64 widen the
// two floats by bit operations and add them with one FP64 addition
// (to_double_add), or use bit operations only (to_double).
#pragma once

#include <cuda_runtime.h>

namespace tprf {

struct dfl {
  float hi, lo;
};

struct __align__(16) cdf {
  dfl x, y;  // real, imaginary
};

__host__ __device__ constexpr dfl kdf(double v) { return dfl{(float)v, (float)(v - (double)(float)v)}; }

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ dfl fast_two_sum(float a, float b) {  // requires |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return dfl{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ dfl dneg(dfl a) { return dfl{-a.hi, -a.lo}; }

__device__ __forceinline__ dfl dadd(dfl a, dfl b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s, e);
}

__device__ __forceinline__ dfl dsub(dfl a, dfl b) { return dadd(a, dneg(b)); }

// a + b without the closing Fast2Sum: hi + lo carries the sum to the same
// accuracy as dadd, but |lo| may exceed half an ulp of hi. TwoSum is exact for
// any inputs and dmul keeps a.lo in full, so a short chain of these adds (the
// levels of one butterfly) followed by one renorm() keeps the error bounded
// relative to the magnitudes of the inputs, as the sloppy dadd does.
__device__ __forceinline__ dfl dadd_lazy(dfl a, dfl b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  return dfl{s, __fadd_rn(e, __fadd_rn(a.lo, b.lo))};
}
__device__ __forceinline__ dfl renorm(dfl a) { return fast_two_sum(a.hi, a.lo); }

__device__ __forceinline__ dfl dmul(dfl a, dfl b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

// a1 b1 - a2 b2 with one rounding-error accumulator
__device__ __forceinline__ dfl ddot_sub(dfl a1, dfl b1, dfl a2, dfl b2) {
  const float p1 = __fmul_rn(a1.hi, b1.hi);
  const float e1 = __fmaf_rn(a1.hi, b1.hi, -p1);
  const float p2 = __fmul_rn(a2.hi, b2.hi);
  const float e2 = __fmaf_rn(a2.hi, b2.hi, -p2);
  float s, es;
  two_sum(p1, -p2, s, es);
  float e = __fadd_rn(es, __fsub_rn(e1, e2));
  e = __fmaf_rn(a1.hi, b1.lo, e);
  e = __fmaf_rn(a1.lo, b1.hi, e);
  e = __fmaf_rn(-a2.hi, b2.lo, e);
  e = __fmaf_rn(-a2.lo, b2.hi, e);
  return fast_two_sum(s, e);
}

// a1 b1 + a2 b2
__device__ __forceinline__ dfl ddot_add(dfl a1, dfl b1, dfl a2, dfl b2) { return ddot_sub(a1, b1, dneg(a2), b2); }

// c - p q + u v: the ddot_sub scheme with the accumulator as a third term. The
// leading parts of c and of the two products meet in two TwoSums; their
// rounding errors, the products' errors, c.lo and the four cross terms go to
// one float, closed by one Fast2Sum (27 float operations against 30 for
// dsub(c, ddot_sub(p, q, u, v))), with the same error bound relative to
// |c| + |p q| + |u v|.
__device__ __forceinline__ dfl dfms2(dfl c, dfl p, dfl q, dfl u, dfl v) {
  const float p1 = __fmul_rn(-p.hi, q.hi);
  const float e1 = __fmaf_rn(-p.hi, q.hi, -p1);
  const float p2 = __fmul_rn(u.hi, v.hi);
  const float e2 = __fmaf_rn(u.hi, v.hi, -p2);
  float s, t1, t2;
  two_sum(c.hi, p1, s, t1);
  two_sum(s, p2, s, t2);
  float e = __fadd_rn(__fadd_rn(t1, t2), __fadd_rn(c.lo, __fadd_rn(e1, e2)));
  e = __fmaf_rn(-p.hi, q.lo, e);
  e = __fmaf_rn(-p.lo, q.hi, e);
  e = __fmaf_rn(u.hi, v.lo, e);
  e = __fmaf_rn(u.lo, v.hi, e);
  return fast_two_sum(s, e);
}

// ---- complex ----------------------------------------------------------------
__device__ __forceinline__ cdf cadd(cdf a, cdf b) { return cdf{dadd(a.x, b.x), dadd(a.y, b.y)}; }
__device__ __forceinline__ cdf csub(cdf a, cdf b) { return cdf{dsub(a.x, b.x), dsub(a.y, b.y)}; }
// butterfly-internal adds (see dadd_lazy) and the renormalisation before a store
__device__ __forceinline__ cdf cadd_lz(cdf a, cdf b) { return cdf{dadd_lazy(a.x, b.x), dadd_lazy(a.y, b.y)}; }
__device__ __forceinline__ cdf csub_lz(cdf a, cdf b) { return cdf{dadd_lazy(a.x, dneg(b.x)), dadd_lazy(a.y, dneg(b.y))}; }
__device__ __forceinline__ cdf cnorm(cdf a) { return cdf{renorm(a.x), renorm(a.y)}; }
__device__ __forceinline__ cdf cmul(cdf a, cdf b) { return cdf{ddot_sub(a.x, b.x, a.y, b.y), ddot_add(a.x, b.y, a.y, b.x)}; }
__device__ __forceinline__ cdf cscale(cdf a, dfl s) { return cdf{dmul(a.x, s), dmul(a.y, s)}; }
__device__ __forceinline__ cdf cconj(cdf a) { return cdf{a.x, dneg(a.y)}; }
// y + k x
__device__ __forceinline__ cdf caxpy(dfl k, cdf x, cdf y) { return cadd(y, cscale(x, k)); }
// acc - a b (the elimination update)
__device__ __forceinline__ cdf cfms_df(cdf a, cdf b, cdf acc) {
  return cdf{dfms2(acc.x, a.x, b.x, a.y, b.y), dfms2(acc.y, a.x, b.y, dneg(a.y), b.x)};
}
// acc - a b without the closing Fast2Sums (dfms2 stops at s + e: the same value,
// |lo| not bounded by half an ulp of hi). Only for a value that goes on into
// further updates; renormalise (cnorm) before a product reads it, a magnitude is
// taken from its high words, or it is converted.
__device__ __forceinline__ dfl dfms2_lazy(dfl c, dfl p, dfl q, dfl u, dfl v) {
  const float p1 = __fmul_rn(-p.hi, q.hi);
  const float e1 = __fmaf_rn(-p.hi, q.hi, -p1);
  const float p2 = __fmul_rn(u.hi, v.hi);
  const float e2 = __fmaf_rn(u.hi, v.hi, -p2);
  float s, t1, t2;
  two_sum(c.hi, p1, s, t1);
  two_sum(s, p2, s, t2);
  float e = __fadd_rn(__fadd_rn(t1, t2), __fadd_rn(c.lo, __fadd_rn(e1, e2)));
  e = __fmaf_rn(-p.hi, q.lo, e);
  e = __fmaf_rn(-p.lo, q.hi, e);
  e = __fmaf_rn(u.hi, v.lo, e);
  e = __fmaf_rn(u.lo, v.hi, e);
  return dfl{s, e};
}
__device__ __forceinline__ cdf cfms_df_lazy(cdf a, cdf b, cdf acc) {
  return cdf{dfms2_lazy(acc.x, a.x, b.x, a.y, b.y), dfms2_lazy(acc.y, a.x, b.y, dneg(a.y), b.x)};
}
// acc + a b
__device__ __forceinline__ cdf cfma_df(cdf a, cdf b, cdf acc) {
  return cdf{dfms2(acc.x, a.y, b.y, a.x, b.x), dfms2(acc.y, dneg(a.x), b.y, a.y, b.x)};
}
template <bool FWD>
__device__ __forceinline__ cdf mul_mi(cdf a) {  // -i a (FWD) or +i a
  return FWD ? cdf{a.y, dneg(a.x)} : cdf{dneg(a.y), a.x};
}

// ---- conversions --------------------------------------------------------------
// All conversions are integer bit operations: on GB300 the FP64 pipe is the
// scarce one, and the conversion instructions would run there.
//
// hi = x truncated to 24 significant bits, lo = the remaining bits (truncated
// to 24 significant bits). Values below 2^-126 in magnitude become 0; NaN and
// infinities keep their class in hi; finite values beyond the float range
// become infinities.
__device__ __forceinline__ dfl split_double(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned h = (unsigned)(b >> 32), l = (unsigned)b;
  const unsigned sign = h & 0x80000000u;
  const int e = (int)((h >> 20) & 0x7ffu);
  const int fe = e - 1023 + 127;
  if (fe <= 0) return dfl{__uint_as_float(sign), 0.f};
  if (fe >= 255) {
    const bool nan = (e == 0x7ff) && (((h & 0xfffffu) | l) != 0u);
    return dfl{__uint_as_float(sign | 0x7f800000u | (nan ? 0x400000u : 0u)), 0.f};
  }
  const float hi = __uint_as_float(sign | ((unsigned)fe << 23) | ((h & 0xfffffu) << 3) | (l >> 29));
  const unsigned r = l & 0x1fffffffu;  // remaining 29 bits, weight 2^(e - 1075)
  if (r == 0u) return dfl{hi, 0.f};
  const int lz = __clz(r);               // >= 3
  const int sh = lz - 8;                 // bring the leading bit to position 23
  const unsigned m = sh >= 0 ? (r << sh) : (r >> (-sh));
  const int le = e - 925 - sh;           // float exponent field of lo
  if (le <= 0) return dfl{hi, 0.f};
  return dfl{hi, __uint_as_float(sign | ((unsigned)le << 23) | (m & 0x7fffffu))};
}

__device__ __forceinline__ double float_to_double_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  if (e == 0u) return __longlong_as_double((long long)sign);
  const unsigned long long ex = (e == 0xffu) ? 0x7ffull : (unsigned long long)(e - 127u + 1023u);
  return __longlong_as_double((long long)(sign | (ex << 52) | ((unsigned long long)(u & 0x7fffffu) << 29)));
}

// hi + lo as a double, by integer arithmetic: lo is aligned to hi's 53-bit
// significand and added or subtracted; lo bits below it are truncated (error
// below one double ulp).
__device__ __forceinline__ double to_double(dfl a) {
  const unsigned hb = __float_as_uint(a.hi), lb = __float_as_uint(a.lo);
  const unsigned eh = (hb >> 23) & 0xffu, el = (lb >> 23) & 0xffu;
  if (eh == 0u) return float_to_double_exact(a.lo);
  if (eh == 0xffu || el == 0u) return float_to_double_exact(a.hi);
  const int d = (int)eh - (int)el;
  if (d < 0 || d >= 53) return float_to_double_exact(a.hi);  // lo below double precision (or not normalised)
  unsigned long long M = (unsigned long long)((hb & 0x7fffffu) | 0x800000u) << 29;  // 53-bit significand
  const unsigned long long Lm = ((unsigned long long)((lb & 0x7fffffu) | 0x800000u) << 29) >> d;
  int e = (int)eh;
  if ((hb ^ lb) & 0x80000000u) {
    M -= Lm;
    while (M != 0ull && M < (1ull << 52)) {
      M <<= 1;
      --e;
    }
    if (M == 0ull) return 0.0;
  } else {
    M += Lm;
    if (M >= (1ull << 53)) {
      M >>= 1;
      ++e;
    }
  }
  const unsigned long long sign = (unsigned long long)(hb & 0x80000000u) << 32;
  return __longlong_as_double((long long)(sign | ((unsigned long long)(e - 127 + 1023) << 52) | (M & ((1ull << 52) - 1))));
}

// hi + lo as a double with one FP64 operation: both floats widened exactly by
// bit operations, then a correctly rounded FP64 addition. Fewer instructions
// than to_double where the FP64 pipe has room (the RPA's outputs).
__device__ __forceinline__ double to_double_add(dfl a) {
  return __dadd_rn(float_to_double_exact(a.hi), float_to_double_exact(a.lo));
}

__device__ __forceinline__ cdf to_cdf(double2 z) { return cdf{split_double(z.x), split_double(z.y)}; }
__device__ __forceinline__ double2 to_double2(cdf z) { return make_double2(to_double(z.x), to_double(z.y)); }

}  // namespace tprf
