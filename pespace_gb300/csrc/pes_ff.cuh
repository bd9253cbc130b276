// Float-float ("double-word") scalar for the sparse node evaluations.
//
// GB300 issues FP64 at 1/64 of its FP32 rate, and the FP64 pipe (which also
// executes FP32<->FP64 conversions) binds the node evaluations of the mixed
// plan.  An FF value is an unevaluated sum hi + lo of two floats with
// |lo| <= ulp(hi)/2, about 48 significant bits: enough for node values that
// feed splines whose own interpolation error is near 1e-9 relative.  Every
// operation runs on the FP32 pipes.
//
// Building blocks (Dekker 1971; Knuth TAOCP vol. 2, 4.2.2; bounds in Joldes,
// Muller and Popescu, "Tight and rigorous error bounds for basic building
// blocks of double-word arithmetic", ACM TOMS 44(2), 2017):
//   two_sum      s + e = a + b exactly (6 flops)
//   fast_two_sum s + e = a + b exactly when |a| >= |b| (3 flops)
//   two_prod     p + e = a * b exactly (1 mul + 1 FMA)
// Addition is the "sloppy" double-word sum (error below 2^-46 (|x| + |y|),
// the same behaviour as FP64 inputs carrying their own rounding); products
// and quotients are accurate to a few 2^-48 relative.
//
// Functions: sqrt and cbrt by one Newton step from the FP32 result; log by
// the atanh series of (m - 1)/(m + 1) after extracting the binary exponent;
// sin and cos by reduction modulo pi/2 (pi/2 split in three floats) and
// Taylor polynomials on |r| <= pi/4 whose leading terms are in FF and whose
// tail is in FP32; sin(x)/x by its Taylor series for |x| <= 2; exp by
// reduction modulo ln 2 and atan by reduction to |x| <= tan(pi/16), each
// with a Taylor polynomial (the FP64 forms had each IMRPhenomHM mode's
// node above its amplitude corner on the FP64 pipe).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include "pes_common.cuh"

namespace pes {

// Out-of-line device functions for the float-float routines that a node
// evaluation calls many times (sin(x)/x six times, sincos four): one copy of
// their code instead of one per call site keeps the fully inlined node
// evaluation within the instruction cache (its top stall was instruction
// fetch; sparse stage 0.45 -> 0.36 ms per step).
#define PES_HD_OUTLINE static __host__ __device__ __noinline__

// Trivially default-constructible (usable in shared memory); the explicit
// conversions let it serve as the value type of the dual numbers (their
// tangents take the head, FP64 constants are split once).
struct FF {
  float hi, lo;
  FF() = default;
  PES_HD explicit FF(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
  PES_HD explicit operator float() const { return hi; }
  PES_HD explicit operator double() const { return (double)hi + (double)lo; }
};

PES_HD FF ff_make(float hi, float lo) { FF r; r.hi = hi; r.lo = lo; return r; }
PES_HD FF ff_from(double x) { return FF(x); }
PES_HD double ff_to(const FF& a) { return (double)a.hi + (double)a.lo; }

PES_HD FF ff_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return ff_make(s, (a - (s - bb)) + (b - bb));
}
PES_HD FF ff_fast_two_sum(float a, float b) {
  const float s = a + b;
  return ff_make(s, b - (s - a));
}
PES_HD FF ff_two_prod(float a, float b) {
  const float p = a * b;
  return ff_make(p, fmaf(a, b, -p));
}

// reciprocal to about 1 ulp: the fast estimate and one Newton step
PES_HD float ff_rcp(float y) {
#ifdef __CUDA_ARCH__
  const float r = __fdividef(1.0f, y);
#else
  const float r = 1.0f / y;
#endif
  return fmaf(r, fmaf(-y, r, 1.0f), r);
}

PES_HD FF operator-(const FF& x) { return ff_make(-x.hi, -x.lo); }
PES_HD FF operator+(const FF& x, const FF& y) {
  FF s = ff_two_sum(x.hi, y.hi);
  s.lo += x.lo + y.lo;
  return ff_fast_two_sum(s.hi, s.lo);
}
PES_HD FF operator-(const FF& x, const FF& y) { return x + (-y); }
PES_HD FF operator*(const FF& x, const FF& y) {
  FF p = ff_two_prod(x.hi, y.hi);
  p.lo = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, p.lo));
  return ff_fast_two_sum(p.hi, p.lo);
}
PES_HD FF ff_mulf(const FF& x, float y) {
  FF p = ff_two_prod(x.hi, y);
  p.lo = fmaf(x.lo, y, p.lo);
  return ff_fast_two_sum(p.hi, p.lo);
}
PES_HD FF ff_addf(const FF& x, float y) {
  FF s = ff_two_sum(x.hi, y);
  s.lo += x.lo;
  return ff_fast_two_sum(s.hi, s.lo);
}
PES_HD FF operator/(const FF& x, const FF& y) {
  const float r = ff_rcp(y.hi);
  const float q1 = x.hi * r;
  const FF p = ff_two_prod(q1, y.hi);  // p.hi is within a few ulps of x.hi: x.hi - p.hi is exact
  const float rem = (((x.hi - p.hi) - p.lo) + x.lo) - q1 * y.lo;
  return ff_fast_two_sum(q1, rem * r);
}

// mixed forms with FP64 constants (folded at compile time for literals)
PES_HD FF operator+(const FF& x, double y) { return x + ff_from(y); }
PES_HD FF operator+(double x, const FF& y) { return ff_from(x) + y; }
PES_HD FF operator-(const FF& x, double y) { return x - ff_from(y); }
PES_HD FF operator-(double x, const FF& y) { return ff_from(x) - y; }
PES_HD FF operator*(const FF& x, double y) { return x * ff_from(y); }
PES_HD FF operator*(double x, const FF& y) { return ff_from(x) * y; }
PES_HD FF operator/(const FF& x, double y) { return x / ff_from(y); }
PES_HD FF operator/(double x, const FF& y) { return ff_from(x) / y; }

PES_HD bool operator<(const FF& a, const FF& b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
PES_HD bool operator>(const FF& a, const FF& b) { return b < a; }
PES_HD bool operator<=(const FF& a, const FF& b) { return !(b < a); }
PES_HD bool operator>=(const FF& a, const FF& b) { return !(a < b); }
PES_HD bool operator<(const FF& a, double b) { return a < ff_from(b); }
PES_HD bool operator>(const FF& a, double b) { return ff_from(b) < a; }
PES_HD bool operator<=(const FF& a, double b) { return !(ff_from(b) < a); }
PES_HD bool operator>=(const FF& a, double b) { return !(a < ff_from(b)); }

PES_HD double val(const FF& x) { return ff_to(x); }
template <> struct Lift<FF> { PES_HD static FF from(double x) { return ff_from(x); } };

PES_HD FF dabs(const FF& x) { return x.hi < 0.0f ? -x : x; }

PES_HD FF dsqrt(const FF& x) {
  if (!(x.hi > 0.0f)) return ff_make(sqrtf(x.hi), 0.0f);
  const float s = sqrtf(x.hi);
  const FF p = ff_two_prod(s, s);
  const float rem = ((x.hi - p.hi) - p.lo) + x.lo;
  return ff_fast_two_sum(s, rem * (0.5f * ff_rcp(s)));
}

// cube root of x > 0: c = cbrtf(hi), then c + (x - c^3) / (3 c^2)
PES_HD FF dcbrt(const FF& x) {
  if (!(x.hi > 0.0f)) return ff_make(cbrtf(x.hi), 0.0f);
  const float c = cbrtf(x.hi);
  const FF c3 = ff_mulf(ff_two_prod(c, c), c);
  const float rem = ((x.hi - c3.hi) - c3.lo) + x.lo;
  return ff_fast_two_sum(c, rem * ff_rcp(3.0f * c * c));
}

// natural log of x > 0: x = 2^k m with m in [sqrt(1/2), sqrt(2)),
// ln m = 2 atanh(s) = 2 s (1 + z/3 + z^2/5 + ...), s = (m - 1)/(m + 1),
// z = s^2 <= 0.0295 (FF for the terms down to z^3/7, FP32 below 1e-7 of the sum).
PES_HD FF dlog(const FF& x) {
  if (!(x.hi > 0.0f)) return ff_make(logf(x.hi), 0.0f);
  int k;
  float mh = frexpf(x.hi, &k);  // x.hi = mh 2^k, mh in [0.5, 1)
  if (mh < 0.70710678f) {
    mh *= 2.0f;
    k -= 1;
  }
  const FF m = ff_make(mh, ldexpf(x.lo, -k));  // exact scaling by a power of two
  const FF s = ff_addf(m, -1.0f) / ff_addf(m, 1.0f);
  const FF z = s * s;
  const float zf = z.hi;
  float t = 1.0f / 21.0f;
  t = fmaf(t, zf, 1.0f / 19.0f);
  t = fmaf(t, zf, 1.0f / 17.0f);
  t = fmaf(t, zf, 1.0f / 15.0f);
  t = fmaf(t, zf, 1.0f / 13.0f);
  t = fmaf(t, zf, 1.0f / 11.0f);
  t = fmaf(t, zf, 1.0f / 9.0f);
  FF q = ff_mulf(z, t) + ff_from(1.0 / 7.0);
  q = q * z + ff_from(1.0 / 5.0);
  q = q * z + ff_from(1.0 / 3.0);
  q = q * z;
  const FF lnm = ff_mulf(s + s * q, 2.0f);
  return ff_mulf(ff_from(0.69314718055994530942), (float)k) + lnm;
}

// exp(x) = 2^k exp(r), x = k ln 2 + r with ln 2 in three parts (k * A exact
// for |k| < 2^12) and |r| <= ln 2 / 2; exp(r) = exp(r/4)^4, exp(r/4) from its
// Taylor series (FF Horner down to the r^4 term, the terms from r^5/5! in
// FP32: below 4e-8 relative, truncation after r^9/9! below 1e-17).  Results
// below the FP32 normal range lose precision (lo underflows first), as any
// FF value does there.
constexpr float kLn2A = 0.693115234375f;  // 2839 / 4096
constexpr float kLn2B = 3.194618329871446e-05f;
constexpr float kLn2C = 1.6465949697480609e-12f;
PES_HD_OUTLINE FF dexp(const FF& x) {
  if (!(x.hi < 88.0f)) return ff_make(x.hi != x.hi ? x.hi : INFINITY, 0.0f);
  if (x.hi < -104.0f) return ff_make(0.0f, 0.0f);
  const float kf = rintf(x.hi * 1.4426950408889634f);
  FF r = ff_addf(x, -kf * kLn2A);  // exact product, FF sum
  r = r - ff_two_prod(kf, kLn2B);
  r = ff_addf(r, -kf * kLn2C);
  const FF q = ff_mulf(r, 0.25f);  // exact
  const float qf = q.hi;
  float t = fmaf(qf, 1.0f / 362880.0f, 1.0f / 40320.0f);
  t = fmaf(t, qf, 1.0f / 5040.0f);
  t = fmaf(t, qf, 1.0f / 720.0f);
  t = fmaf(t, qf, 1.0f / 120.0f);
  FF p = ff_addf(ff_from(1.0 / 24.0), t * qf);
  p = p * q + ff_from(1.0 / 6.0);
  p = p * q + ff_from(0.5);
  p = ff_addf(p * q, 1.0f);
  p = ff_addf(p * q, 1.0f);
  p = p * p;
  p = p * p;
  const int k = (int)kf;
  return ff_make(ldexpf(p.hi, k), ldexpf(p.lo, k));
}

// atan(x): odd; for |x| > 1, pi/2 - atan(1/|x|); two halvings
// atan(a) = 2 atan(a / (1 + sqrt(1 + a^2))) bring |a| below tan(pi/16) =
// 0.199, where atan(a) / a = sum (-1)^n a^2n / (2n + 1) (FF Horner down to
// the a^6 term, the terms from a^8/9 in FP32: below 3e-7 relative,
// truncation after a^18/19 below 5e-16).
PES_HD_OUTLINE FF datan(const FF& x) {
  if (x.hi != x.hi) return x;
  const bool neg = x.hi < 0.0f;
  FF a = neg ? -x : x;
  const bool inv = a.hi > 1.0f;
  if (inv) a = ff_make(1.0f, 0.0f) / a;
#pragma unroll
  for (int h = 0; h < 2; ++h) a = a / ff_addf(dsqrt(ff_addf(a * a, 1.0f)), 1.0f);
  const FF z = a * a;
  const float zf = z.hi;
  float t = fmaf(-zf, 1.0f / 19.0f, 1.0f / 17.0f);
  t = fmaf(-zf, t, 1.0f / 15.0f);
  t = fmaf(-zf, t, 1.0f / 13.0f);
  t = fmaf(-zf, t, 1.0f / 11.0f);
  t = fmaf(-zf, t, 1.0f / 9.0f);
  FF p = ff_addf(ff_from(-1.0 / 7.0), t * zf);
  p = p * z + ff_from(1.0 / 5.0);
  p = p * z + ff_from(-1.0 / 3.0);
  p = ff_addf(p * z, 1.0f);
  FF s = ff_mulf(a * p, 4.0f);  // exact scaling
  if (inv) s = ff_from(1.5707963267948966) - s;
  return neg ? -s : s;
}

// sin and cos of r, |r| <= pi/4 (FF Horner for the terms down to r^9/9! and
// r^8/8!, FP32 for the rest: truncation and tail rounding below 1e-15).
PES_HD void ff_sincos_reduced(const FF& r, FF* s, FF* c) {
  const FF z = r * r;
  const float zf = z.hi;
  float ts = -1.0f / 1307674368000.0f;         // -1/15!
  ts = fmaf(ts, zf, 1.0f / 6227020800.0f);     //  1/13!
  ts = fmaf(ts, zf, -1.0f / 39916800.0f);      // -1/11!
  FF ps = ff_mulf(z, ts) + ff_from(1.0 / 362880.0);
  ps = ps * z + ff_from(-1.0 / 5040.0);
  ps = ps * z + ff_from(1.0 / 120.0);
  ps = ps * z + ff_from(-1.0 / 6.0);
  *s = r + (ps * z) * r;
  float tc = 1.0f / 20922789888000.0f;         //  1/16!
  tc = fmaf(tc, zf, -1.0f / 87178291200.0f);   // -1/14!
  tc = fmaf(tc, zf, 1.0f / 479001600.0f);      //  1/12!
  tc = fmaf(tc, zf, -1.0f / 3628800.0f);       // -1/10!
  FF pc = ff_mulf(z, tc) + ff_from(1.0 / 40320.0);
  pc = pc * z + ff_from(-1.0 / 720.0);
  pc = pc * z + ff_from(1.0 / 24.0);
  pc = pc * z + ff_from(-0.5);
  *c = ff_addf(pc * z, 1.0f);
}

// pi/2 = kHalfPiA + kHalfPiB + kHalfPiC (A has 8 significant bits: k * A exact for |k| < 2^16)
constexpr float kHalfPiA = 1.5703125f;
constexpr float kHalfPiB = 4.838267923332751e-4f;
constexpr float kHalfPiC = 2.5633440682570896e-12f;

// sin and cos of |x| < 2^15 (reduction error below 2^-48 |k| pi/2)
PES_HD_OUTLINE void dsincos(const FF& x, FF* s, FF* c) {
  const float kf = rintf(x.hi * 0.63661977236758134f);
  FF r = ff_addf(x, -kf * kHalfPiA);            // exact product, FF sum
  r = r - ff_two_prod(kf, kHalfPiB);
  r = ff_addf(r, -kf * kHalfPiC);
  FF sr, cr;
  ff_sincos_reduced(r, &sr, &cr);
  const int k = (int)kf;
  FF sv = (k & 1) ? cr : sr;
  FF cv = (k & 1) ? sr : cr;
  if (k & 2) sv = -sv;
  if ((k + 1) & 2) cv = -cv;
  *s = sv;
  *c = cv;
}

// 2 pi = kTwoPiA + kTwoPiB + kTwoPiC (A has 8 significant bits: k * A exact for |k| < 2^16)
constexpr float kTwoPiA = 6.28125f;
constexpr float kTwoPiB = 1.9353071693331003e-3f;
constexpr float kTwoPiC = 1.0253376273028358e-11f;

// x - 2 pi rint(x / 2 pi) for |x| < 2^18 (x.hi - k A is exact: k A is within
// a factor two of x.hi for k != 0)
PES_HD FF ff_wrap_2pi(const FF& x) {
  const float kf = rintf(x.hi * 0.15915494309189535f);
  FF r = ff_addf(x, -kf * kTwoPiA);
  r = r - ff_two_prod(kf, kTwoPiB);
  return ff_addf(r, -kf * kTwoPiC);
}

// 2 pi = kTwoPiWA + kTwoPiWB + kTwoPiWC + kTwoPiWD (A has 5 significant bits:
// k * A exact for |k| < 2^19)
constexpr float kTwoPiWA = 6.25f;
constexpr float kTwoPiWB = 3.318530693650246e-2f;
constexpr float kTwoPiWC = 2.430840251310684e-10f;
constexpr float kTwoPiWD = -4.870820776974614e-18f;
constexpr float kWrapWideMax = 3.2e6f;  // |x| below 2^19 * 2 pi with margin

// x - 2 pi rint(x / 2 pi) for |x| < kWrapWideMax (x.hi - k A is exact: k A is
// within a factor two of x.hi for k != 0); error below 1e-9 rad
PES_HD FF ff_wrap_2pi_wide(const FF& x) {
  const float kf = rintf(x.hi * 0.15915494309189535f);
  FF r = ff_addf(x, -kf * kTwoPiWA);
  r = r - ff_two_prod(kf, kTwoPiWB);
  r = r - ff_two_prod(kf, kTwoPiWC);
  return ff_addf(r, -kf * kTwoPiWD);
}

// x.hi truncated to its leading `bits` significant bits (so that the head
// times a small integer is exact in FP32), and the FF remainder as a float.
PES_HD float ff_head(const FF& x, int bits, float* tail) {
  const unsigned m = ~((1u << (24 - bits)) - 1u);
#ifdef __CUDA_ARCH__
  const float h = __uint_as_float(__float_as_uint(x.hi) & m);
#else
  unsigned u;
  memcpy(&u, &x.hi, 4);
  u &= m;
  float h;
  memcpy(&h, &u, 4);
#endif
  *tail = (x.hi - h) + x.lo;
  return h;
}

// sin(x)/x: Taylor series in z = x^2 for |x| <= 2 (FF for the terms down to
// z^6/13!, FP32 for those below 2e-8; truncation below 2e-16), else sin(x)/x.
PES_HD_OUTLINE FF ff_sinc(const FF& x) {
  if (fabsf(x.hi) <= 2.0f) {
    const FF z = x * x;
    const float zf = z.hi;
    float t = -1.0f / 51090942171709440000.0f;   // -1/21!
    t = fmaf(t, zf, 1.0f / 121645100408832000.0f); //  1/19!
    t = fmaf(t, zf, -1.0f / 355687428096000.0f);   // -1/17!
    t = fmaf(t, zf, 1.0f / 1307674368000.0f);      //  1/15!
    FF p = ff_mulf(z, -t) + ff_from(1.0 / 6227020800.0);
    p = p * z + ff_from(-1.0 / 39916800.0);
    p = p * z + ff_from(1.0 / 362880.0);
    p = p * z + ff_from(-1.0 / 5040.0);
    p = p * z + ff_from(1.0 / 120.0);
    p = p * z + ff_from(-1.0 / 6.0);
    return ff_addf(p * z, 1.0f);
  }
  FF s, c;
  dsincos(x, &s, &c);
  return s / x;
}

// value functions of the dual numbers with FF values
PES_HD FF vsqrt(const FF& x) { return dsqrt(x); }
PES_HD FF vcbrt(const FF& x) { return dcbrt(x); }
PES_HD FF vlog(const FF& x) { return dlog(x); }
PES_HD FF vexp(const FF& x) { return dexp(x); }
PES_HD FF vatan(const FF& x) { return datan(x); }
PES_HD void vsincos(const FF& x, FF* s, FF* c) { dsincos(x, s, c); }

}  // namespace pes
