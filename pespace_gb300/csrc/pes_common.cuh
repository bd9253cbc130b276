// Device-side basics shared by the pespace_gb300 kernels: SI constants of
// pespace/utils/constants.py, complex arithmetic in the order taichi.math uses,
// and a forward-mode dual number for exact parameter derivatives.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define PES_HD __host__ __device__ __forceinline__

namespace pes {

// pespace/utils/constants.py:28-57
constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr double kCSI = 299792458.0;
constexpr double kMRSun = 1.476625038050124729627979840144936351e3;
constexpr double kMTSun = 4.925490947641266978197229498498379006e-6;
constexpr double kYear = 31557600.0;
constexpr double kAU = 149597870700.0;
constexpr double kPc = 3.085677581491367e16;
constexpr double kEulerGamma = 0.5772156649015329;
constexpr double kAUsec = kAU / kCSI;  // orbit.py:12

// ------------------------------------------------------------------ dual numbers
// Forward-mode dual number: a value of type V and N tangents of type D.
//   Dual<N>                FP64 value and tangents (exact derivatives);
//   DualF<N> (D = float)   FP64 value, tangent arithmetic on the FP32 pipes;
//   DualS<N> (V = float)   FP32 value and tangents, for derivative passes whose
//                          values are needed only through the chain rule.
template <int N, class D = double, class V = double>
struct Dual {
  V v;
  D d[N];
};
template <int N> using DualF = Dual<N, float>;
template <int N> using DualS = Dual<N, float, float>;

// value functions in the value's own precision
PES_HD double vsqrt(double x) { return ::sqrt(x); }
PES_HD float vsqrt(float x) { return ::sqrtf(x); }
PES_HD double vexp(double x) { return ::exp(x); }
PES_HD float vexp(float x) { return ::expf(x); }
PES_HD double vlog(double x) { return ::log(x); }
PES_HD float vlog(float x) { return ::logf(x); }
PES_HD double vcbrt(double x) { return ::cbrt(x); }
PES_HD float vcbrt(float x) { return ::cbrtf(x); }
PES_HD double vatan(double x) { return ::atan(x); }
PES_HD float vatan(float x) { return ::atanf(x); }
PES_HD double vpow(double x, double p) { return ::pow(x, p); }
PES_HD float vpow(float x, float p) { return ::powf(x, p); }
// sin and cos for |x| <= 2 from their Taylor series in x^2 (13 terms each;
// truncation below 1e-17 relative), the library routine elsewhere.  The
// response's small phases (link delays with the constellation centre
// factored out) take the series, which costs about half the library's FP64
// operations on this part.
// Series of sin x / x (coefficients (-1)^k / (2k+1)!), cos x ((-1)^k / (2k)!)
// and d/dx (sin x / x) / x ((-1)^k 2k / (2k+1)!), in z = x^2, 13 / 13 / 12 terms:
// truncation below 1e-17 relative for |x| <= 2.
PES_HD double sin_over_x_series(double z) {
  double p = 6.446950284384474e-26;
  p = p * z + -3.868170170630684e-23;
  p = p * z + 1.9572941063391263e-20;
  p = p * z + -8.22063524662433e-18;
  p = p * z + 2.8114572543455206e-15;
  p = p * z + -7.647163731819816e-13;
  p = p * z + 1.6059043836821613e-10;
  p = p * z + -2.505210838544172e-08;
  p = p * z + 2.7557319223985893e-06;
  p = p * z + -0.0001984126984126984;
  p = p * z + 0.008333333333333333;
  p = p * z + -0.16666666666666666;
  p = p * z + 1.0;
  return p;
}
PES_HD double cos_series(double z) {
  double p = 1.6117375710961184e-24;
  p = p * z + -8.896791392450574e-22;
  p = p * z + 4.110317623312165e-19;
  p = p * z + -1.5619206968586225e-16;
  p = p * z + 4.779477332387385e-14;
  p = p * z + -1.1470745597729725e-11;
  p = p * z + 2.08767569878681e-09;
  p = p * z + -2.755731922398589e-07;
  p = p * z + 2.48015873015873e-05;
  p = p * z + -0.001388888888888889;
  p = p * z + 0.041666666666666664;
  p = p * z + -0.5;
  p = p * z + 1.0;
  return p;
}
PES_HD double sinc_deriv_series(double z) {
  double p = 1.5472680682522736e-24;
  p = p * z + -8.509974375387505e-22;
  p = p * z + 3.9145882126782523e-19;
  p = p * z + -1.4797143443923793e-16;
  p = p * z + 4.498331606952833e-14;
  p = p * z + -1.0706029224547743e-11;
  p = p * z + 1.9270852604185937e-09;
  p = p * z + -2.505210838544172e-07;
  p = p * z + 2.2045855379188714e-05;
  p = p * z + -0.0011904761904761906;
  p = p * z + 0.03333333333333333;
  p = p * z + -0.3333333333333333;
  return p;
}

// sin and cos: the series above for |x| <= 2 (the response's small phases,
// link delays with the constellation centre factored out, at about half the
// library's FP64 operations on this part), the library routine elsewhere.
PES_HD void vsincos(double x, double* s, double* c) {
  if (::fabs(x) <= 2.0) {
    const double z = x * x;
    *s = sin_over_x_series(z) * x;
    *c = cos_series(z);
    return;
  }
#ifdef __CUDA_ARCH__
  ::sincos(x, s, c);
#else
  *s = ::sin(x); *c = ::cos(x);
#endif
}

// sin(x)/x and its derivative for |x| <= 2 (1 at x = 0).
PES_HD void sinc_taylor(double x, double* s, double* ds) {
  const double z = x * x;
  *s = sin_over_x_series(z);
  *ds = sinc_deriv_series(z) * x;
}
PES_HD void vsincos(float x, float* s, float* c) {
#ifdef __CUDA_ARCH__
  ::sincosf(x, s, c);
#else
  *s = ::sinf(x); *c = ::cosf(x);
#endif
}

PES_HD double val(double x) { return x; }
template <int N, class D, class V> PES_HD double val(const Dual<N, D, V>& x) { return (double)x.v; }

template <int N, class D = double, class V = double>
PES_HD Dual<N, D, V> mkdual(double x) {
  Dual<N, D, V> r;
  r.v = V(x);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = D(0);
  return r;
}

#define PES_DUAL template <int N, class D, class V> PES_HD
#define PES_DT Dual<N, D, V>
PES_DUAL PES_DT operator+(const PES_DT& a, const PES_DT& b) { PES_DT r; r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
PES_DUAL PES_DT operator-(const PES_DT& a, const PES_DT& b) { PES_DT r; r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
PES_DUAL PES_DT operator-(const PES_DT& a) { PES_DT r; r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i]; return r; }
PES_DUAL PES_DT operator*(const PES_DT& a, const PES_DT& b) { PES_DT r; r.v = a.v * b.v;
  const D av = D(a.v), bv = D(b.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * bv + av * b.d[i]; return r; }
PES_DUAL PES_DT operator/(const PES_DT& a, const PES_DT& b) { PES_DT r; r.v = a.v / b.v;
  const D ib = D(V(1) / b.v), rv = D(r.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - rv * b.d[i]) * ib; return r; }
PES_DUAL PES_DT operator+(const PES_DT& a, double b) { PES_DT r = a; r.v = a.v + V(b); return r; }
PES_DUAL PES_DT operator+(double a, const PES_DT& b) { PES_DT r = b; r.v = V(a) + b.v; return r; }
PES_DUAL PES_DT operator-(const PES_DT& a, double b) { PES_DT r = a; r.v = a.v - V(b); return r; }
PES_DUAL PES_DT operator-(double a, const PES_DT& b) { PES_DT r = -b; r.v = V(a) - b.v; return r; }
PES_DUAL PES_DT operator*(const PES_DT& a, double b) { PES_DT r; r.v = a.v * V(b); const D bb = D(b);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * bb; return r; }
PES_DUAL PES_DT operator*(double a, const PES_DT& b) { PES_DT r; r.v = V(a) * b.v; const D aa = D(a);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = aa * b.d[i]; return r; }
PES_DUAL PES_DT operator/(const PES_DT& a, double b) { PES_DT r; const V bv = V(b); r.v = a.v / bv;
  const D ib = D(V(1) / bv);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * ib; return r; }
PES_DUAL PES_DT operator/(double a, const PES_DT& b) { return mkdual<N, D, V>(a) / b; }
PES_DUAL bool operator<(const PES_DT& a, double b) { return a.v < V(b); }
PES_DUAL bool operator<=(const PES_DT& a, double b) { return a.v <= V(b); }
PES_DUAL bool operator>(const PES_DT& a, double b) { return a.v > V(b); }
PES_DUAL bool operator>=(const PES_DT& a, double b) { return a.v >= V(b); }
PES_DUAL bool operator<(const PES_DT& a, const PES_DT& b) { return a.v < b.v; }
PES_DUAL bool operator>=(const PES_DT& a, const PES_DT& b) { return a.v >= b.v; }

PES_DUAL PES_DT chain1(const PES_DT& a, V fv, V dfv) { PES_DT r; r.v = fv; const D df = D(dfv);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * df; return r; }

// double overloads (device: CUDA libdevice; host: libm)
PES_HD double dsin(double x) { return ::sin(x); }
PES_HD double dcos(double x) { return ::cos(x); }
PES_HD void dsincos(double x, double* s, double* c) { vsincos(x, s, c); }
PES_HD double dexp(double x) { return ::exp(x); }
PES_HD double dlog(double x) { return ::log(x); }
PES_HD double dsqrt(double x) { return ::sqrt(x); }
PES_HD double dcbrt(double x) { return ::cbrt(x); }
PES_HD double datan(double x) { return ::atan(x); }
PES_HD double dpow(double x, double p) { return ::pow(x, p); }
PES_HD double dabs(double x) { return ::fabs(x); }

PES_DUAL PES_DT dsin(const PES_DT& a) { V s, c; vsincos(a.v, &s, &c); return chain1(a, s, c); }
PES_DUAL PES_DT dcos(const PES_DT& a) { V s, c; vsincos(a.v, &s, &c); return chain1(a, c, -s); }
PES_DUAL void dsincos(const PES_DT& a, PES_DT* s, PES_DT* c) {
  V sv, cv; vsincos(a.v, &sv, &cv); *s = chain1(a, sv, cv); *c = chain1(a, cv, -sv); }
PES_DUAL PES_DT dexp(const PES_DT& a) { const V e = vexp(a.v); return chain1(a, e, e); }
PES_DUAL PES_DT dlog(const PES_DT& a) { return chain1(a, vlog(a.v), V(1) / a.v); }
PES_DUAL PES_DT dsqrt(const PES_DT& a) { const V s = vsqrt(a.v); return chain1(a, s, V(0.5) / s); }
PES_DUAL PES_DT dcbrt(const PES_DT& a) { const V c = vcbrt(a.v); return chain1(a, c, V(1) / (V(3) * c * c)); }
PES_DUAL PES_DT datan(const PES_DT& a) { return chain1(a, vatan(a.v), V(1) / (V(1) + a.v * a.v)); }
PES_DUAL PES_DT dpow(const PES_DT& a, double p) { const V pv = V(p), q = vpow(a.v, pv); return chain1(a, q, pv * q / a.v); }
PES_DUAL PES_DT dabs(const PES_DT& a) { return a.v < V(0) ? -a : a; }
#undef PES_DT
#undef PES_DUAL

template <class T> struct Lift { PES_HD static T from(double x); };
template <> struct Lift<double> { PES_HD static double from(double x) { return x; } };
template <> struct Lift<float> { PES_HD static float from(double x) { return (float)x; } };
template <int N, class D, class V> struct Lift<Dual<N, D, V>> {
  PES_HD static Dual<N, D, V> from(double x) { return mkdual<N, D, V>(x); }
};
template <class T> PES_HD T lift(double x) { return Lift<T>::from(x); }

// ------------------------------------------------------------------ complex
template <class T>
struct Cx {
  T re, im;
};
template <class T> PES_HD Cx<T> cx(const T& a, const T& b) { Cx<T> r; r.re = a; r.im = b; return r; }
template <class T> PES_HD Cx<T> operator+(const Cx<T>& a, const Cx<T>& b) { return cx(a.re + b.re, a.im + b.im); }
template <class T> PES_HD Cx<T> operator-(const Cx<T>& a, const Cx<T>& b) { return cx(a.re - b.re, a.im - b.im); }
// taichi.math.cmul ordering: (x0 y0 - x1 y1, x0 y1 + x1 y0)
template <class T> PES_HD Cx<T> cmul(const Cx<T>& a, const Cx<T>& b) {
  return cx(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <class T, class S> PES_HD Cx<T> cscale(const S& s, const Cx<T>& a) { return cx(s * a.re, s * a.im); }

// ------------------------------------------------------------------ status
enum : int32_t {
  kSampleOk = 0,
  kSampleNonFinite = 1,   // NaN/Inf in the inputs or the result
  kSampleOutOfDomain = 2, // q < 1, |chi| >= 1, |cos i| > 1, |sin b| > 1
};

}  // namespace pes
