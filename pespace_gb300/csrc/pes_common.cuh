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
// Forward-mode dual number: FP64 value and N tangents of type D (double for
// exact derivatives; float to run the tangent arithmetic on the FP32 pipes
// while the value stays FP64).
template <int N, class D = double>
struct Dual {
  double v;
  D d[N];
};
template <int N> using DualF = Dual<N, float>;

PES_HD double val(double x) { return x; }
template <int N, class D> PES_HD double val(const Dual<N, D>& x) { return x.v; }

template <int N, class D = double>
PES_HD Dual<N, D> mkdual(double x) {
  Dual<N, D> r;
  r.v = x;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = D(0);
  return r;
}

#define PES_DUAL template <int N, class D> PES_HD
PES_DUAL Dual<N, D> operator+(const Dual<N, D>& a, const Dual<N, D>& b) { Dual<N, D> r; r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
PES_DUAL Dual<N, D> operator-(const Dual<N, D>& a, const Dual<N, D>& b) { Dual<N, D> r; r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
PES_DUAL Dual<N, D> operator-(const Dual<N, D>& a) { Dual<N, D> r; r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i]; return r; }
PES_DUAL Dual<N, D> operator*(const Dual<N, D>& a, const Dual<N, D>& b) { Dual<N, D> r; r.v = a.v * b.v;
  const D av = D(a.v), bv = D(b.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * bv + av * b.d[i]; return r; }
PES_DUAL Dual<N, D> operator/(const Dual<N, D>& a, const Dual<N, D>& b) { Dual<N, D> r; r.v = a.v / b.v;
  const D ib = D(1.0 / b.v), rv = D(r.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - rv * b.d[i]) * ib; return r; }
PES_DUAL Dual<N, D> operator+(const Dual<N, D>& a, double b) { Dual<N, D> r = a; r.v = a.v + b; return r; }
PES_DUAL Dual<N, D> operator+(double a, const Dual<N, D>& b) { Dual<N, D> r = b; r.v = a + b.v; return r; }
PES_DUAL Dual<N, D> operator-(const Dual<N, D>& a, double b) { Dual<N, D> r = a; r.v = a.v - b; return r; }
PES_DUAL Dual<N, D> operator-(double a, const Dual<N, D>& b) { Dual<N, D> r = -b; r.v = a - b.v; return r; }
PES_DUAL Dual<N, D> operator*(const Dual<N, D>& a, double b) { Dual<N, D> r; r.v = a.v * b; const D bb = D(b);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * bb; return r; }
PES_DUAL Dual<N, D> operator*(double a, const Dual<N, D>& b) { Dual<N, D> r; r.v = a * b.v; const D aa = D(a);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = aa * b.d[i]; return r; }
PES_DUAL Dual<N, D> operator/(const Dual<N, D>& a, double b) { Dual<N, D> r; r.v = a.v / b; const D ib = D(1.0 / b);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * ib; return r; }
PES_DUAL Dual<N, D> operator/(double a, const Dual<N, D>& b) { return mkdual<N, D>(a) / b; }
PES_DUAL bool operator<(const Dual<N, D>& a, double b) { return a.v < b; }
PES_DUAL bool operator<=(const Dual<N, D>& a, double b) { return a.v <= b; }
PES_DUAL bool operator>(const Dual<N, D>& a, double b) { return a.v > b; }
PES_DUAL bool operator>=(const Dual<N, D>& a, double b) { return a.v >= b; }
PES_DUAL bool operator<(const Dual<N, D>& a, const Dual<N, D>& b) { return a.v < b.v; }
PES_DUAL bool operator>=(const Dual<N, D>& a, const Dual<N, D>& b) { return a.v >= b.v; }

PES_DUAL Dual<N, D> chain1(const Dual<N, D>& a, double fv, double dfv) { Dual<N, D> r; r.v = fv; const D df = D(dfv);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * df; return r; }

// double overloads (device: CUDA libdevice; host: libm)
PES_HD double dsin(double x) { return ::sin(x); }
PES_HD double dcos(double x) { return ::cos(x); }
PES_HD void dsincos(double x, double* s, double* c) {
#ifdef __CUDA_ARCH__
  ::sincos(x, s, c);
#else
  *s = ::sin(x); *c = ::cos(x);
#endif
}
PES_HD double dexp(double x) { return ::exp(x); }
PES_HD double dlog(double x) { return ::log(x); }
PES_HD double dsqrt(double x) { return ::sqrt(x); }
PES_HD double dcbrt(double x) { return ::cbrt(x); }
PES_HD double datan(double x) { return ::atan(x); }
PES_HD double dpow(double x, double p) { return ::pow(x, p); }
PES_HD double dabs(double x) { return ::fabs(x); }

PES_DUAL Dual<N, D> dsin(const Dual<N, D>& a) { double s, c; dsincos(a.v, &s, &c); return chain1(a, s, c); }
PES_DUAL Dual<N, D> dcos(const Dual<N, D>& a) { double s, c; dsincos(a.v, &s, &c); return chain1(a, c, -s); }
PES_DUAL void dsincos(const Dual<N, D>& a, Dual<N, D>* s, Dual<N, D>* c) {
  double sv, cv; dsincos(a.v, &sv, &cv); *s = chain1(a, sv, cv); *c = chain1(a, cv, -sv); }
PES_DUAL Dual<N, D> dexp(const Dual<N, D>& a) { double e = ::exp(a.v); return chain1(a, e, e); }
PES_DUAL Dual<N, D> dlog(const Dual<N, D>& a) { return chain1(a, ::log(a.v), 1.0 / a.v); }
PES_DUAL Dual<N, D> dsqrt(const Dual<N, D>& a) { double s = ::sqrt(a.v); return chain1(a, s, 0.5 / s); }
PES_DUAL Dual<N, D> dcbrt(const Dual<N, D>& a) { double c = ::cbrt(a.v); return chain1(a, c, 1.0 / (3.0 * c * c)); }
PES_DUAL Dual<N, D> datan(const Dual<N, D>& a) { return chain1(a, ::atan(a.v), 1.0 / (1.0 + a.v * a.v)); }
PES_DUAL Dual<N, D> dpow(const Dual<N, D>& a, double p) { double q = ::pow(a.v, p); return chain1(a, q, p * q / a.v); }
PES_DUAL Dual<N, D> dabs(const Dual<N, D>& a) { return a.v < 0.0 ? -a : a; }
#undef PES_DUAL

template <class T> struct Lift { PES_HD static T from(double x); };
template <> struct Lift<double> { PES_HD static double from(double x) { return x; } };
template <int N, class D> struct Lift<Dual<N, D>> { PES_HD static Dual<N, D> from(double x) { return mkdual<N, D>(x); } };
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
