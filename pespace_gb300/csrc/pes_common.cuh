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
template <int N>
struct Dual {
  double v;
  double d[N];
};

PES_HD double val(double x) { return x; }
template <int N> PES_HD double val(const Dual<N>& x) { return x.v; }

template <int N>
PES_HD Dual<N> mkdual(double x) {
  Dual<N> r;
  r.v = x;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = 0.0;
  return r;
}

template <int N> PES_HD Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) { Dual<N> r; r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
template <int N> PES_HD Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) { Dual<N> r; r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
template <int N> PES_HD Dual<N> operator-(const Dual<N>& a) { Dual<N> r; r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i]; return r; }
template <int N> PES_HD Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) { Dual<N> r; r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
template <int N> PES_HD Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) { Dual<N> r; r.v = a.v / b.v; const double ib = 1.0 / b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib; return r; }
template <int N> PES_HD Dual<N> operator+(const Dual<N>& a, double b) { Dual<N> r = a; r.v = a.v + b; return r; }
template <int N> PES_HD Dual<N> operator+(double a, const Dual<N>& b) { Dual<N> r = b; r.v = a + b.v; return r; }
template <int N> PES_HD Dual<N> operator-(const Dual<N>& a, double b) { Dual<N> r = a; r.v = a.v - b; return r; }
template <int N> PES_HD Dual<N> operator-(double a, const Dual<N>& b) { Dual<N> r = -b; r.v = a - b.v; return r; }
template <int N> PES_HD Dual<N> operator*(const Dual<N>& a, double b) { Dual<N> r; r.v = a.v * b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b; return r; }
template <int N> PES_HD Dual<N> operator*(double a, const Dual<N>& b) { Dual<N> r; r.v = a * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a * b.d[i]; return r; }
template <int N> PES_HD Dual<N> operator/(const Dual<N>& a, double b) { Dual<N> r; r.v = a.v / b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / b; return r; }
template <int N> PES_HD Dual<N> operator/(double a, const Dual<N>& b) { return mkdual<N>(a) / b; }
template <int N> PES_HD bool operator<(const Dual<N>& a, double b) { return a.v < b; }
template <int N> PES_HD bool operator<=(const Dual<N>& a, double b) { return a.v <= b; }
template <int N> PES_HD bool operator>(const Dual<N>& a, double b) { return a.v > b; }
template <int N> PES_HD bool operator>=(const Dual<N>& a, double b) { return a.v >= b; }
template <int N> PES_HD bool operator<(const Dual<N>& a, const Dual<N>& b) { return a.v < b.v; }
template <int N> PES_HD bool operator>=(const Dual<N>& a, const Dual<N>& b) { return a.v >= b.v; }

template <int N> PES_HD Dual<N> chain1(const Dual<N>& a, double fv, double dfv) { Dual<N> r; r.v = fv;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * dfv; return r; }

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

template <int N> PES_HD Dual<N> dsin(const Dual<N>& a) { double s, c; dsincos(a.v, &s, &c); return chain1(a, s, c); }
template <int N> PES_HD Dual<N> dcos(const Dual<N>& a) { double s, c; dsincos(a.v, &s, &c); return chain1(a, c, -s); }
template <int N> PES_HD void dsincos(const Dual<N>& a, Dual<N>* s, Dual<N>* c) {
  double sv, cv; dsincos(a.v, &sv, &cv); *s = chain1(a, sv, cv); *c = chain1(a, cv, -sv); }
template <int N> PES_HD Dual<N> dexp(const Dual<N>& a) { double e = ::exp(a.v); return chain1(a, e, e); }
template <int N> PES_HD Dual<N> dlog(const Dual<N>& a) { return chain1(a, ::log(a.v), 1.0 / a.v); }
template <int N> PES_HD Dual<N> dsqrt(const Dual<N>& a) { double s = ::sqrt(a.v); return chain1(a, s, 0.5 / s); }
template <int N> PES_HD Dual<N> dcbrt(const Dual<N>& a) { double c = ::cbrt(a.v); return chain1(a, c, 1.0 / (3.0 * c * c)); }
template <int N> PES_HD Dual<N> datan(const Dual<N>& a) { return chain1(a, ::atan(a.v), 1.0 / (1.0 + a.v * a.v)); }
template <int N> PES_HD Dual<N> dpow(const Dual<N>& a, double p) { double q = ::pow(a.v, p); return chain1(a, q, p * q / a.v); }
template <int N> PES_HD Dual<N> dabs(const Dual<N>& a) { return a.v < 0.0 ? -a : a; }

template <class T> struct Lift { PES_HD static T from(double x); };
template <> struct Lift<double> { PES_HD static double from(double x) { return x; } };
template <int N> struct Lift<Dual<N>> { PES_HD static Dual<N> from(double x) { return mkdual<N>(x); } };
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
