// Host check of the float-float arithmetic (pespace_gb300/csrc/pes_ff.cuh)
// against long double: prints the largest errors of each operation and
// function over seeded inputs, one "name value" pair per line.
#include <cmath>
#include <cstdio>
#include <random>

#include "../../pespace_gb300/csrc/pes_ff.cuh"

using namespace pes;

static long double ld(const FF& x) { return (long double)x.hi + (long double)x.lo; }

int main() {
  std::mt19937_64 rng(2026);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  double e_add = 0, e_mul = 0, e_div = 0, e_sqrt = 0, e_cbrt = 0, e_log = 0, e_sin = 0, e_cos = 0, e_sinc = 0,
         e_wrap = 0, e_wrapw = 0, e_exp = 0, e_atan = 0;
  const long double two_pi = 6.283185307179586476925286766559L;
  for (int it = 0; it < 400000; ++it) {
    const double a = std::pow(10.0, -6.0 + 12.0 * U(rng)), b = std::pow(10.0, -6.0 + 12.0 * U(rng));
    const FF fa = ff_from(a), fb = ff_from(U(rng) < 0.5 ? -b : b);
    const long double A = ld(fa), B = ld(fb);
    e_add = std::fmax(e_add, (double)(fabsl(ld(fa + fb) - (A + B)) / (fabsl(A) + fabsl(B))));
    e_mul = std::fmax(e_mul, (double)(fabsl(ld(fa * fb) - A * B) / fabsl(A * B)));
    e_div = std::fmax(e_div, (double)(fabsl(ld(fa / fb) - A / B) / fabsl(A / B)));
    e_sqrt = std::fmax(e_sqrt, (double)(fabsl(ld(dsqrt(fa)) - sqrtl(A)) / sqrtl(A)));
    e_cbrt = std::fmax(e_cbrt, (double)(fabsl(ld(dcbrt(fa)) - cbrtl(A)) / cbrtl(A)));
    e_log = std::fmax(e_log, (double)(fabsl(ld(dlog(fa)) - logl(A)) / fmaxl(1.0L, fabsl(logl(A)))));
    const FF x = ff_from((2.0 * U(rng) - 1.0) * 3000.0);
    FF s, c;
    dsincos(x, &s, &c);
    e_sin = std::fmax(e_sin, (double)fabsl(ld(s) - sinl(ld(x))));
    e_cos = std::fmax(e_cos, (double)fabsl(ld(c) - cosl(ld(x))));
    const FF z = ff_from((2.0 * U(rng) - 1.0) * 6.0);
    const long double Z = ld(z);
    e_sinc = std::fmax(e_sinc, (double)fabsl(ld(ff_sinc(z)) - (Z == 0 ? 1.0L : sinl(Z) / Z)));
    const FF w = ff_from((2.0 * U(rng) - 1.0) * 2.0e5), ww = ff_from((2.0 * U(rng) - 1.0) * 3.1e6);
    const long double dw = ld(ff_wrap_2pi(w)) - ld(w), dww = ld(ff_wrap_2pi_wide(ww)) - ld(ww);
    e_wrap = std::fmax(e_wrap, (double)fabsl(dw - roundl(dw / two_pi) * two_pi));
    e_wrapw = std::fmax(e_wrapw, (double)fabsl(dww - roundl(dww / two_pi) * two_pi));
    const FF ex = ff_from(-60.0 + 80.0 * U(rng));
    e_exp = std::fmax(e_exp, (double)(fabsl(ld(dexp(ex)) - expl(ld(ex))) / expl(ld(ex))));
    const FF at = ff_from((U(rng) < 0.5 ? -1.0 : 1.0) * std::pow(10.0, -5.0 + 10.0 * U(rng)));
    e_atan = std::fmax(e_atan, (double)fabsl(ld(datan(at)) - atanl(ld(at))));
  }
  std::printf("add %.3e\nmul %.3e\ndiv %.3e\nsqrt %.3e\ncbrt %.3e\nlog %.3e\nsin %.3e\ncos %.3e\nsinc %.3e\n"
              "wrap %.3e\nwrap_wide %.3e\nexp %.3e\natan %.3e\n",
              e_add, e_mul, e_div, e_sqrt, e_cbrt, e_log, e_sin, e_cos, e_sinc, e_wrap, e_wrapw, e_exp, e_atan);
  return 0;
}
