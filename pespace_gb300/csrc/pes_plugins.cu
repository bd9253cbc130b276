// Granular drop-in entry points: one per reference plugin method (orbit
// vectors, single-link response, TDI combination, Whittle likelihood) plus the
// IMRPhenomD waveform producer.  FP64 throughout, one thread per frequency.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "pes_abi_common.cuh"
#include "pes_physics.cuh"

namespace pes {

static thread_local char g_error[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_error, sizeof(g_error), fmt, ap);
  va_end(ap);
}

// ------------------------------------------------------------------ kernels
__global__ void k_orbit_vectors(PesOrbit o, const double* __restrict__ t, int64_t n, double* __restrict__ out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double nn[3][3], xx[3][3];
  constellation<double>(o, t[i], nn, xx);
  double* o18 = out + 18 * i;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      o18[3 * a + j] = nn[a][j];
      o18[9 + 3 * a + j] = xx[a][j];
    }
}

__global__ void k_response_links(PesOrbit o, Polar<double> pol, const double* __restrict__ freqs, int64_t n,
                                 int nmodes, const double2* __restrict__ hp, const double2* __restrict__ hc,
                                 const double* __restrict__ tf, double tc, double2* __restrict__ links) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double f = freqs[i];
  // antenna.py:435: exp(-2 pi i f tc)
  Cx<double> ts;
  dsincos(-2.0 * kPi * f * tc, &ts.im, &ts.re);
  Cx<double> acc[6];
  for (int m = 0; m < nmodes; ++m) {
    double2 a = hp[m * n + i], b = hc[m * n + i];
    Cx<double> p = cmul(cx(a.x, a.y), ts), c = cmul(cx(b.x, b.y), ts);
    Cx<double> L[6];
    single_links<double>(o, f, p, c, tf[m * n + i] + tc, pol, L);
#pragma unroll
    for (int l = 0; l < 6; ++l) acc[l] = (m == 0) ? L[l] : acc[l] + L[l];
  }
#pragma unroll
  for (int l = 0; l < 6; ++l) links[l * n + i] = make_double2(acc[l].re, acc[l].im);
}

__global__ void k_tdi(const double* __restrict__ freqs, int64_t n, double arm, int gen20, int orth,
                      const double2* __restrict__ links, double2* __restrict__ out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  Cx<double> D, P, L[6], C[3];
  tdi_factors(freqs[i], arm, gen20, D, P);
#pragma unroll
  for (int l = 0; l < 6; ++l) {
    double2 v = links[l * n + i];
    L[l] = cx(v.x, v.y);
  }
  tdi_channels<double>(D, P, orth, L, C);
#pragma unroll
  for (int c = 0; c < 3; ++c) out[c * n + i] = make_double2(C[c].re, C[c].im);
}

constexpr int kWhittleThreads = 256;
constexpr int kWhittleMaxBlocks = 1024;

__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  return r;  // valid in thread 0
}

// pass 1: each block sums a fixed, contiguous range of bins
__global__ void k_whittle_partial(const double2* __restrict__ d, const double2* __restrict__ h,
                                  const double* __restrict__ S, int nchan, int64_t n, int64_t per_block,
                                  double* __restrict__ partial) {
  __shared__ double sh[32];
  const int64_t lo = blockIdx.x * per_block;
  const int64_t hi = min(n, lo + per_block);
  double acc = 0.0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    double ip = 0.0;
    for (int c = 0; c < nchan; ++c) {
      double2 a = d[c * n + i], b = h[c * n + i];
      double rr = a.x - b.x, ri = a.y - b.y;
      ip += (rr * rr + ri * ri) / S[c * n + i];
    }
    acc += ip;
  }
  double r = block_sum(acc, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = r;
}

// pass 2: one block sums the partials in a fixed order
__global__ void k_whittle_final(const double* __restrict__ partial, int nblk, double scale, double* __restrict__ out) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) acc += partial[i];
  double r = block_sum(acc, sh);
  if (threadIdx.x == 0) out[0] = scale * r;
}

// Scratch of the allocation-free Whittle entry point: one partial sum per block
// of k_whittle_partial (at most kWhittleMaxBlocks).  8 KB that every device
// which loads this library keeps until the process exits.
constexpr int kNoAllocPartials = kWhittleMaxBlocks;
static __device__ __align__(256) double g_whittle_scratch[kNoAllocPartials];

// Device address of g_whittle_scratch for each device, looked up on the first
// call made with that device current.
constexpr int kMaxDevices = 64;
static std::mutex g_scratch_mu;
static double* g_scratch_ptr[kMaxDevices] = {};

static int whittle_scratch(double** out) {
  int dev = -1;
  PES_CHECK_CUDA(cudaGetDevice(&dev));
  PES_REQUIRE(dev >= 0 && dev < kMaxDevices, "pes_whittle_lnl_noalloc: device index %d unsupported", dev);
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (g_scratch_ptr[dev] == nullptr) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_whittle_scratch);
    if (e != cudaSuccess) {
      set_error("pes_whittle_lnl_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev,
                cudaGetErrorString(e));
      return PES_ECUDA;
    }
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  return PES_OK;
}

struct ThetaArg {
  double v[11];
};

// h22 = A e^{-i Psi}; hp = pfac h22, hc = -i cfac h22; t(f) from dPsi/df.
__global__ void k_phenomd(ThetaArg th, double f_ref, double f_cut, const double* __restrict__ freqs, int64_t n,
                          double2* __restrict__ hp, double2* __restrict__ hc, double* __restrict__ tf) {
  __shared__ PhenomDCoef<double> c;
  if (threadIdx.x == 0) phenomd_setup<double>(th.v, f_ref, c);
  __syncthreads();
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double f = freqs[i];
  const double Mf = c.Msec * f;
  if (f > f_cut || Mf > kMfCut) {
    hp[i] = make_double2(0.0, 0.0);
    hc[i] = make_double2(0.0, 0.0);
    tf[i] = 0.0;
    return;
  }
  double amp, psi, t;
  phenomd_eval<double>(c, Mf, amp, psi, t);
  double s, co;
  dsincos(psi, &s, &co);
  hp[i] = make_double2(c.pfac * amp * co, -(c.pfac * amp * s));
  hc[i] = make_double2(-(c.cfac * amp * s), -(c.cfac * amp * co));
  tf[i] = t;
}

// IMRPhenomHM modes on a frequency array: block (x, mode); h_lm = A e^{-i Psi},
// hp = P_lm h_lm, hc = i C_lm h_lm, t(f) = dPsi_lm/df / (2 pi); zero above the
// cut and above the mode's mapped Mf = 0.2.  Outputs mode-major (6, n).
__global__ void k_phenomhm(ThetaArg th, double f_ref, double f_cut, const double* __restrict__ freqs, int64_t n,
                           double2* __restrict__ hp, double2* __restrict__ hc, double* __restrict__ tf) {
  __shared__ PhenomDCoef<double> c;
  __shared__ PhenomHMCoef<double> h;
  if (threadIdx.x == 0) {
    phenomd_setup<double>(th.v, f_ref, c);
    phenomhm_setup<double>(th.v, c, h);
  }
  __syncthreads();
  const int k = blockIdx.y;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t o = (int64_t)k * n + i;
  const double f = freqs[i];
  double amp = 0.0, psi = 0.0, t = 0.0, f22 = 0.0;
  if (f <= f_cut) phenomhm_eval<double>(c, h, k, c.Msec * f, amp, psi, t, &f22);
  if (f > f_cut || f22 > kMfCut) {
    hp[o] = make_double2(0.0, 0.0);
    hc[o] = make_double2(0.0, 0.0);
    tf[o] = 0.0;
    return;
  }
  double s, co;
  dsincos(psi, &s, &co);
  const double ap = h.md[k].P * amp, ac = h.md[k].C * amp;
  hp[o] = make_double2(ap * co, -(ap * s));
  hc[o] = make_double2(ac * s, ac * co);
  tf[o] = t;
}

}  // namespace pes

using namespace pes;

// ------------------------------------------------------------------ C ABI
// ------------------------------------------------------------------ PN t(f)
// Post-Newtonian time-frequency map of the reference's lalsimulation interface
// (pespace/waveform/interface_lalsim.py:297-482): aligned-spin TaylorF2 phase
// Psi(x) = sum_k (a_k + b_k ln(pi x)) x^((k-5)/3), x = M f, and
// t(f) = -M/(2 pi) (Psi'(x) - Psi'(x_ISCO)) below x_ISCO = 6^-3/2 / pi, 0 above.
// The coefficient table is the published expansion the reference uses (its
// 4PN spin-orbit term carries pi^2, interface_lalsim.py:435-444).
constexpr double kPnXIsco = 0.021658244478713225;  // M f at the ISCO, 1 / (6^(3/2) pi)

struct PnCoef {
  double a[9];      // a_0..a_8 (a_5 = 0)
  double b5, b6, b8;
  double msec;      // total mass [s]
  double d_isco;    // Psi'(x_ISCO)
};

__device__ double pn_dpsi(const PnCoef& c, double x) {
  // Psi'(x) = sum_k (k-5)/3 a_k x^((k-8)/3) + b5/x + b6 x^(-2/3) (ln(pi x)/3 + 1) + b8 (ln(pi x) + 1):
  // Horner in w = x^(-1/3) for the power terms (exponents -8/3 .. 0)
  const double w = 1.0 / cbrt(x);
  double p = (-5.0 / 3.0) * c.a[0];
  p = p * w + (-4.0 / 3.0) * c.a[1];
  p = p * w + (-1.0) * c.a[2];
  p = p * w + (-2.0 / 3.0) * c.a[3];
  p = p * w + (-1.0 / 3.0) * c.a[4];
  p = p * w;                              // k = 5: no power term
  p = p * w + (1.0 / 3.0) * c.a[6];
  p = p * w + (2.0 / 3.0) * c.a[7];
  p = p * w + c.a[8];
  const double lp = log(kPi * x);
  const double w2 = w * w;
  return p + c.b5 * w2 * w + c.b6 * w2 * (lp * (1.0 / 3.0) + 1.0) + c.b8 * (lp + 1.0);
}

__device__ void pn_coefficients(double m1, double m2, double chi1, double chi2, PnCoef& c) {
  const double mt = m1 + m2;
  const double eta = m1 * m2 / (mt * mt), e2 = eta * eta, e3 = e2 * eta;
  const double dl = sqrt(fmax(0.0, 1.0 - 4.0 * eta));
  const double xa = 0.5 * (chi1 - chi2), xs = 0.5 * (chi1 + chi2);
  const double pi = kPi, pi2 = kPi * kPi, pi13 = cbrt(kPi), pi23 = pi13 * pi13;
  const double pfac = -3.0 / (128.0 * eta);
  const double c2 = 3715.0 / 756.0 + 55.0 / 9.0 * eta;
  const double c3 = -16.0 * pi + 113.0 / 3.0 * dl * xa + (113.0 / 3.0 - 76.0 / 3.0 * eta) * xs;
  const double c4 = 15293365.0 / 508032.0 + 27145.0 / 504.0 * eta + 3085.0 / 72.0 * e2 +
                    (-405.0 / 8.0 + 200.0 * eta) * xa * xa - 405.0 / 4.0 * dl * xa * xs +
                    (-405.0 / 8.0 + 5.0 / 2.0 * eta) * xs * xs;
  const double c5l = (38645.0 / 756.0 - 65.0 / 9.0 * eta) * pi + (-732985.0 / 2268.0 - 140.0 / 9.0 * eta) * dl * xa +
                     (-732985.0 / 2268.0 + 24260.0 / 81.0 * eta + 340.0 / 9.0 * e2) * xs;
  const double c6 = 11583231236531.0 / 4694215680.0 - 640.0 / 3.0 * pi2 - 6848.0 / 21.0 * kEulerGamma +
                    (-15737765635.0 / 3048192.0 + 2255.0 / 12.0 * pi2) * eta + 76055.0 / 1728.0 * e2 -
                    127825.0 / 1296.0 * e3 - 0.69314718055994531 * 13696.0 / 21.0 + 2270.0 / 3.0 * pi * dl * xa +
                    (2270.0 / 3.0 - 520.0 * eta) * pi * xs + (75515.0 / 144.0 - 8225.0 / 18.0 * eta) * dl * xs * xa +
                    (75515.0 / 288.0 - 263245.0 / 252.0 * eta - 480.0 * e2) * xa * xa +
                    (75515.0 / 288.0 - 232415.0 / 504.0 * eta + 1255.0 / 9.0 * e2) * xs * xs;
  const double c7 =
      (77096675.0 / 254016.0 + 378515.0 / 1512.0 * eta - 74045.0 / 756.0 * e2) * pi +
      (-25150083775.0 / 3048192.0 + 26804935.0 / 6048.0 * eta - 1985.0 / 48.0 * e2) * dl * xa +
      (-25150083775.0 / 3048192.0 + 10566655595.0 / 762048.0 * eta - 1042165.0 / 3024.0 * e2 + 5345.0 / 36.0 * e3) * xs -
      1140.0 * pi * dl * xa * xs + (-570.0 + 2240.0 * eta) * pi * xa * xa + (-570.0 + 40.0 * eta) * pi * xs * xs +
      (14585.0 / 8.0 - 215.0 / 2.0 * eta) * dl * xa * xs * xs + (14585.0 / 8.0 - 7270.0 * eta + 80.0 * e2) * xa * xa * xs +
      (14585.0 / 24.0 - 2380.0 * eta) * dl * xa * xa * xa +
      (14585.0 / 24.0 - 475.0 / 6.0 * eta + 100.0 / 3.0 * e2) * xs * xs * xs;
  const double c8 = (233915.0 / 168.0 - 99185.0 / 252.0 * eta) * dl * xa +
                    (233915.0 / 168.0 - 3970375.0 / 2268.0 * eta + 19655.0 / 189.0 * e2) * xs;
  c.a[0] = pfac / (pi * pi23);
  c.a[1] = 0.0;
  c.a[2] = pfac * c2 / pi;
  c.a[3] = pfac * c3 / pi23;
  c.a[4] = pfac * c4 / pi13;
  c.a[5] = 0.0;
  c.a[6] = pfac * c6 * pi13;
  c.a[7] = pfac * c7 * pi23;
  c.a[8] = pfac * c8 * pi2;
  c.b5 = pfac * c5l;
  c.b6 = pfac * (-6848.0 / 63.0) * pi13;
  c.b8 = -c.a[8];
  c.msec = mt * kMTSun;
  c.d_isco = pn_dpsi(c, kPnXIsco);
}

// grid (ceil(n / 256), B): thread 0 of each block sets up the sample's coefficients
__global__ void k_pn_tf(const double* __restrict__ params, int64_t n, const double* __restrict__ freqs,
                        double* __restrict__ tf) {
  __shared__ PnCoef c;
  const int64_t b = blockIdx.y;
  if (threadIdx.x == 0) {
    const double* q = params + 4 * b;
    pn_coefficients(q[0], q[1], q[2], q[3], c);
  }
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x = freqs[i] * c.msec;
  tf[b * n + i] = (x < kPnXIsco && x > 0.0) ? -c.msec / (2.0 * kPi) * (pn_dpsi(c, x) - c.d_isco) : 0.0;
}

// ------------------------------------------------ time-domain Michelson TDI
// TDMichelsonConstantEqualArm.update_tdi_response (pespace/detector/tdi.py:
// 1460-1600): every output sample i combines the six single-link series at
// the undelayed sample i + added and, for each delay k = 0..max_delay-1, the
// linear interpolation left + (right - left) * frac_k between samples
// i + shift_k and i + shift_k + 1 (utils.py:83-100).  The shifts, fractions and
// `added` are the reference's expressions on Python floats (tdi.py:1449-1454,
// 1469-1491), evaluated on the host by td_layout.  The arithmetic keeps the
// reference's order with no contraction (explicit round-to-nearest adds and
// multiplies), so the result is bit-identical to a left-to-right evaluation.
//
// Each block stages the window [i0, i0 + kTdTile + added + 1) of its six link
// series in shared memory with coalesced loads, and beside it the differences
// right - left of neighbouring samples: every delay that reads a sample pair
// reuses its difference (the same subtraction of the same operands), which
// takes 6 instead of 6 max_delay FP64 subtractions per output sample.  Per
// output sample the unique traffic is 6 x 8 B read and 3 x 8 B written, but
// the reference's operation order leaves about 145 unfused FP64 operations,
// so the FP64 pipe (1/64 of the FP32 rate) binds, not HBM.  A window beyond
// kTdMaxWindow samples (added > 1535, e.g. sub-0.04 s sampling) reads
// through the L1 and subtracts per delay instead.

struct TdLayout {
  int max_delay;
  int64_t added;
  int64_t shift[7];
  double frac[7];
  double rs2, rs6, rs3;  // sqrt(2), sqrt(6), sqrt(3), correctly rounded
};

constexpr int kTdThreads = 256;
constexpr int kTdTile = 512;
constexpr int kTdMaxWindow = 2048;  // values and differences: 12 x 2048 x 8 B = 192 KB of shared memory

// Python's float // and % (CPython's divmod: floor of (a - fmod(a, b)) / b,
// rounded to the nearest integer when it lands within half of one).
static void py_divmod(double a, double b, double* floordiv, double* mod) {
  double m = std::fmod(a, b);
  double div = (a - m) / b;
  if (m != 0.0) {
    if ((b < 0) != (m < 0)) {
      m += b;
      div -= 1.0;
    }
  } else {
    m = std::copysign(0.0, b);
  }
  double fd;
  if (div != 0.0) {
    fd = std::floor(div);
    if (div - fd > 0.5) fd += 1.0;
  } else {
    fd = std::copysign(0.0, a / b);
  }
  *floordiv = fd;
  *mod = m;
}

static void td_layout(double arm, double dt, int gen20, TdLayout& lay) {
  lay.max_delay = gen20 ? 7 : 3;
  double q, r;
  py_divmod(lay.max_delay * arm, dt, &q, &r);
  lay.added = (int64_t)(q + 1.0);  // int(max_num_delay * armlength // delta_time + 1)
  for (int k = 0; k < 7; ++k) {
    lay.shift[k] = 0;
    lay.frac[k] = 0.0;
  }
  for (int k = 0; k < lay.max_delay; ++k) {
    const int nd = k + 1;
    py_divmod(nd * arm, dt, &q, &r);
    lay.frac[k] = 1.0 - r / dt;  // 1 - (num_delay * armlength % delta_time) / delta_time
    py_divmod((lay.max_delay - nd) * arm, dt, &q, &r);
    lay.shift[k] = (int64_t)q;  // (max_num_delay - num_delay) * armlength // delta_time
  }
  lay.rs2 = std::sqrt(2.0);
  lay.rs6 = std::sqrt(6.0);
  lay.rs3 = std::sqrt(3.0);
}

// grid (ceil(n / kTdTile), B); links [B][6][n_ext] in the order link12, link21,
// link23, link32, link31, link13; out [B][3][n].
template <int kMaxDelay, bool kStaged>
__global__ void __launch_bounds__(kTdThreads) k_td_tdi(TdLayout lay, const double* __restrict__ links, int64_t n_ext,
                                                       int64_t n, int orth, double* __restrict__ out) {
  extern __shared__ double td_win[];  // [6][win] values, then [6][win] differences
  const double* src = links + (int64_t)blockIdx.y * 6 * n_ext;
  double* dst = out + (int64_t)blockIdx.y * 3 * n;
  const int64_t i0 = (int64_t)blockIdx.x * kTdTile;
  const int64_t win = kTdTile + lay.added + 1;
  double* td_dif = td_win + 6 * win;
  if (kStaged) {
    const int64_t avail = n_ext - i0;
#pragma unroll 1
    for (int l = 0; l < 6; ++l) {
      const double* s = src + (int64_t)l * n_ext + i0;
      double* w = td_win + l * win;
#pragma unroll 4
      for (int64_t j = threadIdx.x; j < win; j += kTdThreads) w[j] = j < avail ? __ldg(s + j) : 0.0;
    }
    __syncthreads();
#pragma unroll 1
    for (int l = 0; l < 6; ++l) {
      const double* w = td_win + l * win;
      double* df = td_dif + l * win;
#pragma unroll 4
      for (int64_t j = threadIdx.x; j + 1 < win; j += kTdThreads) df[j] = __dsub_rn(w[j + 1], w[j]);
    }
    __syncthreads();
  }
  // X = sum of the "plus" terms, then minus the "minus" terms, in the order of
  // tdi.py:1506-1591 (k = -1: the undelayed sample); Y and Z are the cyclic
  // relabelling 1 -> 2 -> 3 -> 1, i.e. link index l -> (l + 2) mod 6.
  constexpr int kTerms = kMaxDelay + 1;
  constexpr int xp[8] = {5, 4, 0, 1, 0, 1, 5, 4};
  constexpr int xm[8] = {0, 1, 5, 4, 5, 4, 0, 1};
#pragma unroll 1
  for (int r = 0; r < kTdTile / kTdThreads; ++r) {
    const int64_t t = threadIdx.x + r * kTdThreads;
    const int64_t i = i0 + t;
    if (i >= n) break;
    auto at = [&](int l, int64_t off) -> double {
      return kStaged ? td_win[l * win + t + off] : __ldg(src + (int64_t)l * n_ext + i + off);
    };
    auto term = [&](int l, int k) -> double {
      if (k < 0) return at(l, lay.added);
      const double left = at(l, lay.shift[k]);
      const double dif = kStaged ? td_dif[l * win + t + lay.shift[k]] : __dsub_rn(at(l, lay.shift[k] + 1), left);
      return __dadd_rn(left, __dmul_rn(dif, lay.frac[k]));
    };
    double ch[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double acc = term((xp[0] + 2 * c) % 6, -1);
#pragma unroll
      for (int j = 1; j < kTerms; ++j) acc = __dadd_rn(acc, term((xp[j] + 2 * c) % 6, j - 1));
#pragma unroll
      for (int j = 0; j < kTerms; ++j) acc = __dsub_rn(acc, term((xm[j] + 2 * c) % 6, j - 1));
      ch[c] = acc;
    }
    if (orth) {
      const double X = ch[0], Y = ch[1], Z = ch[2];
      dst[i] = __ddiv_rn(__dsub_rn(Z, X), lay.rs2);
      dst[n + i] = __ddiv_rn(__dadd_rn(__dsub_rn(X, __dmul_rn(2.0, Y)), Z), lay.rs6);
      dst[2 * n + i] = __ddiv_rn(__dadd_rn(__dadd_rn(X, Y), Z), lay.rs3);
    } else {
      dst[i] = ch[0];
      dst[n + i] = ch[1];
      dst[2 * n + i] = ch[2];
    }
  }
}

template <int kMaxDelay>
static int launch_td_tdi(const TdLayout& lay, const double* links, int64_t B, int64_t n_ext, int64_t n, int orth,
                         double* out, cudaStream_t st) {
  const dim3 grid((unsigned)((n + kTdTile - 1) / kTdTile), (unsigned)B);
  const int64_t win = kTdTile + lay.added + 1;
  if (win <= kTdMaxWindow) {
    const size_t smem = (size_t)12 * win * sizeof(double);
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(k_td_tdi<kMaxDelay, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem);
      if (e != cudaSuccess) {
        set_error("pes_td_tdi_combination: %s", cudaGetErrorString(e));
        return PES_ECUDA;
      }
    }
    k_td_tdi<kMaxDelay, true><<<grid, kTdThreads, smem, st>>>(lay, links, n_ext, n, orth, out);
  } else {
    k_td_tdi<kMaxDelay, false><<<grid, kTdThreads, 0, st>>>(lay, links, n_ext, n, orth, out);
  }
  PES_CHECK_LAUNCH();
  return PES_OK;
}

// Float-float variant (pes_td_tdi_combination_mixed): the same combination on
// the FP32 pipe.  Each block scales its window by a power of two (its largest
// exponent to 2^0, exact) and splits every double into a float-float pair from
// the bits alone (integer operations: the FP64 pipe is not used on the way
// in); interpolations, sums and the A/E/T combination run in float-float
// (about 2^-46 of the operands per operation); each channel goes back to a
// double from the bits and one FP64 add.  Scaled magnitudes below 2^-126
// (2^-126 of the window's largest link sample) flush to zero; a NaN or an
// infinity among the inputs gives NaN in the outputs that read it.
struct TdLayoutFF {
  int max_delay;
  int64_t added;
  int64_t shift[7];
  float2 frac[7];      // the weights as float-float pairs
  float2 rs2, rs6, rs3;  // 1/sqrt(2), 1/sqrt(6), 1/sqrt(3) as float-float pairs
};

static float2 ff_pair(double x) {
  const float h = (float)x;
  return make_float2(h, (float)(x - (double)h));
}

static void td_layout_ff(const TdLayout& lay, TdLayoutFF& out) {
  out.max_delay = lay.max_delay;
  out.added = lay.added;
  for (int k = 0; k < 7; ++k) {
    out.shift[k] = lay.shift[k];
    out.frac[k] = ff_pair(lay.frac[k]);
  }
  out.rs2 = ff_pair(1.0 / std::sqrt(2.0));
  out.rs6 = ff_pair(1.0 / std::sqrt(6.0));
  out.rs3 = ff_pair(1.0 / std::sqrt(3.0));
}

// x * 2^-scale as a float-float pair: head = sign, exponent and the top 23
// fraction bits; tail = the other 29 fraction bits, normalised (truncated to
// 24 significant bits).
__device__ __forceinline__ FF td_split(double x, int scale) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int E = (int)((b >> 52) & 0x7FF);
  if (E == 0x7FF) return ff_make(__uint_as_float(0x7fc00000u), 0.0f);
  const int e = E - 1023 - scale;
  if (E == 0 || e < -126) return ff_make(0.0f, 0.0f);
  const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  const float hi = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | (unsigned)(m >> 29));
  const unsigned r = (unsigned)(m & 0x1FFFFFFFull);
  float lo = 0.0f;
  if (r != 0u) {
    const int lz = __clz((int)r);    // r < 2^29: 3 <= lz <= 31
    const int el = e - 52 + 31 - lz;  // exponent of r's leading bit
    if (el >= -126) {
      const unsigned frac = (unsigned)((((unsigned long long)r << (lz + 1)) & 0xFFFFFFFFull) >> 9);
      lo = __uint_as_float(sign | ((unsigned)(el + 127) << 23) | frac);
    }
  }
  return ff_make(hi, lo);
}

// float f * 2^scale as a double, from the bits
__device__ __forceinline__ double td_widen(float f, int scale) {
  const unsigned u = __float_as_uint(f);
  const int ef = (int)((u >> 23) & 0xFF);
  if (ef == 0xFF) return __longlong_as_double(0x7ff8000000000000ll);
  const int ed = ef - 127 + 1023 + scale;
  if (ef == 0 || ed <= 0) return 0.0;
  if (ed >= 0x7FF) return __longlong_as_double((long long)(((unsigned long long)(u >> 31) << 63) | 0x7ff0000000000000ull));
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  return __longlong_as_double((long long)(sign | ((unsigned long long)ed << 52) |
                                          ((unsigned long long)(u & 0x7FFFFFu) << 29)));
}

template <int kMaxDelay>
__global__ void __launch_bounds__(kTdThreads) k_td_tdi_ff(TdLayoutFF lay, const double* __restrict__ links,
                                                          int64_t n_ext, int64_t n, int orth,
                                                          double* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char td_raw[];
  const int64_t win = kTdTile + lay.added + 1;
  FF* val = reinterpret_cast<FF*>(td_raw);  // [6][win]: the doubles first, then their float-float pairs
  FF* dif = val + 6 * win;                  // [6][win]: right - left
  double* raw = reinterpret_cast<double*>(td_raw);
  __shared__ int wmax[kTdThreads / 32];
  const double* src = links + (int64_t)blockIdx.y * 6 * n_ext;
  double* dst = out + (int64_t)blockIdx.y * 3 * n;
  const int64_t i0 = (int64_t)blockIdx.x * kTdTile;
  const int64_t avail = n_ext - i0;
  int emax = 0;  // largest finite biased exponent in the window
#pragma unroll 1
  for (int l = 0; l < 6; ++l) {
    const double* s = src + (int64_t)l * n_ext + i0;
    double* w = raw + l * win;
#pragma unroll 4
    for (int64_t j = threadIdx.x; j < win; j += kTdThreads) {
      const double x = j < avail ? __ldg(s + j) : 0.0;
      w[j] = x;
      const int E = (int)(((unsigned long long)__double_as_longlong(x) >> 52) & 0x7FF);
      if (E != 0x7FF) emax = max(emax, E);
    }
  }
  emax = __reduce_max_sync(0xffffffffu, emax);
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = emax;
  __syncthreads();
#pragma unroll
  for (int w = 0; w < kTdThreads / 32; ++w) emax = max(emax, wmax[w]);
  const int scale = emax - 1023;  // the window's largest magnitude maps into [1, 2)
  // each thread rewrites the slots it loaded: doubles -> float-float pairs in place
#pragma unroll 1
  for (int l = 0; l < 6; ++l) {
    double* w = raw + l * win;
    FF* v = val + l * win;
#pragma unroll 4
    for (int64_t j = threadIdx.x; j < win; j += kTdThreads) v[j] = td_split(w[j], scale);
  }
  __syncthreads();
#pragma unroll 1
  for (int l = 0; l < 6; ++l) {
    const FF* v = val + l * win;
    FF* df = dif + l * win;
#pragma unroll 4
    for (int64_t j = threadIdx.x; j + 1 < win; j += kTdThreads) df[j] = v[j + 1] - v[j];
  }
  __syncthreads();
  constexpr int kTerms = kMaxDelay + 1;
  constexpr int xp[8] = {5, 4, 0, 1, 0, 1, 5, 4};
  constexpr int xm[8] = {0, 1, 5, 4, 5, 4, 0, 1};
#pragma unroll 1
  for (int r = 0; r < kTdTile / kTdThreads; ++r) {
    const int64_t t = threadIdx.x + r * kTdThreads;
    const int64_t i = i0 + t;
    if (i >= n) break;
    auto term = [&](int l, int k) -> FF {
      if (k < 0) return val[l * win + t + lay.added];
      const int64_t o = l * win + t + lay.shift[k];
      const float2 f = lay.frac[k];
      return val[o] + dif[o] * ff_make(f.x, f.y);
    };
    FF ch[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      FF acc = term((xp[0] + 2 * c) % 6, -1);
#pragma unroll
      for (int j = 1; j < kTerms; ++j) acc = acc + term((xp[j] + 2 * c) % 6, j - 1);
#pragma unroll
      for (int j = 0; j < kTerms; ++j) acc = acc - term((xm[j] + 2 * c) % 6, j - 1);
      ch[c] = acc;
    }
    FF o3[3];
    if (orth) {
      const FF X = ch[0], Y = ch[1], Z = ch[2];
      o3[0] = (Z - X) * ff_make(lay.rs2.x, lay.rs2.y);
      o3[1] = (X - ff_mulf(Y, 2.0f) + Z) * ff_make(lay.rs6.x, lay.rs6.y);
      o3[2] = (X + Y + Z) * ff_make(lay.rs3.x, lay.rs3.y);
    } else {
      o3[0] = ch[0];
      o3[1] = ch[1];
      o3[2] = ch[2];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) dst[(int64_t)c * n + i] = __dadd_rn(td_widen(o3[c].hi, scale), td_widen(o3[c].lo, scale));
  }
}

template <int kMaxDelay>
static int launch_td_tdi_ff(const TdLayout& lay, const double* links, int64_t B, int64_t n_ext, int64_t n, int orth,
                            double* out, cudaStream_t st) {
  TdLayoutFF lf;
  td_layout_ff(lay, lf);
  const dim3 grid((unsigned)((n + kTdTile - 1) / kTdTile), (unsigned)B);
  const int64_t win = kTdTile + lay.added + 1;
  const size_t smem = (size_t)12 * win * sizeof(FF);  // [6][win] values + [6][win] differences, float pairs
  if (win > kTdMaxWindow) {
    set_error("pes_td_tdi_combination_mixed: the longest delay (%lld samples) exceeds %d",
              (long long)lay.added, kTdMaxWindow - kTdTile - 1);
    return PES_EINVAL;
  }
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_td_tdi_ff<kMaxDelay>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) {
      set_error("pes_td_tdi_combination_mixed: %s", cudaGetErrorString(e));
      return PES_ECUDA;
    }
  }
  k_td_tdi_ff<kMaxDelay><<<grid, kTdThreads, smem, st>>>(lf, links, n_ext, n, orth, out);
  PES_CHECK_LAUNCH();
  return PES_OK;
}

extern "C" {

const char* pes_last_error(void) { return pes::g_error; }
int pes_version(void) { return 1; }

int pes_orbit_vectors(const PesOrbit* orbit, const double* time, int64_t n, double* out, void* stream) {
  PES_REQUIRE(orbit && (n == 0 || (time && out)), "pes_orbit_vectors: null pointer");
  PES_REQUIRE(n >= 0, "pes_orbit_vectors: n < 0");
  PES_REQUIRE(orbit->kind == 0 || orbit->kind == 1, "pes_orbit_vectors: unknown orbit kind %d", orbit->kind);
  if (n == 0) return PES_OK;
  k_orbit_vectors<<<ceil_div(n, 128), 128, 0, as_stream(stream)>>>(*orbit, time, n, out);
  PES_CHECK_LAUNCH();
  return PES_OK;
}

int pes_polarization(double lam, double beta, double psi, double* plus9, double* cross9, double* k3) {
  PES_REQUIRE(plus9 && cross9 && k3, "pes_polarization: null pointer");
  Polar<double> p;
  make_polar<double>(lam, ::sin(beta), ::cos(beta), psi, p);
  const int ii[6] = {0, 0, 0, 1, 1, 2}, jj[6] = {0, 1, 2, 1, 2, 2};
  for (int m = 0; m < 6; ++m) {
    plus9[3 * ii[m] + jj[m]] = plus9[3 * jj[m] + ii[m]] = p.P[m];
    cross9[3 * ii[m] + jj[m]] = cross9[3 * jj[m] + ii[m]] = p.X[m];
  }
  for (int j = 0; j < 3; ++j) k3[j] = p.k[j];
  return PES_OK;
}

int pes_response_links(const PesOrbit* orbit, const double* freqs, int64_t n, int32_t n_modes, const double* hp,
                       const double* hc, const double* tf, double lam, double beta, double psi, double tc,
                       double* links, void* stream) {
  PES_REQUIRE(orbit, "pes_response_links: null orbit");
  PES_REQUIRE(n >= 0 && n_modes >= 1, "pes_response_links: bad sizes n=%lld modes=%d", (long long)n, n_modes);
  PES_REQUIRE(orbit->kind == 0 || orbit->kind == 1, "pes_response_links: unknown orbit kind %d", orbit->kind);
  if (n == 0) return PES_OK;
  PES_REQUIRE(freqs && hp && hc && tf && links, "pes_response_links: null pointer");
  Polar<double> pol;
  make_polar<double>(lam, ::sin(beta), ::cos(beta), psi, pol);
  k_response_links<<<ceil_div(n, 128), 128, 0, as_stream(stream)>>>(
      *orbit, pol, freqs, n, n_modes, reinterpret_cast<const double2*>(hp), reinterpret_cast<const double2*>(hc),
      tf, tc, reinterpret_cast<double2*>(links));
  PES_CHECK_LAUNCH();
  return PES_OK;
}

int pes_tdi_combination(const double* freqs, int64_t n, double arm_sec, int32_t generation, int32_t orthogonal,
                        const double* links, double* out, void* stream) {
  PES_REQUIRE(generation == 15 || generation == 20, "pes_tdi_combination: unsupported generation %d", generation);
  PES_REQUIRE(n >= 0, "pes_tdi_combination: n < 0");
  if (n == 0) return PES_OK;
  PES_REQUIRE(freqs && links && out, "pes_tdi_combination: null pointer");
  k_tdi<<<ceil_div(n, 128), 128, 0, as_stream(stream)>>>(freqs, n, arm_sec, generation == 20, orthogonal != 0,
                                                          reinterpret_cast<const double2*>(links),
                                                          reinterpret_cast<double2*>(out));
  PES_CHECK_LAUNCH();
  return PES_OK;
}

int64_t pes_whittle_workspace_len(int64_t n) {
  if (n <= 0) return 1;
  int64_t blocks = (n + 4 * kWhittleThreads - 1) / (4 * kWhittleThreads);
  return blocks < kWhittleMaxBlocks ? blocks : kWhittleMaxBlocks;
}

int pes_whittle_lnl(const double* data, const double* response, const double* psd, int32_t n_chan, int64_t n,
                    double df, double* workspace, int64_t workspace_len, double* out, void* stream) {
  PES_REQUIRE(n_chan >= 1 && n_chan <= 3, "pes_whittle_lnl: n_chan must be 1..3, got %d", n_chan);
  PES_REQUIRE(n >= 0, "pes_whittle_lnl: n < 0");
  PES_REQUIRE(out, "pes_whittle_lnl: null out");
  const int64_t nblk = pes_whittle_workspace_len(n);
  PES_REQUIRE(workspace && workspace_len >= nblk, "pes_whittle_lnl: workspace needs %lld doubles",
              (long long)nblk);
  cudaStream_t st = as_stream(stream);
  if (n == 0) {
    PES_CHECK_CUDA(cudaMemsetAsync(out, 0, sizeof(double), st));
    return PES_OK;
  }
  PES_REQUIRE(data && response && psd, "pes_whittle_lnl: null pointer");
  const int64_t per_block = (n + nblk - 1) / nblk;
  k_whittle_partial<<<(unsigned)nblk, kWhittleThreads, 0, st>>>(reinterpret_cast<const double2*>(data),
                                                                 reinterpret_cast<const double2*>(response), psd,
                                                                 n_chan, n, per_block, workspace);
  PES_CHECK_LAUNCH();
  k_whittle_final<<<1, kWhittleThreads, 0, st>>>(workspace, (int)nblk, -2.0 * df, out);
  PES_CHECK_LAUNCH();
  return PES_OK;
}

int pes_whittle_lnl_noalloc(const double* data, const double* response, const double* psd, int32_t n_chan,
                            int64_t n, double df, double* out, void* stream) {
  PES_REQUIRE(n_chan >= 1 && n_chan <= 3, "pes_whittle_lnl_noalloc: n_chan must be 1..3, got %d", n_chan);
  PES_REQUIRE(n >= 0 && n <= PES_WHITTLE_NOALLOC_MAX_BINS,
              "pes_whittle_lnl_noalloc: n = %lld outside [0, %lld]", (long long)n,
              (long long)PES_WHITTLE_NOALLOC_MAX_BINS);
  PES_REQUIRE(out, "pes_whittle_lnl_noalloc: null out");
  const int64_t nblk = pes_whittle_workspace_len(n);
  PES_REQUIRE(nblk <= kNoAllocPartials, "pes_whittle_lnl_noalloc: %lld partial sums exceed the %d-entry scratch",
              (long long)nblk, kNoAllocPartials);
  double* scratch = nullptr;
  int rc = whittle_scratch(&scratch);
  if (rc != PES_OK) return rc;
  cudaStream_t st = as_stream(stream);
  if (n == 0) {
    PES_CHECK_CUDA(cudaMemsetAsync(out, 0, sizeof(double), st));
    return PES_OK;
  }
  PES_REQUIRE(data && response && psd, "pes_whittle_lnl_noalloc: null pointer");
  // every partial the final pass reads is written by the first pass, so the
  // scratch needs no clearing between calls
  const int64_t per_block = (n + nblk - 1) / nblk;
  k_whittle_partial<<<(unsigned)nblk, kWhittleThreads, 0, st>>>(reinterpret_cast<const double2*>(data),
                                                                 reinterpret_cast<const double2*>(response), psd,
                                                                 n_chan, n, per_block, scratch);
  PES_CHECK_LAUNCH();
  k_whittle_final<<<1, kWhittleThreads, 0, st>>>(scratch, (int)nblk, -2.0 * df, out);
  PES_CHECK_LAUNCH();
  return PES_OK;
}

int pes_phenomd(const double* theta, const double* freqs, int64_t n, double f_ref, double f_cut_hz, double* hp,
                double* hc, double* tf, void* stream) {
  PES_REQUIRE(theta, "pes_phenomd: null theta");
  PES_REQUIRE(n >= 0, "pes_phenomd: n < 0");
  if (n == 0) return PES_OK;
  PES_REQUIRE(freqs && hp && hc && tf, "pes_phenomd: null pointer");
  ThetaArg th;
  for (int j = 0; j < 11; ++j) th.v[j] = theta[j];
  k_phenomd<<<ceil_div(n, 128), 128, 0, as_stream(stream)>>>(th, f_ref, f_cut_hz, freqs, n,
                                                             reinterpret_cast<double2*>(hp),
                                                             reinterpret_cast<double2*>(hc), tf);
  PES_CHECK_LAUNCH();
  return PES_OK;
}

int pes_phenomhm(const double* theta, const double* freqs, int64_t n, double f_ref, double f_cut_hz, double* hp,
                 double* hc, double* tf, void* stream) {
  PES_REQUIRE(theta, "pes_phenomhm: null theta");
  PES_REQUIRE(n >= 0, "pes_phenomhm: n < 0");
  if (n == 0) return PES_OK;
  PES_REQUIRE(freqs && hp && hc && tf, "pes_phenomhm: null pointer");
  ThetaArg th;
  for (int j = 0; j < 11; ++j) th.v[j] = theta[j];
  k_phenomhm<<<dim3(ceil_div(n, 128), kHMModes), 128, 0, as_stream(stream)>>>(
      th, f_ref, f_cut_hz, freqs, n, reinterpret_cast<double2*>(hp), reinterpret_cast<double2*>(hc), tf);
  PES_CHECK_LAUNCH();
  return PES_OK;
}

int pes_pn_tf(const double* params, int64_t B, const double* freqs, int64_t n, double* tf, void* stream) {
  PES_REQUIRE(B >= 0 && n >= 0, "pes_pn_tf: negative size (B = %lld, n = %lld)", (long long)B, (long long)n);
  PES_REQUIRE(B <= 65535, "pes_pn_tf: at most 65535 parameter sets per call, got %lld", (long long)B);
  if (B == 0 || n == 0) return PES_OK;
  PES_REQUIRE(params && freqs && tf, "pes_pn_tf: null pointer");
  k_pn_tf<<<dim3(ceil_div(n, 256), (unsigned)B), 256, 0, as_stream(stream)>>>(params, n, freqs, tf);
  PES_CHECK_LAUNCH();
  return PES_OK;
}

int pes_td_tdi_layout(double arm_sec, double delta_time, int32_t generation, int64_t* added, int32_t* max_delay,
                      int64_t* shifts, double* fracs) {
  PES_REQUIRE(generation == 15 || generation == 20, "pes_td_tdi_layout: unsupported generation %d", generation);
  PES_REQUIRE(std::isfinite(arm_sec) && arm_sec > 0.0 && std::isfinite(delta_time) && delta_time > 0.0,
              "pes_td_tdi_layout: arm length and sampling step must be finite and > 0 (%g, %g)", arm_sec,
              delta_time);
  PES_REQUIRE(added && max_delay && shifts && fracs, "pes_td_tdi_layout: null pointer");
  PES_REQUIRE(7.0 * arm_sec / delta_time < 1e9, "pes_td_tdi_layout: delay of %g samples too long",
              7.0 * arm_sec / delta_time);
  TdLayout lay;
  td_layout(arm_sec, delta_time, generation == 20, lay);
  *added = lay.added;
  *max_delay = lay.max_delay;
  for (int k = 0; k < lay.max_delay; ++k) {
    shifts[k] = lay.shift[k];
    fracs[k] = lay.frac[k];
  }
  return PES_OK;
}

int pes_td_tdi_combination(const double* links, int64_t B, int64_t n_ext, int64_t n, double arm_sec,
                           double delta_time, int32_t generation, int32_t orthogonal, double* out, void* stream) {
  PES_REQUIRE(generation == 15 || generation == 20, "pes_td_tdi_combination: unsupported generation %d",
              generation);
  PES_REQUIRE(std::isfinite(arm_sec) && arm_sec > 0.0 && std::isfinite(delta_time) && delta_time > 0.0,
              "pes_td_tdi_combination: arm length and sampling step must be finite and > 0 (%g, %g)", arm_sec,
              delta_time);
  PES_REQUIRE(B >= 0 && B <= 65535 && n >= 0 && n_ext >= 0,
              "pes_td_tdi_combination: bad sizes (B = %lld, n = %lld, n_ext = %lld)", (long long)B, (long long)n,
              (long long)n_ext);
  PES_REQUIRE(n <= (int64_t)kTdTile * 0x7FFFFFFF, "pes_td_tdi_combination: %lld samples exceed the launch grid",
              (long long)n);
  PES_REQUIRE(7.0 * arm_sec / delta_time < 1e9, "pes_td_tdi_combination: delay of %g samples too long",
              7.0 * arm_sec / delta_time);
  TdLayout lay;
  td_layout(arm_sec, delta_time, generation == 20, lay);
  for (int k = 0; k < lay.max_delay; ++k)  // every read stays in [i, i + added]
    PES_REQUIRE(lay.shift[k] >= 0 && lay.shift[k] + 1 <= lay.added,
                "pes_td_tdi_combination: delay layout out of range (shift %lld, added %lld)",
                (long long)lay.shift[k], (long long)lay.added);
  PES_REQUIRE(n_ext >= n + lay.added,
              "pes_td_tdi_combination: %lld link samples for %lld outputs, need n + %lld (the longest delay)",
              (long long)n_ext, (long long)n, (long long)lay.added);
  if (B == 0 || n == 0) return PES_OK;
  PES_REQUIRE(links && out, "pes_td_tdi_combination: null pointer");
  const cudaStream_t st = as_stream(stream);
  return generation == 20 ? launch_td_tdi<7>(lay, links, B, n_ext, n, orthogonal != 0, out, st)
                          : launch_td_tdi<3>(lay, links, B, n_ext, n, orthogonal != 0, out, st);
}

int pes_td_tdi_combination_mixed(const double* links, int64_t B, int64_t n_ext, int64_t n, double arm_sec,
                                 double delta_time, int32_t generation, int32_t orthogonal, double* out,
                                 void* stream) {
  PES_REQUIRE(generation == 15 || generation == 20, "pes_td_tdi_combination_mixed: unsupported generation %d",
              generation);
  PES_REQUIRE(std::isfinite(arm_sec) && arm_sec > 0.0 && std::isfinite(delta_time) && delta_time > 0.0,
              "pes_td_tdi_combination_mixed: arm length and sampling step must be finite and > 0 (%g, %g)",
              arm_sec, delta_time);
  PES_REQUIRE(B >= 0 && B <= 65535 && n >= 0 && n_ext >= 0,
              "pes_td_tdi_combination_mixed: bad sizes (B = %lld, n = %lld, n_ext = %lld)", (long long)B,
              (long long)n, (long long)n_ext);
  PES_REQUIRE(n <= (int64_t)kTdTile * 0x7FFFFFFF, "pes_td_tdi_combination_mixed: %lld samples exceed the launch grid",
              (long long)n);
  PES_REQUIRE(7.0 * arm_sec / delta_time < 1e9, "pes_td_tdi_combination_mixed: delay of %g samples too long",
              7.0 * arm_sec / delta_time);
  TdLayout lay;
  td_layout(arm_sec, delta_time, generation == 20, lay);
  for (int k = 0; k < lay.max_delay; ++k)  // every read stays in [i, i + added]
    PES_REQUIRE(lay.shift[k] >= 0 && lay.shift[k] + 1 <= lay.added,
                "pes_td_tdi_combination_mixed: delay layout out of range (shift %lld, added %lld)",
                (long long)lay.shift[k], (long long)lay.added);
  PES_REQUIRE(n_ext >= n + lay.added,
              "pes_td_tdi_combination_mixed: %lld link samples for %lld outputs, need n + %lld (the longest delay)",
              (long long)n_ext, (long long)n, (long long)lay.added);
  PES_REQUIRE(kTdTile + lay.added + 1 <= kTdMaxWindow,
              "pes_td_tdi_combination_mixed: the longest delay (%lld samples) exceeds %d", (long long)lay.added,
              kTdMaxWindow - kTdTile - 1);
  if (B == 0 || n == 0) return PES_OK;
  PES_REQUIRE(links && out, "pes_td_tdi_combination_mixed: null pointer");
  const cudaStream_t st = as_stream(stream);
  return generation == 20 ? launch_td_tdi_ff<7>(lay, links, B, n_ext, n, orthogonal != 0, out, st)
                          : launch_td_tdi_ff<3>(lay, links, B, n_ext, n, orthogonal != 0, out, st);
}

}  // extern "C"
