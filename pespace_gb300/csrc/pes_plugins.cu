// Granular drop-in entry points: one per reference plugin method (orbit
// vectors, single-link response, TDI combination, Whittle likelihood) plus the
// IMRPhenomD waveform producer.  FP64 throughout, one thread per frequency.
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

}  // namespace pes

using namespace pes;

// ------------------------------------------------------------------ C ABI
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

}  // extern "C"
