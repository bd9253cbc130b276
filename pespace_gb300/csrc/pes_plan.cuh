// Plan object shared by the batched-likelihood translation units.
#pragma once

#include <utility>
#include <vector>

#include "pes_abi_common.cuh"
#include "pes_physics.cuh"

namespace pes {

// Cached TDI factors of one bin: delay D = exp(-2 pi i f L), generation prefactor P.
struct __align__(32) TdiFactor {
  double dre, dim, pre, pim;
};

// Device-visible, by-value copy of the plan's constants and data pointers.
struct PlanDev {
  int64_t nbins;
  int64_t k0;
  double f_step;
  double df;
  double f_ref;
  double cut_factor;
  int32_t n_det;
  int32_t chan_mask;
  int32_t approximant;  // PES_APPROX_*
  int32_t pad;
  PesOrbit orbit[PES_MAX_DETECTORS];
  const double2* data;   // [n_det][3][nbins]
  const double* w;       // [n_det][3][nbins] inverse PSD, zero on channels outside chan_mask
  const TdiFactor* tdi;    // [n_det][nbins] (D.re, D.im, P.re, P.im)
  const double* suffix;  // [nbins + 1]: sum over bins >= k of sum_det sum_c |d|^2 w
};

// Per-sample state produced by the set-up kernel.
template <class T>
struct SampleBlock {
  PhenomDCoef<T> wf;
  Polar<T> pol;
  T tc;
  double fcut;
  int64_t kcut;    // bins [0, kcut) carry a model
  int32_t status;  // PES_SAMPLE_*
  int32_t pad;
};

// Mixed-precision plan buffers (allocated only for PES_PRECISION_MIXED).
struct MixedBuffers;

// Kernel classes for the measurement hooks.
enum KernelClass : int {
  kKSetup = 0,
  kKDenseFp64 = 1,
  kKFinalize = 2,
  kKSparse = 3,
  kKSpline = 4,
  kKDenseMixed = 5,
  kKAdjoint = 6,
  kKOther = 7,
};

// Threads per block of the per-sample kernels (set-up, ranges, kink): each
// thread runs a long FP64 chain, and GB300 issues FP64 at 2 lanes per cycle
// per SM, so small blocks spread the samples over all SMs instead of
// queueing 64 lanes on each SM's FP64 pipe.
// The default; a plan's lnL launches use PesPlan::sample_threads, which
// PES_OPT_SAMPLE_THREADS (the autotuner) may change.
constexpr int kPerSampleThreads = 8;

struct Profiler {
  bool enabled = false;
  int64_t launches[PES_KERNEL_CLASSES] = {};
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  std::vector<cudaEvent_t> pool;
  cudaEvent_t take() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
};

}  // namespace pes

struct PesPlan {
  PesPlanDesc desc;
  int device;
  pes::PlanDev dev;
  double2* data = nullptr;
  double* w = nullptr;
  pes::TdiFactor* tdi = nullptr;
  double* suffix = nullptr;
  double* d_row = nullptr;     // [nbins] per-bin sum_det sum_c |d|^2 w (suffix source)
  void* blocks = nullptr;      // per-sample SampleBlock<T> (largest T)
  void* hm_blocks = nullptr;   // per-sample PhenomHMCoef<T> (IMRPhenomHM plans; largest T)
  size_t blocks_bytes = 0;
  double* partial = nullptr;   // [max_batch][nblk][1 + NT]
  size_t partial_len = 0;
  int32_t* status = nullptr;   // [max_batch] internal status when the caller passes NULL
  unsigned data_set_mask = 0;
  pes::MixedBuffers* mixed = nullptr;
  int sample_threads = pes::kPerSampleThreads;  // block size of the per-sample lnL kernels (PES_OPT_SAMPLE_THREADS)
  void* fisher_blocks = nullptr;     // [max_batch] SampleBlock<Dual<11>> (first Fisher call)
  double* fisher_partial = nullptr;  // [max_batch][blocks][66]
  pes::Profiler prof;
};

namespace pes {
// the plan's per-sample IMRPhenomHM mode coefficients in scalar type T (null for IMRPhenomD plans)
template <class T>
inline PhenomHMCoef<T>* hm_blocks(PesPlan* p) {
  return reinterpret_cast<PhenomHMCoef<T>*>(p->hm_blocks);
}

// Brackets one kernel launch for the measurement hooks (a no-op unless enabled).
struct ProfScope {
  PesPlan* p;
  int cls;
  cudaStream_t st;
  cudaEvent_t e1 = nullptr;
  ProfScope(PesPlan* p_, int cls_, cudaStream_t st_) : p(p_), cls(cls_), st(st_) {
    p->prof.launches[cls] += 1;
    if (p->prof.enabled) {
      e1 = p->prof.take();
      cudaEventRecord(e1, st);
    }
  }
  ~ProfScope() {
    if (p->prof.enabled) {
      cudaEvent_t e2 = p->prof.take();
      cudaEventRecord(e2, st);
      p->prof.pending.push_back({cls, {e1, e2}});
    }
  }
};
}  // namespace pes

namespace pes {

constexpr int kGradTangents = 4;  // tangents per gradient pass (3 passes for 11 parameters)


// ------------------------------------------------------------------ scalar helpers
template <class T> struct Seed;
template <> struct Seed<double> {
  PES_HD static double make(double v, int) { return v; }
  static constexpr int N = 0;
};
template <int N, class D, class V> struct Seed<Dual<N, D, V>> {
  PES_HD static Dual<N, D, V> make(double v, int slot) {
    Dual<N, D, V> r = mkdual<N, D, V>(v);
    if (slot >= 0 && slot < N) r.d[slot] = D(1);
    return r;
  }
  static constexpr int NT = N;
};
template <class T> struct NumTangents { static constexpr int value = 0; };
template <int N, class D, class V> struct NumTangents<Dual<N, D, V>> { static constexpr int value = N; };

template <class T> PES_HD void scalar_to(const T& x, double* out);
template <> PES_HD void scalar_to<double>(const double& x, double* out) { out[0] = x; }
template <int N, class D, class V> PES_HD void scalar_to(const Dual<N, D, V>& x, double* out) {
  out[0] = x.v;
#pragma unroll
  for (int i = 0; i < N; ++i) out[1 + i] = x.d[i];
}

// true when parameters are in the model's domain
PES_HD bool theta_in_domain(const double* t) {
  for (int j = 0; j < 11; ++j)
    if (!isfinite(t[j])) return false;
  return t[1] >= 1.0 && t[1] <= 1000.0 && fabs(t[2]) < 1.0 && fabs(t[3]) < 1.0 && fabs(t[5]) <= 1.0 &&
         fabs(t[7]) <= 1.0;
}

// bins [0, kcut) satisfy f <= fcut and Msec f <= mf_max (both monotone in f)
PES_HD int64_t find_kcut(const PlanDev& P, double Msec, double fcut, double mf_max = kMfCut) {
  int64_t lo = 0, hi = P.nbins;  // invariant: live(i) for i < lo, !live(i) for i >= hi
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    double f = (double)(P.k0 + mid) * P.f_step;
    bool live = (f <= fcut) && (Msec * f <= mf_max);
    if (live) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// IMRPhenomHM container of mode k at f, time-shifted by t_c as the reference
// does (antenna.py:435-441): hp, hc times exp(-2 pi i f t_c), tf + t_c.
// False when the mode is above its mapped Mf = 0.2.
template <class T>
__device__ __forceinline__ bool hm_mode_container(const SampleBlock<T>& b, const PhenomHMCoef<T>& h, int k, double f,
                                                  const Cx<T>& ts, Cx<T>& hp, Cx<T>& hc, T& tft) {
  const T Mf = b.wf.Msec * f;
  T amp, psi, tf, f22;
  phenomhm_eval<T>(b.wf, h, k, Mf, amp, psi, tf, &f22);
  if (val(f22) > kMfCut) return false;
  T s, c;
  dsincos(psi, &s, &c);
  // h_lm = amp e^{-i psi}; hp = P h_lm, hc = i C h_lm
  const T ap = h.md[k].P * amp, ac = h.md[k].C * amp;
  hp = cmul(cx(ap * c, -(ap * s)), ts);
  hc = cmul(cx(ac * s, ac * c), ts);
  tft = tf + b.tc;
  return true;
}

// ------------------------------------------------------------------ kernels
// hmb: the samples' IMRPhenomHM mode coefficients (IMRPhenomHM plans; may be null otherwise)
template <class T>
__global__ void k_setup(PlanDev P, const double* __restrict__ theta, int64_t B, int pass,
                        SampleBlock<T>* __restrict__ blocks, PhenomHMCoef<T>* __restrict__ hmb) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= B) return;
  constexpr int NT = NumTangents<T>::value;
  double raw[11];
  for (int j = 0; j < 11; ++j) raw[j] = theta[11 * s + j];
  SampleBlock<T>& b = blocks[s];
  if (!theta_in_domain(raw)) {
    b.status = kSampleOutOfDomain;
    b.kcut = 0;
    b.fcut = 0.0;
    return;
  }
  T th[11];
  for (int j = 0; j < 11; ++j) th[j] = Seed<T>::make(raw[j], NT > 0 ? j - pass * NT : -1);
  phenomd_setup<T>(th, P.f_ref, b.wf);
  const bool hm = P.approximant == PES_APPROX_PHENOMHM;
  if (hm) phenomhm_setup<T>(th, b.wf, hmb[s]);
  T sb = th[7];
  T cb = dsqrt((1.0 - sb) * (1.0 + sb));
  make_polar<T>(th[6], sb, cb, th[8], b.pol);
  b.tc = th[10];
  const double Msec = val(b.wf.Msec);
  const double fmax = (double)(P.k0 + P.nbins - 1) * P.f_step + 1.0;
  double fcut = fmax;
  // the model's cut: cut_factor times the largest ringdown frequency of its modes
  const double frd = hm ? val(hmb[s].fRDmax) : val(b.wf.fRD);
  if (P.cut_factor > 0.0) fcut = fmin(fmax, P.cut_factor * frd / Msec);
  b.fcut = fcut;
  double mf_max = kMfCut;  // PhenomD: zero above Mf = 0.2; HM: each mode above its mapped Mf = 0.2
  if (hm)
    for (int k = 1; k < kHMModes; ++k) {
      const double mk = kMfCut / val(hmb[s].md[k].Rholm);
      mf_max = mk > mf_max ? mk : mf_max;
    }
  b.kcut = find_kcut(P, Msec, fcut, mf_max);
  b.status = kSampleOk;
}


// out[k] = sum_{i >= k} row[i] for k = 0..n (FP64, fixed order; set-up only)
void suffix_sum(int64_t n, const double* row, double* out, cudaStream_t st);

int mixed_create(PesPlan* p);
void mixed_destroy(PesPlan* p);
int mixed_ingest(PesPlan* p, int det, const double* data, const double* psd, cudaStream_t st);
int mixed_model(PesPlan* p, const double* theta_dev, double* out, cudaStream_t st);
int mixed_work(PesPlan* p, int64_t B, const std::vector<int64_t>& kcut, const std::vector<int32_t>& ok,
               int64_t* out, cudaStream_t st);
int mixed_lnl(PesPlan* p, const double* theta, int64_t B, double* lnl, double* grad, int32_t* status,
              cudaStream_t st);
// read (set == 0) or write the dense stage's staging choice of the gradient pass
void mixed_stage_option(PesPlan* p, int set, int64_t* value);
void mixed_refine_option(PesPlan* p, int set, int64_t* value);
}  // namespace pes
