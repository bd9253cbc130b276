// Batched lnL / lnL+gradient plans: set-up, data ingestion and the dense FP64
// path (every bin evaluated in FP64: waveform -> links -> TDI -> residual,
// fused, with a deterministic two-pass reduction per sample).
#include <cstring>
#include <cmath>
#include <cstdlib>
#include <new>

#include "pes_plan.cuh"

namespace pes {

constexpr int kDenseThreads = 128;
constexpr int kDenseBinsPerThread = 4;
constexpr int kDenseBinsPerBlock = kDenseThreads * kDenseBinsPerThread;

// IMRPhenomHM: the six modes' links summed per detector (antenna.py:446-458),
// then TDI; residual sum over detectors and channels.
template <class T>
__device__ __forceinline__ T bin_residual_hm(const PlanDev& P, const SampleBlock<T>& b, const PhenomHMCoef<T>& h,
                                             int64_t i) {
  const double f = (double)(P.k0 + i) * P.f_step;
  Cx<T> ts;
  dsincos((-2.0 * kPi * f) * b.tc, &ts.im, &ts.re);
  T sum = lift<T>(0.0);
  for (int d = 0; d < P.n_det; ++d) {
    Cx<T> La[6];
#pragma unroll
    for (int l = 0; l < 6; ++l) La[l] = cx(lift<T>(0.0), lift<T>(0.0));
#pragma unroll 1
    for (int k = 0; k < kHMModes; ++k) {
      Cx<T> hp, hc, L[6];
      T tft;
      if (!hm_mode_container<T>(b, h, k, f, ts, hp, hc, tft)) continue;
      single_links<T>(P.orbit[d], f, hp, hc, tft, b.pol, L);
#pragma unroll
      for (int l = 0; l < 6; ++l) La[l] = La[l] + L[l];
    }
    Cx<T> C[3];
    const TdiFactor dp = P.tdi[d * P.nbins + i];
    tdi_channels<T>(cx(dp.dre, dp.dim), cx(dp.pre, dp.pim), 1, La, C);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      if (!((P.chan_mask >> ch) & 1)) continue;
      const size_t off = ((size_t)d * 3 + ch) * P.nbins + i;
      const double2 dv = P.data[off];
      T rr = dv.x - C[ch].re, ri = dv.y - C[ch].im;
      sum = sum + (rr * rr + ri * ri) * P.w[off];
    }
  }
  return sum;
}

// Model (A/E/T) of every detector at one dense bin, accumulated into the
// residual sum sum_det sum_c |d - h|^2 w.
template <class T>
__device__ __forceinline__ T bin_residual(const PlanDev& P, const SampleBlock<T>& b, const PhenomHMCoef<T>* h,
                                          int64_t i) {
  if (P.approximant == PES_APPROX_PHENOMHM) return bin_residual_hm<T>(P, b, *h, i);
  const double f = (double)(P.k0 + i) * P.f_step;
  T Mf = b.wf.Msec * f;
  T amp, psi, tf;
  phenomd_eval<T>(b.wf, Mf, amp, psi, tf);
  T s, c;
  dsincos(psi, &s, &c);
  T ap = b.wf.pfac * amp, ac = b.wf.cfac * amp;
  Cx<T> hp = cx(ap * c, -(ap * s));
  Cx<T> hc = cx(-(ac * s), -(ac * c));
  Cx<T> ts;
  dsincos((-2.0 * kPi * f) * b.tc, &ts.im, &ts.re);
  hp = cmul(hp, ts);
  hc = cmul(hc, ts);
  T tft = tf + b.tc;
  T sum = lift<T>(0.0);
  for (int d = 0; d < P.n_det; ++d) {
    Cx<T> L[6], C[3];
    single_links<T>(P.orbit[d], f, hp, hc, tft, b.pol, L);
    const TdiFactor dp = P.tdi[d * P.nbins + i];
    tdi_channels<T>(cx(dp.dre, dp.dim), cx(dp.pre, dp.pim), 1, L, C);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      if (!((P.chan_mask >> ch) & 1)) continue;
      const size_t off = ((size_t)d * 3 + ch) * P.nbins + i;
      const double2 dv = P.data[off];
      T rr = dv.x - C[ch].re, ri = dv.y - C[ch].im;
      sum = sum + (rr * rr + ri * ri) * P.w[off];
    }
  }
  return sum;
}

template <class T>
__global__ void __launch_bounds__(kDenseThreads) k_dense_fp64(PlanDev P, const SampleBlock<T>* __restrict__ blocks,
                                                              const PhenomHMCoef<T>* __restrict__ hmb, int nblk,
                                                              double* __restrict__ partial) {
  constexpr int NV = 1 + NumTangents<T>::value;
  __shared__ SampleBlock<T> sb;
  __shared__ double red[kDenseThreads / 32][NV];
  const int s = blockIdx.y;
  {
    const int n8 = sizeof(SampleBlock<T>) / 8;
    const double* src = reinterpret_cast<const double*>(&blocks[s]);
    double* dst = reinterpret_cast<double*>(&sb);
    for (int j = threadIdx.x; j < n8; j += blockDim.x) dst[j] = src[j];
  }
  __syncthreads();
  T acc = lift<T>(0.0);
  if (sb.status == kSampleOk) {
    const int64_t base = (int64_t)blockIdx.x * kDenseBinsPerBlock + threadIdx.x;
#pragma unroll 1
    for (int j = 0; j < kDenseBinsPerThread; ++j) {
      const int64_t i = base + (int64_t)j * kDenseThreads;
      if (i < sb.kcut) acc = acc + bin_residual<T>(P, sb, hmb ? hmb + s : nullptr, i);
    }
  }
  double v[NV];
  scalar_to(acc, v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int c = 0; c < NV; ++c) {
    double x = v[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (l == 0) red[w][c] = x;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double x = 0.0;
#pragma unroll
    for (int k = 0; k < kDenseThreads / 32; ++k) x += red[k][threadIdx.x];
    partial[((size_t)s * nblk + blockIdx.x) * NV + threadIdx.x] = x;
  }
}

template <class T>
__global__ void k_finalize(PlanDev P, const SampleBlock<T>* __restrict__ blocks, int64_t B, int nblk,
                           const double* __restrict__ partial, int pass, double* __restrict__ lnl,
                           double* __restrict__ grad, int32_t* __restrict__ status) {
  constexpr int NT = NumTangents<T>::value;
  constexpr int NV = 1 + NT;
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= B) return;
  const SampleBlock<T>& b = blocks[s];
  if (b.status != kSampleOk) {
    if (pass == 0) {
      lnl[s] = -INFINITY;
      if (status) status[s] = b.status;
    }
    if (grad)
      for (int j = 0; j < NT; ++j)
        if (pass * NT + j < 11) grad[11 * s + pass * NT + j] = 0.0;
    return;
  }
  double acc[NV];
  for (int c = 0; c < NV; ++c) acc[c] = 0.0;
  for (int k = 0; k < nblk; ++k)
    for (int c = 0; c < NV; ++c) acc[c] += partial[((size_t)s * nblk + k) * NV + c];
  const double scale = -2.0 * P.df;
  if (pass == 0) {
    double v = scale * (acc[0] + P.suffix[b.kcut]);
    lnl[s] = v;
    if (status) status[s] = isfinite(v) ? kSampleOk : kSampleNonFinite;
  }
  if (grad)
    for (int j = 0; j < NT; ++j)
      if (pass * NT + j < 11) grad[11 * s + pass * NT + j] = scale * acc[1 + j];
}

// Dense A/E/T (or X/Y/Z) model of one detector (parity/debug path).
__global__ void k_model_tdi(PlanDev P, const SampleBlock<double>* __restrict__ blocks,
                            const PhenomHMCoef<double>* __restrict__ hmb, int det, int orth, double2* __restrict__ out) {
  __shared__ SampleBlock<double> sb;
  if (threadIdx.x == 0) sb = blocks[0];
  __syncthreads();
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.nbins) return;
  Cx<double> C[3] = {cx(0.0, 0.0), cx(0.0, 0.0), cx(0.0, 0.0)};
  if (sb.status == kSampleOk && i < sb.kcut && P.approximant == PES_APPROX_PHENOMHM) {
    const double f = (double)(P.k0 + i) * P.f_step;
    Cx<double> ts, La[6];
    dsincos((-2.0 * kPi * f) * sb.tc, &ts.im, &ts.re);
    for (int l = 0; l < 6; ++l) La[l] = cx(0.0, 0.0);
    for (int k = 0; k < kHMModes; ++k) {
      Cx<double> hp, hc, L[6];
      double tft;
      if (!hm_mode_container<double>(sb, hmb[0], k, f, ts, hp, hc, tft)) continue;
      single_links<double>(P.orbit[det], f, hp, hc, tft, sb.pol, L);
      for (int l = 0; l < 6; ++l) La[l] = La[l] + L[l];
    }
    const TdiFactor dp = P.tdi[det * P.nbins + i];
    tdi_channels<double>(cx(dp.dre, dp.dim), cx(dp.pre, dp.pim), orth, La, C);
  } else if (sb.status == kSampleOk && i < sb.kcut) {
    const double f = (double)(P.k0 + i) * P.f_step;
    double Mf = sb.wf.Msec * f;
    double amp, psi, tf, s, c;
    phenomd_eval<double>(sb.wf, Mf, amp, psi, tf);
    dsincos(psi, &s, &c);
    double ap = sb.wf.pfac * amp, ac = sb.wf.cfac * amp;
    Cx<double> hp = cx(ap * c, -(ap * s)), hc = cx(-(ac * s), -(ac * c)), ts;
    dsincos((-2.0 * kPi * f) * sb.tc, &ts.im, &ts.re);
    Cx<double> L[6];
    single_links<double>(P.orbit[det], f, cmul(hp, ts), cmul(hc, ts), tf + sb.tc, sb.pol, L);
    const TdiFactor dp = P.tdi[det * P.nbins + i];
    tdi_channels<double>(cx(dp.dre, dp.dim), cx(dp.pre, dp.pim), orth, L, C);
  }
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) out[ch * P.nbins + i] = make_double2(C[ch].re, C[ch].im);
}

// Data ingestion: inverse PSD (masked), TDI factor cache, per-bin |d|^2 w rows.
__global__ void k_ingest(PlanDev P, int det, int gen20, const double2* __restrict__ d_in,
                         const double* __restrict__ psd_in, double2* __restrict__ data, double* __restrict__ w,
                         TdiFactor* __restrict__ tdi) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.nbins) return;
  const double f = (double)(P.k0 + i) * P.f_step;
  Cx<double> D, Pf;
  tdi_factors(f, P.orbit[det].arm_sec, gen20, D, Pf);
  tdi[det * P.nbins + i] = TdiFactor{D.re, D.im, Pf.re, Pf.im};
  for (int ch = 0; ch < 3; ++ch) {
    const size_t off = ((size_t)det * 3 + ch) * P.nbins + i;
    data[off] = d_in[ch * P.nbins + i];
    w[off] = ((P.chan_mask >> ch) & 1) ? 1.0 / psd_in[ch * P.nbins + i] : 0.0;
  }
}

__global__ void k_row_norm(PlanDev P, const double2* __restrict__ data, const double* __restrict__ w,
                           double* __restrict__ row) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.nbins) return;
  double acc = 0.0;
  for (int d = 0; d < P.n_det; ++d)
    for (int ch = 0; ch < 3; ++ch) {
      const size_t off = ((size_t)d * 3 + ch) * P.nbins + i;
      const double2 v = data[off];
      acc += (v.x * v.x + v.y * v.y) * w[off];
    }
  row[i] = acc;
}

// suffix[k] = sum_{i >= k} row[i] (set-up only): one block; every thread sums
// its contiguous chunk, thread 0 turns the chunk totals into the carries from
// the chunks above (fixed order), and every thread writes its chunk.
constexpr int kSuffixThreads = 1024;
__global__ void __launch_bounds__(kSuffixThreads) k_suffix(int64_t n, const double* __restrict__ row,
                                                           double* __restrict__ suffix) {
  __shared__ double part[kSuffixThreads];
  const int t = threadIdx.x;
  const int64_t chunk = (n + kSuffixThreads - 1) / kSuffixThreads;
  const int64_t lo = min(n, (int64_t)t * chunk), hi = min(n, lo + chunk);
  double acc = 0.0;
  for (int64_t i = hi - 1; i >= lo; --i) acc += row[i];
  part[t] = acc;
  __syncthreads();
  if (t == 0) {
    double c = 0.0;
    for (int u = kSuffixThreads - 1; u >= 0; --u) {
      const double v = part[u];
      part[u] = c;
      c += v;
    }
    suffix[n] = 0.0;
  }
  __syncthreads();
  double c = part[t];
  for (int64_t i = hi - 1; i >= lo; --i) {
    c += row[i];
    suffix[i] = c;
  }
}

void suffix_sum(int64_t n, const double* row, double* out, cudaStream_t st) {
  k_suffix<<<1, kSuffixThreads, 0, st>>>(n, row, out);
}

// ------------------------------------------------------------------ host driver
template <class T>
int run_dense(PesPlan* p, const double* theta, int64_t B, int pass, double* lnl, double* grad, int32_t* status,
              cudaStream_t st) {
  SampleBlock<T>* blocks = reinterpret_cast<SampleBlock<T>*>(p->blocks);
  {
    ProfScope ps(p, kKSetup, st);
    k_setup<T><<<ceil_div(B, p->sample_threads), p->sample_threads, 0, st>>>(p->dev, theta, B, pass, blocks,
                                                                            hm_blocks<T>(p));
  }
  PES_CHECK_LAUNCH();
  const int nblk = (int)ceil_div(p->desc.nbins, kDenseBinsPerBlock);
  dim3 grid(nblk, (unsigned)B);
  {
    ProfScope ps(p, kKDenseFp64, st);
    k_dense_fp64<T><<<grid, kDenseThreads, 0, st>>>(p->dev, blocks, hm_blocks<T>(p), nblk, p->partial);
  }
  PES_CHECK_LAUNCH();
  {
    ProfScope ps(p, kKFinalize, st);
    k_finalize<T><<<ceil_div(B, 64), 64, 0, st>>>(p->dev, blocks, B, nblk, p->partial, pass, lnl, grad, status);
  }
  PES_CHECK_LAUNCH();
  return PES_OK;
}

}  // namespace pes

using namespace pes;

extern "C" {

int pes_plan_create(const PesPlanDesc* desc, PesPlan** out) {
  PES_REQUIRE(desc && out, "pes_plan_create: null pointer");
  *out = nullptr;
  PES_REQUIRE(desc->nbins > 0 && desc->nbins < (int64_t(1) << 31), "pes_plan_create: nbins out of range");
  PES_REQUIRE(desc->n_det >= 1 && desc->n_det <= PES_MAX_DETECTORS, "pes_plan_create: n_det must be 1..%d",
              PES_MAX_DETECTORS);
  PES_REQUIRE(desc->chan_mask >= 1 && desc->chan_mask <= 7, "pes_plan_create: chan_mask must be 1..7");
  PES_REQUIRE(desc->precision == PES_PRECISION_FP64 || desc->precision == PES_PRECISION_MIXED,
              "pes_plan_create: unknown precision %d", desc->precision);
  PES_REQUIRE(desc->max_batch >= 1 && desc->max_batch <= 65535, "pes_plan_create: max_batch must be 1..65535");
  PES_REQUIRE(desc->approximant == PES_APPROX_PHENOMD || desc->approximant == PES_APPROX_PHENOMHM,
              "pes_plan_create: unknown approximant %d", desc->approximant);
  PES_REQUIRE(desc->f_step > 0 && desc->df > 0, "pes_plan_create: f_step and df must be positive");
  for (int d = 0; d < desc->n_det; ++d) {
    PES_REQUIRE(desc->det[d].generation == 15 || desc->det[d].generation == 20,
                "pes_plan_create: detector %d generation must be 15 or 20", d);
    PES_REQUIRE(desc->det[d].orbit.kind == 0 || desc->det[d].orbit.kind == 1,
                "pes_plan_create: detector %d orbit kind", d);
  }
  PesPlan* p = new (std::nothrow) PesPlan();
  if (!p) return PES_ENOMEM;
  p->desc = *desc;
  cudaGetDevice(&p->device);
  PlanDev& D = p->dev;
  D.nbins = desc->nbins;
  D.k0 = desc->k0;
  D.f_step = desc->f_step;
  D.df = desc->df;
  D.f_ref = desc->f_ref;
  D.cut_factor = desc->cut_factor;
  D.n_det = desc->n_det;
  D.chan_mask = desc->chan_mask;
  D.approximant = desc->approximant;
  D.pad = 0;
  for (int d = 0; d < desc->n_det; ++d) D.orbit[d] = desc->det[d].orbit;
  const int64_t n = desc->nbins;
  const int nd = desc->n_det;
  const int64_t B = desc->max_batch;
  const int nblk = (int)ceil_div(n, kDenseBinsPerBlock);
  p->blocks_bytes = (size_t)B * sizeof(SampleBlock<Dual<kGradTangents>>);
  p->partial_len = (size_t)B * nblk * (1 + kGradTangents);
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = cudaMalloc(&p->data, sizeof(double2) * nd * 3 * n);
  if (e == cudaSuccess) e = cudaMalloc(&p->w, sizeof(double) * nd * 3 * n);
  if (e == cudaSuccess) e = cudaMalloc(&p->tdi, sizeof(TdiFactor) * nd * n);
  if (e == cudaSuccess) e = cudaMalloc(&p->suffix, sizeof(double) * (n + 1));
  if (e == cudaSuccess) e = cudaMalloc(&p->d_row, sizeof(double) * n);
  if (e == cudaSuccess) e = cudaMalloc(&p->blocks, p->blocks_bytes);
  if (e == cudaSuccess && desc->approximant == PES_APPROX_PHENOMHM)  // the largest scalar: the Fisher duals
    e = cudaMalloc(&p->hm_blocks, (size_t)B * sizeof(PhenomHMCoef<Dual<11>>));
  if (e == cudaSuccess && desc->precision == PES_PRECISION_FP64)
    e = cudaMalloc(&p->partial, sizeof(double) * p->partial_len);
  if (e == cudaSuccess) e = cudaMalloc(&p->status, sizeof(int32_t) * B);
  if (e != cudaSuccess) {
    set_error("pes_plan_create: cudaMalloc failed: %s", cudaGetErrorString(e));
    pes_plan_destroy(p);
    return PES_ENOMEM;
  }
  cudaMemset(p->data, 0, sizeof(double2) * nd * 3 * n);
  cudaMemset(p->w, 0, sizeof(double) * nd * 3 * n);
  D.data = p->data;
  D.w = p->w;
  D.tdi = p->tdi;
  D.suffix = p->suffix;
  if (desc->precision == PES_PRECISION_MIXED) {
    int rc = mixed_create(p);
    if (rc != PES_OK) {
      pes_plan_destroy(p);
      return rc;
    }
  }
  *out = p;
  return PES_OK;
}

int pes_plan_destroy(PesPlan* p) {
  if (!p) return PES_OK;
  for (auto& e : p->prof.pending) {
    cudaEventDestroy(e.second.first);
    cudaEventDestroy(e.second.second);
  }
  for (auto e : p->prof.pool) cudaEventDestroy(e);
  if (p->mixed) mixed_destroy(p);
  cudaFree(p->fisher_blocks);
  cudaFree(p->fisher_partial);
  cudaFree(p->data);
  cudaFree(p->w);
  cudaFree(p->tdi);
  cudaFree(p->suffix);
  cudaFree(p->d_row);
  cudaFree(p->blocks);
  if (p->hm_blocks) cudaFree(p->hm_blocks);
  cudaFree(p->partial);
  cudaFree(p->status);
  delete p;
  return PES_OK;
}

int pes_plan_set_data(PesPlan* p, int32_t det, const double* data, const double* psd, void* stream) {
  PES_REQUIRE(p, "pes_plan_set_data: null plan");
  PES_REQUIRE(det >= 0 && det < p->desc.n_det, "pes_plan_set_data: detector %d out of range", det);
  PES_REQUIRE(data && psd, "pes_plan_set_data: null pointer");
  cudaStream_t st = as_stream(stream);
  const int64_t n = p->desc.nbins;
  k_ingest<<<ceil_div(n, 256), 256, 0, st>>>(p->dev, det, p->desc.det[det].generation == 20,
                                             reinterpret_cast<const double2*>(data), psd, p->data, p->w, p->tdi);
  PES_CHECK_LAUNCH();
  k_row_norm<<<ceil_div(n, 256), 256, 0, st>>>(p->dev, p->data, p->w, p->d_row);
  PES_CHECK_LAUNCH();
  k_suffix<<<1, kSuffixThreads, 0, st>>>(n, p->d_row, p->suffix);
  PES_CHECK_LAUNCH();
  p->data_set_mask |= 1u << det;
  if (p->mixed) {
    int rc = mixed_ingest(p, det, data, psd, st);
    if (rc != PES_OK) return rc;
  }
  PES_CHECK_CUDA(cudaStreamSynchronize(st));
  return PES_OK;
}

static int check_batch(PesPlan* p, const double* theta, int64_t B, const double* lnl) {
  PES_REQUIRE(p, "null plan");
  PES_REQUIRE(B >= 0 && B <= p->desc.max_batch, "batch size %lld outside [0, max_batch=%d]", (long long)B,
              p->desc.max_batch);
  PES_REQUIRE(B == 0 || (theta && lnl), "null theta or lnl");
  unsigned need = (1u << p->desc.n_det) - 1u;
  PES_REQUIRE((p->data_set_mask & need) == need, "data not set for every detector (pes_plan_set_data)");
  return PES_OK;
}

int pes_lnl_batch(PesPlan* p, const double* theta, int64_t B, double* lnl, int32_t* status, void* stream) {
  int rc = check_batch(p, theta, B, lnl);
  if (rc != PES_OK) return rc;
  if (B == 0) return PES_OK;
  cudaStream_t st = as_stream(stream);
  if (p->desc.precision == PES_PRECISION_MIXED) return mixed_lnl(p, theta, B, lnl, nullptr, status, st);
  return run_dense<double>(p, theta, B, 0, lnl, nullptr, status, st);
}

int pes_lnl_grad_batch(PesPlan* p, const double* theta, int64_t B, double* lnl, double* grad, int32_t* status,
                       void* stream) {
  int rc = check_batch(p, theta, B, lnl);
  if (rc != PES_OK) return rc;
  PES_REQUIRE(B == 0 || grad, "pes_lnl_grad_batch: null grad");
  if (B == 0) return PES_OK;
  cudaStream_t st = as_stream(stream);
  if (p->desc.precision == PES_PRECISION_MIXED) return mixed_lnl(p, theta, B, lnl, grad, status, st);
  constexpr int NT = kGradTangents;
  for (int pass = 0; pass * NT < 11; ++pass) {
    rc = run_dense<Dual<NT>>(p, theta, B, pass, lnl, grad, status, st);
    if (rc != PES_OK) return rc;
  }
  return PES_OK;
}

int pes_plan_model_tdi(PesPlan* p, int32_t det, int32_t orthogonal, const double* theta, double* out,
                       void* stream) {
  PES_REQUIRE(p && theta && out, "pes_plan_model_tdi: null pointer");
  PES_REQUIRE(det >= 0 && det < p->desc.n_det, "pes_plan_model_tdi: detector out of range");
  PES_REQUIRE(p->desc.precision == PES_PRECISION_FP64 || orthogonal,
              "pes_plan_model_tdi: mixed plans model the A/E/T channels only");
  cudaStream_t st = as_stream(stream);
  double* d_theta = nullptr;
  PES_CHECK_CUDA(cudaMallocAsync(&d_theta, 11 * sizeof(double), st));
  PES_CHECK_CUDA(cudaMemcpyAsync(d_theta, theta, 11 * sizeof(double), cudaMemcpyHostToDevice, st));
  if (p->desc.precision == PES_PRECISION_MIXED) {
    const size_t n3 = (size_t)3 * p->desc.nbins;
    double* all = nullptr;
    PES_CHECK_CUDA(cudaMallocAsync(&all, sizeof(double2) * p->desc.n_det * n3, st));
    int rc = mixed_model(p, d_theta, all, st);
    if (rc != PES_OK) return rc;
    PES_CHECK_CUDA(cudaMemcpyAsync(out, all + 2 * n3 * det, sizeof(double2) * n3, cudaMemcpyDeviceToDevice, st));
    PES_CHECK_CUDA(cudaFreeAsync(all, st));
    PES_CHECK_CUDA(cudaFreeAsync(d_theta, st));
    return PES_OK;
  }
  SampleBlock<double>* blocks = reinterpret_cast<SampleBlock<double>*>(p->blocks);
  k_setup<double><<<1, 1, 0, st>>>(p->dev, d_theta, 1, 0, blocks, hm_blocks<double>(p));
  PES_CHECK_LAUNCH();
  k_model_tdi<<<ceil_div(p->desc.nbins, 128), 128, 0, st>>>(p->dev, blocks, hm_blocks<double>(p), det, orthogonal != 0,
                                                            reinterpret_cast<double2*>(out));
  PES_CHECK_LAUNCH();
  PES_CHECK_CUDA(cudaFreeAsync(d_theta, st));
  return PES_OK;
}

int pes_plan_profile(PesPlan* p, int32_t enable) {
  PES_REQUIRE(p, "pes_plan_profile: null plan");
  p->prof.enabled = enable != 0;
  return PES_OK;
}

int pes_plan_set_option(PesPlan* p, int32_t option, int64_t value) {
  PES_REQUIRE(p, "pes_plan_set_option: null plan");
  switch (option) {
    case PES_OPT_DENSE_STAGE:
      PES_REQUIRE(value == 0 || value == 1, "pes_plan_set_option: PES_OPT_DENSE_STAGE takes 0 or 1, got %lld",
                  (long long)value);
      if (p->mixed) mixed_stage_option(p, 1, &value);
      return PES_OK;
    case PES_OPT_SAMPLE_THREADS:
      PES_REQUIRE(value >= 1 && value <= 128, "pes_plan_set_option: PES_OPT_SAMPLE_THREADS takes 1..128, got %lld",
                  (long long)value);
      p->sample_threads = (int)value;
      return PES_OK;
    case PES_OPT_REFINE_ALL:
      PES_REQUIRE(value == 0 || value == 1, "pes_plan_set_option: PES_OPT_REFINE_ALL takes 0 or 1, got %lld",
                  (long long)value);
      if (p->mixed) mixed_refine_option(p, 1, &value);
      return PES_OK;
    default:
      break;
  }
  ::pes::set_error("pes_plan_set_option: unknown option %d", option);
  return PES_EINVAL;
}

int pes_plan_get_option(PesPlan* p, int32_t option, int64_t* value) {
  PES_REQUIRE(p && value, "pes_plan_get_option: null pointer");
  switch (option) {
    case PES_OPT_DENSE_STAGE:
      *value = 0;
      if (p->mixed) mixed_stage_option(p, 0, value);
      return PES_OK;
    case PES_OPT_SAMPLE_THREADS:
      *value = p->sample_threads;
      return PES_OK;
    case PES_OPT_REFINE_ALL:
      *value = 0;
      if (p->mixed) mixed_refine_option(p, 0, value);
      return PES_OK;
    default:
      break;
  }
  ::pes::set_error("pes_plan_get_option: unknown option %d", option);
  return PES_EINVAL;
}

int pes_plan_stats(PesPlan* p, int64_t* launches, double* device_ms) {
  PES_REQUIRE(p && launches && device_ms, "pes_plan_stats: null pointer");
  for (int k = 0; k < PES_KERNEL_CLASSES; ++k) {
    launches[k] = p->prof.launches[k];
    device_ms[k] = 0.0;
    p->prof.launches[k] = 0;
  }
  for (auto& e : p->prof.pending) {
    float ms = 0.0f;
    PES_CHECK_CUDA(cudaEventSynchronize(e.second.second));
    PES_CHECK_CUDA(cudaEventElapsedTime(&ms, e.second.first, e.second.second));
    device_ms[e.first] += ms;
    p->prof.pool.push_back(e.second.first);
    p->prof.pool.push_back(e.second.second);
  }
  p->prof.pending.clear();
  return PES_OK;
}

int pes_plan_work(PesPlan* p, int64_t B, int64_t* out, void* stream) {
  PES_REQUIRE(p && out, "pes_plan_work: null pointer");
  PES_REQUIRE(B >= 0 && B <= p->desc.max_batch, "pes_plan_work: B must be 0..max_batch");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  PES_CHECK_CUDA(cudaStreamSynchronize(st));
  // the forward set-up blocks hold kcut and status at the same offsets for every scalar type
  std::vector<unsigned char> raw((size_t)B * sizeof(SampleBlock<double>));
  if (B > 0) PES_CHECK_CUDA(cudaMemcpy(raw.data(), p->blocks, raw.size(), cudaMemcpyDeviceToHost));
  std::vector<int64_t> kcut(B);
  std::vector<int32_t> ok(B);
  for (int64_t s = 0; s < B; ++s) {
    SampleBlock<double> b;
    std::memcpy(&b, raw.data() + (size_t)s * sizeof(SampleBlock<double>), sizeof(b));
    ok[s] = b.status == kSampleOk;
    kcut[s] = ok[s] ? b.kcut : 0;
  }
  for (int k = 0; k < 6; ++k) out[k] = 0;
  for (int64_t s = 0; s < B; ++s) out[3] += ok[s];
  if (p->desc.precision == PES_PRECISION_MIXED) return mixed_work(p, B, kcut, ok, out, st);
  for (int64_t s = 0; s < B; ++s) out[1] += kcut[s] * p->desc.n_det;
  return PES_OK;
}

const char* pes_kernel_class_name(int32_t k) {
  static const char* names[PES_KERNEL_CLASSES] = {"setup", "dense_fp64", "finalize", "sparse_stage",
                                                  "spline", "dense_mixed", "adjoint", "other"};
  return (k >= 0 && k < PES_KERNEL_CLASSES) ? names[k] : "";
}

}  // extern "C"
