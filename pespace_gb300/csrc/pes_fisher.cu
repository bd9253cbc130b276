// Fisher matrices of the batched plans, pespace/inference/fisher.py:27-162:
// F_ij = 4 df Re sum_{det, c, f} conj(dh_i) dh_j / S_c(f).  FP64 plans take
// the derivatives of the A/E/T model with respect to the 11 parameters by
// forward-mode dual numbers in FP64 at every live bin (the same per-bin model
// as the FP64 plan; IMRPhenomHM: the six modes' links summed per detector);
// mixed IMRPhenomD plans by FP32 duals with the model's structure
// (k_fisher_fast below), mixed IMRPhenomHM plans as the FP64 ones.
// A block of 64 threads evaluates 64 bins of one detector, stores
// sqrt(w) dh in shared memory, and its threads then form the 66 pair sums of
// those bins; per-block partials are summed in a fixed order.
#include "pes_plan.cuh"

namespace pes {

constexpr int kFisherThreads = 64;
constexpr int kFisherBlocks = 48;  // blocks per sample, grid-stride over the live bins
constexpr int kPairs = 66;         // a <= b of 11 parameters
using FisherScalar = Dual<11>;

__device__ __forceinline__ void pair_of(int p, int& a, int& b) {
  a = 0;
  while (p >= 11 - a) {
    p -= 11 - a;
    ++a;
  }
  b = a + p;
}

// hmb: the samples' IMRPhenomHM mode coefficients (IMRPhenomHM plans: the
// six modes' links summed per detector, antenna.py:446-458), else null.
__global__ void __launch_bounds__(kFisherThreads) k_fisher_bins(PlanDev P,
                                                                const SampleBlock<FisherScalar>* __restrict__ blocks,
                                                                const PhenomHMCoef<FisherScalar>* __restrict__ hmb,
                                                                double* __restrict__ partial) {
  using T = FisherScalar;
  __shared__ SampleBlock<T> sb;
  __shared__ double dh[kFisherThreads][3][22];  // sqrt(w) dRe h / dtheta_a, then sqrt(w) dIm h / dtheta_a
  const int s = blockIdx.y, t = threadIdx.x;
  {
    const int n8 = sizeof(SampleBlock<T>) / 8;
    const double* src = reinterpret_cast<const double*>(&blocks[s]);
    double* dst = reinterpret_cast<double*>(&sb);
    for (int j = t; j < n8; j += kFisherThreads) dst[j] = src[j];
  }
  __syncthreads();
  int pa[2], pb[2];
  bool own[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int p = t + k * kFisherThreads;
    own[k] = p < kPairs;
    pair_of(own[k] ? p : 0, pa[k], pb[k]);
  }
  double acc[2] = {0.0, 0.0};
  if (sb.status == kSampleOk) {
    for (int64_t base = (int64_t)blockIdx.x * kFisherThreads; base < sb.kcut;
         base += (int64_t)gridDim.x * kFisherThreads) {
      const int64_t i = base + t;
      const bool live = i < sb.kcut;
      const double f = (double)(P.k0 + (live ? i : 0)) * P.f_step;
      Cx<T> hp, hc, ts;
      T tft;
      if (live) {
        dsincos((-2.0 * kPi * f) * sb.tc, &ts.im, &ts.re);
        if (!hmb) {
          T Mf = sb.wf.Msec * f;
          T amp, psi, tf;
          phenomd_eval<T>(sb.wf, Mf, amp, psi, tf);
          T sn, cs;
          dsincos(psi, &sn, &cs);
          T ap = sb.wf.pfac * amp, ac = sb.wf.cfac * amp;
          hp = cx(ap * cs, -(ap * sn));
          hc = cx(-(ac * sn), -(ac * cs));
          hp = cmul(hp, ts);
          hc = cmul(hc, ts);
          tft = tf + sb.tc;
        }
      }
      for (int d = 0; d < P.n_det; ++d) {
        if (live) {
          Cx<T> L[6], C[3];
          if (hmb) {
#pragma unroll
            for (int l = 0; l < 6; ++l) L[l] = cx(lift<T>(0.0), lift<T>(0.0));
#pragma unroll 1
            for (int k = 0; k < kHMModes; ++k) {
              Cx<T> mhp, mhc, Lk[6];
              T mtft;
              if (!hm_mode_container<T>(sb, hmb[s], k, f, ts, mhp, mhc, mtft)) continue;
              single_links<T>(P.orbit[d], f, mhp, mhc, mtft, sb.pol, Lk);
#pragma unroll
              for (int l = 0; l < 6; ++l) L[l] = L[l] + Lk[l];
            }
          } else {
            single_links<T>(P.orbit[d], f, hp, hc, tft, sb.pol, L);
          }
          const TdiFactor dp = P.tdi[d * P.nbins + i];
          tdi_channels<T>(cx(dp.dre, dp.dim), cx(dp.pre, dp.pim), 1, L, C);
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const double sw = sqrt(P.w[((size_t)d * 3 + c) * P.nbins + i]);  // zero off the channel mask
#pragma unroll
            for (int a = 0; a < 11; ++a) {
              dh[t][c][a] = sw * C[c].re.d[a];
              dh[t][c][11 + a] = sw * C[c].im.d[a];
            }
          }
        } else {
#pragma unroll
          for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int a = 0; a < 22; ++a) dh[t][c][a] = 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          if (!own[k]) continue;
          const int a = pa[k], b = pb[k];
          double x = 0.0;
          for (int u = 0; u < kFisherThreads; ++u)
#pragma unroll
            for (int c = 0; c < 3; ++c) x += dh[u][c][a] * dh[u][c][b] + dh[u][c][11 + a] * dh[u][c][11 + b];
          acc[k] += x;
        }
        __syncthreads();
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 2; ++k)
    if (own[k]) partial[((size_t)s * gridDim.x + blockIdx.x) * kPairs + t + k * kFisherThreads] = acc[k];
}

__global__ void k_fisher_final(const SampleBlock<FisherScalar>* __restrict__ blocks, int64_t B, int nblk,
                               double scale, const double* __restrict__ partial, double* __restrict__ fisher,
                               int32_t* __restrict__ status) {
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (tid >= B * kPairs) return;
  const int64_t s = tid / kPairs;
  const int p = (int)(tid % kPairs);
  int a, b;
  pair_of(p, a, b);
  const bool ok = blocks[s].status == kSampleOk;
  double x = 0.0;
  for (int k = 0; k < nblk; ++k) x += partial[((size_t)s * nblk + k) * kPairs + p];
  const double v = ok ? scale * x : NAN;
  fisher[s * 121 + a * 11 + b] = v;
  fisher[s * 121 + b * 11 + a] = v;
  if (status && p == 0) status[s] = blocks[s].status;
}

// Fisher matrices of mixed plans in FP32, by the structure of the model:
// h_c = A Y_c(T, lambda, sin beta, psi, cos iota) exp(-i phase), T = t(f) + t_c,
// phase = Psi + 2 pi f (k.x0(T, lambda, sin beta) + t_c), with A, Psi, t(f)
// depending on the mass and spin parameters only.  Its derivatives are
//   dh/dtheta = (d(A Y)/dtheta - i A Y dphase/dtheta) exp(-i phase),
// and the phase factor cancels in conj(dh_a) dh_b, so the Fisher needs no
// phase values: PhenomD runs with FP32 duals over the four mass/spin
// parameters (A, dPsi, dt), the response per unit amplitude with FP32 duals
// over (T, lambda, sin beta, psi, cos iota); ln D_L and phi_c are analytic
// (dh = -h and 2 i h).  A block of 128 threads evaluates 128 bins of one
// detector, stores sqrt(w) times the 11 complex derivatives in shared memory,
// and threads 0..65 each sum one pair over those bins (FP32 within the block,
// FP64 across blocks, fixed order).  Amplitudes are scaled by
// PC / (MRSUN MTSUN) and the weights by its inverse square to stay in FP32 range.
constexpr int kFastThreads = 128;
// ln Mc, q, chi_1, chi_2: float-float values and tangents (the phase tangents
// are sums of large cancelling terms; FP32 tangents left 1e-4 errors in F_qq
// at mass ratios near 7)
using FM = Dual<4, FF, FF>;
using FR = DualS<5>;  // T, lambda, sin beta, psi, cos iota

struct FisherFastBlock {
  PhenomDCoef<FM> wf;
  Polar<FR> pol;
  FR pfac, cfac;
  float tc;
  int32_t status;
  int64_t kcut;
};

__global__ void __launch_bounds__(kFastThreads) k_fisher_fast(PlanDev P,
                                                              const SampleBlock<FisherScalar>* __restrict__ blocks,
                                                              double* __restrict__ partial) {
  __shared__ FisherFastBlock sb;
  __shared__ OrbitF orb[PES_MAX_DETECTORS];
  __shared__ float dh[kFastThreads][3][22];  // sqrt(w) dRe h / dtheta_a, then sqrt(w) dIm h / dtheta_a
  const int s = blockIdx.y, t = threadIdx.x;
  {
    // narrow the FP64 coefficient block (11 tangents in parameter order)
    const SampleBlock<FisherScalar>& g = blocks[s];
    constexpr int nwf = (int)(sizeof(PhenomDCoef<FisherScalar>) / sizeof(FisherScalar));
    constexpr int npol = (int)(sizeof(Polar<FisherScalar>) / sizeof(FisherScalar));
    static_assert(sizeof(PhenomDCoef<FM>) / sizeof(FM) == nwf, "coefficient block must be an array of scalars");
    static_assert(sizeof(Polar<FR>) / sizeof(FR) == npol, "polarisation block must be an array of scalars");
    const FisherScalar* ws = reinterpret_cast<const FisherScalar*>(&g.wf);
    FM* wd = reinterpret_cast<FM*>(&sb.wf);
    for (int k = t; k < nwf; k += blockDim.x) {
      wd[k].v = ff_from(ws[k].v);
#pragma unroll
      for (int a = 0; a < 4; ++a) wd[k].d[a] = ff_from(ws[k].d[a]);
    }
    const FisherScalar* ps = reinterpret_cast<const FisherScalar*>(&g.pol);
    FR* pd = reinterpret_cast<FR*>(&sb.pol);
    for (int k = t; k < npol; k += blockDim.x) {
      pd[k].v = (float)ps[k].v;
      pd[k].d[0] = 0.0f;
      pd[k].d[1] = (float)ps[k].d[6];  // lambda
      pd[k].d[2] = (float)ps[k].d[7];  // sin beta
      pd[k].d[3] = (float)ps[k].d[8];  // psi
      pd[k].d[4] = 0.0f;
    }
    if (t == 0) {
      sb.pfac.v = (float)g.wf.pfac.v;
      sb.cfac.v = (float)g.wf.cfac.v;
#pragma unroll
      for (int a = 0; a < 4; ++a) sb.pfac.d[a] = sb.cfac.d[a] = 0.0f;
      sb.pfac.d[4] = (float)g.wf.pfac.d[5];  // cos iota
      sb.cfac.d[4] = (float)g.wf.cfac.d[5];
      sb.tc = (float)g.tc.v;
      sb.status = g.status;
      sb.kcut = g.kcut;
    }
    if (t < P.n_det) orb[t] = orbit_f(P.orbit[t]);
  }
  __syncthreads();
  const float scale = (float)(kPc / (kMRSun * kMTSun));
  const double inv_scale2 = 1.0 / ((double)scale * (double)scale);
  int pa = 0, pb = 0;
  pair_of(t < kPairs ? t : 0, pa, pb);
  double acc = 0.0;
  if (sb.status == kSampleOk) {
    for (int64_t base = (int64_t)blockIdx.x * kFastThreads; base < sb.kcut;
         base += (int64_t)gridDim.x * kFastThreads) {
      const int64_t i = base + t;
      const bool live = i < sb.kcut;
      const float f = (float)((double)(P.k0 + (live ? i : 0)) * P.f_step);
      FM amp, psi, tf;
      if (live) {
        phenomd_eval<FM>(sb.wf, sb.wf.Msec * f, amp, psi, tf);
        amp = amp * scale;
      }
      for (int d = 0; d < P.n_det; ++d) {
        if (live) {
          Cx<FR> Y[3];
          FR kx0;
          {
            FR T = lift<FR>(0.0);
            T.v = tf.v.hi + sb.tc;
            T.d[0] = 1.0f;
            const FR zero = lift<FR>(0.0);
            Cx<FR> L[6];
            single_links_impl<true, FR>(orb[d], f, cx(sb.pfac, zero), cx(zero, -sb.cfac), T, sb.pol, L, &kx0);
            const TdiFactor tdb = P.tdi[(size_t)d * P.nbins + i];
            tdi_channels_t<true, FR>(cx(lift<FR>((float)tdb.dre), lift<FR>((float)tdb.dim)),
                                     cx(lift<FR>((float)tdb.pre), lift<FR>((float)tdb.pim)), 1, L, Y);
          }
          const float A = amp.v.hi, tp = 6.283185307179586f * f;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const float sw = (float)sqrt(P.w[((size_t)d * 3 + c) * P.nbins + i] * inv_scale2);  // 0 off the mask
            const FR& Yr = Y[c].re;
            const FR& Yi = Y[c].im;
            const float ar = A * Yr.v, ai = A * Yi.v;  // A Y
            float ur[11], ui[11];
#pragma unroll
            for (int k = 0; k < 4; ++k) {  // ln Mc, q, chi_1, chi_2
              const float dA = amp.d[k].hi, dt = tf.d[k].hi;
              const float ph = psi.d[k].hi + tp * kx0.d[0] * dt;
              ur[k] = dA * Yr.v + A * Yr.d[0] * dt + ai * ph;
              ui[k] = dA * Yi.v + A * Yi.d[0] * dt - ar * ph;
            }
            ur[4] = -ar;  // ln D_L: dh = -h
            ui[4] = -ai;
            ur[5] = A * Yr.d[4];  // cos iota
            ui[5] = A * Yi.d[4];
            ur[6] = A * Yr.d[1] + ai * tp * kx0.d[1];  // lambda
            ui[6] = A * Yi.d[1] - ar * tp * kx0.d[1];
            ur[7] = A * Yr.d[2] + ai * tp * kx0.d[2];  // sin beta
            ui[7] = A * Yi.d[2] - ar * tp * kx0.d[2];
            ur[8] = A * Yr.d[3];  // psi
            ui[8] = A * Yi.d[3];
            ur[9] = -2.0f * ai;  // phi_c: dh = 2 i h
            ui[9] = 2.0f * ar;
            const float pt = tp * (kx0.d[0] + 1.0f);  // t_c
            ur[10] = A * Yr.d[0] + ai * pt;
            ui[10] = A * Yi.d[0] - ar * pt;
#pragma unroll
            for (int a = 0; a < 11; ++a) {
              dh[t][c][a] = sw * ur[a];
              dh[t][c][11 + a] = sw * ui[a];
            }
          }
        } else {
#pragma unroll
          for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int a = 0; a < 22; ++a) dh[t][c][a] = 0.0f;
        }
        __syncthreads();
        if (t < kPairs) {
          float x = 0.0f;
          for (int u = 0; u < kFastThreads; ++u)
#pragma unroll
            for (int c = 0; c < 3; ++c)
              x = fmaf(dh[u][c][pa], dh[u][c][pb], fmaf(dh[u][c][11 + pa], dh[u][c][11 + pb], x));
          acc += (double)x;
        }
        __syncthreads();
      }
    }
  }
  if (t < kPairs) partial[((size_t)s * gridDim.x + blockIdx.x) * kPairs + t] = acc;
}

}  // namespace pes

using namespace pes;

extern "C" int pes_fisher_batch(PesPlan* p, const double* theta, int64_t B, double* fisher, int32_t* status,
                                void* stream) {
  PES_REQUIRE(p, "pes_fisher_batch: null plan");
  PES_REQUIRE(B >= 0 && B <= p->desc.max_batch, "pes_fisher_batch: batch size %lld outside [0, max_batch=%d]",
              (long long)B, p->desc.max_batch);
  PES_REQUIRE(B == 0 || (theta && fisher), "pes_fisher_batch: null theta or fisher");
  const unsigned need = (1u << p->desc.n_det) - 1u;
  PES_REQUIRE((p->data_set_mask & need) == need, "pes_fisher_batch: PSD not set for every detector (pes_plan_set_data)");
  if (B == 0) return PES_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (!p->fisher_blocks) {
    const int64_t M = p->desc.max_batch;
    PES_CHECK_CUDA(cudaMalloc(&p->fisher_blocks, sizeof(SampleBlock<FisherScalar>) * M));
    PES_CHECK_CUDA(cudaMalloc(&p->fisher_partial, sizeof(double) * M * kFisherBlocks * kPairs));
  }
  auto* blocks = reinterpret_cast<SampleBlock<FisherScalar>*>(p->fisher_blocks);
  k_setup<FisherScalar><<<(unsigned)ceil_div(B, kPerSampleThreads), kPerSampleThreads, 0, st>>>(
      p->dev, theta, B, 0, blocks, hm_blocks<FisherScalar>(p));
  PES_CHECK_LAUNCH();
  const bool hm = p->desc.approximant == PES_APPROX_PHENOMHM;
  if (p->mixed && !hm)  // mixed IMRPhenomD plans: FP32 structured derivatives
    k_fisher_fast<<<dim3(kFisherBlocks, (unsigned)B), kFastThreads, 0, st>>>(p->dev, blocks, p->fisher_partial);
  else  // FP64 plans and IMRPhenomHM: FP64 dual numbers through the whole model
    k_fisher_bins<<<dim3(kFisherBlocks, (unsigned)B), kFisherThreads, 0, st>>>(
        p->dev, blocks, hm ? hm_blocks<FisherScalar>(p) : nullptr, p->fisher_partial);
  PES_CHECK_LAUNCH();
  k_fisher_final<<<(unsigned)ceil_div(B * kPairs, 128), 128, 0, st>>>(blocks, B, kFisherBlocks, 4.0 * p->dev.df,
                                                                       p->fisher_partial, fisher, status);
  PES_CHECK_LAUNCH();
  return PES_OK;
}
