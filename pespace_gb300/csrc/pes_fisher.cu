// Fisher matrices of the batched plans, pespace/inference/fisher.py:27-162:
// F_ij = 4 df Re sum_{det, c, f} conj(dh_i) dh_j / S_c(f), the derivatives of
// the A/E/T model with respect to the 11 parameters taken by forward-mode dual
// numbers in FP64 at every live bin (the same per-bin model as the FP64 plan).
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

__global__ void __launch_bounds__(kFisherThreads) k_fisher_bins(PlanDev P,
                                                                const SampleBlock<FisherScalar>* __restrict__ blocks,
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
      Cx<T> hp, hc;
      T tft;
      if (live) {
        T Mf = sb.wf.Msec * f;
        T amp, psi, tf;
        phenomd_eval<T>(sb.wf, Mf, amp, psi, tf);
        T sn, cs;
        dsincos(psi, &sn, &cs);
        T ap = sb.wf.pfac * amp, ac = sb.wf.cfac * amp;
        hp = cx(ap * cs, -(ap * sn));
        hc = cx(-(ac * sn), -(ac * cs));
        Cx<T> ts;
        dsincos((-2.0 * kPi * f) * sb.tc, &ts.im, &ts.re);
        hp = cmul(hp, ts);
        hc = cmul(hc, ts);
        tft = tf + sb.tc;
      }
      for (int d = 0; d < P.n_det; ++d) {
        if (live) {
          Cx<T> L[6], C[3];
          single_links<T>(P.orbit[d], f, hp, hc, tft, sb.pol, L);
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
  k_setup<FisherScalar><<<(unsigned)ceil_div(B, kPerSampleThreads), kPerSampleThreads, 0, st>>>(p->dev, theta, B, 0, blocks);
  PES_CHECK_LAUNCH();
  k_fisher_bins<<<dim3(kFisherBlocks, (unsigned)B), kFisherThreads, 0, st>>>(p->dev, blocks, p->fisher_partial);
  PES_CHECK_LAUNCH();
  k_fisher_final<<<(unsigned)ceil_div(B * kPairs, 128), 128, 0, st>>>(blocks, B, kFisherBlocks, 4.0 * p->dev.df,
                                                                       p->fisher_partial, fisher, status);
  PES_CHECK_LAUNCH();
  return PES_OK;
}
