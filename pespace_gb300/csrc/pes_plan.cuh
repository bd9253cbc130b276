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
  size_t blocks_bytes = 0;
  double* partial = nullptr;   // [max_batch][nblk][1 + NT]
  size_t partial_len = 0;
  int32_t* status = nullptr;   // [max_batch] internal status when the caller passes NULL
  unsigned data_set_mask = 0;
  pes::MixedBuffers* mixed = nullptr;
  pes::Profiler prof;
};

namespace pes {
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
int mixed_create(PesPlan* p);
void mixed_destroy(PesPlan* p);
int mixed_set_data(PesPlan* p, cudaStream_t st);
int mixed_lnl(PesPlan* p, const double* theta, int64_t B, double* lnl, double* grad, int32_t* status,
              cudaStream_t st);
}  // namespace pes
