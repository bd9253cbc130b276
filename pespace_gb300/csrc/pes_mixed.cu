// Mixed-precision batched path (sparse FP64 grid + FP32 dense spline bulk).
#include "pes_plan.cuh"

namespace pes {

struct MixedBuffers {
  int unused;
};

int mixed_create(PesPlan* p) {
  (void)p;
  set_error("mixed precision plans are not available in this build");
  return PES_EINVAL;
}
void mixed_destroy(PesPlan* p) { delete p->mixed; p->mixed = nullptr; }
int mixed_set_data(PesPlan*, cudaStream_t) { return PES_OK; }
int mixed_lnl(PesPlan*, const double*, int64_t, double*, double*, int32_t*, cudaStream_t) {
  set_error("mixed precision plans are not available in this build");
  return PES_EINVAL;
}

}  // namespace pes
