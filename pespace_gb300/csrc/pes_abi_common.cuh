// Host-side helpers shared by the C-ABI translation units: error recording,
// CUDA error mapping and stream conversion.
#pragma once

#include <cstdio>
#include <cstring>
#include <cuda_runtime.h>

#include "../../include/pespace_gb300.h"

namespace pes {

void set_error(const char* fmt, ...);

#define PES_CHECK_CUDA(call)                                                  \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) {                                                  \
      ::pes::set_error("%s: %s (%s:%d)", #call, cudaGetErrorString(e_),       \
                       __FILE__, __LINE__);                                   \
      return PES_ECUDA;                                                       \
    }                                                                         \
  } while (0)

#define PES_CHECK_LAUNCH()                                                    \
  do {                                                                        \
    cudaError_t e_ = cudaGetLastError();                                      \
    if (e_ != cudaSuccess) {                                                  \
      ::pes::set_error("kernel launch: %s (%s:%d)", cudaGetErrorString(e_),   \
                       __FILE__, __LINE__);                                   \
      return PES_ECUDA;                                                       \
    }                                                                         \
  } while (0)

#define PES_REQUIRE(cond, ...)                                                \
  do {                                                                        \
    if (!(cond)) {                                                            \
      ::pes::set_error(__VA_ARGS__);                                          \
      return PES_EINVAL;                                                      \
    }                                                                         \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline unsigned int ceil_div(long long a, long long b) { return (unsigned int)((a + b - 1) / b); }

}  // namespace pes
