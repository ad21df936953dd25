// Shared definitions of the GB300 closed-shell CC engine (device + host).
#pragma once
#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "../../include/scess_cc.h"

namespace scess {

// A CUDA or engine failure travels as an exception inside the library and is
// turned into an SCESS_ERR_* status at the C ABI.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define SCESS_CUDA(call)                                                              \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) {                                                          \
      if (e_ == cudaErrorMemoryAllocation)                                            \
        throw ::scess::Error(SCESS_ERR_OOM, std::string("out of device memory: ") + #call); \
      throw ::scess::Error(SCESS_ERR_CUDA, std::string(cudaGetErrorString(e_)) + " at " + \
                                               __FILE__ + ":" + std::to_string(__LINE__)); \
    }                                                                                 \
  } while (0)

// Every kernel launch of the engine is followed by SCESS_CHECK_LAUNCH(), which
// also counts it (scess_launch_count()).
extern std::atomic<long long> g_launches;
#define SCESS_CHECK_LAUNCH()                                   \
  do {                                                         \
    ::scess::g_launches.fetch_add(1, std::memory_order_relaxed); \
    SCESS_CUDA(cudaGetLastError());                            \
  } while (0)

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline int64_t round_up(int64_t a, int64_t b) { return ceil_div(a, b) * b; }

constexpr int kNumSMs = 152;  // GB300: 2 dies x 76 SMs

}  // namespace scess
