// Fixed device scratch of mcg_trace_cases_static. The array itself lives in
// mcg_trace_static.cu; this header gives its layout to the engine translation
// units, which launch the trace kernel on it.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/mcell_gb300.h"

namespace mcg {

constexpr size_t trace_static_up(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

// byte offsets of the per-call buffers inside the scratch (each 256-byte aligned)
struct TraceStaticLayout {
  static constexpr size_t kCases = MCG_TRACE_STATIC_MAX_CASES;
  static constexpr size_t ids = 0;                                                                    // uint64 [cases]
  static constexpr size_t idx = trace_static_up(ids + 8 * kCases);                                    // uint32 [cases]
  static constexpr size_t disp = trace_static_up(idx + 4 * kCases);                                   // double [cases][3]
  static constexpr size_t rrf = trace_static_up(disp + 24 * kCases);                                  // double [cases]
  static constexpr size_t tst = trace_static_up(rrf + 8 * kCases);                                    // double [cases]
  static constexpr size_t draws = trace_static_up(tst + 8 * kCases);                                  // uint32 [MAX_DRAWS]
  static constexpr size_t out = trace_static_up(draws + 4 * (size_t)MCG_TRACE_STATIC_MAX_DRAWS);      // double [cases][265]
  static constexpr size_t bytes = trace_static_up(out + 8 * (size_t)MCG_TRACE_RESULT_SIZE * kCases);
};

// Device address of the scratch on the current device (cudaGetSymbolAddress with
// that device current). The first call on a device also loads the module that
// holds the array (CUDA loads modules lazily), which takes its device memory;
// engines call it once, when they are created, and keep the address. Returns an
// MCG_* code.
int trace_static_scratch(unsigned char** addr, std::string& err);

// idx[c] = position of the live molecule whose id is want[c]; slots of ids that
// are not live are left untouched (the caller fills them with 0xFFFFFFFF first).
cudaError_t launch_find_ids(const uint64_t* uid, uint32_t n_live, const uint64_t* want, uint32_t n_cases,
                            uint32_t* idx, cudaStream_t stream);

}  // namespace mcg
