// Scratch memory of mcg_trace_cases_static: one statically sized __device__
// array per device instead of buffers from cudaMalloc, so that the call makes
// no device allocation. Its size is fixed at build time by
// MCG_TRACE_STATIC_MAX_CASES and MCG_TRACE_STATIC_MAX_DRAWS (about 0.6 MB).
#include "mcg_trace_static.h"

namespace mcg {

namespace {

// Every device context holds its own copy of this array. Nothing in it has to
// start at zero: each call resets the index slots it uses and the trace kernel
// writes every output double of every case it runs.
static __device__ __align__(256) unsigned char g_trace_scratch[TraceStaticLayout::bytes];

__global__ void k_find_ids(const uint64_t* uid, uint32_t n, const uint64_t* want, uint32_t nc, uint32_t* idx) {
  __shared__ uint64_t w[MCG_TRACE_STATIC_MAX_CASES];
  for (uint32_t c = threadIdx.x; c < nc; c += blockDim.x) w[c] = want[c];
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint64_t u = uid[i];
    for (uint32_t c = 0; c < nc; c++)
      if (w[c] == u) idx[c] = i;  // live ids are unique: at most one writer per slot
  }
}

}  // namespace

int trace_static_scratch(unsigned char** addr, std::string& err) {
  // resolved per call (engines call it once, when they are created): an address
  // cached across engines would go stale after a cudaDeviceReset in the process
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_trace_scratch);
  if (e != cudaSuccess || !p) {
    err = std::string("cudaGetSymbolAddress of the trace scratch: ") + cudaGetErrorString(e);
    return MCG_ERR_CUDA;
  }
  *addr = static_cast<unsigned char*>(p);
  return MCG_OK;
}

cudaError_t launch_find_ids(const uint64_t* uid, uint32_t n_live, const uint64_t* want, uint32_t n_cases,
                            uint32_t* idx, cudaStream_t stream) {
  if (n_live == 0 || n_cases == 0) return cudaSuccess;
  const uint32_t blocks = (n_live + 255) / 256 < 1024u ? (n_live + 255) / 256 : 1024u;
  k_find_ids<<<blocks, 256, 0, stream>>>(uid, n_live, want, n_cases, idx);
  return cudaGetLastError();
}

}  // namespace mcg
