// fp64 instantiation of the engine. Built with -fmad=false so that every
// product and sum is rounded like MCell4's CPU build (no fused multiply-add).
#include "mcg_engine.cuh"

namespace mcg {
DeviceEngine* make_engine_f64() { return new DeviceEngineT<double>(); }
// the countdown is shared by every engine of the process (one inline definition)
void set_alloc_failure(long long after) { alloc_failure_countdown().store(after < 0 ? -1 : after); }

// reaction decisions on injected draws (one per case): kind 0 test_bimolecular over a
// class of npw[c] pathways (cum[c][MAXPW]) at scaling[c], kind 1 which_unimolecular;
// out[c] = pathway, or -1 for no reaction
__global__ void k_rxn_decisions(int kind, uint32_t n, const double* cum, const uint32_t* npw, const double* scaling,
                                const uint32_t* draws, int32_t* out) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  InjectedDraws d;
  d.d = draws + c;
  d.n = 1;
  d.used = 0;
  d.over = false;
  const int np = (int)min(max(npw[c], 1u), (uint32_t)MAXPW);
  out[c] = kind == 0 ? test_bimolecular(cum + (size_t)c * MAXPW, np, scaling[c], d.u32())
                     : which_unimolecular(cum + (size_t)c * MAXPW, np, d);
}

// parity harness of the reaction decisions (k_rxn_decisions); test infrastructure of
// the C ABI, with its own short-lived buffers
int rxn_decisions(int kind, uint32_t n, const double* cum, const uint32_t* npw, const double* scaling,
                  const uint32_t* draws, int32_t* out, std::string& err) {
  if (n == 0) return 0;
  AllocSet a;
  double *d_cum, *d_sc;
  uint32_t *d_np, *d_dr;
  int32_t* d_out;
  MCG_CUDA(a.get(&d_cum, sizeof(double) * MAXPW * n));
  MCG_CUDA(a.get(&d_sc, sizeof(double) * n));
  MCG_CUDA(a.get(&d_np, sizeof(uint32_t) * n));
  MCG_CUDA(a.get(&d_dr, sizeof(uint32_t) * n));
  MCG_CUDA(a.get(&d_out, sizeof(int32_t) * n));
  MCG_CUDA(cudaMemcpy(d_cum, cum, sizeof(double) * MAXPW * n, cudaMemcpyHostToDevice));
  MCG_CUDA(cudaMemcpy(d_sc, scaling, sizeof(double) * n, cudaMemcpyHostToDevice));
  MCG_CUDA(cudaMemcpy(d_np, npw, sizeof(uint32_t) * n, cudaMemcpyHostToDevice));
  MCG_CUDA(cudaMemcpy(d_dr, draws, sizeof(uint32_t) * n, cudaMemcpyHostToDevice));
  k_rxn_decisions<<<(n + 127) / 128, 128>>>(kind, n, d_cum, d_np, d_sc, d_dr, d_out);
  MCG_CUDA(cudaGetLastError());
  MCG_CUDA(cudaMemcpy(out, d_out, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
  return 0;
}

// one thread draws the whole release from the injected stream, as the reference's
// single generator does
__global__ void k_release_positions(int shape, uint32_t n, const double* c, const double* dia, const uint32_t* draws,
                                    uint32_t ndraws, double* out, uint32_t* used) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  InjectedDraws d;
  d.d = draws;
  d.n = ndraws;
  d.used = 0;
  d.over = false;
  for (uint32_t i = 0; i < n; i++) {
    V3<double> p;
    release_point(shape, c, dia, d, p);
    out[3 * i] = p.x;
    out[3 * i + 1] = p.y;
    out[3 * i + 2] = p.z;
  }
  *used = d.over ? 0xFFFFFFFFu : d.used;
}

int release_positions(int shape, uint32_t n, const double* center, const double* diameter, const uint32_t* draws,
                      uint32_t ndraws, double* out, uint32_t* used, std::string& err) {
  AllocSet a;
  double *d_c, *d_out;
  uint32_t *d_dr, *d_used;
  MCG_CUDA(a.get(&d_c, sizeof(double) * 6));
  MCG_CUDA(a.get(&d_out, sizeof(double) * 3 * std::max<uint32_t>(n, 1)));
  MCG_CUDA(a.get(&d_dr, sizeof(uint32_t) * std::max<uint32_t>(ndraws, 1)));
  MCG_CUDA(a.get(&d_used, sizeof(uint32_t)));
  const double cd[6] = {center[0], center[1], center[2], diameter[0], diameter[1], diameter[2]};
  MCG_CUDA(cudaMemcpy(d_c, cd, sizeof(cd), cudaMemcpyHostToDevice));
  if (ndraws) MCG_CUDA(cudaMemcpy(d_dr, draws, sizeof(uint32_t) * ndraws, cudaMemcpyHostToDevice));
  k_release_positions<<<1, 1>>>(shape, n, d_c, d_c + 3, d_dr, ndraws, d_out, d_used);
  MCG_CUDA(cudaGetLastError());
  MCG_CUDA(cudaMemcpy(out, d_out, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost));
  MCG_CUDA(cudaMemcpy(used, d_used, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  return 0;
}

}  // namespace mcg
