// Device engine for one model (templated on the position precision). Owns all
// device memory of the model and one CUDA stream; iterations run without host
// synchronisation, blocks of two iterations are replayed from CUDA graphs.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstring>
#include <unordered_map>

#include "mcg_engine.h"
#include "mcg_kernels.cuh"
#include "mcg_trace_static.h"

namespace mcg {

#define MCG_CUDA(call)                                                             \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      err = std::string(#call) + ": " + cudaGetErrorString(e_);                    \
      return -2;                                                                   \
    }                                                                              \
  } while (0)

template <typename T>
class DeviceEngineT : public DeviceEngine {
 public:
  ~DeviceEngineT() override { release(); }

  int init(const HostSetup& hs, const ChemHost& ch, const std::vector<uint8_t>& wall_class, uint64_t seed,
           uint64_t capacity, std::string& err) override {
    // a blocking stream: setup copies on the legacy default stream are ordered before its kernels
    MCG_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamDefault));
    int dev = 0;
    MCG_CUDA(cudaGetDevice(&dev));
    MCG_CUDA(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev));
    {
      // k_diffuse runs persistent warps: exactly as many blocks as can be resident
      int bps = 1;
      MCG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_diffuse<T>, TPB, 0));
      diffuse_grid_ = std::max(1, bps) * sms_;
    }
    nsp_ = ch.nsp;
    nw_ = hs.nw;
    // geometry
    Geo<T>& g = base_.g;
    g.origin = v3<T>((T)hs.origin[0], (T)hs.origin[1], (T)hs.origin[2]);
    g.opposite = v3<T>((T)hs.opposite[0], (T)hs.opposite[1], (T)hs.opposite[2]);
    g.part_edge = (T)hs.part_edge;
    g.sp_edge = (T)hs.sp_edge;
    g.sp_rcp = (T)hs.sp_rcp;
    g.R = (T)hs.R;
    g.nsub = (int)hs.nsub;
    g.nsub2 = (int)(hs.nsub * hs.nsub);
    g.nsp = (int)ch.nsp;
    std::vector<P4<T>> rej(std::max<uint32_t>(nw_, 1));
    std::vector<WallFace<T>> face(std::max<uint32_t>(nw_, 1));
    for (uint32_t w = 0; w < nw_; w++) {
      const double* o = &hs.wall[(size_t)w * 24];
      rej[w].x = (T)o[0];
      rej[w].y = (T)o[1];
      rej[w].z = (T)o[2];
      rej[w].w = (T)o[3];
      face[w].u = v3<T>((T)o[4], (T)o[5], (T)o[6]);
      face[w].v = v3<T>((T)o[7], (T)o[8], (T)o[9]);
      face[w].uv1u = (T)o[10];
      face[w].uv2u = (T)o[11];
      face[w].uv2v = (T)o[12];
      face[w].v0 = v3<T>((T)o[13], (T)o[14], (T)o[15]);
      face[w].v1 = v3<T>((T)o[16], (T)o[17], (T)o[18]);
      face[w].v2 = v3<T>((T)o[19], (T)o[20], (T)o[21]);
    }
    // wall list entries on the device: wall index << 8 | octant mask
    std::vector<uint32_t> ent(std::max<size_t>(hs.wsp_list.size(), 1), 0);
    for (size_t k = 0; k < hs.wsp_list.size(); k++) ent[k] = (hs.wsp_list[k] << 8) | hs.wsp_mask[k];
    if (alloc_copy(&d_wrej_, rej, err) || alloc_copy(&d_wface_, face, err) || alloc_copy(&d_wsp_off_, hs.wsp_off, err) ||
        alloc_copy(&d_wsp_list_, ent, err) ||
        alloc_copy(&d_wclass_, wall_class.empty() ? std::vector<uint8_t>(1, 0) : wall_class, err))
      return -2;
    g.wrej = d_wrej_;
    g.wface = d_wface_;
    g.wsp_off = d_wsp_off_;
    g.wsp_list = d_wsp_list_;
    g.wall_class = d_wclass_;
    // chemistry
    Chem c;
    std::memset(&c, 0, sizeof(c));
    c.nsp = (int)ch.nsp;
    for (int a = 0; a < MAXSP; a++) {
      c.space_step[a] = ch.space_step[a];
      c.unimol_k[a] = ch.unimol_k[a];
      c.uni_prod[a][0] = ch.uni_prod[a][0];
      c.uni_prod[a][1] = ch.uni_prod[a][1];
      for (int b = 0; b < MAXSP; b++) {
        c.bimol_p[a][b] = ch.bimol_p[a][b];
        c.bimol_prod[a][b][0] = ch.bimol_prod[a][b][0];
        c.bimol_prod[a][b][1] = ch.bimol_prod[a][b][1];
        if (ch.bimol_p[a][b] >= 0) c.partners[a] |= 1u << b;
      }
    }
    for (uint32_t w = 0; w < nw_; w++)
      for (uint32_t a = 0; a < ch.nsp; a++)
        if (wall_class[(size_t)w * ch.nsp + a]) c.can_volwall[a] = 1;
    MCG_CUDA(cudaMalloc(&d_chem_, sizeof(Chem)));
    MCG_CUDA(cudaMemcpy(d_chem_, &c, sizeof(Chem), cudaMemcpyHostToDevice));
    g.chem = d_chem_;
    base_.seed = seed;
    base_.debug_uid = ~0ull;
    base_.debug_log = nullptr;
    {
      // occupants are binned per subpartition octant while the key space stays small
      const uint64_t base_keys = (uint64_t)hs.nsub * hs.nsub * hs.nsub * ch.nsp;
      g.oct_shift = base_keys * 8 <= (1ull << 26) ? 3 : 0;
      nkeys_ = (uint32_t)(base_keys << g.oct_shift);
    }
    base_.nkeys = nkeys_;
    ntiles_ = (nkeys_ + SCAN_TILE - 1) / SCAN_TILE;
    base_.traj_cap = traj_cap_;
    MCG_CUDA(cudaMalloc(&d_cnt_, sizeof(Counters)));
    MCG_CUDA(cudaMemset(d_cnt_, 0, sizeof(Counters)));
    base_.cnt = d_cnt_;
    for (int k = 0; k < 2; k++) {
      MCG_CUDA(cudaMalloc(&d_start_[k], sizeof(uint32_t) * (nkeys_ + 1)));
      MCG_CUDA(cudaMemset(d_start_[k], 0, sizeof(uint32_t) * (nkeys_ + 1)));
    }
    MCG_CUDA(cudaMalloc(&d_counts_, sizeof(uint32_t) * nkeys_));
    MCG_CUDA(cudaMemset(d_counts_, 0, sizeof(uint32_t) * nkeys_));
    MCG_CUDA(cudaMalloc(&d_cursor_, sizeof(uint32_t) * nkeys_));
    MCG_CUDA(cudaMemset(d_cursor_, 0, sizeof(uint32_t) * nkeys_));
    MCG_CUDA(cudaMalloc(&d_tile_, sizeof(uint32_t) * (ntiles_ + 1)));
    MCG_CUDA(cudaMalloc(&d_traj_, sizeof(unsigned long long) * traj_cap_ * nsp_));
    MCG_CUDA(cudaMemset(d_traj_, 0, sizeof(unsigned long long) * traj_cap_ * nsp_));
    base_.start = d_start_[0];
    base_.nstart = d_start_[1];
    base_.counts = d_counts_;
    base_.cursor = d_cursor_;
    base_.tile_sum = d_tile_;
    base_.traj = d_traj_;
    if (capacity) {
      if (ensure_capacity(capacity, err)) return -2;
    }
    return 0;
  }

  int add_molecules(uint64_t n, const double* pos, const uint32_t* species, uint64_t uid0, std::string& err) override {
    if (n == 0) return 0;
    uint64_t live = 0;
    if (read_counters(err)) return -2;
    live = cnt_.n_live;
    if (live + n > 0xFFFFFFF0ull) {
      err = "too many molecules for 32-bit indices";
      return -3;
    }
    if (live + n > cap_ && ensure_capacity(std::max<uint64_t>((live + n) * 3 / 2, 1024), err)) return -2;
    if (n > base_.prod_cap && ensure_prod(n, err)) return -2;
    std::vector<Product<T>> stage(n);
    for (uint64_t i = 0; i < n; i++) {
      if (species[i] >= nsp_) {
        err = "species index out of range";
        return -1;
      }
      stage[i].pos.x = (T)pos[3 * i];
      stage[i].pos.y = (T)pos[3 * i + 1];
      stage[i].pos.z = (T)pos[3 * i + 2];
      uint32_t meta = species[i] | META_SCHEDULE_UNIMOL;
      std::memcpy(&stage[i].pos.w, &meta, sizeof(meta));
      if (sizeof(T) == 8) {
        uint64_t m64 = meta;
        std::memcpy(&stage[i].pos.w, &m64, sizeof(m64));
      }
      stage[i].birth = 0;
      stage[i].uid = uid0 + i;
      stage[i].tuni = TIME_FOREVER;
      const double* p = pos + 3 * i;
      if (!(p[0] >= origin_d(0) && p[1] >= origin_d(1) && p[2] >= origin_d(2) && p[0] < opp_d(0) && p[1] < opp_d(1) &&
            p[2] < opp_d(2))) {
        err = "molecule outside the partition";
        return -4;
      }
    }
    MCG_CUDA(cudaMemcpyAsync(base_.prod, stage.data(), sizeof(Product<T>) * n, cudaMemcpyHostToDevice, stream_));
    // counters: staged molecules sit in the product list, already "diffused"
    Counters c = cnt_;
    c.n_prod = (uint32_t)n;
    c.n_prod_done = (uint32_t)n;
    c.prod_hi = (uint32_t)n;
    MCG_CUDA(cudaMemcpyAsync(d_cnt_, &c, sizeof(Counters), cudaMemcpyHostToDevice, stream_));
    State<T> s = state(parity_);
    k_rebin_count<T><<<grid(live + n), TPB, 0, stream_>>>(s, (uint32_t)n);
    k_scan_tiles<T><<<ntiles_, TPB, 0, stream_>>>(s);
    k_scan_top<T><<<1, TPB, 0, stream_>>>(s, ntiles_);
    k_scan_apply<T><<<ntiles_, TPB, 0, stream_>>>(s);
    k_scatter<T><<<grid(live + n), TPB, 0, stream_>>>(s, 0, 0);
    launches_ += 5;
    MCG_CUDA(cudaGetLastError());
    MCG_CUDA(cudaStreamSynchronize(stream_));
    if (read_counters(err)) return -2;
    Counters c2 = cnt_;
    c2.n_live = std::min<uint32_t>(c2.n_live_next, (uint32_t)cap_);
    c2.n_prod = c2.n_prod_done = c2.prod_hi = 0;
    MCG_CUDA(cudaMemcpy(d_cnt_, &c2, sizeof(Counters), cudaMemcpyHostToDevice));
    parity_ ^= 1;  // the staged arrays became the current ones
    cnt_ = c2;
    invalidate_graphs();
    return status_to_error(c2.status, err);
  }

  int step(uint32_t n, std::string& err) override {
    if (cap_ == 0) {
      err = "no molecules";
      return -1;
    }
    uint32_t done = 0;
    while (done < n) {
      if (n - done >= 2 && use_graphs_ && !profile_) {
        cudaGraphExec_t& ge = graph_[parity_];
        if (!ge) {
          if (capture(parity_, err)) return -2;
        }
        MCG_CUDA(cudaGraphLaunch(ge, stream_));
        launches_ += 2 * kernels_per_iteration_;
        done += 2;  // two iterations return to the same parity
      } else {
        launch_iteration(state(parity_), profile_);
        MCG_CUDA(cudaGetLastError());
        parity_ ^= 1;
        done += 1;
      }
    }
    iterations_ += n;
    return 0;
  }

  int sync(std::string& err) override {
    MCG_CUDA(cudaStreamSynchronize(stream_));
    if (read_counters(err)) return -2;
    return status_to_error(cnt_.status, err);
  }

  int counts(uint64_t* out, std::string& err) override {
    int rc = sync(err);
    if (rc) return rc;
    if (cnt_.iteration > 0) {
      // species counts of the last finished iteration, accumulated by k_scatter
      const uint64_t row = (cnt_.iteration - 1) % traj_cap_;
      std::vector<unsigned long long> h(nsp_);
      MCG_CUDA(cudaMemcpy(h.data(), d_traj_ + row * nsp_, sizeof(unsigned long long) * nsp_, cudaMemcpyDeviceToHost));
      for (uint32_t a = 0; a < nsp_; a++) out[a] = h[a];
      return 0;
    }
    std::vector<uint32_t> st(nkeys_ + 1);
    MCG_CUDA(cudaMemcpy(st.data(), state(parity_).start, sizeof(uint32_t) * (nkeys_ + 1), cudaMemcpyDeviceToHost));
    for (uint32_t a = 0; a < nsp_; a++) out[a] = 0;
    for (uint32_t k = 0; k < nkeys_; k++) out[(k >> base_.g.oct_shift) % nsp_] += st[k + 1] - st[k];
    return 0;
  }

  int trajectory(uint32_t n, uint64_t* out, std::string& err) override {
    int rc = sync(err);
    if (rc) return rc;
    if (n > iterations_ || n > traj_cap_ - 1) {
      err = "trajectory longer than the iterations run or the ring";
      return -1;
    }
    std::vector<unsigned long long> h((size_t)traj_cap_ * nsp_);
    MCG_CUDA(cudaMemcpy(h.data(), d_traj_, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    const uint64_t last = cnt_.iteration;  // rows 0..iteration-1 hold finished iterations
    for (uint32_t k = 0; k < n; k++) {
      uint64_t it = last - n + k;
      for (uint32_t a = 0; a < nsp_; a++) out[(size_t)k * nsp_ + a] = h[(it % traj_cap_) * nsp_ + a];
    }
    return 0;
  }

  int download(uint64_t capn, double* pos, uint32_t* species, uint64_t* ids, uint64_t* n_out,
               std::string& err) override {
    int rc = sync(err);
    if (rc) return rc;
    const uint32_t n = cnt_.n_live;
    *n_out = n;
    if (n == 0) return 0;
    State<T> s = state(parity_);
    std::vector<P4<T>> p(n);
    std::vector<uint64_t> u(n);
    MCG_CUDA(cudaMemcpy(p.data(), s.a_pos, sizeof(P4<T>) * n, cudaMemcpyDeviceToHost));
    MCG_CUDA(cudaMemcpy(u.data(), s.a_uid, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost));
    for (uint64_t i = 0; i < std::min<uint64_t>(n, capn); i++) {
      if (pos) {
        pos[3 * i] = (double)p[i].x;
        pos[3 * i + 1] = (double)p[i].y;
        pos[3 * i + 2] = (double)p[i].z;
      }
      uint32_t meta;
      if (sizeof(T) == 8) {
        uint64_t m64;
        std::memcpy(&m64, &p[i].w, 8);
        meta = (uint32_t)m64;
      } else {
        std::memcpy(&meta, &p[i].w, 4);
      }
      if (species) species[i] = meta & META_SPECIES_MASK;
      if (ids) ids[i] = u[i];
    }
    return 0;
  }

  int trace(uint32_t nc, const uint64_t* ids, const double* disp, const uint32_t* draws, uint32_t ndraws,
            const double* rrf, const double* tst, double* out, std::string& err) override {
    int rc = sync(err);
    if (rc) return rc;
    const uint32_t n = cnt_.n_live;
    State<T> s = state(parity_);
    std::vector<uint64_t> u(n);
    MCG_CUDA(cudaMemcpy(u.data(), s.a_uid, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost));
    std::unordered_map<uint64_t, uint32_t> where;
    for (uint32_t i = 0; i < n; i++) where[u[i]] = i;
    std::vector<uint32_t> idx(nc);
    for (uint32_t c = 0; c < nc; c++) {
      auto it = where.find(ids[c]);
      if (it == where.end()) {
        err = "traced molecule id is not live";
        return -1;
      }
      idx[c] = it->second;
    }
    uint32_t* d_idx;
    double *d_disp, *d_rrf, *d_tst, *d_out;
    uint32_t* d_draws;
    MCG_CUDA(cudaMalloc(&d_idx, sizeof(uint32_t) * nc));
    MCG_CUDA(cudaMalloc(&d_disp, sizeof(double) * 3 * nc));
    MCG_CUDA(cudaMalloc(&d_rrf, sizeof(double) * nc));
    MCG_CUDA(cudaMalloc(&d_tst, sizeof(double) * nc));
    MCG_CUDA(cudaMalloc(&d_out, sizeof(double) * 265 * nc));
    MCG_CUDA(cudaMalloc(&d_draws, sizeof(uint32_t) * std::max<uint64_t>((uint64_t)ndraws * nc, 1)));
    MCG_CUDA(cudaMemcpy(d_idx, idx.data(), sizeof(uint32_t) * nc, cudaMemcpyHostToDevice));
    MCG_CUDA(cudaMemcpy(d_disp, disp, sizeof(double) * 3 * nc, cudaMemcpyHostToDevice));
    MCG_CUDA(cudaMemcpy(d_rrf, rrf, sizeof(double) * nc, cudaMemcpyHostToDevice));
    MCG_CUDA(cudaMemcpy(d_tst, tst, sizeof(double) * nc, cudaMemcpyHostToDevice));
    if (ndraws) MCG_CUDA(cudaMemcpy(d_draws, draws, sizeof(uint32_t) * ndraws * nc, cudaMemcpyHostToDevice));
    k_trace_cases<T><<<(nc + 127) / 128, 128, 0, stream_>>>(s, nc, d_idx, d_disp, d_draws, ndraws, d_rrf, d_tst, d_out);
    launches_ += 1;
    MCG_CUDA(cudaGetLastError());
    MCG_CUDA(cudaStreamSynchronize(stream_));
    MCG_CUDA(cudaMemcpy(out, d_out, sizeof(double) * 265 * nc, cudaMemcpyDeviceToHost));
    cudaFree(d_idx);
    cudaFree(d_disp);
    cudaFree(d_rrf);
    cudaFree(d_tst);
    cudaFree(d_out);
    cudaFree(d_draws);
    return 0;
  }

  int trace_static(uint32_t nc, const uint64_t* ids, const double* disp, const uint32_t* draws, uint32_t ndraws,
                   const double* rrf, const double* tst, double* out, std::string& err) override {
    int rc = sync(err);
    if (rc) return rc;
    unsigned char* sc = nullptr;
    rc = trace_static_scratch(&sc, err);
    if (rc) return rc;
    if (nc == 0) return 0;
    using L = TraceStaticLayout;
    uint64_t* d_ids = reinterpret_cast<uint64_t*>(sc + L::ids);
    uint32_t* d_idx = reinterpret_cast<uint32_t*>(sc + L::idx);
    double* d_disp = reinterpret_cast<double*>(sc + L::disp);
    double* d_rrf = reinterpret_cast<double*>(sc + L::rrf);
    double* d_tst = reinterpret_cast<double*>(sc + L::tst);
    uint32_t* d_draws = reinterpret_cast<uint32_t*>(sc + L::draws);
    double* d_out = reinterpret_cast<double*>(sc + L::out);
    State<T> s = state(parity_);
    // molecule ids -> positions in the current (sorted) arrays, on the device
    MCG_CUDA(cudaMemcpyAsync(d_ids, ids, sizeof(uint64_t) * nc, cudaMemcpyHostToDevice, stream_));
    MCG_CUDA(cudaMemsetAsync(d_idx, 0xFF, sizeof(uint32_t) * nc, stream_));
    MCG_CUDA(launch_find_ids(s.a_uid, cnt_.n_live, d_ids, nc, d_idx, stream_));
    uint32_t idx[MCG_TRACE_STATIC_MAX_CASES];
    MCG_CUDA(cudaMemcpyAsync(idx, d_idx, sizeof(uint32_t) * nc, cudaMemcpyDeviceToHost, stream_));
    MCG_CUDA(cudaStreamSynchronize(stream_));
    for (uint32_t c = 0; c < nc; c++)
      if (idx[c] == NONE) {
        err = "traced molecule id is not live";
        return -1;
      }
    MCG_CUDA(cudaMemcpyAsync(d_disp, disp, sizeof(double) * 3 * nc, cudaMemcpyHostToDevice, stream_));
    MCG_CUDA(cudaMemcpyAsync(d_rrf, rrf, sizeof(double) * nc, cudaMemcpyHostToDevice, stream_));
    MCG_CUDA(cudaMemcpyAsync(d_tst, tst, sizeof(double) * nc, cudaMemcpyHostToDevice, stream_));
    if (ndraws)
      MCG_CUDA(cudaMemcpyAsync(d_draws, draws, sizeof(uint32_t) * ndraws * nc, cudaMemcpyHostToDevice, stream_));
    k_trace_cases<T><<<(nc + 127) / 128, 128, 0, stream_>>>(s, nc, d_idx, d_disp, d_draws, ndraws, d_rrf, d_tst, d_out);
    launches_ += cnt_.n_live ? 2 : 1;
    MCG_CUDA(cudaGetLastError());
    MCG_CUDA(cudaMemcpyAsync(out, d_out, sizeof(double) * MCG_TRACE_RESULT_SIZE * nc, cudaMemcpyDeviceToHost, stream_));
    MCG_CUDA(cudaStreamSynchronize(stream_));
    return 0;
  }

  void set_options(int use_graphs, int profile) override {
    use_graphs_ = use_graphs != 0;
    profile_ = profile != 0;
  }

  int profile(double* out, std::string& err) override {
    MCG_CUDA(cudaStreamSynchronize(stream_));
    for (int k = 0; k < 6; k++) out[k] = 0;
    for (auto& ev : prof_) {
      float ms;
      MCG_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[4]));
      out[0] += ms;
      MCG_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
      out[1] += ms;
      MCG_CUDA(cudaEventElapsedTime(&ms, ev[1], ev[2]));
      out[2] += ms;
      MCG_CUDA(cudaEventElapsedTime(&ms, ev[2], ev[3]));
      out[3] += ms;
      MCG_CUDA(cudaEventElapsedTime(&ms, ev[3], ev[4]));
      out[4] += ms;
      for (int k = 0; k < 5; k++) cudaEventDestroy(ev[k]);
    }
    out[5] = (double)prof_.size();
    prof_.clear();
    return 0;
  }

  int debug_molecule(uint64_t uid, std::string& err) override {
    if (!d_debug_) {
      MCG_CUDA(cudaMalloc(&d_debug_, sizeof(double) * 64 * 271));
    }
    MCG_CUDA(cudaMemset(d_debug_, 0, sizeof(double) * 64 * 271));
    base_.debug_uid = uid;
    base_.debug_log = d_debug_;
    invalidate_graphs();
    return 0;
  }

  int debug_log(double* out, std::string& err) override {
    MCG_CUDA(cudaStreamSynchronize(stream_));
    if (!d_debug_) {
      err = "no molecule is being logged";
      return -1;
    }
    MCG_CUDA(cudaMemcpy(out, d_debug_, sizeof(double) * 64 * 271, cudaMemcpyDeviceToHost));
    return 0;
  }

  int escapes(double* out, uint32_t cap, uint32_t* n, std::string& err) override {
    MCG_CUDA(cudaStreamSynchronize(stream_));
    if (read_counters(err)) return -2;
    *n = cnt_.n_esc;
    for (uint32_t k = 0; k < std::min<uint32_t>(std::min<uint32_t>(cap, cnt_.n_esc), 8); k++)
      for (int q = 0; q < 12; q++) out[k * 12 + q] = cnt_.esc[k][q];
    return 0;
  }

  void stats(uint64_t* iterations, uint64_t* mol_steps, uint64_t* launches) override {
    std::string e;
    sync(e);
    if (iterations) *iterations = iterations_;
    if (mol_steps) *mol_steps = cnt_.mol_steps;
    if (launches) *launches = launches_;
  }

  static constexpr int kernels_per_iteration_ = 15;

 private:
  template <typename V>
  int alloc_copy(V** d, const std::vector<V>& h, std::string& err) {
    MCG_CUDA(cudaMalloc((void**)d, sizeof(V) * std::max<size_t>(h.size(), 1)));
    if (!h.empty()) MCG_CUDA(cudaMemcpy(*d, h.data(), sizeof(V) * h.size(), cudaMemcpyHostToDevice));
    return 0;
  }
  double origin_d(int k) const { return (double)(&base_.g.origin.x)[k]; }
  double opp_d(int k) const { return (double)(&base_.g.opposite.x)[k]; }
  unsigned grid(uint64_t n) const {
    uint64_t b = (n + TPB - 1) / TPB;
    uint64_t mx = (uint64_t)sms_ * 8;
    return (unsigned)std::max<uint64_t>(1, std::min(b, mx));
  }

  int read_counters(std::string& err) {
    MCG_CUDA(cudaMemcpy(&cnt_, d_cnt_, sizeof(Counters), cudaMemcpyDeviceToHost));
    return 0;
  }

  // molecule arrays: 2 sorted buffers (current / next) plus per-iteration scratch
  int ensure_capacity(uint64_t cap, std::string& err) {
    if (cap <= cap_) return 0;
    if (cap_ != 0 && cnt_.n_live != 0) {
      // grow while keeping the current molecules: copy into the new buffers
      std::string e2;
      if (sync(e2) < -1) return -2;
    }
    P4<T>* np[2];
    uint64_t* nu[2];
    T* nt[2];
    for (int k = 0; k < 2; k++) {
      MCG_CUDA(cudaMalloc(&np[k], sizeof(P4<T>) * cap));
      MCG_CUDA(cudaMalloc(&nu[k], sizeof(uint64_t) * cap));
      MCG_CUDA(cudaMalloc(&nt[k], sizeof(T) * cap));
      if (cap_) {
        MCG_CUDA(cudaMemcpy(np[k], pos_[k], sizeof(P4<T>) * cap_, cudaMemcpyDeviceToDevice));
        MCG_CUDA(cudaMemcpy(nu[k], uid_[k], sizeof(uint64_t) * cap_, cudaMemcpyDeviceToDevice));
        MCG_CUDA(cudaMemcpy(nt[k], tuni_[k], sizeof(T) * cap_, cudaMemcpyDeviceToDevice));
        cudaFree(pos_[k]);
        cudaFree(uid_[k]);
        cudaFree(tuni_[k]);
      }
      pos_[k] = np[k];
      uid_[k] = nu[k];
      tuni_[k] = nt[k];
    }
    cudaFree(d_b_pos_);
    cudaFree(d_st_);
    cudaFree(d_claim_);
    cudaFree(d_props_);
    cudaFree(d_losers_);
    cudaFree(d_redo_);
    MCG_CUDA(cudaMalloc(&d_b_pos_, sizeof(P4<T>) * cap));
    MCG_CUDA(cudaMalloc(&d_st_, cap));
    MCG_CUDA(cudaMalloc(&d_claim_, sizeof(uint64_t) * cap));
    MCG_CUDA(cudaMemset(d_claim_, 0xFF, sizeof(uint64_t) * cap));
    uint64_t pc = std::max<uint64_t>(4096, cap / 8);
    MCG_CUDA(cudaMalloc(&d_props_, sizeof(Proposal) * pc));
    MCG_CUDA(cudaMalloc(&d_losers_, sizeof(uint32_t) * 2 * pc));
    MCG_CUDA(cudaMalloc(&d_redo_, sizeof(Proposal) * pc));
    base_.prop_cap = (uint32_t)pc;
    cap_ = cap;
    base_.cap = (uint32_t)cap;
    if (ensure_prod(std::max<uint64_t>(4096, cap / 4), err)) return -2;
    invalidate_graphs();
    return 0;
  }

  int ensure_prod(uint64_t pc, std::string& err) {
    if (pc <= base_.prod_cap) return 0;
    cudaFree(d_prod_);
    cudaFree(d_pst_);
    MCG_CUDA(cudaMalloc(&d_prod_, sizeof(Product<T>) * pc));
    MCG_CUDA(cudaMalloc(&d_pst_, pc));
    base_.prod_cap = (uint32_t)pc;
    base_.prod = d_prod_;
    base_.pst = d_pst_;
    invalidate_graphs();
    return 0;
  }

  State<T> state(int parity) const {
    State<T> s = base_;
    s.a_pos = pos_[parity];
    s.a_uid = uid_[parity];
    s.a_tuni = tuni_[parity];
    s.n_pos = pos_[parity ^ 1];
    s.n_uid = uid_[parity ^ 1];
    s.n_tuni = tuni_[parity ^ 1];
    s.start = d_start_[parity];
    s.nstart = d_start_[parity ^ 1];
    s.b_pos = d_b_pos_;
    s.st = d_st_;
    s.claim = d_claim_;
    s.props = d_props_;
    s.losers = d_losers_;
    s.redo_props = d_redo_;
    s.prod = d_prod_;
    s.pst = d_pst_;
    return s;
  }

  // records an event on the engine stream when profiling (not during graph capture)
  void mark(int k, bool prof) {
    if (!prof) return;
    if (k == 0) prof_.emplace_back();
    cudaEventCreate(&prof_.back()[k]);
    cudaEventRecord(prof_.back()[k], stream_);
  }

  void launch_iteration(const State<T>& s, bool prof = false) {
    const unsigned g = grid(cap_);
    const unsigned gs = (unsigned)std::max(1, sms_);
    mark(0, prof);
    k_diffuse<T><<<diffuse_grid_, TPB, 0, stream_>>>(s);
    mark(1, prof);
    k_resolve<T><<<gs, TPB, 0, stream_>>>(s);
    k_collect_losers<T><<<gs, TPB, 0, stream_>>>(s);
    k_reset_claims<T><<<gs, TPB, 0, stream_>>>(s);
    k_redo<T><<<1, TPB, 0, stream_>>>(s);
    mark(2, prof);
    k_prod_window<T><<<1, 1, 0, stream_>>>(s);
    k_products<T><<<gs, TPB, 0, stream_>>>(s);
    k_prod_window<T><<<1, 1, 0, stream_>>>(s);
    k_products<T><<<gs, TPB, 0, stream_>>>(s);
    k_prod_window<T><<<1, 1, 0, stream_>>>(s);
    mark(3, prof);
    k_scan_tiles<T><<<ntiles_, TPB, 0, stream_>>>(s);
    k_scan_top<T><<<1, TPB, 0, stream_>>>(s, ntiles_);
    k_scan_apply<T><<<ntiles_, TPB, 0, stream_>>>(s);
    k_scatter<T><<<g, TPB, 0, stream_>>>(s, 1, 1);
    k_end<T><<<1, 1, 0, stream_>>>(s);
    mark(4, prof);
    launches_ += kernels_per_iteration_;
  }

  int capture(int parity, std::string& err) {
    cudaGraph_t gr;
    MCG_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    uint64_t l0 = launches_;
    launch_iteration(state(parity));
    launch_iteration(state(parity ^ 1));
    launches_ = l0;
    MCG_CUDA(cudaStreamEndCapture(stream_, &gr));
    MCG_CUDA(cudaGraphInstantiate(&graph_[parity], gr, 0));
    cudaGraphDestroy(gr);
    return 0;
  }

  void invalidate_graphs() {
    for (int k = 0; k < 2; k++) {
      if (graph_[k]) cudaGraphExecDestroy(graph_[k]);
      graph_[k] = nullptr;
    }
  }

  void release() {
    invalidate_graphs();
    for (int k = 0; k < 2; k++) {
      cudaFree(pos_[k]);
      cudaFree(uid_[k]);
      cudaFree(tuni_[k]);
      cudaFree(d_start_[k]);
    }
    cudaFree(d_b_pos_);
    cudaFree(d_st_);
    cudaFree(d_claim_);
    cudaFree(d_props_);
    cudaFree(d_losers_);
    cudaFree(d_redo_);
    cudaFree(d_prod_);
    cudaFree(d_pst_);
    cudaFree(d_counts_);
    cudaFree(d_cursor_);
    cudaFree(d_tile_);
    cudaFree(d_traj_);
    cudaFree(d_cnt_);
    cudaFree(d_debug_);
    cudaFree(d_chem_);
    cudaFree(d_wrej_);
    cudaFree(d_wface_);
    cudaFree(d_wsp_off_);
    cudaFree(d_wsp_list_);
    cudaFree(d_wclass_);
    if (stream_) cudaStreamDestroy(stream_);
  }

  State<T> base_{};
  cudaStream_t stream_ = nullptr;
  int sms_ = 1;
  int diffuse_grid_ = 1;
  int parity_ = 0;
  bool use_graphs_ = true;
  bool profile_ = false;
  std::vector<std::array<cudaEvent_t, 5>> prof_;
  cudaGraphExec_t graph_[2] = {nullptr, nullptr};
  uint32_t nsp_ = 0, nw_ = 0, nkeys_ = 0, ntiles_ = 0, traj_cap_ = 65536;
  uint64_t cap_ = 0, iterations_ = 0, launches_ = 0;
  Counters cnt_{};
  P4<T>* pos_[2] = {nullptr, nullptr};
  uint64_t* uid_[2] = {nullptr, nullptr};
  T* tuni_[2] = {nullptr, nullptr};
  uint32_t* d_start_[2] = {nullptr, nullptr};
  P4<T>* d_b_pos_ = nullptr;
  uint8_t* d_st_ = nullptr;
  uint64_t* d_claim_ = nullptr;
  Proposal* d_props_ = nullptr;
  uint32_t* d_losers_ = nullptr;
  Proposal* d_redo_ = nullptr;
  Product<T>* d_prod_ = nullptr;
  uint8_t* d_pst_ = nullptr;
  uint32_t *d_counts_ = nullptr, *d_cursor_ = nullptr, *d_tile_ = nullptr;
  unsigned long long* d_traj_ = nullptr;
  Counters* d_cnt_ = nullptr;
  double* d_debug_ = nullptr;
  Chem* d_chem_ = nullptr;
  P4<T>* d_wrej_ = nullptr;
  WallFace<T>* d_wface_ = nullptr;
  uint32_t *d_wsp_off_ = nullptr, *d_wsp_list_ = nullptr;
  uint8_t* d_wclass_ = nullptr;
};

}  // namespace mcg
