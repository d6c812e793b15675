// Device engine (templated on the position precision). Owns all device memory
// and one CUDA stream. It holds a table of replicas — independent models, each
// with its own mesh, partition grid, reactions, seed and iteration budget — whose
// molecules share one set of sorted arrays, so every kernel of an iteration
// covers all replicas. Iterations run without host synchronisation; blocks of
// two iterations are replayed from CUDA graphs. Adding or removing replicas
// re-sorts the molecules once (the key space is laid out again).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <array>
#include <climits>
#include <cstddef>
#include <cmath>
#include <cstring>
#include <memory>
#include <thread>
#include <unordered_map>

#include <random>

#include "mcg_engine.h"
#include "mcg_kernels.cuh"
#include "mcg_region.h"
#include "mcg_trace_static.h"

namespace mcg {

// Device allocations go through dev_malloc. A test hook (mcg_inject_device_alloc_failure)
// can make one of them fail as if the device were out of memory, so that the error
// paths (status codes, no leak, the engine left as it was) run without exhausting HBM.
inline std::atomic<long long>& alloc_failure_countdown() {
  static std::atomic<long long> c{-1};
  return c;
}
template <typename P>
inline cudaError_t dev_malloc(P** p, size_t bytes) {
  *p = nullptr;
  if (alloc_failure_countdown().load() >= 0 && alloc_failure_countdown().fetch_sub(1) == 0)
    return cudaErrorMemoryAllocation;
  return cudaMalloc((void**)p, bytes);
}

// The allocations of one resize: freed together unless the resize commits them, so a
// failed resize leaks nothing and leaves the engine's buffers as they were.
struct AllocSet {
  std::vector<void*> ptrs;
  bool keep = false;
  AllocSet() = default;
  AllocSet(const AllocSet&) = delete;
  AllocSet& operator=(const AllocSet&) = delete;
  ~AllocSet() {
    if (!keep)
      for (void* p : ptrs) cudaFree(p);
  }
  template <typename P>
  cudaError_t get(P** p, size_t bytes) {
    cudaError_t e = dev_malloc(p, bytes);
    if (e == cudaSuccess) ptrs.push_back((void*)*p);
    return e;
  }
};

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

  int create(uint32_t nsp, uint32_t max_rep, uint64_t capacity, std::string& err) override {
    if (nsp == 0 || nsp > (uint32_t)MAXSP || max_rep == 0 || max_rep > MAX_REPLICAS) {
      err = "invalid species count or replica slots";
      return -1;
    }
    // a non-blocking stream, and every copy and memset of the engine is ordered on it:
    // nothing synchronises with the legacy default stream, so engines driven from
    // other threads (a serving loop) do not disturb a graph capture on this one
    MCG_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    int dev = 0;
    MCG_CUDA(cudaGetDevice(&dev));
    dev_ = dev;
    MCG_CUDA(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev));
    // the fixed scratch of the allocation-free trace (mcg_trace_cases_static): its
    // module is loaded, and its device memory taken, here rather than on the first
    // such call (which may come when device memory is fully committed, or while
    // another thread captures a graph)
    {
      const int rc = trace_static_scratch(&static_scratch_, err);
      if (rc) return rc;
    }
    {
      // k_diffuse runs persistent warps: as many blocks as can be resident. It uses no
      // shared memory; its spills and per-thread arrays live in local memory, cached in
      // L1, so the whole L1/shared carveout goes to L1.
#ifndef MCG_DIFFUSE_CARVEOUT
#define MCG_DIFFUSE_CARVEOUT 0
#endif
      if (MCG_DIFFUSE_CARVEOUT >= 0) {
        MCG_CUDA(cudaFuncSetAttribute(k_diffuse<T, false>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                      MCG_DIFFUSE_CARVEOUT));
        MCG_CUDA(cudaFuncSetAttribute(k_diffuse<T, true>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                      MCG_DIFFUSE_CARVEOUT));
      }
      int bps = 1;
      MCG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_diffuse<T, false>, TPB, 0));
      bps_max_ = std::max(1, bps);
      diffuse_grid_ = bps_max_ * sms_;
    }
    nsp_ = nsp;
    max_rep_ = max_rep;
    reps_.assign(max_rep, Rep());
    geos_h_.assign(max_rep, Geo<T>{});
    for (uint32_t r = 0; r < max_rep; r++) {
      geos_h_[r].mode = REP_DROP;  // free slot: no keys, no molecules
      geos_h_[r].nsp = (int)nsp;
      geos_h_[r].rep = r;
    }
    MCG_CUDA(dev_malloc(&d_geos_, sizeof(Geo<T>) * max_rep));
    MCG_CUDA(cudaMemcpyAsync(d_geos_, geos_h_.data(), sizeof(Geo<T>) * max_rep, cudaMemcpyHostToDevice, stream_));
    // count trajectory ring: [row][replica][species], at most 64 MB
    const uint64_t row_bytes = sizeof(unsigned long long) * (uint64_t)max_rep * nsp;
    traj_cap_ = (uint32_t)std::max<uint64_t>(64, std::min<uint64_t>(65536, (64ull << 20) / row_bytes));
    MCG_CUDA(dev_malloc(&d_traj_, row_bytes * traj_cap_));
    MCG_CUDA(cudaMemsetAsync(d_traj_, 0, row_bytes * traj_cap_, stream_));
    MCG_CUDA(dev_malloc(&d_cnt_, sizeof(Counters)));
    MCG_CUDA(cudaMemsetAsync(d_cnt_, 0, sizeof(Counters), stream_));
    base_.geos = d_geos_;
    base_.n_rep = max_rep;
    base_.nsp = (int)nsp;
    base_.traj_cap = traj_cap_;
    base_.traj = d_traj_;
    base_.cnt = d_cnt_;
    base_.debug_uid = ~0ull;
    base_.debug_log = nullptr;
    base_.maxc = MAXC;
    base_.maxset = MAXSET;
    if (capacity && ensure_capacity(capacity, err)) return -2;
    return 0;
  }

  int add_replicas(const ReplicaSpec* specs, uint32_t n, uint32_t* out_reps, std::string& err) override {
    if (n == 0) return 0;
    if (read_counters(err)) return -2;
    std::vector<uint32_t> slots;
    for (uint32_t r = 0; r < max_rep_ && slots.size() < n; r++)
      if (!reps_[r].used) slots.push_back(r);
    if (slots.size() < n) {
      err = "no free replica slot";
      return -3;
    }
    uint64_t n_new = 0;
    for (uint32_t k = 0; k < n; k++) n_new += specs[k].n_mol;
    if (cnt_.n_live + n_new > 0xFFFFFFF0ull) {
      err = "too many molecules for 32-bit indices";
      return -3;
    }
    // any failure before the re-sort leaves the engine as it was: the new slots are
    // freed and the key space laid out again without them (it needs no new memory then)
    auto undo = [&](int rc) {
      for (uint32_t k = 0; k < n; k++) free_replica(slots[k]);
      std::string e2;
      layout_keys(e2);
      return rc;
    };
    for (uint32_t k = 0; k < n; k++) {
      const ReplicaSpec& sp = specs[k];
      const uint32_t r = slots[k];
      int rc = upload_replica(sp, r, err);
      if (rc) return undo(rc);
      reps_[r].next_uid = sp.n_mol;
      out_reps[k] = r;
    }
    bool any_cv = false;
    for (uint32_t k = 0; k < n; k++) any_cv = any_cv || !specs[k].counted.empty();
    if (any_cv && !d_cv_count_) {
      int rc = alloc_counted(err);
      if (rc) return undo(rc);
    }
    // room for the new molecules before the key space changes
    if (cnt_.n_live + n_new > cap_) {
      int rc = ensure_capacity(std::max<uint64_t>((cnt_.n_live + n_new) * 3 / 2, 1024), err);
      if (rc) return undo(rc);
    }
    if (n_new > base_.prod_cap) {
      int rc = ensure_prod(n_new, err);
      if (rc) return undo(rc);
    }
    int rc = layout_keys(err);
    if (rc) return undo(rc);
    // the molecules, staged on the device once the replicas' grids are there
    uint64_t staged = 0;
    for (uint32_t k = 0; k < n; k++) {
      rc = stage_on_device(slots[k], specs[k].n_mol, specs[k].pos, specs[k].species, 0, staged, err);
      if (rc) return undo(rc);
      staged += specs[k].n_mol;
    }
    return rebin(nullptr, n_new, err, true);
  }

  // counted-volume count arrays (allocated when the first replica counts a volume)
  int alloc_counted(std::string& err) {
    {
      const size_t nq = (size_t)max_rep_ * nsp_ * MAX_COUNTED;
      cv_traj_cap_ = std::min<uint32_t>(traj_cap_, 4096);
      AllocSet a;
      uint32_t *cc, *cn, *ct;
      MCG_CUDA(a.get(&cc, sizeof(uint32_t) * nq));
      MCG_CUDA(a.get(&cn, sizeof(uint32_t) * nq));
      MCG_CUDA(a.get(&ct, sizeof(uint32_t) * nq * cv_traj_cap_));
      MCG_CUDA(cudaMemsetAsync(cc, 0, sizeof(uint32_t) * nq, stream_));
      MCG_CUDA(cudaMemsetAsync(cn, 0, sizeof(uint32_t) * nq, stream_));
      MCG_CUDA(cudaMemsetAsync(ct, 0, sizeof(uint32_t) * nq * cv_traj_cap_, stream_));
      a.keep = true;
      d_cv_count_ = cc;
      d_cv_now_ = cn;
      d_cv_traj_ = ct;
      base_.cv_count = d_cv_count_;
      base_.cv_now = d_cv_now_;
      base_.cv_traj = d_cv_traj_;
      base_.cv_traj_cap = cv_traj_cap_;
    }
    return 0;
  }

  int remove_replicas(const uint32_t* reps, uint32_t n, std::string& err) override {
    if (n == 0) return 0;
    for (uint32_t k = 0; k < n; k++)
      if (reps[k] >= max_rep_ || !reps_[reps[k]].used) {
        err = "no such replica";
        return -1;
      }
    int rc = sync(err);
    if (rc) return rc;
    for (uint32_t k = 0; k < n; k++) {
      geos_h_[reps[k]].mode = REP_DROP;  // its molecules leave with the re-binning below
      reps_[reps[k]].used = false;
    }
    rc = layout_keys(err);
    if (rc) return rc;
    rc = rebin(nullptr, 0, err);
    if (rc) return rc;
    for (uint32_t k = 0; k < n; k++) free_replica(reps[k]);
    return 0;
  }

  int add_molecules(uint32_t rep, uint64_t n, const double* pos, const uint32_t* species, uint64_t uid0,
                    std::string& err) override {
    if (n == 0) return 0;
    if (rep >= max_rep_ || !reps_[rep].used) {
      err = "no such replica";
      return -1;
    }
    if (read_counters(err)) return -2;
    if (cnt_.n_live + n > 0xFFFFFFF0ull) {
      err = "too many molecules for 32-bit indices";
      return -3;
    }
    if (cnt_.n_live + n > cap_ && ensure_capacity(std::max<uint64_t>((cnt_.n_live + n) * 3 / 2, 1024), err))
      return -2;
    if (n > base_.prod_cap && ensure_prod(n, err)) return -2;
    int rc = stage_on_device(rep, n, pos, species, uid0, 0, err);
    if (rc) return rc;
    reps_[rep].next_uid = std::max<uint64_t>(reps_[rep].next_uid, uid0 + n);
    return rebin(nullptr, n, err, true);
  }

  // host molecule arrays staged into the product list at `offset` on the device
  // (k_stage_upload); the input is checked before anything is kept
  int stage_on_device(uint32_t r, uint64_t n, const double* pos, const uint32_t* species, uint64_t uid0,
                      uint64_t offset, std::string& err) {
    if (n == 0) return 0;
    AllocSet tmp;
    double* d_pos;
    uint32_t *d_sp, *d_err;
    MCG_CUDA(tmp.get(&d_pos, sizeof(double) * 3 * n));
    MCG_CUDA(tmp.get(&d_sp, sizeof(uint32_t) * n));
    MCG_CUDA(tmp.get(&d_err, sizeof(uint32_t)));
    MCG_CUDA(cudaMemcpyAsync(d_pos, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, stream_));
    MCG_CUDA(cudaMemcpyAsync(d_sp, species, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, stream_));
    MCG_CUDA(cudaMemsetAsync(d_err, 0, sizeof(uint32_t), stream_));
    k_stage_upload<T><<<grid(n), TPB, 0, stream_>>>(state(parity_), r, (uint32_t)n, d_pos, d_sp, uid0,
                                                     (uint32_t)offset, nsp_, d_err);
    launches_ += 1;
    MCG_CUDA(cudaGetLastError());
    uint32_t bad = 0;
    MCG_CUDA(d2h(&bad, d_err, sizeof(uint32_t)));
    if (bad & 1u) {
      err = "species index out of range";
      return -1;
    }
    if (bad & 2u) {
      err = "molecule outside the partition";
      return -4;
    }
    return 0;
  }

  int step(uint32_t n, std::string& err) override {
    if (nkeys_ == 0) {
      err = "no replica to step";
      return -1;
    }
    // a model without molecules yet (a release may add them later) steps on empty arrays,
    // as the reference's event does with an empty molecule list
    if (cap_ == 0 && ensure_capacity(1024, err)) return -2;
    uint32_t done = 0;
    while (done < n) {
      if (use_graphs_ && !profile_) {
        // two iterations return to the same parity; a single one (a caller stepping one
        // iteration at a time) flips it
        const int k = n - done >= 2 ? 2 : 1;
        cudaGraphExec_t& ge = graph_[parity_ + 2 * (k - 1)];
        if (!ge) {
          if (capture(parity_, k, err)) return -2;
        }
        MCG_CUDA(cudaGraphLaunch(ge, stream_));
        launches_ += (uint64_t)k * kernels_per_iteration();
        done += k;
        if (k == 1) parity_ ^= 1;
      } else {
        launch_iteration(state(parity_), profile_);
        MCG_CUDA(cudaGetLastError());
        parity_ ^= 1;
        done += 1;
      }
    }
    iterations_ += n;
    pending_iters_ += n;
    return 0;
  }

  int sync(std::string& err) override {
    // the counters' copy is ordered after all queued work and waited for: one round trip
    if (read_counters(err)) return -2;
    return status_to_error(cnt_.status, err);
  }

  int counts(uint32_t rep, uint64_t* out, std::string& err) override {
    if (rep >= max_rep_ || !reps_[rep].used) {
      err = "no such replica";
      return -1;
    }
    const Geo<T>& g = geos_h_[rep];
    {
      // one round trip: the counters and the row the queued iterations will have
      // written (each iteration advances the engine's iteration by one), then checked
      const uint64_t it = (uint64_t)cnt_.iteration + pending_iters_;
      if (it > g.it0 && it > rebin_it_ && it <= 0xFFFFFFFFull) {
        const uint64_t row = (it - 1) % traj_cap_;
        unsigned long long h[MAXSP];
        Counters c;
        MCG_CUDA(cudaMemcpyAsync(&c, d_cnt_, sizeof(Counters), cudaMemcpyDeviceToHost, stream_));
        MCG_CUDA(cudaMemcpyAsync(h, d_traj_ + (row * max_rep_ + rep) * nsp_, sizeof(unsigned long long) * nsp_,
                                 cudaMemcpyDeviceToHost, stream_));
        MCG_CUDA(cudaStreamSynchronize(stream_));
        cnt_ = c;
        pending_iters_ = 0;
        int rc = status_to_error(cnt_.status, err);
        if (rc) return rc;
        if (cnt_.iteration == it) {
          for (uint32_t a = 0; a < nsp_; a++) out[a] = h[a];
          return 0;
        }
      }
    }
    int rc = sync(err);
    if (rc) return rc;
    if (cnt_.iteration > g.it0 && cnt_.iteration > rebin_it_) {
      // species counts of the last finished iteration (k_end)
      const uint64_t row = (cnt_.iteration - 1) % traj_cap_;
      std::vector<unsigned long long> h(nsp_);
      MCG_CUDA(d2h(h.data(), d_traj_ + (row * max_rep_ + rep) * nsp_, sizeof(unsigned long long) * nsp_));
      for (uint32_t a = 0; a < nsp_; a++) out[a] = h[a];
      return 0;
    }
    // before the replica's first iteration: from the start offsets of its key ranges
    const uint32_t span = g.n3 << g.oct_shift;
    const uint32_t* st = state(parity_).start;
    for (uint32_t a = 0; a < nsp_; a++) {
      uint32_t lo = 0, hi = 0;
      MCG_CUDA(d2h(&lo, st + g.kbase + a * span, sizeof(uint32_t)));
      MCG_CUDA(d2h(&hi, st + g.kbase + (a + 1) * span, sizeof(uint32_t)));
      out[a] = hi - lo;
    }
    return 0;
  }

  // Non-blocking counts. The copy of the counters and of the row the queued iterations
  // will have written goes on the stream after them, into pinned slots, followed by an
  // event; the wait is on that event alone, so iterations queued after the request keep
  // running while the host reads. Before a replica's first iteration since its
  // molecules were added the counts come from the start offsets, read at once.
  int request_counts(uint32_t rep, uint64_t* ticket, std::string& err) override {
    if (rep >= max_rep_ || !reps_[rep].used) {
      err = "no such replica";
      return -1;
    }
    if (!cslot_host_) {
      MCG_CUDA(cudaMallocHost(&cslot_host_, sizeof(CountSlotHost) * NCSLOT));
      for (int k = 0; k < NCSLOT; k++) {
        MCG_CUDA(cudaEventCreateWithFlags(&cslot_ev_[k], cudaEventDisableTiming));
        cslot_ticket_[k] = 0;
      }
    }
    const uint64_t t = next_ticket_;
    const int k = (int)(t % NCSLOT);
    CountSlotHost& h = cslot_host_[k];
    const Geo<T>& g = geos_h_[rep];
    const uint64_t it = (uint64_t)cnt_.iteration + pending_iters_;
    if (it > g.it0 && it > rebin_it_ && it <= 0xFFFFFFFFull) {
      const uint64_t row = (it - 1) % traj_cap_;
      // the counters' head (through the status word and the iteration: 64 bytes) is
      // all the wait reads, not the escape records after it
      static_assert(offsetof(Counters, mol_steps) == 64, "counters head");
      MCG_CUDA(cudaMemcpyAsync(&h.c, d_cnt_, offsetof(Counters, mol_steps), cudaMemcpyDeviceToHost, stream_));
      MCG_CUDA(cudaMemcpyAsync(h.n, d_traj_ + (row * max_rep_ + rep) * nsp_, sizeof(unsigned long long) * nsp_,
                               cudaMemcpyDeviceToHost, stream_));
      cslot_it_[k] = it;
    } else {
      uint64_t out[MAXSP];
      int rc = counts(rep, out, err);
      if (rc) return rc;
      for (uint32_t a = 0; a < nsp_; a++) h.n[a] = out[a];
      h.c = cnt_;
      cslot_it_[k] = cnt_.iteration;
    }
    MCG_CUDA(cudaEventRecord(cslot_ev_[k], stream_));
    cslot_ticket_[k] = t;
    next_ticket_++;
    *ticket = t;
    return 0;
  }

  int wait_counts(uint64_t ticket, uint64_t* out, std::string& err) override {
    const int k = (int)(ticket % NCSLOT);
    if (!cslot_host_ || ticket == 0 || cslot_ticket_[k] != ticket) {
      err = "unknown ticket, or one whose slot a later request took";
      return -1;
    }
    MCG_CUDA(cudaEventSynchronize(cslot_ev_[k]));
    const CountSlotHost& h = cslot_host_[k];
    int rc = status_to_error(h.c.status, err);
    if (rc) return rc;
    if (h.c.iteration != cslot_it_[k]) {
      err = "the counts of the requested iteration were not written";
      return -2;
    }
    for (uint32_t a = 0; a < nsp_; a++) out[a] = h.n[a];
    return 0;
  }

  int trajectory(uint32_t rep, uint32_t n, uint64_t* out, std::string& err) override {
    int rc = sync(err);
    if (rc) return rc;
    if (rep >= max_rep_ || !reps_[rep].used) {
      err = "no such replica";
      return -1;
    }
    const uint64_t ran = cnt_.iteration - geos_h_[rep].it0;
    if (n > ran || n > traj_cap_ - 1) {
      err = "trajectory longer than the iterations run or the ring";
      return -1;
    }
    const uint64_t last = cnt_.iteration;  // rows 0..iteration-1 hold finished iterations
    std::vector<unsigned long long> h((size_t)n * nsp_);
    uint32_t k = 0;
    while (k < n) {
      const uint64_t row = (last - n + k) % traj_cap_;
      const uint32_t rows = (uint32_t)std::min<uint64_t>(n - k, traj_cap_ - row);
      MCG_CUDA(cudaMemcpy2DAsync(h.data() + (size_t)k * nsp_, sizeof(unsigned long long) * nsp_,
                                 d_traj_ + (row * max_rep_ + rep) * nsp_, sizeof(unsigned long long) * nsp_ * max_rep_,
                                 sizeof(unsigned long long) * nsp_, rows, cudaMemcpyDeviceToHost, stream_));
      MCG_CUDA(cudaStreamSynchronize(stream_));
      k += rows;
    }
    for (size_t q = 0; q < h.size(); q++) out[q] = h[q];
    return 0;
  }

  int download(uint32_t rep, uint64_t capn, double* pos, uint32_t* species, uint64_t* ids, uint64_t* n_out,
               std::string& err) override {
    int rc = sync(err);
    if (rc) return rc;
    if (rep >= max_rep_ || !reps_[rep].used) {
      err = "no such replica";
      return -1;
    }
    const Geo<T>& g = geos_h_[rep];
    State<T> s = state(parity_);
    uint32_t lo = 0, hi = 0;
    MCG_CUDA(d2h(&lo, s.start + g.kbase, sizeof(uint32_t)));
    MCG_CUDA(d2h(&hi, s.start + g.kbase + nsp_ * (g.n3 << g.oct_shift), sizeof(uint32_t)));
    const uint32_t n = hi - lo;
    *n_out = n;
    if (n == 0) return 0;
    std::vector<P4<T>> p(n);
    std::vector<uint64_t> u(n);
    MCG_CUDA(d2h(p.data(), s.a_pos + lo, sizeof(P4<T>) * n));
    MCG_CUDA(d2h(u.data(), s.a_uid + lo, sizeof(uint64_t) * n));
    for (uint64_t i = 0; i < std::min<uint64_t>(n, capn); i++) {
      if (pos) {
        pos[3 * i] = (double)p[i].x;
        pos[3 * i + 1] = (double)p[i].y;
        pos[3 * i + 2] = (double)p[i].z;
      }
      if (species) species[i] = host_meta(p[i]) & META_SPECIES_MASK;
      if (ids) ids[i] = u[i];
    }
    return 0;
  }

  int export_state(uint32_t rep, uint64_t capn, double* pos, uint32_t* species, uint64_t* ids, double* tuni,
                   uint8_t* flags, uint64_t* n_out, uint64_t* iteration, std::string& err) override {
    int rc = download(rep, capn, pos, species, ids, n_out, err);
    if (rc) return rc;
    *iteration = cnt_.iteration - geos_h_[rep].it0;
    const uint64_t n = std::min<uint64_t>(*n_out, capn);
    if (n == 0 || (!tuni && !flags)) return 0;
    const Geo<T>& g = geos_h_[rep];
    State<T> s = state(parity_);
    uint32_t lo = 0;
    MCG_CUDA(d2h(&lo, s.start + g.kbase, sizeof(uint32_t)));
    std::vector<P4<T>> p(n);
    std::vector<T> t(n);
    MCG_CUDA(d2h(p.data(), s.a_pos + lo, sizeof(P4<T>) * n));
    MCG_CUDA(d2h(t.data(), s.a_tuni + lo, sizeof(T) * n));
    for (uint64_t i = 0; i < n; i++) {
      if (tuni) tuni[i] = (double)t[i];
      if (flags) flags[i] = (uint8_t)(((host_meta(p[i]) & META_SCHEDULE_UNIMOL) ? 1 : 0) | (meta_cv(host_meta(p[i])) << 1));
    }
    return 0;
  }

  int release(uint32_t rep, uint32_t species, uint64_t n, int shape, const double* center, const double* diameter,
              uint32_t object, uint64_t seed, std::string& err) override {
    if (rep >= max_rep_ || !reps_[rep].used) {
      err = "no such replica";
      return -1;
    }
    if (species >= nsp_ || shape < REL_SPHERE || shape > REL_INSIDE || n == 0 || n > 0xFFFFFFF0ull) {
      err = "invalid release";
      return -1;
    }
    const Rep& R = reps_[rep];
    const Geo<T>& g = geos_h_[rep];
    ReleaseDesc d{};
    d.rep = rep;
    d.species = species;
    d.n = (uint32_t)n;
    d.object = object;
    d.shape = shape;
    d.seed = seed;
    d.uid0 = R.next_uid;
    double lo[3], hi[3];
    if (shape == REL_INSIDE) {
      if (!R.has_obj || object >= R.obj_llf.size() / 3 || R.obj_llf[3 * object] > R.obj_urb[3 * object]) {
        err = "release inside an object: no walls of that object (mcg_set_wall_objects)";
        return -1;
      }
      for (int a = 0; a < 3; a++) {
        d.llf[a] = lo[a] = R.obj_llf[3 * object + a];
        d.urb[a] = hi[a] = R.obj_urb[3 * object + a];
        d.leaf_llf[0][a] = d.llf[a];
      }
      d.expr[0] = (int32_t)object;
      d.n_expr = 1;
    } else {
      for (int a = 0; a < 3; a++) {
        d.center[a] = center[a];
        d.diameter[a] = diameter[a];
        lo[a] = center[a] - 0.5 * std::fabs(diameter[a]);
        hi[a] = center[a] + 0.5 * std::fabs(diameter[a]);
      }
    }
    const double o[3] = {(double)g.origin.x, (double)g.origin.y, (double)g.origin.z};
    const double q[3] = {(double)g.opposite.x, (double)g.opposite.y, (double)g.opposite.z};
    for (int a = 0; a < 3; a++)
      if (!(lo[a] >= o[a] && hi[a] < q[a])) {
        err = "release region outside the partition";
        return -4;
      }
    if (read_counters(err)) return -2;
    const uint64_t live = cnt_.n_live;
    if (live + n > cap_ && ensure_capacity(std::max<uint64_t>((live + n) * 3 / 2, 1024), err)) return -2;
    if (n > base_.prod_cap && ensure_prod(n, err)) return -2;
    k_release<T><<<grid(n), TPB, 0, stream_>>>(state(parity_), d);
    launches_ += 1;
    MCG_CUDA(cudaGetLastError());
    reps_[rep].next_uid += n;
    return rebin(nullptr, n, err);
  }

  // the descriptor of a release into a region expression: its program, the box of each
  // leaf object, the expression's box (inside the partition), and the count (method
  // and number or concentration, the reference's rules; single_draw for an
  // expression's approximate concentration count)
  int region_desc(uint32_t rep, uint32_t species, int method, int64_t number, double concentration,
                  double length_unit, const int32_t* expr, uint32_t n_expr, ReleaseDesc& d, int64_t& count,
                  std::string& err) {
    if (rep >= max_rep_ || !reps_[rep].used) {
      err = "no such replica";
      return -1;
    }
    const Rep& R = reps_[rep];
    if (species >= nsp_ || (method != 0 && method != 1)) {
      err = "invalid release";
      return -1;
    }
    if (!R.has_obj) {
      err = "region releases need the walls' objects (mcg_set_wall_objects)";
      return -1;
    }
    const uint32_t nobj = (uint32_t)(R.obj_llf.size() / 3);
    if (!region_expr_valid(expr, n_expr, nobj)) {
      err = "invalid region expression (postfix program of objects and operators, at most 15 tokens)";
      return -1;
    }
    d = ReleaseDesc{};
    d.rep = rep;
    d.species = species;
    d.shape = REL_INSIDE;
    d.n_expr = n_expr;
    for (uint32_t k = 0; k < n_expr; k++) {
      d.expr[k] = expr[k];
      if (expr[k] < 0) continue;
      const uint32_t o = (uint32_t)expr[k];
      if (R.obj_llf[3 * o] > R.obj_urb[3 * o]) {
        err = "region expression: an object without walls";
        return -1;
      }
      for (int a = 0; a < 3; a++) d.leaf_llf[k][a] = R.obj_llf[3 * o + a];
    }
    region_expr_bbox(expr, n_expr, R.obj_llf.data(), R.obj_urb.data(), d.llf, d.urb);
    const Geo<T>& g = geos_h_[rep];
    const double o[3] = {(double)g.origin.x, (double)g.origin.y, (double)g.origin.z};
    const double q[3] = {(double)g.opposite.x, (double)g.opposite.y, (double)g.opposite.z};
    for (int a = 0; a < 3; a++)
      if (!(d.llf[a] >= o[a] && d.urb[a] < q[a])) {
        err = "release region outside the partition";
        return -4;
      }
    if (method == 1) {
      // num_vol_mols_from_conc (release_event.cpp:826-856): one object's volume, exact;
      // an expression's bounding box, approximate (each draw counts)
      if (!(concentration >= 0) || !(length_unit > 0)) {
        err = "invalid concentration or length unit";
        return -1;
      }
      double vol;
      if (n_expr == 1) {
        vol = R.obj_vol[(uint32_t)expr[0]];
      } else {
        vol = (d.urb[0] - d.llf[0]) * (d.urb[1] - d.llf[1]) * (d.urb[2] - d.llf[2]);
        d.single_draw = 1;
      }
      const double num = concentration_number(concentration, vol, length_unit);
      if (!(num >= 0) || num > 2147483647.0) {  // check_max_release_count (:497-506)
        err = "concentration release of more than INT_MAX molecules";
        return -1;
      }
      count = (int64_t)(uint32_t)num;
    } else {
      count = number;
    }
    if (count > (int64_t)0xFFFFFFF0ll || count < -(int64_t)0xFFFFFFF0ll) {
      err = "invalid release";
      return -1;
    }
    return 0;
  }

  // the molecules of d.species inside d's region, in id order
  int vacuum_candidates(const ReleaseDesc& d, std::vector<std::pair<uint64_t, uint32_t>>& cand, std::string& err) {
    if (read_counters(err)) return -2;
    const uint32_t n = cnt_.n_live;
    cand.clear();
    if (n == 0) return 0;
    AllocSet tmp;
    uint64_t* d_ids;
    uint32_t *d_idx, *d_cnt;
    MCG_CUDA(tmp.get(&d_ids, sizeof(uint64_t) * n));
    MCG_CUDA(tmp.get(&d_idx, sizeof(uint32_t) * n));
    MCG_CUDA(tmp.get(&d_cnt, sizeof(uint32_t)));
    MCG_CUDA(cudaMemsetAsync(d_cnt, 0, sizeof(uint32_t), stream_));
    k_vacuum_candidates<T><<<grid(n), TPB, 0, stream_>>>(state(parity_), d, d_ids, d_idx, d_cnt);
    launches_ += 1;
    MCG_CUDA(cudaGetLastError());
    uint32_t m = 0;
    MCG_CUDA(d2h(&m, d_cnt, sizeof(uint32_t)));
    std::vector<uint64_t> ids(m);
    std::vector<uint32_t> idx(m);
    if (m) {
      MCG_CUDA(d2h(ids.data(), d_ids, sizeof(uint64_t) * m));
      MCG_CUDA(d2h(idx.data(), d_idx, sizeof(uint32_t) * m));
    }
    cand.resize(m);
    for (uint32_t k = 0; k < m; k++) cand[k] = {ids[k], idx[k]};
    std::sort(cand.begin(), cand.end());
    return 0;
  }

  int release_region(uint32_t rep, uint32_t species, int method, int64_t number, double concentration,
                     double length_unit, const int32_t* expr, uint32_t n_expr, uint64_t seed, int64_t* done,
                     std::string& err) override {
    ReleaseDesc d;
    int64_t count = 0;
    int rc = region_desc(rep, species, method, number, concentration, length_unit, expr, n_expr, d, count, err);
    if (rc) return rc;
    *done = 0;
    if (count == 0) return 0;
    if (count < 0) {
      // vacuum_inside_regions: the candidates in id order, each removed with the
      // probability of the removals left over the candidates left
      std::vector<std::pair<uint64_t, uint32_t>> cand;
      if ((rc = vacuum_candidates(d, cand, err))) return rc;
      std::vector<uint8_t> chosen(cand.size());
      std::mt19937_64 gen(seed);
      const int removed = select_for_removal((uint32_t)cand.size(), (uint32_t)(-count), [&]() {
        return (double)(uint32_t)(gen() >> 32) * (1.0 / 4294967296.0);
      }, chosen.data());
      if (removed == 0) return 0;
      const uint32_t n = cnt_.n_live;
      std::vector<uint8_t> mask(n, 0);
      for (size_t k = 0; k < cand.size(); k++)
        if (chosen[k]) mask[cand[k].second] = 1;
      AllocSet tmp;
      uint8_t* d_mask;
      MCG_CUDA(tmp.get(&d_mask, n));
      MCG_CUDA(cudaMemcpyAsync(d_mask, mask.data(), n, cudaMemcpyHostToDevice, stream_));
      if ((rc = rebin(nullptr, 0, err, false, d_mask))) return rc;
      *done = -(int64_t)removed;
      return 0;
    }
    if (read_counters(err)) return -2;
    const uint64_t live = cnt_.n_live, n = (uint64_t)count;
    if (live + n > cap_ && ensure_capacity(std::max<uint64_t>((live + n) * 3 / 2, 1024), err)) return -2;
    if (n > base_.prod_cap && ensure_prod(n, err)) return -2;
    d.n = (uint32_t)n;
    d.seed = seed;
    d.uid0 = reps_[rep].next_uid;
    k_release<T><<<grid(n), TPB, 0, stream_>>>(state(parity_), d);
    launches_ += 1;
    MCG_CUDA(cudaGetLastError());
    reps_[rep].next_uid += n;
    if ((rc = rebin(nullptr, n, err, false, nullptr, 1))) return rc;
    *done = (int64_t)cnt_.n_live - (int64_t)live;
    return 0;
  }

  uint64_t next_molecule_id(uint32_t rep) override {
    return rep < max_rep_ && reps_[rep].used ? reps_[rep].next_uid : 0;
  }

  int release_region_harness(uint32_t rep, uint32_t species, int method, int64_t number, double concentration,
                             double length_unit, const int32_t* expr, uint32_t n_expr, const uint32_t* draws,
                             uint32_t n_draws, double* pos, uint32_t cap, uint32_t* n_pos, uint64_t* removed,
                             uint32_t* n_removed, uint32_t* used, std::string& err) override {
    ReleaseDesc d;
    int64_t count = 0;
    int rc = region_desc(rep, species, method, number, concentration, length_unit, expr, n_expr, d, count, err);
    if (rc) return rc;
    *n_pos = 0;
    *n_removed = 0;
    *used = 0;
    if (count < 0) {
      std::vector<std::pair<uint64_t, uint32_t>> cand;
      if ((rc = vacuum_candidates(d, cand, err))) return rc;
      std::vector<uint8_t> chosen(cand.size());
      uint32_t k = 0;
      bool over = false;
      select_for_removal((uint32_t)cand.size(), (uint32_t)(-count), [&]() {
        if (k >= n_draws) {
          over = true;
          return 0.0;
        }
        return (double)draws[k++] * (1.0 / 4294967296.0);
      }, chosen.data());
      uint32_t nr = 0;
      for (size_t q = 0; q < cand.size(); q++)
        if (chosen[q]) {
          if (nr < cap) removed[nr] = cand[q].first;
          nr++;
        }
      *n_removed = nr;
      *used = over ? 0xFFFFFFFFu : k;
      return 0;
    }
    d.n = (uint32_t)count;
    AllocSet tmp;
    uint32_t *d_draws, *d_out_n;
    double* d_pos;
    MCG_CUDA(tmp.get(&d_draws, sizeof(uint32_t) * std::max<uint32_t>(n_draws, 1)));
    MCG_CUDA(tmp.get(&d_pos, sizeof(double) * 3 * std::max<uint32_t>(cap, 1)));
    MCG_CUDA(tmp.get(&d_out_n, sizeof(uint32_t) * 2));
    if (n_draws) MCG_CUDA(cudaMemcpyAsync(d_draws, draws, sizeof(uint32_t) * n_draws, cudaMemcpyHostToDevice, stream_));
    k_release_region_harness<T><<<1, 32, 0, stream_>>>(state(parity_), d, d_draws, n_draws, d_pos, cap, d_out_n,
                                                        d_out_n + 1);
    launches_ += 1;
    MCG_CUDA(cudaGetLastError());
    uint32_t out2[2];
    MCG_CUDA(d2h(out2, d_out_n, sizeof(out2)));
    *n_pos = out2[0];
    *used = out2[1];
    if (out2[0] && cap) MCG_CUDA(d2h(pos, d_pos, sizeof(double) * 3 * std::min(cap, out2[0])));
    return 0;
  }

  int import_state(uint32_t rep, uint64_t n, const double* pos, const uint32_t* species, const uint64_t* ids,
                   const double* tuni, const uint8_t* flags, uint64_t iteration, std::string& err) override {
    if (rep >= max_rep_ || !reps_[rep].used) {
      err = "no such replica";
      return -1;
    }
    if (read_counters(err)) return -2;
    if (iterations_ != 0 || cnt_.n_live != 0 || iteration > 0xFFFFFFF0ull) {
      err = "a checkpoint is loaded into a prepared engine before any molecule or iteration";
      return -1;
    }
    std::unique_ptr<Product<T>[]> stage(new Product<T>[n]);  // filled by stage_molecules
    int rc = stage_molecules(rep, n, pos, species, 0, stage.get(), err);
    if (rc) return rc;
    for (uint64_t i = 0; i < n; i++) {
      stage[i].uid = ids[i];
      stage[i].tuni = tuni[i];
      put_meta(stage[i].pos, make_meta(species[i], rep,
                                       ((flags[i] & 1) ? META_SCHEDULE_UNIMOL : 0) | ((uint32_t)(flags[i] >> 1) << META_CV_SHIFT)));
      reps_[rep].next_uid = std::max<uint64_t>(reps_[rep].next_uid, ids[i] + 1);
    }
    // the engine continues at the checkpoint's iteration: the replica's random streams
    // (seed, molecule id, iteration) pick up where they stopped
    Counters c = cnt_;
    c.iteration = (uint32_t)iteration;
    MCG_CUDA(cudaMemcpyAsync(d_cnt_, &c, sizeof(Counters), cudaMemcpyHostToDevice, stream_));
    cnt_ = c;
    geos_h_[rep].it0 = 0;
    MCG_CUDA(cudaMemcpyAsync(d_geos_, geos_h_.data(), sizeof(Geo<T>) * max_rep_, cudaMemcpyHostToDevice, stream_));
    rc = rebin(stage.get(), n, err);
    rebin_it_ = cnt_.iteration;
    return rc;
  }

  int counted_counts(uint32_t rep, uint64_t* out, std::string& err) override {
    int rc = sync(err);
    if (rc) return rc;
    if (rep >= max_rep_ || !reps_[rep].used || !reps_[rep].n_cv || !d_cv_now_) {
      err = "no counted objects in this model";
      return -1;
    }
    const uint32_t nc = reps_[rep].n_cv;
    std::vector<uint32_t> h((size_t)nsp_ * MAX_COUNTED);
    MCG_CUDA(d2h(h.data(), d_cv_now_ + (size_t)rep * nsp_ * MAX_COUNTED, sizeof(uint32_t) * h.size()));
    for (uint32_t a = 0; a < nsp_; a++)
      for (uint32_t k = 0; k < nc; k++) out[a * nc + k] = h[a * MAX_COUNTED + k];
    return 0;
  }

  int counted_trajectory(uint32_t rep, uint32_t n, uint64_t* out, std::string& err) override {
    int rc = sync(err);
    if (rc) return rc;
    if (rep >= max_rep_ || !reps_[rep].used || !reps_[rep].n_cv || !d_cv_traj_) {
      err = "no counted objects in this model";
      return -1;
    }
    if (n > cnt_.iteration - geos_h_[rep].it0 || n > cv_traj_cap_ - 1) {
      err = "trajectory longer than the iterations run or the ring";
      return -1;
    }
    const uint32_t nc = reps_[rep].n_cv;
    const size_t nq = (size_t)max_rep_ * nsp_ * MAX_COUNTED;
    std::vector<uint32_t> h((size_t)nsp_ * MAX_COUNTED);
    for (uint32_t k = 0; k < n; k++) {
      const uint64_t row = (cnt_.iteration - n + k) % cv_traj_cap_;
      MCG_CUDA(d2h(h.data(), d_cv_traj_ + row * nq + (size_t)rep * nsp_ * MAX_COUNTED, sizeof(uint32_t) * h.size()));
      for (uint32_t a = 0; a < nsp_; a++)
        for (uint32_t o = 0; o < nc; o++) out[((size_t)k * nsp_ + a) * nc + o] = h[a * MAX_COUNTED + o];
    }
    return 0;
  }

  int replica_rows(uint32_t rep, uint32_t* n_counted, uint64_t* since_added, std::string& err) override {
    int rc = sync(err);
    if (rc) return rc;
    if (rep >= max_rep_ || !reps_[rep].used) {
      err = "no such replica";
      return -1;
    }
    *n_counted = reps_[rep].n_cv;
    *since_added = cnt_.iteration - geos_h_[rep].it0;
    return 0;
  }

  int replica_iterations(uint32_t rep, uint64_t* done, std::string& err) override {
    int rc = sync(err);
    if (rc) return rc;
    if (rep >= max_rep_ || !reps_[rep].used) {
      err = "no such replica";
      return -1;
    }
    const Geo<T>& g = geos_h_[rep];
    *done = std::min<uint64_t>(cnt_.iteration, g.it_end) - g.it0;
    return 0;
  }

  uint64_t replica_bytes(uint32_t rep) override {
    if (rep >= max_rep_ || !reps_[rep].used) return 0;
    return reps_[rep].bytes + (uint64_t)reps_[rep].span * 16;
  }

  uint64_t device_bytes() override {
    uint64_t b = (uint64_t)cap_ * (2 * (sizeof(P4<T>) + 8 + sizeof(T)) + sizeof(P4<T>) + 1 + 8);
    b += (uint64_t)base_.prop_cap * (2 * sizeof(Proposal) + 8) + (uint64_t)base_.prod_cap * (sizeof(Product<T>) + 1);
    b += (uint64_t)key_alloc_ * 16 + (uint64_t)traj_cap_ * max_rep_ * nsp_ * 8;
    for (uint32_t r = 0; r < max_rep_; r++)
      if (reps_[r].used) b += reps_[r].bytes;
    return b;
  }

  int trace(uint32_t nc, const uint64_t* ids, const double* disp, const uint32_t* draws, uint32_t ndraws,
            const double* rrf, const double* tst, double* out, std::string& err) override {
    int rc = sync(err);
    if (rc) return rc;
    const uint32_t n = cnt_.n_live;
    State<T> s = state(parity_);
    std::vector<uint64_t> u(n);
    MCG_CUDA(d2h(u.data(), s.a_uid, sizeof(uint64_t) * n));
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
    AllocSet tmp;  // freed on every return
    MCG_CUDA(tmp.get(&d_idx, sizeof(uint32_t) * nc));
    MCG_CUDA(tmp.get(&d_disp, sizeof(double) * 3 * nc));
    MCG_CUDA(tmp.get(&d_rrf, sizeof(double) * nc));
    MCG_CUDA(tmp.get(&d_tst, sizeof(double) * nc));
    MCG_CUDA(tmp.get(&d_out, sizeof(double) * 265 * nc));
    MCG_CUDA(tmp.get(&d_draws, sizeof(uint32_t) * std::max<uint64_t>((uint64_t)ndraws * nc, 1)));
    MCG_CUDA(cudaMemcpyAsync(d_idx, idx.data(), sizeof(uint32_t) * nc, cudaMemcpyHostToDevice, stream_));
    MCG_CUDA(cudaMemcpyAsync(d_disp, disp, sizeof(double) * 3 * nc, cudaMemcpyHostToDevice, stream_));
    MCG_CUDA(cudaMemcpyAsync(d_rrf, rrf, sizeof(double) * nc, cudaMemcpyHostToDevice, stream_));
    MCG_CUDA(cudaMemcpyAsync(d_tst, tst, sizeof(double) * nc, cudaMemcpyHostToDevice, stream_));
    if (ndraws) MCG_CUDA(cudaMemcpyAsync(d_draws, draws, sizeof(uint32_t) * ndraws * nc, cudaMemcpyHostToDevice, stream_));
    k_trace_cases<T><<<(nc + 127) / 128, 128, 0, stream_>>>(s, nc, d_idx, d_disp, d_draws, ndraws, d_rrf, d_tst, d_out);
    launches_ += 1;
    MCG_CUDA(cudaGetLastError());
    MCG_CUDA(cudaStreamSynchronize(stream_));
    MCG_CUDA(d2h(out, d_out, sizeof(double) * 265 * nc));
    return 0;
  }

  int trace_static(uint32_t nc, const uint64_t* ids, const double* disp, const uint32_t* draws, uint32_t ndraws,
                   const double* rrf, const double* tst, double* out, std::string& err) override {
    int cur = -1;
    MCG_CUDA(cudaGetDevice(&cur));
    if (cur != dev_) {
      err = "mcg_trace_cases_static: the calling thread's current device is not the engine's";
      return -1;
    }
    int rc = sync(err);
    if (rc) return rc;
    unsigned char* sc = static_scratch_;
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

  int set_trace_limits(int maxc, int maxset, std::string& err) override {
    if (maxc < 1 || maxc > MAXC || maxset < 1 || maxset > MAXSET) {
      err = "trace limits out of range (1..16 candidates, 1..48 subpartitions)";
      return -1;
    }
    base_.maxc = maxc;
    base_.maxset = maxset;
    invalidate_graphs();
    return 0;
  }

  int fallbacks(uint64_t* out, std::string& err) override {
    int rc = sync(err);
    if (rc) return rc;
    out[0] = cnt_.warn_coll_overflow;
    out[1] = cnt_.warn_set_overflow;
    out[2] = cnt_.warn_inside_redo;
    return 0;
  }

  int inside_tests(uint32_t rep, uint32_t n, const double* pos, int kind, uint32_t obj, uint32_t* out,
                   std::string& err) override {
    int rc = sync(err);
    if (rc) return rc;
    if (rep >= max_rep_ || !reps_[rep].used) {
      err = "no such replica";
      return -1;
    }
    const Rep& R = reps_[rep];
    double llf[3] = {0, 0, 0};
    if (kind == 1) {
      if (!R.has_obj || obj >= R.obj_llf.size() / 3 || R.obj_llf[3 * obj] > R.obj_urb[3 * obj]) {
        err = "no walls of that object (mcg_set_wall_objects)";
        return -1;
      }
      for (int a = 0; a < 3; a++) llf[a] = R.obj_llf[3 * obj + a];
    } else if (!R.n_cv) {
      err = "no counted objects in this model";
      return -1;
    } else if (!R.has_obj) {
      err = "counted objects need wall objects";
      return -1;
    }
    if (n == 0) return 0;
    AllocSet tmp;
    double *d_pos, *d_llf;
    uint32_t* d_out;
    MCG_CUDA(tmp.get(&d_pos, sizeof(double) * 3 * n));
    MCG_CUDA(tmp.get(&d_llf, sizeof(double) * 3));
    MCG_CUDA(tmp.get(&d_out, sizeof(uint32_t) * n));
    MCG_CUDA(cudaMemcpyAsync(d_pos, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, stream_));
    MCG_CUDA(cudaMemcpyAsync(d_llf, llf, sizeof(double) * 3, cudaMemcpyHostToDevice, stream_));
    k_inside_tests<T><<<grid(n), TPB, 0, stream_>>>(state(parity_), rep, n, d_pos, kind, obj, d_llf, d_out);
    launches_ += 1;
    MCG_CUDA(cudaGetLastError());
    MCG_CUDA(d2h(out, d_out, sizeof(uint32_t) * n));
    return 0;
  }

  void set_options(int use_graphs, int profile) override {
    use_graphs_ = use_graphs != 0;
    profile_ = profile != 0;
  }

  int set_diffuse_blocks_per_sm(int blocks, std::string& err) override {
    if (blocks < 0 || blocks > bps_max_) {
      err = "diffuse blocks per SM out of range";
      return -1;
    }
    diffuse_grid_ = (blocks ? blocks : bps_max_) * sms_;
    invalidate_graphs();
    return 0;
  }

  int max_diffuse_blocks_per_sm() override { return bps_max_; }

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
      MCG_CUDA(dev_malloc(&d_debug_, sizeof(double) * 64 * 271));
    }
    MCG_CUDA(cudaMemsetAsync(d_debug_, 0, sizeof(double) * 64 * 271, stream_));
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
    MCG_CUDA(d2h(out, d_debug_, sizeof(double) * 64 * 271));
    return 0;
  }

  int escapes(double* out, uint32_t cap, uint32_t* n, std::string& err) override {
    MCG_CUDA(cudaStreamSynchronize(stream_));
    if (read_counters(err)) return -2;
    *n = cnt_.n_esc;
    for (uint32_t k = 0; k < std::min<uint32_t>(std::min<uint32_t>(cap, cnt_.n_esc), 8); k++)
      for (int q = 0; q < 13; q++) out[k * 13 + q] = cnt_.esc[k][q];
    return 0;
  }

  void stats(uint64_t* iterations, uint64_t* mol_steps, uint64_t* launches) override {
    std::string e;
    sync(e);
    if (iterations) *iterations = iterations_;
    if (mol_steps) *mol_steps = cnt_.mol_steps;
    if (launches) *launches = launches_;
  }

  int kernels_per_iteration() const { return (prod_chain_ ? 15 : 13) + 3 * GRID_REDO_ROUNDS; }
  bool prod_chain_ = true;  // two products passes (layout_keys decides)

 private:
  // host view of one replica slot
  struct Rep {
    bool used = false;
    uint32_t span = 0;      // sort keys: nsp * n3 << oct_shift
    uint64_t bytes = 0;     // device bytes of its mesh, wall lists and tables
    uint64_t next_uid = 0;  // next molecule id for uploads
    P4<T>* wrej = nullptr;
    WallFace<T>* wface = nullptr;
    uint32_t* wsp_off = nullptr;
    uint32_t* wsp_list = nullptr;
    uint64_t* wsp_cells = nullptr;
    uint32_t* wsp_cm = nullptr;
    uint64_t* wsp_cellent = nullptr;
    uint8_t* wclass = nullptr;
    Chem* chem = nullptr;
    double* w64 = nullptr;  // fp32 engines: fp64 wall constants for the tie-breaks
    uint16_t* wall_obj = nullptr;  // geometry object of each wall
    bool has_obj = false;
    uint32_t n_cv = 0;     // counted objects
    double wall_density = 0;  // wall-list entries per subpartition (orders the key space)
    // counts before the replica's first iteration (the t = 0 row of its count files):
    // per species in the world, and per species and counted object
    std::vector<uint64_t> init_world, init_cv;
    std::vector<double> obj_llf, obj_urb;  // bounding box of each object's walls
    std::vector<double> obj_vol;           // volume of each closed object
    bool uni_products = false;             // some unimolecular reaction has products
    // host copies for placing fp32 molecules: wall planes (n xyz, d), walls per
    // subpartition, and the grid
    std::vector<double> planes;
    std::vector<uint32_t> h_wsp_off, h_wsp_list;
    double origin[3] = {0, 0, 0}, sp_rcp = 1;
    uint32_t nsub = 1;
  };

  // Rounding a position to fp32 can put a molecule that lies within a few ulps of
  // a wall on the plane or behind it, from where it would leave without a hit.
  // Such molecules are moved along the wall normal to 1e-4 internal units (or 8
  // ulps of the coordinates, if larger) from the plane, on their own side, before
  // rounding; the walls checked are those listed for the molecule's subpartition
  // (every wall within the reaction radius of it).
  void place_fp32(const Rep& R, double* p) const {
    if (sizeof(T) != 4 || R.planes.empty()) return;
    int ix[3];
    for (int a = 0; a < 3; a++) {
      ix[a] = (int)((p[a] - R.origin[a]) * R.sp_rcp);
      ix[a] = std::min(std::max(ix[a], 0), (int)R.nsub - 1);
    }
    const size_t sp = (size_t)ix[0] + (size_t)ix[1] * R.nsub + (size_t)ix[2] * R.nsub * R.nsub;
    const double mag = std::max(std::fabs(p[0]), std::max(std::fabs(p[1]), std::fabs(p[2])));
    const double margin = std::max(1e-4, 8.0 * mag * 1.1920928955078125e-07);
    for (int pass = 0; pass < 2; pass++) {  // a second pass only after a move (edges, corners)
      bool moved = false;
      for (uint32_t k = R.h_wsp_off[sp]; k < R.h_wsp_off[sp + 1]; k++) {
        const double* pl = &R.planes[4 * (size_t)R.h_wsp_list[k]];
        const double dd = pl[0] * p[0] + pl[1] * p[1] + pl[2] * p[2] - pl[3];
        if (std::fabs(dd) >= margin) continue;
        const double shift = (dd >= 0 ? margin : -margin) - dd;
        for (int a = 0; a < 3; a++) p[a] += shift * pl[a];
        moved = true;
      }
      if (!moved) break;
    }
  }

  // device -> host copy ordered on the engine stream; returns when the data is there
  cudaError_t d2h(void* h, const void* d, size_t n) {
    cudaError_t e = cudaMemcpyAsync(h, d, n, cudaMemcpyDeviceToHost, stream_);
    return e != cudaSuccess ? e : cudaStreamSynchronize(stream_);
  }

  static uint32_t host_meta(const P4<T>& p) {
    if (sizeof(T) == 8) {
      uint64_t m64;
      std::memcpy(&m64, &p.w, 8);
      return (uint32_t)m64;
    }
    uint32_t m;
    std::memcpy(&m, &p.w, 4);
    return m;
  }

  static void put_meta(P4<T>& p, uint32_t meta) {
    if (sizeof(T) == 8) {
      uint64_t m64 = meta;
      std::memcpy(&p.w, &m64, 8);
    } else {
      std::memcpy(&p.w, &meta, 4);
    }
  }

  template <typename V>
  int alloc_copy(V** d, const std::vector<V>& h, uint64_t& bytes, std::string& err) {
    const size_t sz = sizeof(V) * std::max<size_t>(h.size(), 1);
    MCG_CUDA(dev_malloc((void**)d, sz));
    bytes += sz;
    if (!h.empty()) MCG_CUDA(cudaMemcpyAsync(*d, h.data(), sizeof(V) * h.size(), cudaMemcpyHostToDevice, stream_));
    return 0;
  }

  // device copies of one model's walls, wall lists and reaction tables; its Geo entry
  int upload_replica(const ReplicaSpec& sp, uint32_t r, std::string& err) {
    const HostSetup& hs = *sp.hs;
    const ChemHost& ch = *sp.chem;
    const std::vector<uint8_t>& wall_class = *sp.wall_class;
    Rep& R = reps_[r];
    R = Rep();
    Geo<T> g{};
    g.origin = v3<T>((T)hs.origin[0], (T)hs.origin[1], (T)hs.origin[2]);
    g.opposite = v3<T>((T)hs.opposite[0], (T)hs.opposite[1], (T)hs.opposite[2]);
    g.part_edge = (T)hs.part_edge;
    g.sp_edge = (T)hs.sp_edge;
    g.sp_rcp = (T)hs.sp_rcp;
    g.R = (T)hs.R;
    g.nsub = (int)hs.nsub;
    g.nsub2 = (int)(hs.nsub * hs.nsub);
    g.nsp = (int)nsp_;
    g.n3 = hs.nsub * hs.nsub * hs.nsub;
    g.rcp_n = 1.0f / (float)hs.nsub;
    g.rcp_n2 = 1.0f / (float)(hs.nsub * hs.nsub);
    for (int a = 0; a < 3; a++) g.origin64[a] = hs.origin[a];
    g.sp_edge64 = hs.sp_edge;
    g.sp_rcp64 = hs.sp_rcp;
    const uint64_t base_keys = (uint64_t)g.n3 * nsp_;
    // occupants are binned per subpartition octant while the key space stays small
    g.oct_shift = (sp.octants && base_keys * 8 <= (1ull << 26)) ? 3 : 0;
    if ((base_keys << g.oct_shift) >= (1ull << 31)) {
      err = "subpartition grid too large";
      return -1;
    }
    g.rep = r;
    g.it0 = cnt_.iteration;
    g.it_end = sp.n_iterations ? cnt_.iteration + sp.n_iterations : UINT_MAX;
    g.mode = REP_RUN;
    g.seed = sp.seed;
    const uint32_t nw = hs.nw;
    std::vector<P4<T>> rej(std::max<uint32_t>(nw, 1));
    std::vector<WallFace<T>> face(std::max<uint32_t>(nw, 1));
    for (uint32_t w = 0; w < nw; w++) {
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
    // wall lists on the device: wall indices and the 4x4x4 cell mask of each entry
    std::vector<uint32_t> ent(std::max<size_t>(hs.wsp_list.size(), 1), 0);
    std::vector<uint64_t> cells(std::max<size_t>(hs.wsp_list.size(), 1), ~0ull);
    for (size_t k = 0; k < hs.wsp_list.size(); k++) {
      ent[k] = hs.wsp_list[k];
      cells[k] = hs.wsp_cells[k];
    }
    // per-cell entry masks of the subpartitions that list 1-64 walls: the wall search
    // then loads one mask per cell its segment touches instead of testing every entry
    const uint32_t n3h = hs.nsub * hs.nsub * hs.nsub;
    std::vector<uint32_t> cm(n3h, NONE);
    std::vector<uint64_t> cellent;
    for (uint32_t sp = 0; sp < n3h; sp++) {
      const uint32_t b = hs.wsp_off[sp], e = hs.wsp_off[sp + 1];
      if (e == b || e - b > 64) continue;
      cm[sp] = (uint32_t)(cellent.size() / 64);
      cellent.resize(cellent.size() + 64, 0);
      uint64_t* blk = &cellent[cellent.size() - 64];
      for (uint32_t k = b; k < e; k++)
        for (int c = 0; c < 64; c++)
          if ((hs.wsp_cells[k] >> c) & 1ull) blk[c] |= 1ull << (k - b);
    }
    if (cellent.empty()) cellent.assign(64, 0);
    Chem c;
    std::memset(&c, 0, sizeof(c));
    static_assert(MAXPW == MAX_PATHWAYS, "pathway tables of host and device differ");
    c.nsp = (int)ch.nsp;
    for (int a = 0; a < MAXSP; a++) {
      c.space_step[a] = ch.space_step[a];
      c.unimol_k[a] = ch.unimol_k[a];
      c.uni_npw[a] = (int8_t)ch.uni_npw[a];
      for (int k = 0; k < MAXPW; k++) {
        c.uni_cum[a][k] = ch.uni_cum[a][k];
        c.uni_prod[a][k][0] = (int8_t)ch.uni_prod[a][k][0];
        c.uni_prod[a][k][1] = (int8_t)ch.uni_prod[a][k][1];
      }
      for (int b = 0; b < MAXSP; b++) {
        c.bimol_p[a][b] = ch.bimol_p[a][b];
        c.bimol_npw[a][b] = (int8_t)ch.bimol_npw[a][b];
        for (int k = 0; k < MAXPW; k++) {
          c.bimol_cum[a][b][k] = ch.bimol_cum[a][b][k];
          c.bimol_prod[a][b][k][0] = (int8_t)ch.bimol_prod[a][b][k][0];
          c.bimol_prod[a][b][k][1] = (int8_t)ch.bimol_prod[a][b][k][1];
        }
        if (ch.bimol_npw[a][b] > 0) c.partners[a] |= 1u << b;
      }
    }
    for (uint32_t w = 0; w < nw; w++)
      for (uint32_t a = 0; a < ch.nsp; a++)
        if (wall_class[(size_t)w * ch.nsp + a]) c.can_volwall[a] = 1;
    // a unimolecular reaction with products: a product can make products in its birth step
    R.uni_products = false;
    for (uint32_t a = 0; a < ch.nsp; a++)
      for (int k = 0; k < (int)ch.uni_npw[a]; k++)
        if (ch.uni_prod[a][k][0] >= 0 || ch.uni_prod[a][k][1] >= 0) R.uni_products = true;
    R.used = true;  // from here on free_replica() releases what was allocated
    if (alloc_copy(&R.wrej, rej, R.bytes, err) || alloc_copy(&R.wface, face, R.bytes, err) ||
        alloc_copy(&R.wsp_off, hs.wsp_off, R.bytes, err) || alloc_copy(&R.wsp_list, ent, R.bytes, err) ||
        alloc_copy(&R.wsp_cells, cells, R.bytes, err) || alloc_copy(&R.wsp_cm, cm, R.bytes, err) ||
        alloc_copy(&R.wsp_cellent, cellent, R.bytes, err) ||
        alloc_copy(&R.wclass, wall_class.empty() ? std::vector<uint8_t>(1, 0) : wall_class, R.bytes, err) ||
        alloc_copy(&R.chem, std::vector<Chem>(1, c), R.bytes, err))
      return -2;
    g.wrej = R.wrej;
    g.wface = R.wface;
    g.wsp_off = R.wsp_off;
    g.wsp_list = R.wsp_list;
    g.wsp_cells = R.wsp_cells;
    g.wsp_cm = R.wsp_cm;
    g.wsp_cellent = R.wsp_cellent;
    g.wall_class = R.wclass;
    g.chem = R.chem;
    g.w64 = nullptr;
    if (sizeof(T) == 4) {
      std::vector<double> w64(16 * (size_t)std::max<uint32_t>(nw, 1), 0.0);
      for (uint32_t w = 0; w < nw; w++) {
        const double* o = &hs.wall[(size_t)w * 24];
        double* q = &w64[16 * (size_t)w];
        for (int k = 0; k < 10; k++) q[k] = o[k];  // normal, d, unit_u, unit_v
        q[10] = o[13];                               // v0
        q[11] = o[14];
        q[12] = o[15];
        q[13] = o[10];                               // uv_vert1_u, uv_vert2 u v
        q[14] = o[11];
        q[15] = o[12];
      }
      if (alloc_copy(&R.w64, w64, R.bytes, err)) return -2;
      g.w64 = R.w64;
    }
    g.wall_obj = nullptr;
    if (sp.wall_obj && sp.wall_obj->size() == nw && nw) {
      if (alloc_copy(&R.wall_obj, *sp.wall_obj, R.bytes, err)) return -2;
      g.wall_obj = R.wall_obj;
      R.has_obj = true;
      uint32_t nobj = 0;
      for (uint16_t o : *sp.wall_obj) nobj = std::max<uint32_t>(nobj, (uint32_t)o + 1);
      R.obj_llf.assign(3 * (size_t)nobj, 1e300);
      R.obj_urb.assign(3 * (size_t)nobj, -1e300);
      for (uint32_t w = 0; w < nw; w++) {
        const uint32_t ob = (*sp.wall_obj)[w];
        for (int v = 0; v < 3; v++)
          for (int a = 0; a < 3; a++) {
            const double x = hs.wall[(size_t)w * 24 + 13 + 3 * v + a];
            R.obj_llf[3 * ob + a] = std::min(R.obj_llf[3 * ob + a], x);
            R.obj_urb[3 * ob + a] = std::max(R.obj_urb[3 * ob + a], x);
          }
      }
      // the objects' volumes (concentration releases), from the walls' vertices
      std::vector<double> vx(9 * (size_t)nw);
      std::vector<uint32_t> tri(3 * (size_t)nw);
      for (uint32_t w = 0; w < nw; w++)
        for (int v = 0; v < 3; v++) {
          tri[3 * (size_t)w + v] = 3 * w + v;
          for (int a = 0; a < 3; a++) vx[9 * (size_t)w + 3 * v + a] = hs.wall[(size_t)w * 24 + 13 + 3 * v + a];
        }
      const MeshView mv{3 * nw, vx.data(), nw, tri.data(), sp.wall_obj->data()};
      R.obj_vol.assign(nobj, 0.0);
      for (uint32_t ob = 0; ob < nobj; ob++)
        if (R.obj_llf[3 * ob] <= R.obj_urb[3 * ob]) object_volume(mv, ob, &R.obj_vol[ob]);
    }
    g.n_cv = 0;
    if (!sp.counted.empty()) {
      if (!g.wall_obj || sp.counted.size() > MAX_COUNTED) {
        err = "counted objects need wall objects (mcg_set_wall_objects), at most 7";
        return -1;
      }
      g.n_cv = (uint32_t)sp.counted.size();
      for (uint32_t k = 0; k < g.n_cv; k++) g.cv_obj[k] = sp.counted[k];
      R.n_cv = g.n_cv;
    }
    R.span = (uint32_t)(base_keys << g.oct_shift);
    R.wall_density = (double)hs.wsp_list.size() / (double)g.n3;
    if (sizeof(T) == 4) {
      R.planes.resize(4 * (size_t)nw);
      for (uint32_t w = 0; w < nw; w++)
        for (int k = 0; k < 4; k++) R.planes[4 * (size_t)w + k] = hs.wall[(size_t)w * 24 + k];
      R.h_wsp_off = hs.wsp_off;
      R.h_wsp_list = hs.wsp_list;
      for (int a = 0; a < 3; a++) R.origin[a] = hs.origin[a];
      R.sp_rcp = hs.sp_rcp;
      R.nsub = hs.nsub;
    }
    geos_h_[r] = g;
    return 0;
  }

  void free_replica(uint32_t r) {
    Rep& R = reps_[r];
    cudaFree(R.wrej);
    cudaFree(R.wface);
    cudaFree(R.wsp_off);
    cudaFree(R.wsp_list);
    cudaFree(R.wsp_cells);
    cudaFree(R.wsp_cm);
    cudaFree(R.wsp_cellent);
    cudaFree(R.wclass);
    cudaFree(R.chem);
    cudaFree(R.w64);
    cudaFree(R.wall_obj);
    R = Rep();
    Geo<T> g{};
    g.mode = REP_DROP;
    g.nsp = (int)nsp_;
    g.rep = r;
    geos_h_[r] = g;
  }

  // molecules of replica r into the staging list (checked against its partition)
  int stage_molecules(uint32_t r, uint64_t n, const double* pos, const uint32_t* species, uint64_t uid0,
                      Product<T>* stage, std::string& err) {
    const Geo<T>& g = geos_h_[r];
    const double o[3] = {(double)g.origin.x, (double)g.origin.y, (double)g.origin.z};
    const double q[3] = {(double)g.opposite.x, (double)g.opposite.y, (double)g.opposite.z};
    // large uploads are staged by all host threads (independent ranges; the wall-plane
    // checks of place_fp32 dominate: ~4 ns per molecule on 8 Arm cores)
    auto work = [&](uint64_t a, uint64_t b) -> int {
      for (uint64_t i = a; i < b; i++) {
        if (species[i] >= nsp_) return -1;
        double p[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        if (!(p[0] >= o[0] && p[1] >= o[1] && p[2] >= o[2] && p[0] < q[0] && p[1] < q[1] && p[2] < q[2])) return -4;
        place_fp32(reps_[r], p);
        Product<T> m;
        m.pos.x = (T)p[0];
        m.pos.y = (T)p[1];
        m.pos.z = (T)p[2];
        put_meta(m.pos, make_meta(species[i], r, META_SCHEDULE_UNIMOL));
        m.birth = 0;
        m.uid = uid0 + i;
        m.tuni = TIME_FOREVER;
        stage[i] = m;
      }
      return 0;
    };
    const unsigned nt = n < 200000 ? 1u : std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    std::vector<int> rcs(nt, 0);
    std::vector<std::thread> th;
    for (unsigned t = 1; t < nt; t++) th.emplace_back([&, t] { rcs[t] = work(n * t / nt, n * (t + 1) / nt); });
    rcs[0] = work(0, n / nt);
    for (auto& x : th) x.join();
    for (int rc : rcs) {
      if (rc == -1) err = "species index out of range";
      if (rc == -4) err = "molecule outside the partition";
      if (rc) return rc;
    }
    return 0;
  }

  // key ranges of the used replicas in slot order; grows the key arrays when needed
  // Replicas whose molecules cost most per step (most walls per subpartition) come
  // first in the key space: the persistent diffuse warps take molecules in key
  // order, so the slow ones start early instead of forming the kernel's tail.
  int layout_keys(std::string& err) {
    // the second products pass (products of products' unimolecular reactions in their
    // birth step) only where some replica's chemistry can make them
    prod_chain_ = false;
    for (uint32_t r = 0; r < max_rep_; r++) prod_chain_ = prod_chain_ || (reps_[r].used && reps_[r].uni_products);
    std::vector<uint32_t> order;
    for (uint32_t r = 0; r < max_rep_; r++) order.push_back(r);
    std::stable_sort(order.begin(), order.end(), [this](uint32_t a, uint32_t b) {
      return reps_[a].wall_density > reps_[b].wall_density;
    });
    uint64_t k = 0;
    for (uint32_t r : order) {
      geos_h_[r].kbase = (uint32_t)k;
      if (reps_[r].used) k += reps_[r].span;
    }
    if (k >= 0xFFFFFFF0ull) {
      err = "sort key space of the replicas exceeds 32 bits";
      return -3;
    }
    nkeys_ = (uint32_t)k;
    if (nkeys_ > key_alloc_) {
      const uint64_t na = std::max<uint64_t>(nkeys_, (uint64_t)key_alloc_ * 5 / 4);
      AllocSet a;
      uint32_t *st[2], *cn, *cu, *ti;
      for (int p = 0; p < 2; p++) MCG_CUDA(a.get(&st[p], sizeof(uint32_t) * (na + 1)));
      MCG_CUDA(a.get(&cn, sizeof(uint32_t) * na));
      MCG_CUDA(a.get(&cu, sizeof(uint32_t) * na));
      MCG_CUDA(a.get(&ti, sizeof(uint32_t) * ((na + SCAN_TILE - 1) / SCAN_TILE + 1)));
      for (int p = 0; p < 2; p++) MCG_CUDA(cudaMemsetAsync(st[p], 0, sizeof(uint32_t) * (na + 1), stream_));
      MCG_CUDA(cudaMemsetAsync(cn, 0, sizeof(uint32_t) * na, stream_));
      MCG_CUDA(cudaMemsetAsync(cu, 0, sizeof(uint32_t) * na, stream_));
      a.keep = true;
      for (int p = 0; p < 2; p++) {
        cudaFree(d_start_[p]);
        d_start_[p] = st[p];
      }
      cudaFree(d_counts_);
      cudaFree(d_cursor_);
      cudaFree(d_tile_);
      d_counts_ = cn;
      d_cursor_ = cu;
      d_tile_ = ti;
      key_alloc_ = (uint32_t)na;
    }
    base_.nkeys = nkeys_;
    ntiles_ = (nkeys_ + SCAN_TILE - 1) / SCAN_TILE;
    MCG_CUDA(cudaMemcpyAsync(d_geos_, geos_h_.data(), sizeof(Geo<T>) * max_rep_, cudaMemcpyHostToDevice, stream_));
    invalidate_graphs();
    return 0;
  }

  // re-sorts the live molecules plus the staged ones into the other sorted arrays
  // (molecules of dropped replicas are left out); counters must be fresh
  int rebin(const Product<T>* stage, uint64_t n, std::string& err, bool init_cv = false,
            const uint8_t* d_remove = nullptr, int staged_status = 0) {
    const uint64_t live = cnt_.n_live;
    if (live + n > 0xFFFFFFF0ull) {
      err = "too many molecules for 32-bit indices";
      return -3;
    }
    if (live + n > cap_ && ensure_capacity(std::max<uint64_t>((live + n) * 3 / 2, 1024), err)) return -2;
    if (n > base_.prod_cap && ensure_prod(n, err)) return -2;
    if (nkeys_ == 0) {
      // no replica left: nothing to sort
      Counters c = cnt_;
      c.n_live = 0;
      MCG_CUDA(cudaMemcpyAsync(d_cnt_, &c, sizeof(Counters), cudaMemcpyHostToDevice, stream_));
      cnt_ = c;
      return 0;
    }
    // staged molecules come from the host, or (stage == nullptr) are already in the list
    if (n && stage) MCG_CUDA(cudaMemcpyAsync(base_.prod, stage, sizeof(Product<T>) * n, cudaMemcpyHostToDevice, stream_));
    // staged molecules sit in the product list, already "diffused"
    Counters c = cnt_;
    c.n_prod = (uint32_t)n;
    c.n_prod_done = (uint32_t)n;
    c.prod_hi = (uint32_t)n;
    MCG_CUDA(cudaMemcpyAsync(d_cnt_, &c, sizeof(Counters), cudaMemcpyHostToDevice, stream_));
    State<T> s = state(parity_);
    if (init_cv && n && d_cv_count_) {
      k_cv_init<T><<<grid(n), TPB, 0, stream_>>>(s, (uint32_t)n);
      launches_ += 1;
    }
    k_rebin_count<T><<<grid(live + n), TPB, 0, stream_>>>(s, (uint32_t)n, d_remove, staged_status);
    k_scan_tiles<T><<<ntiles_, TPB, 0, stream_>>>(s);
    k_scan_top<T><<<1, TPB, 0, stream_>>>(s, ntiles_);
    k_scan_apply<T><<<ntiles_, TPB, 0, stream_>>>(s);
    k_scatter<T><<<grid(live + n), TPB, 0, stream_>>>(s, 0);
    launches_ += 5;
    if (d_cv_count_) {
      k_publish_cv<T><<<1, TPB, 0, stream_>>>(s);
      launches_ += 1;
    }
    MCG_CUDA(cudaGetLastError());
    MCG_CUDA(cudaStreamSynchronize(stream_));
    if (read_counters(err)) return -2;
    Counters c2 = cnt_;
    c2.n_live = std::min<uint32_t>(c2.n_live_next, (uint32_t)cap_);
    c2.n_prod = c2.n_prod_done = c2.prod_hi = 0;
    MCG_CUDA(cudaMemcpyAsync(d_cnt_, &c2, sizeof(Counters), cudaMemcpyHostToDevice, stream_));
    parity_ ^= 1;  // the re-binned arrays became the current ones
    cnt_ = c2;
    rebin_it_ = cnt_.iteration;
    invalidate_graphs();
    if (int rc = capture_initial_counts(err)) return rc;
    return status_to_error(c2.status, err);
  }

  // counts of every replica that has not run an iteration yet, from the start offsets
  // of its key ranges (and its counted-volume counts as just published)
  int capture_initial_counts(std::string& err) {
    const uint32_t* st = state(parity_).start;
    for (uint32_t r = 0; r < max_rep_; r++) {
      if (!reps_[r].used || geos_h_[r].it0 < cnt_.iteration) continue;
      const Geo<T>& g = geos_h_[r];
      const size_t span = (size_t)g.n3 << g.oct_shift;
      std::vector<uint32_t> b(nsp_ + 1);
      MCG_CUDA(cudaMemcpy2DAsync(b.data(), sizeof(uint32_t), st + g.kbase, sizeof(uint32_t) * span, sizeof(uint32_t),
                                 nsp_ + 1, cudaMemcpyDeviceToHost, stream_));
      Rep& R = reps_[r];
      if (R.n_cv && d_cv_now_) {
        std::vector<uint32_t> h((size_t)nsp_ * MAX_COUNTED);
        MCG_CUDA(cudaMemcpyAsync(h.data(), d_cv_now_ + (size_t)r * nsp_ * MAX_COUNTED, sizeof(uint32_t) * h.size(),
                                 cudaMemcpyDeviceToHost, stream_));
        MCG_CUDA(cudaStreamSynchronize(stream_));
        R.init_cv.assign((size_t)nsp_ * R.n_cv, 0);
        for (uint32_t a = 0; a < nsp_; a++)
          for (uint32_t k = 0; k < R.n_cv; k++) R.init_cv[a * R.n_cv + k] = h[a * MAX_COUNTED + k];
      }
      MCG_CUDA(cudaStreamSynchronize(stream_));
      R.init_world.assign(nsp_, 0);
      for (uint32_t a = 0; a < nsp_; a++) R.init_world[a] = b[a + 1] - b[a];
    }
    return 0;
  }

 public:
  int initial_counts(uint32_t rep, uint64_t* world, uint64_t* inside, std::string& err) override {
    if (rep >= max_rep_ || !reps_[rep].used || reps_[rep].init_world.size() != nsp_) {
      err = "no initial counts for this replica";
      return -1;
    }
    const Rep& R = reps_[rep];
    for (uint32_t a = 0; a < nsp_; a++) world[a] = R.init_world[a];
    if (inside)
      for (size_t k = 0; k < R.init_cv.size(); k++) inside[k] = R.init_cv[k];
    return 0;
  }

 private:

  unsigned grid(uint64_t n) const {
    uint64_t b = (n + TPB - 1) / TPB;
    uint64_t mx = (uint64_t)sms_ * 8;
    return (unsigned)std::max<uint64_t>(1, std::min(b, mx));
  }

  int read_counters(std::string& err) {
    MCG_CUDA(d2h(&cnt_, d_cnt_, sizeof(Counters)));
    pending_iters_ = 0;
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
    // every new buffer first; the old ones are replaced only when all exist
    AllocSet a;
    P4<T>* np[2];
    uint64_t* nu[2];
    T* nt[2];
    for (int k = 0; k < 2; k++) {
      MCG_CUDA(a.get(&np[k], sizeof(P4<T>) * cap));
      MCG_CUDA(a.get(&nu[k], sizeof(uint64_t) * cap));
      MCG_CUDA(a.get(&nt[k], sizeof(T) * cap));
    }
    // every molecule can propose once per iteration (dense models at high rates
    // propose with a large share of their molecules)
    const uint64_t pc = std::max<uint64_t>(4096, cap);
    P4<T>* nb;
    uint8_t* nst;
    uint64_t* ncl;
    Proposal *npr, *nre;
    uint32_t* nlo;
    MCG_CUDA(a.get(&nb, sizeof(P4<T>) * cap));
    MCG_CUDA(a.get(&nst, cap));
    MCG_CUDA(a.get(&ncl, sizeof(uint64_t) * cap));
    MCG_CUDA(a.get(&npr, sizeof(Proposal) * pc));
    MCG_CUDA(a.get(&nlo, sizeof(uint32_t) * 2 * pc));
    MCG_CUDA(a.get(&nre, sizeof(Proposal) * pc));
    // products: at most one per reactant of a bimolecular reaction with two products
    Product<T>* nprod = nullptr;
    uint8_t* npst = nullptr;
    if (pc > base_.prod_cap) {
      MCG_CUDA(a.get(&nprod, sizeof(Product<T>) * pc));
      MCG_CUDA(a.get(&npst, pc));
    }
    for (int k = 0; k < 2 && cap_; k++) {
      MCG_CUDA(cudaMemcpyAsync(np[k], pos_[k], sizeof(P4<T>) * cap_, cudaMemcpyDeviceToDevice, stream_));
      MCG_CUDA(cudaMemcpyAsync(nu[k], uid_[k], sizeof(uint64_t) * cap_, cudaMemcpyDeviceToDevice, stream_));
      MCG_CUDA(cudaMemcpyAsync(nt[k], tuni_[k], sizeof(T) * cap_, cudaMemcpyDeviceToDevice, stream_));
    }
    MCG_CUDA(cudaMemsetAsync(ncl, 0xFF, sizeof(uint64_t) * cap, stream_));
    MCG_CUDA(cudaStreamSynchronize(stream_));
    a.keep = true;
    for (int k = 0; k < 2; k++) {
      cudaFree(pos_[k]);
      cudaFree(uid_[k]);
      cudaFree(tuni_[k]);
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
    d_b_pos_ = nb;
    d_st_ = nst;
    d_claim_ = ncl;
    d_props_ = npr;
    d_losers_ = nlo;
    d_redo_ = nre;
    base_.prop_cap = (uint32_t)pc;
    cap_ = cap;
    base_.cap = (uint32_t)cap;
    if (nprod) adopt_prod(nprod, npst, pc);
    invalidate_graphs();
    return 0;
  }

  int ensure_prod(uint64_t pc, std::string& err) {
    if (pc <= base_.prod_cap) return 0;
    AllocSet a;
    Product<T>* nprod;
    uint8_t* npst;
    MCG_CUDA(a.get(&nprod, sizeof(Product<T>) * pc));
    MCG_CUDA(a.get(&npst, pc));
    a.keep = true;
    adopt_prod(nprod, npst, pc);
    invalidate_graphs();
    return 0;
  }

  void adopt_prod(Product<T>* prod, uint8_t* pst, uint64_t pc) {
    cudaFree(d_prod_);
    cudaFree(d_pst_);
    d_prod_ = prod;
    d_pst_ = pst;
    base_.prod_cap = (uint32_t)pc;
    base_.prod = d_prod_;
    base_.pst = d_pst_;
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
    s.counts = d_counts_;
    s.cursor = d_cursor_;
    s.tile_sum = d_tile_;
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
    if (s.debug_log)
      k_diffuse<T, true><<<diffuse_grid_, TPB, 0, stream_>>>(s);
    else
      k_diffuse<T, false><<<diffuse_grid_, TPB, 0, stream_>>>(s);
    mark(1, prof);
    k_resolve<T><<<gs, TPB, 0, stream_>>>(s);
    k_collect_losers<T><<<gs, TPB, 0, stream_>>>(s);
    k_reset_claims<T><<<gs, TPB, 0, stream_>>>(s);
    for (int r = 0; r < GRID_REDO_ROUNDS; r++) {
      k_redo_trace<T><<<diffuse_grid_, TPB, 0, stream_>>>(s, r);
      k_redo_commit<T><<<gs, TPB, 0, stream_>>>(s, r);
      k_redo_next<T><<<gs, TPB, 0, stream_>>>(s, r);
    }
    k_redo<T><<<1, TPB, 0, stream_>>>(s);
    mark(2, prof);
    k_prod_window<T><<<1, 1, 0, stream_>>>(s);
    k_products<T><<<2 * gs, TPB, 0, stream_>>>(s);
    k_prod_window<T><<<1, 1, 0, stream_>>>(s);
    if (prod_chain_) {
      k_products<T><<<2 * gs, TPB, 0, stream_>>>(s);
      k_prod_window<T><<<1, 1, 0, stream_>>>(s);
    }
    mark(3, prof);
    k_scan_tiles<T><<<ntiles_, TPB, 0, stream_>>>(s);
    k_scan_top<T><<<1, TPB, 0, stream_>>>(s, ntiles_);
    k_scan_apply<T><<<ntiles_, TPB, 0, stream_>>>(s);
    k_scatter<T><<<g, TPB, 0, stream_>>>(s, 1);
    k_end<T><<<1, TPB, 0, stream_>>>(s);
    mark(4, prof);
    launches_ += kernels_per_iteration();
  }

  // graph of `iters` (1 or 2) iterations starting at `parity`
  int capture(int parity, int iters, std::string& err) {
    cudaGraph_t gr;
    MCG_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    uint64_t l0 = launches_;
    launch_iteration(state(parity));
    if (iters == 2) launch_iteration(state(parity ^ 1));
    launches_ = l0;
    MCG_CUDA(cudaStreamEndCapture(stream_, &gr));
    MCG_CUDA(cudaGraphInstantiate(&graph_[parity + 2 * (iters - 1)], gr, 0));
    cudaGraphDestroy(gr);
    return 0;
  }

  void invalidate_graphs() {
    for (int k = 0; k < 4; k++) {
      if (graph_[k]) cudaGraphExecDestroy(graph_[k]);
      graph_[k] = nullptr;
    }
  }

  void release() {
    invalidate_graphs();
    for (uint32_t r = 0; r < reps_.size(); r++)
      if (reps_[r].used) free_replica(r);
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
    cudaFree(d_geos_);
    cudaFree(d_cv_count_);
    cudaFree(d_cv_now_);
    cudaFree(d_cv_traj_);
    if (cslot_host_) {
      for (int k = 0; k < NCSLOT; k++) cudaEventDestroy(cslot_ev_[k]);
      cudaFreeHost(cslot_host_);
      cslot_host_ = nullptr;
    }
    if (stream_) cudaStreamDestroy(stream_);
  }

  State<T> base_{};
  cudaStream_t stream_ = nullptr;
  int dev_ = 0;                             // device the engine was created on
  unsigned char* static_scratch_ = nullptr;  // that device's fixed trace scratch
  int sms_ = 1;
  int bps_max_ = 1;
  int diffuse_grid_ = 1;
  int parity_ = 0;
  bool use_graphs_ = true;
  bool profile_ = false;
  std::vector<std::array<cudaEvent_t, 5>> prof_;
  cudaGraphExec_t graph_[4] = {nullptr, nullptr, nullptr, nullptr};  // [parity + 2 * (iterations - 1)]
  uint64_t pending_iters_ = 0;  // iterations queued since the counters were last read
  // pinned slots of the non-blocking counts (request_counts / wait_counts)
  struct CountSlotHost {
    Counters c;
    unsigned long long n[MAXSP];
  };
  static constexpr int NCSLOT = 8;
  CountSlotHost* cslot_host_ = nullptr;
  cudaEvent_t cslot_ev_[NCSLOT] = {};
  uint64_t cslot_ticket_[NCSLOT] = {};
  uint64_t cslot_it_[NCSLOT] = {};
  uint64_t next_ticket_ = 1;
  uint32_t nsp_ = 0, max_rep_ = 0, nkeys_ = 0, key_alloc_ = 0, ntiles_ = 0, traj_cap_ = 65536;
  uint64_t cap_ = 0, iterations_ = 0, launches_ = 0;
  uint64_t rebin_it_ = 0;  // engine iteration of the last re-sort (counts then come from the starts)
  Counters cnt_{};
  std::vector<Rep> reps_;
  std::vector<Geo<T>> geos_h_;
  Geo<T>* d_geos_ = nullptr;
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
  uint32_t *d_cv_count_ = nullptr, *d_cv_now_ = nullptr, *d_cv_traj_ = nullptr;
  uint32_t cv_traj_cap_ = 0;
};

}  // namespace mcg
