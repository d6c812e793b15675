// Kernels of one diffuse-react iteration (templated on the position precision).
//
// Schedule of one iteration, all on the engine's stream, no host round trip
// (so a block of iterations can be captured in a CUDA graph):
//   k_diffuse      one thread per molecule: unimolecular schedule, displacement,
//                  ray trace, first firing reaction -> proposal; survivors are
//                  counted into the (subpartition, species) histogram
//   k_resolve      a proposal wins if it holds the minimum claim key on both
//                  molecules; winners kill both reactants and emit products
//   k_collect_losers / k_reset_claims
//   k_redo_*       losers re-trace with used-up partners excluded, in rounds
//                  over the whole GPU, then the rest in one CTA (k_redo),
//                  until every proposal is decided
//   k_products     newborn products diffuse for the rest of the step (twice)
//   k_scan_*       histogram -> start offsets of the sorted ranges
//   k_scatter      survivors move into the next iteration's sorted arrays
//                  (warp-aggregated atomics per key), species are counted
//   k_end          iteration bookkeeping
// This replaces MCell4's serial loop over the molecule schedule
// (DiffuseReactEvent::diffuse_molecules, diffuse_react_event.cpp:67-161), the
// per-subpartition reactant maps (partition.h:354-418), the sort by subpartition
// (sort_mols_by_subpart_event.cpp:62-97) and defragmentation
// (defragmentation_event.cpp:31-116), which the counting sort subsumes.
#pragma once

#include "mcg_device.cuh"

namespace mcg {

constexpr int TPB = 256;
// resident blocks of k_diffuse the register allocation must allow (occupancy vs spills)
#ifndef MCG_DIFFUSE_MIN_BLOCKS
#define MCG_DIFFUSE_MIN_BLOCKS 8
#endif
constexpr int SCAN_TILE = 2048;
constexpr int REDO_ROUNDS = 64;      // loser rounds in the one-CTA pass
constexpr int GRID_REDO_ROUNDS = 3;  // loser rounds over the whole GPU before it
constexpr uint64_t CLAIM_FREE = ~0ull;

struct Counters {
  uint32_t n_live;       // molecules in the current sorted arrays
  uint32_t n_live_next;  // survivors after this iteration
  uint32_t n_props;      // proposals made in k_diffuse
  uint32_t redo_n[GRID_REDO_ROUNDS + 1];  // losers entering loser round r (redo_n[0] from the first resolution)
  uint32_t redo_np[GRID_REDO_ROUNDS];     // proposals made in grid loser round r
  uint32_t n_prod;       // products created this iteration
  uint32_t n_prod_done;  // products already diffused
  uint32_t prod_hi;      // end of the products pass window
  uint32_t work;         // next molecule handed to a k_diffuse warp
  uint32_t status;       // ST_* bits
  uint32_t iteration;
  unsigned long long mol_steps;
  unsigned long long warn_coll_overflow;  // traces that refilled a full candidate page
  unsigned long long warn_set_overflow;   // traces that scanned partners along the walk
  unsigned long long warn_inside_redo;    // inside tests whose ray met an edge (see counted_volume_bits)
  // first escapes (diagnostics): uid, species, iteration, start xyz, displacement xyz, final xyz, replica
  uint32_t n_esc;
  double esc[8][13];
};

struct Proposal {
  uint32_t i, partner;
  uint32_t cv;  // counted-volume bits of the reactant at the collision (the products')
  uint32_t pw;  // pathway of the reaction class that fired
  uint64_t key;
  double t_abs;
  double x, y, z;
};

template <typename T>
struct Product {
  P4<T> pos;       // birth position, then final position (meta in w)
  double birth;    // time within the iteration
  uint64_t uid;
  double tuni;     // unimolecular time relative to the next iteration start
};

// state of one engine instance as the kernels see it
template <typename T>
struct State {
  const Geo<T>* __restrict__ geos;  // [n_rep] replica table
  uint32_t n_rep;                   // replica slots (used or free)
  int nsp;                          // species per replica
  uint64_t debug_uid;  // molecule whose steps are logged into debug_log (diagnostics)
  double* debug_log;   // [64 iterations][271] or null
  uint32_t cap, prod_cap, prop_cap, nkeys, traj_cap;
  int maxc, maxset;  // candidate page and partner list capacities (MAXC, MAXSET; tests lower them)
  // current sorted molecules and the next iteration's
  P4<T>* a_pos;
  uint64_t* a_uid;
  T* a_tuni;
  P4<T>* n_pos;
  uint64_t* n_uid;
  T* n_tuni;
  uint32_t* start;   // [nkeys + 1] of the current arrays
  uint32_t* nstart;  // [nkeys + 1] of the next arrays
  uint32_t* counts;  // [nkeys] histogram of the next iteration
  uint32_t* cursor;  // [nkeys]
  uint32_t* tile_sum;
  // this iteration
  P4<T>* b_pos;      // final positions
  uint8_t* st;       // 0 survivor, 1 proposer, 2 dead
  uint64_t* claim;
  Proposal* props;
  uint32_t* losers;
  Proposal* redo_props;
  Product<T>* prod;
  uint8_t* pst;      // product status
  unsigned long long* traj;  // [traj_cap][n_rep][nsp] species counts after each iteration
  // counted volumes (null when no replica counts any): molecules inside counted
  // object k per (replica, species): accumulated by k_scatter, published by k_end
  uint32_t* cv_count;  // [n_rep][nsp][MAX_COUNTED] of the iteration being sorted
  uint32_t* cv_now;    // [n_rep][nsp][MAX_COUNTED] after the last iteration or upload
  uint32_t* cv_traj;   // [cv_traj_cap][n_rep][nsp][MAX_COUNTED]
  uint32_t cv_traj_cap;
  Counters* cnt;
};

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  // splitmix64 finalizer: a bijection on 64-bit words
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31; }

// slot in a list filled through a counter, with one atomic per group of lanes that
// arrive together (a counter hit by every thread on its own serialises at its cache
// line: on GB300 that costs more than the work of a short kernel)
__device__ __forceinline__ uint32_t warp_slot(uint32_t* counter) {
  const unsigned am = __activemask();
  const int leader = __ffs(am) - 1;
  uint32_t b = 0;
  if ((int)lane_id() == leader) b = atomicAdd(counter, (uint32_t)__popc(am));
  b = __shfl_sync(am, b, leader);
  return b + (uint32_t)__popc(am & ((1u << lane_id()) - 1u));
}

// histogram add with one atomic per distinct key in the warp
__device__ __forceinline__ void warp_count(uint32_t* counts, uint32_t key, bool active) {
  unsigned mask = __ballot_sync(0xffffffffu, active);
  if (!active) return;
  unsigned peers = __match_any_sync(mask, key);
  if ((int)lane_id() == __ffs(peers) - 1) atomicAdd(&counts[key], (uint32_t)__popc(peers));
}

// Box-Muller pairs from 4 draws -> 3 standard normals
template <typename T>
__device__ __forceinline__ V3<T> gauss3(PhiloxDraws& d) {
  const uint4 w = d.ph.next4();
  const uint32_t a = w.x, b = w.y, c = w.z, e = w.w;
  if (sizeof(T) == 8) {
    double u1 = ((double)a + 0.5) * (1.0 / 4294967296.0), u2 = (double)b * (1.0 / 4294967296.0);
    double u3 = ((double)c + 0.5) * (1.0 / 4294967296.0), u4 = (double)e * (1.0 / 4294967296.0);
    double r1 = sqrt(-2.0 * log(u1)), r2 = sqrt(-2.0 * log(u3));
    double s1, c1, s2, c2;
    sincospi(2.0 * u2, &s1, &c1);
    sincospi(2.0 * u4, &s2, &c2);
    (void)s2;
    return v3<T>((T)(r1 * c1), (T)(r1 * s1), (T)(r2 * c2));
  } else {
    float u1 = ((float)a + 0.5f) * (1.0f / 4294967296.0f), u2 = (float)b * (1.0f / 4294967296.0f);
    float u3 = ((float)c + 0.5f) * (1.0f / 4294967296.0f), u4 = (float)e * (1.0f / 4294967296.0f);
    float r1 = sqrtf(-2.0f * logf(u1)), r2 = sqrtf(-2.0f * logf(u3));
    float s1, c1, s2, c2;
    sincospif(2.0f * u2, &s1, &c1);
    sincospif(2.0f * u4, &s2, &c2);
    (void)s2;
    return v3<T>((T)(r1 * c1), (T)(r1 * s1), (T)(r2 * c2));
  }
}

// sort key: (replica, species, subpartition, octant within the subpartition). The
// species-major order inside a replica makes each (replica, species) one contiguous
// key range, so species counts are differences of two scan offsets.
template <typename T>
__device__ __forceinline__ uint32_t key_of(const Geo<T>& g, V3<T> p, uint32_t species) {
  int x, y, z;
  sub3(g, p, x, y, z);
  const uint32_t sp = sub_of3(g, x, y, z);
  const uint32_t oct = g.oct_shift ? octant_of(g, p, x, y, z) : 0u;
  return g.kbase + (((species * g.n3 + sp) << g.oct_shift) | oct);
}

template <typename T>
__device__ __forceinline__ const Geo<T>& geo_of(const State<T>& s, uint32_t meta) {
  return s.geos[meta_rep(meta)];
}

// key of a record from its own meta word
template <typename T>
__device__ __forceinline__ uint32_t key_of_rec(const State<T>& s, const P4<T>& b) {
  const uint32_t m = meta_of(b);
  return key_of(geo_of(s, m), v3<T>(b.x, b.y, b.z), m & META_SPECIES_MASK);
}

// exact fallbacks a trace took (rare), one count per trace
template <typename T>
__device__ __forceinline__ void count_fallbacks(const State<T>& s, uint32_t terr) {
  if (terr & ST_COLL_OVERFLOW) atomicAdd(&s.cnt->warn_coll_overflow, 1ull);
  if (terr & ST_SET_OVERFLOW) atomicAdd(&s.cnt->warn_set_overflow, 1ull);
}

template <typename T>
__device__ void add_product(const State<T>& s, int species, uint32_t rep, uint32_t cv, V3<T> pos, double birth,
                            uint64_t uid) {
  if (species < 0) return;
  const uint32_t k = warp_slot(&s.cnt->n_prod);
  if (k >= s.prod_cap) {
    atomicOr(&s.cnt->status, ST_CAPACITY);
    return;
  }
  Product<T> p;
  p.pos.x = pos.x;
  p.pos.y = pos.y;
  p.pos.z = pos.z;
  set_meta(p.pos, make_meta((uint32_t)species, rep, META_SCHEDULE_UNIMOL | (cv << META_CV_SHIFT)));
  p.birth = birth;
  p.uid = uid;
  p.tuni = TIME_FOREVER;
  s.prod[k] = p;
}

// unimolecular outcome: the pathway (which_unimolecular, one more draw of the
// molecule's stream when the class has several), the molecule is destroyed, products
// appear at its position (react_unimol_single_molecule / outcome_unimolecular,
// diffuse_react_event.cpp:1809-1813, :2939). it: the replica's own iteration.
template <typename T>
__device__ __noinline__ void unimol_products(const State<T>& s, const Geo<T>& g, int species, uint32_t cv, V3<T> pos,
                                             double t, uint64_t uid, uint32_t it, PhiloxDraws draws) {
  const Chem& ch = *g.chem;
  const int pw = which_unimolecular(ch.uni_cum[species], ch.uni_npw[species], draws);
  for (int k = 0; k < 2; k++) {
    int ps = ch.uni_prod[species][pw][k];
    if (ps >= 0)
      add_product(s, ps, g.rep, cv, pos, t, mix64(uid ^ ((uint64_t)(it + 1) << 40) ^ (0xA5ull << 32) ^ (uint64_t)k));
  }
}

// Outcome of one molecule's step in the main pass. Shared by k_diffuse and k_redo.
struct StepDecision {
  int kind;  // 0 survivor, 1 proposal, 2 dead
};

// anomaly log for the host (the first 8 of an iteration): uid, species + 1000 * kind
// (1 escape, 2 watchdog), iteration, start xyz, displacement xyz, final xyz, replica
template <typename T>
__device__ __noinline__ void log_anomaly(const State<T>& s, const Geo<T>& g, uint64_t uid, int species, bool escaped,
                                         uint32_t it, V3<T> start, V3<T> disp, V3<T> end) {
  const uint32_t k = atomicAdd(&s.cnt->n_esc, 1u);
  if (k >= 8) return;
  const double rec[13] = {(double)uid,    (double)species + 1000.0 * (escaped ? 1 : 2),
                          (double)it,     (double)start.x,
                          (double)start.y, (double)start.z,
                          (double)disp.x, (double)disp.y,
                          (double)disp.z, (double)end.x,
                          (double)end.y,  (double)end.z,
                          (double)g.rep};
  for (int q = 0; q < 13; q++) s.cnt->esc[k][q] = rec[q];
}

// Items a warp takes at a time when a pass has n items (molecules, products, losers)
// for nwarps warps: the fewest lanes (a power of two) that still cover all items in
// one round. Scattered items diverge, so a full warp of them costs nearly 32 traces
// in a row; spread thin, the pass costs about one.
__device__ __forceinline__ uint32_t lanes_per_warp(uint32_t n, uint32_t nwarps) {
  uint32_t per = 32;
  while (per > 1 && (uint64_t)nwarps * (per / 2) >= n) per >>= 1;
  return per;
}

// returns 0 survivor, 1 proposal, 2 dead, 3 survivor of a frozen replica (not stepped);
// key: the next iteration's sort key of a survivor.
// LOG: the build that can log one molecule's events (mcg_debug_molecule)
template <typename T, bool LOG = true>
__device__ __forceinline__ int run_molecule(const State<T>& s, uint32_t i, const uint8_t* dead, Proposal* prop_out,
                                            uint32_t& err, uint32_t& key) {
  P4<T> rec = s.a_pos[i];
  uint32_t meta = meta_of(rec);
  const Geo<T>& g = geo_of(s, meta);
  const uint32_t mode = (g.mode == REP_RUN && s.cnt->iteration >= g.it_end) ? REP_FROZEN : g.mode;
  if (mode != REP_RUN) {
    if (mode == REP_DROP) return 2;
    s.b_pos[i] = rec;  // frozen: stays as it is until the replica is collected
    key = key_of(g, v3<T>(rec.x, rec.y, rec.z), meta & META_SPECIES_MASK);
    return 3;
  }
  const Chem& ch = *g.chem;
  const uint32_t it = s.cnt->iteration - g.it0;  // the replica's own iteration
  const uint64_t uid = s.a_uid[i];
  const int species = (int)(meta & META_SPECIES_MASK);
  // the step's time bookkeeping runs in T: fp32 keeps the FP64 pipe out of the common path
  T tuni = s.a_tuni[i];
  V3<T> pos = v3<T>(rec.x, rec.y, rec.z);
  PhiloxDraws draws;
  draws.ph.init(g.seed, uid, it, 0);
  // pick_unimol_rxn_class_and_set_rxn_time (diffuse_react_event.cpp:1731) on first diffusion
  if (meta & META_SCHEDULE_UNIMOL) {
    tuni = (T)(ch.unimol_k[species] >= 0 ? time_of_unimol(ch.unimol_k[species], draws) : TIME_FOREVER);
  }
  if (tuni <= (T)0) {
    // scheduled at or before the start of the step: react first (diffuse_single_molecule :214-223)
    unimol_products(s, g, species, meta_cv(meta), pos, 0.0, uid, it, draws);
    return 2;
  }
  // get_max_time (:164-198) with the barrier at the end of the iteration
  T max_time = 1;
  if (tuni < max_time) max_time = tuni;
  // compute_vol_displacement (diffusion_utils.inl:366-432), time_step = 1
  T steps = 1, t_steps = 1;
  if (t_steps > max_time) {
    t_steps = max_time;
    steps = max_time;
  }
  if (steps < (T)EPS) {
    steps = (T)EPS;
    t_steps = (T)EPS;
  }
  const T space_step = (T)ch.space_step[species];
  T scl = space_step;
  T r_rate_factor = 1;
  if (steps != (T)1) {
    T rate_factor = sqrt(steps);
    r_rate_factor = (T)1 / rate_factor;
    scl = rate_factor * space_step;
  }
  TraceOut<T> r;
  V3<T> disp = v3<T>(0, 0, 0);
  if (scl != (T)0) {
    V3<T> gz = gauss3<T>(draws);
    const T rsqrt2 = (T)0.70710678118654752440;
    disp = v3<T>(scl * gz.x * rsqrt2, scl * gz.y * rsqrt2, scl * gz.z * rsqrt2);
    Cells<T> cells;
    cells.pos = s.a_pos;
    cells.uid = s.a_uid;
    cells.start = s.start;
    cells.dead = dead;
    cells.maxc = s.maxc;
    cells.maxset = s.maxset;
    if (LOG) {
      MaybeEvents ev;
      ev.out = nullptr;
      if (uid == s.debug_uid && s.debug_log) {
        // per-iteration record of one chosen molecule: 9 + 32*8 result doubles, start xyz, displacement xyz
        ev.out = s.debug_log + (size_t)(it % 64) * 271;
        for (int q = 0; q < 271; q++) ev.out[q] = 0;
        ev.out[265] = (double)pos.x;
        ev.out[266] = (double)pos.y;
        ev.out[267] = (double)pos.z;
        ev.out[268] = (double)disp.x;
        ev.out[269] = (double)disp.y;
        ev.out[270] = (double)disp.z;
      }
      r = trace_molecule<T>(g, cells, i, pos, species, disp, r_rate_factor, t_steps, (T)0, draws, ev);
      if (ev.out) {
        ev.out[0] = r.status;
        ev.out[1] = (double)r.pos.x;
        ev.out[2] = (double)r.pos.y;
        ev.out[3] = (double)r.pos.z;
        ev.out[4] = r.subpart;
        ev.out[5] = it;
      }
    } else {
      NoEvents ev;  // production kernel: no event code in the hot path
      r = trace_molecule<T>(g, cells, i, pos, species, disp, r_rate_factor, t_steps, (T)0, draws, ev);
    }
    if (r.err & (ST_COLL_OVERFLOW | ST_SET_OVERFLOW)) count_fallbacks(s, r.err);
    err |= r.err;
  } else {
    r.status = 0;
    r.pos = pos;
    r.cv_mask = 0;
    r.cv_val = 0;
  }
  if (r.status == 1) {
    Proposal p;
    p.i = i;
    p.partner = r.partner;
    p.pw = (uint32_t)r.pathway;
    const float tf = (float)r.t_abs;
    // earliest reaction wins; the molecule index makes keys unique within the iteration
    p.key = ((uint64_t)__float_as_uint(tf < 0.f ? 0.f : tf) << 32) | i;
    p.t_abs = (double)r.t_abs;
    p.cv = cv_after(meta_cv(meta), r);
    p.x = (double)r.rxn_pos.x;
    p.y = (double)r.rxn_pos.y;
    p.z = (double)r.rxn_pos.z;
    *prop_out = p;
    return 1;
  }
  if (r.status == 2) return 2;
  if (max_time < (T)1) {
    // the unimolecular reaction happens where the molecule stopped
    unimol_products(s, g, species, cv_after(meta_cv(meta), r), r.pos, (double)tuni, uid, it, draws);
    return 2;
  }
  const bool escaped = !in_partition(g, r.pos);
  if (escaped || (r.err & ST_WATCHDOG)) log_anomaly(s, g, uid, species, escaped, it, pos, disp, r.pos);
  if (escaped) {
    err |= ST_ESCAPE;  // the reference stops with a fatal error; here the molecule is dropped
    return 2;
  }
  P4<T> out;
  out.x = r.pos.x;
  out.y = r.pos.y;
  out.z = r.pos.z;
  // schedule flag consumed; counted-volume bits as left by the crossings
  set_meta(out, make_meta((uint32_t)species, g.rep, cv_after(meta_cv(meta), r) << META_CV_SHIFT));
  s.b_pos[i] = out;
  key = key_of(g, r.pos, (uint32_t)species);
  if (meta & META_SCHEDULE_UNIMOL) s.a_tuni[i] = tuni;  // keep the drawn time for the scatter
  return 0;
}

template <typename T, bool LOG>
__global__ void __launch_bounds__(TPB, MCG_DIFFUSE_MIN_BLOCKS) k_diffuse(State<T> s) {
  const uint32_t n = s.cnt->n_live;
  uint32_t err = 0;
  uint32_t steps = 0;
  // persistent warps: each warp takes the next `per` molecules (in sorted order) until
  // none are left, so long-running warps near walls do not leave SMs idle at the end.
  // A warp's lanes diverge and run largely one after another, so a warp's batch costs
  // about its lanes' traces in a row: in fp32 a model with fewer molecules than 32 per
  // warp spreads them thinner (its step then takes a few traces' time, not 32). fp64
  // keeps full warps: a warp instruction holds GB300's narrow FP64 pipe as long with
  // 2 lanes as with 32.
  const uint32_t per = sizeof(T) == 4 ? lanes_per_warp(n, gridDim.x * (TPB / 32)) : 32u;
  for (;;) {
    uint32_t base = 0;
    if (lane_id() == 0) base = atomicAdd(&s.cnt->work, per);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) break;
    uint32_t i = base + lane_id();
    bool active = lane_id() < per && i < n;
    int kind = 2;
    uint32_t key = 0;
    if (active) {
      Proposal p;
      kind = run_molecule<T, LOG>(s, i, nullptr, &p, err, key);
      if (kind == 3)
        kind = 0;  // frozen replica: kept, not stepped
      else
        steps++;
      s.st[i] = (uint8_t)kind;
      if (kind == 1) {
        const uint32_t k = warp_slot(&s.cnt->n_props);
        if (k < s.prop_cap) {
          s.props[k] = p;
          atomicMin((unsigned long long*)&s.claim[i], (unsigned long long)p.key);
          atomicMin((unsigned long long*)&s.claim[p.partner], (unsigned long long)p.key);
        } else {
          err |= ST_CAPACITY;
        }
      }
    }
    warp_count(s.counts, key, active && kind == 0);
  }
  if (err & (ST_CAPACITY | ST_ESCAPE | ST_WATCHDOG))
    atomicOr(&s.cnt->status, err & (ST_CAPACITY | ST_ESCAPE | ST_WATCHDOG));
  // the warps leave the loop together: one molecule-step count per warp
  steps = __reduce_add_sync(0xffffffffu, steps);
  if (lane_id() == 0 && steps) atomicAdd(&s.cnt->mol_steps, (unsigned long long)steps);
}

// a winning proposal: both reactants die, products appear at the collision point
// (outcome_bimolecular / outcome_products_random, diffuse_react_event.cpp:1833, :2446)
template <typename T>
__device__ void commit(const State<T>& s, const Proposal& p) {
  const uint32_t ma = meta_of(s.a_pos[p.i]);
  const Geo<T>& g = geo_of(s, ma);
  const Chem& ch = *g.chem;
  const uint32_t it = s.cnt->iteration - g.it0;
  s.st[p.i] = 2;
  if (s.st[p.partner] == 0) {
    // the partner had finished its own step: take it out of the histogram
    atomicSub(&s.counts[key_of_rec(s, s.b_pos[p.partner])], 1u);
  }
  s.st[p.partner] = 2;
  const int sa = (int)(ma & META_SPECIES_MASK);
  const int sb = (int)(meta_of(s.a_pos[p.partner]) & META_SPECIES_MASK);
  const uint64_t uid = s.a_uid[p.i];
  for (int k = 0; k < 2; k++) {
    int ps = ch.bimol_prod[sa][sb][p.pw][k];
    if (ps >= 0) {
      add_product(s, ps, g.rep, p.cv, v3<T>((T)p.x, (T)p.y, (T)p.z), p.t_abs,
                  mix64(uid ^ ((uint64_t)(it + 1) << 40) ^ (0x5Aull << 32) ^ (uint64_t)k));
    }
  }
}

template <typename T>
__global__ void k_resolve(State<T> s) {
  uint32_t n = min(s.cnt->n_props, s.prop_cap);
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const Proposal p = s.props[k];
    if (s.claim[p.i] == p.key && s.claim[p.partner] == p.key) commit(s, p);
  }
}

template <typename T>
__global__ void k_collect_losers(State<T> s) {
  uint32_t n = min(s.cnt->n_props, s.prop_cap);
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const Proposal p = s.props[k];
    if (s.st[p.i] == 1) {
      s.losers[warp_slot(&s.cnt->redo_n[0])] = p.i;  // losers <= n_props <= prop_cap
    }
  }
}

template <typename T>
__global__ void k_reset_claims(State<T> s) {
  uint32_t n = min(s.cnt->n_props, s.prop_cap);
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const Proposal p = s.props[k];
    s.claim[p.i] = CLAIM_FREE;
    s.claim[p.partner] = CLAIM_FREE;
  }
}

// Losers (their partner was taken by an earlier-keyed reaction) re-trace their
// step in rounds: each replays its own draws (counter-based RNG) with every
// used-up molecule excluded, and proposes again or finishes; the proposals of a
// round are resolved like the first ones. The first GRID_REDO_ROUNDS rounds run
// over the whole GPU (three launches each, empty when nothing is left: dense
// models at high rates lose a large share of their proposals), the rest in one
// CTA. Round r reads its losers from half (r & 1) of the loser buffer and
// their count from redo_n[r], and appends the next round's to the other half.

// one loser re-traced: a new proposal (counted in *n_props) or a final state
template <typename T>
__device__ __forceinline__ void redo_one(const State<T>& s, uint32_t i, uint32_t* n_props, uint32_t& err) {
  Proposal p;
  uint32_t key = 0;
  int kind = run_molecule(s, i, s.st, &p, err, key);
  if (kind == 1) {
    s.st[i] = 1;
    const uint32_t k = warp_slot(n_props);
    s.redo_props[k] = p;  // k < number of losers <= prop_cap
    atomicMin((unsigned long long*)&s.claim[i], (unsigned long long)p.key);
    atomicMin((unsigned long long*)&s.claim[p.partner], (unsigned long long)p.key);
  } else if (kind == 0 || kind == 3) {
    s.st[i] = 0;
    atomicAdd(&s.counts[key], 1u);
  } else {
    s.st[i] = (uint8_t)kind;
  }
}

template <typename T>
__global__ void __launch_bounds__(TPB) k_redo_trace(State<T> s, int round) {
  const uint32_t n = min(s.cnt->redo_n[round], s.prop_cap);
  const uint32_t* cur = s.losers + (size_t)(round & 1) * s.prop_cap;
  uint32_t err = 0;
  // losers are few and scattered: as few per warp as covers them in one round (as in
  // k_products), so the round takes about one trace
  const uint32_t nwarps = gridDim.x * (TPB / 32);
  const uint32_t per = lanes_per_warp(n, nwarps);
  const uint32_t lane = lane_id();
  if (lane < per)
    for (uint32_t l = (blockIdx.x * (TPB / 32) + threadIdx.x / 32) * per + lane; l < n; l += nwarps * per)
      redo_one(s, cur[l], &s.cnt->redo_np[round], err);
  if (err & (ST_CAPACITY | ST_ESCAPE | ST_WATCHDOG))
    atomicOr(&s.cnt->status, err & (ST_CAPACITY | ST_ESCAPE | ST_WATCHDOG));
}

template <typename T>
__global__ void k_redo_commit(State<T> s, int round) {
  const uint32_t n = s.cnt->redo_np[round];
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const Proposal p = s.redo_props[k];
    if (s.claim[p.i] == p.key && s.claim[p.partner] == p.key) commit(s, p);
  }
}

// proposals that lost again become the next round's losers; claims are released
template <typename T>
__global__ void k_redo_next(State<T> s, int round) {
  const uint32_t n = s.cnt->redo_np[round];
  uint32_t* next = s.losers + (size_t)((round + 1) & 1) * s.prop_cap;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const Proposal p = s.redo_props[k];
    if (s.st[p.i] == 1) next[warp_slot(&s.cnt->redo_n[round + 1])] = p.i;
    s.claim[p.i] = CLAIM_FREE;
    s.claim[p.partner] = CLAIM_FREE;
  }
}

// the remaining rounds in one CTA
template <typename T>
__global__ void __launch_bounds__(TPB) k_redo(State<T> s) {
  __shared__ uint32_t n_cur, n_next, n_rp;
  uint32_t err = 0;
  if (threadIdx.x == 0) n_cur = min(s.cnt->redo_n[GRID_REDO_ROUNDS], s.prop_cap);
  __syncthreads();
  int half = GRID_REDO_ROUNDS & 1;
  for (int round = 0; round < REDO_ROUNDS; round++) {
    if (n_cur == 0) break;
    const uint32_t* cur = s.losers + (size_t)half * s.prop_cap;
    uint32_t* next = s.losers + (size_t)(half ^ 1) * s.prop_cap;
    if (threadIdx.x == 0) {
      n_next = 0;
      n_rp = 0;
    }
    __syncthreads();
    for (uint32_t l = threadIdx.x; l < n_cur; l += blockDim.x) redo_one(s, cur[l], &n_rp, err);
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < n_rp; k += blockDim.x) {
      const Proposal p = s.redo_props[k];
      if (s.claim[p.i] == p.key && s.claim[p.partner] == p.key) commit(s, p);
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < n_rp; k += blockDim.x) {
      const Proposal p = s.redo_props[k];
      if (s.st[p.i] == 1) next[atomicAdd(&n_next, 1u)] = p.i;
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < n_rp; k += blockDim.x) {
      const Proposal p = s.redo_props[k];
      s.claim[p.i] = CLAIM_FREE;
      s.claim[p.partner] = CLAIM_FREE;
    }
    __syncthreads();
    if (threadIdx.x == 0) n_cur = n_next;
    half ^= 1;
    __syncthreads();
  }
  if (n_cur != 0) {
    // undecided after the round limit: report and drop them as dead rather than loop on
    if (threadIdx.x == 0) atomicOr(&s.cnt->status, ST_WATCHDOG);
    const uint32_t* cur = s.losers + (size_t)half * s.prop_cap;
    for (uint32_t l = threadIdx.x; l < n_cur; l += blockDim.x) s.st[cur[l]] = 2;
  }
  if (err & (ST_CAPACITY | ST_ESCAPE | ST_WATCHDOG))
    atomicOr(&s.cnt->status, err & (ST_CAPACITY | ST_ESCAPE | ST_WATCHDOG));
}

// Products diffuse the rest of the step from their birth time (the queue of new
// diffuse actions, diffuse_react_event.cpp:122-129, 2883-2886). Products do not
// react with other molecules in the step they are born in.
template <typename T>
__global__ void __launch_bounds__(TPB) k_products(State<T> s) {
  const uint32_t b0 = s.cnt->n_prod_done;
  const uint32_t b1 = s.cnt->prod_hi;
  const uint32_t it_engine = s.cnt->iteration;
  uint32_t err = 0;
  // products are scattered over the model: spread thin over the warps (2,000 products
  // on 2,432 warps: one each); large windows still fill whole warps
  const uint32_t nwarps = gridDim.x * (TPB / 32);
  const uint32_t per = lanes_per_warp(b1 > b0 ? b1 - b0 : 0u, nwarps);
  const uint32_t lane = lane_id();
  for (uint32_t base = b0 + (blockIdx.x * (TPB / 32) + threadIdx.x / 32) * per; base < b1; base += nwarps * per) {
    uint32_t k = base + lane;
    bool active = lane < per && k < b1;
    uint32_t key = 0;
    bool survive = false;
    if (active) {
      Product<T> p = s.prod[k];
      const uint32_t meta = meta_of(p.pos);
      const int species = (int)(meta & META_SPECIES_MASK);
      const Geo<T>& g = geo_of(s, meta);
      const Chem& ch = *g.chem;
      const uint32_t it = it_engine - g.it0;
      PhiloxDraws draws;
      draws.ph.init(g.seed, p.uid, it, 1);
      double unimol_time = TIME_FOREVER;
      if (ch.unimol_k[species] >= 0) unimol_time = p.birth + time_of_unimol(ch.unimol_k[species], draws);
      double max_time = 1.0 - p.birth;
      if (unimol_time < p.birth + max_time) max_time = unimol_time - p.birth;
      V3<T> pos = v3<T>(p.pos.x, p.pos.y, p.pos.z);
      const V3<T> start = pos;
      V3<T> disp = v3<T>(0, 0, 0);
      uint32_t werr = 0;
      uint32_t cv = meta_cv(meta);
      bool dead = false;
      if (max_time <= 0.0) {
        unimol_products(s, g, species, meta_cv(meta), pos, unimol_time, p.uid, it, draws);
        dead = true;
      } else {
        double steps = 1.0, t_steps = 1.0;
        if (t_steps > max_time) {
          t_steps = max_time;
          steps = max_time;
        }
        if (steps < EPS) {
          steps = EPS;
          t_steps = EPS;
        }
        double scl = ch.space_step[species], r_rate_factor = 1.0;
        if (steps != 1.0) {
          double rf = sqrt(steps);
          r_rate_factor = 1.0 / rf;
          scl = rf * ch.space_step[species];
        }
        if (scl != 0.0) {
          V3<T> gz = gauss3<T>(draws);
          disp = v3<T>((T)(scl * (double)gz.x * 0.70710678118654752440),
                       (T)(scl * (double)gz.y * 0.70710678118654752440),
                       (T)(scl * (double)gz.z * 0.70710678118654752440));
          Cells<T> cells;
          cells.pos = s.a_pos;
          cells.uid = s.a_uid;
          cells.start = s.start;
          cells.dead = s.st;
          cells.maxc = s.maxc;
          cells.maxset = s.maxset;
          NoEvents ev;
          TraceOut<T> r = trace_molecule<T>(g, cells, NONE, pos, species, disp, (T)r_rate_factor, (T)t_steps,
                                            (T)p.birth, draws, ev, false);
          if (r.err & (ST_COLL_OVERFLOW | ST_SET_OVERFLOW)) count_fallbacks(s, r.err);
          err |= r.err;
          werr = r.err & ST_WATCHDOG;
          cv = cv_after(cv, r);
          if (r.status == 2) {
            dead = true;
          } else {
            pos = r.pos;
          }
        }
        if (!dead && unimol_time < 1.0) {
          unimol_products(s, g, species, cv, pos, unimol_time, p.uid, it, draws);
          dead = true;
        }
      }
      const bool escaped = !dead && !in_partition(g, pos);
      if (escaped || werr) log_anomaly(s, g, p.uid, species, escaped, it, start, disp, pos);
      if (escaped) {
        err |= ST_ESCAPE;
        dead = true;
      }
      if (!dead) {
        p.pos.x = pos.x;
        p.pos.y = pos.y;
        p.pos.z = pos.z;
        set_meta(p.pos, make_meta((uint32_t)species, g.rep, cv << META_CV_SHIFT));
        p.tuni = unimol_time - 1.0;
        s.prod[k] = p;
        key = key_of(g, pos, (uint32_t)species);
        survive = true;
      }
      s.pst[k] = survive ? 0 : 2;
    }
    warp_count(s.counts, key, active && survive);
  }
  __syncthreads();
  if (err & (ST_CAPACITY | ST_ESCAPE | ST_WATCHDOG))
    atomicOr(&s.cnt->status, err & (ST_CAPACITY | ST_ESCAPE | ST_WATCHDOG));
}

// window of products for the next pass: [done, hi) where hi is a snapshot taken
// before the pass, so products created during a pass go to the next one
template <typename T>
__global__ void k_prod_window(State<T> s) {
  s.cnt->n_prod_done = s.cnt->prod_hi;
  s.cnt->prod_hi = min(s.cnt->n_prod, s.prod_cap);
}

// ---- exclusive scan of the histogram (3 phases over tiles of SCAN_TILE keys)

template <typename T>
__global__ void k_scan_tiles(State<T> s) {
  __shared__ uint32_t red[TPB / 32];
  const uint32_t b = blockIdx.x * SCAN_TILE;
  uint32_t sum = 0;
  for (uint32_t k = b + threadIdx.x; k < min(b + SCAN_TILE, s.nkeys); k += TPB) sum += s.counts[k];
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
  if (lane_id() == 0) red[threadIdx.x >> 5] = sum;
  __syncthreads();
  if (threadIdx.x < 32) {
    uint32_t v = threadIdx.x < TPB / 32 ? red[threadIdx.x] : 0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) s.tile_sum[blockIdx.x] = v;
  }
}

__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t warp_tot[TPB / 32];
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if ((int)lane_id() >= o) x += y;
  }
  if (lane_id() == 31) warp_tot[threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x < 32) {
    uint32_t w = threadIdx.x < TPB / 32 ? warp_tot[threadIdx.x] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if ((int)threadIdx.x >= o) w += y;
    }
    if (threadIdx.x < TPB / 32) warp_tot[threadIdx.x] = w;
  }
  __syncthreads();
  uint32_t warp_off = (threadIdx.x >> 5) ? warp_tot[(threadIdx.x >> 5) - 1] : 0;
  *total = warp_tot[TPB / 32 - 1];
  __syncthreads();
  return warp_off + x - v;
}

template <typename T>
__global__ void k_scan_top(State<T> s, uint32_t ntiles) {
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint32_t b = 0; b < ntiles; b += TPB) {
    uint32_t k = b + threadIdx.x;
    uint32_t v = k < ntiles ? s.tile_sum[k] : 0;
    uint32_t tot;
    uint32_t ex = block_excl_scan(v, &tot);
    if (k < ntiles) s.tile_sum[k] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    s.cnt->n_live_next = carry;
    if (carry > s.cap) atomicOr(&s.cnt->status, ST_CAPACITY);
  }
}

template <typename T>
__global__ void k_scan_apply(State<T> s) {
  const uint32_t b = blockIdx.x * SCAN_TILE;
  uint32_t carry = s.tile_sum[blockIdx.x];
  __shared__ uint32_t sh_carry;
  for (uint32_t c = 0; c < SCAN_TILE; c += TPB) {
    uint32_t k = b + c + threadIdx.x;
    uint32_t v = k < s.nkeys ? s.counts[k] : 0;
    uint32_t tot;
    uint32_t ex = block_excl_scan(v, &tot);
    if (k < s.nkeys) {
      s.nstart[k] = carry + ex;
      s.counts[k] = 0;
      s.cursor[k] = 0;
    }
    carry += tot;
  }
  (void)sh_carry;
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) s.nstart[s.nkeys] = carry;
}

// ---- scatter into the next sorted arrays

template <typename T>
__device__ __forceinline__ void scatter_one(const State<T>& s, bool active, const P4<T>& pos, uint64_t uid, T tuni,
                                            bool count_cv) {
  uint32_t key = 0;
  if (active) key = key_of_rec(s, pos);
  unsigned mask = __ballot_sync(0xffffffffu, active);
  if (!active) return;
  unsigned peers = __match_any_sync(mask, key);
  int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if ((int)lane_id() == leader) base = atomicAdd(&s.cursor[key], (uint32_t)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  uint32_t rank = __popc(peers & ((1u << lane_id()) - 1));
  uint32_t slot = s.nstart[key] + base + rank;
  if (slot < s.cap) {
    s.n_pos[slot] = pos;
    s.n_uid[slot] = uid;
    s.n_tuni[slot] = tuni;
  }
  if (count_cv) {
    // molecules inside counted objects, one atomic per (replica, species, object) of the peers
    const uint32_t m = meta_of(pos);
    const uint32_t cv = meta_cv(m);
    const uint32_t cell = (meta_rep(m) * (uint32_t)s.nsp + (m & META_SPECIES_MASK)) * MAX_COUNTED;
    for (uint32_t k = 0; k < MAX_COUNTED; k++) {
      const bool in = (cv >> k) & 1u;
      const unsigned im = __ballot_sync(peers, in);
      if (!in) continue;
      const unsigned same = __match_any_sync(im, cell + k);
      if ((int)lane_id() == __ffs(same) - 1) atomicAdd(&s.cv_count[cell + k], (uint32_t)__popc(same));
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(TPB) k_scatter(State<T> s, int tuni_shift) {
  const uint32_t n = s.cnt->n_live;
  const bool count_cv = s.cv_count != nullptr;
  for (uint32_t base = blockIdx.x * TPB; base < n; base += gridDim.x * TPB) {
    uint32_t i = base + threadIdx.x;
    bool active = i < n && s.st[i] == 0;
    P4<T> p;
    uint64_t uid = 0;
    T tuni = 0;
    if (active) {
      p = s.b_pos[i];
      uid = s.a_uid[i];
      tuni = s.a_tuni[i] - (T)tuni_shift;
    }
    scatter_one(s, active, p, uid, tuni, count_cv);
  }
  const uint32_t np = min(s.cnt->n_prod, s.prod_cap);
  for (uint32_t base = blockIdx.x * TPB; base < np; base += gridDim.x * TPB) {
    uint32_t k = base + threadIdx.x;
    bool active = k < np && k < s.cnt->n_prod_done && s.pst[k] == 0;
    P4<T> p;
    uint64_t uid = 0;
    T tuni = 0;
    if (active) {
      Product<T> q = s.prod[k];
      p = q.pos;
      uid = q.uid;
      tuni = (T)q.tuni;
    }
    scatter_one(s, active, p, uid, tuni, count_cv);
  }
}

// species counts of every replica after the sort: each (replica, species) is one
// contiguous key range of the next arrays, so its count is a difference of two
// start offsets
template <typename T>
__device__ void count_species(const State<T>& s, uint32_t row) {
  const uint32_t nq = s.n_rep * (uint32_t)s.nsp;
  for (uint32_t q = threadIdx.x; q < nq; q += blockDim.x) {
    const Geo<T>& g = s.geos[q / (uint32_t)s.nsp];
    const uint32_t a = q % (uint32_t)s.nsp;
    const uint32_t span = g.n3 << g.oct_shift;
    const uint32_t k0 = g.kbase + a * span;
    s.traj[(size_t)row * nq + q] = g.mode == REP_DROP ? 0ull : (unsigned long long)(s.nstart[k0 + span] - s.nstart[k0]);
  }
}

// counted-volume counts of the sort just done: to the latest counts (and, after an
// iteration, to the trajectory ring); the accumulator is cleared
template <typename T>
__device__ void publish_cv(const State<T>& s, uint32_t it, bool to_ring) {
  if (!s.cv_count) return;
  const uint32_t nq = s.n_rep * (uint32_t)s.nsp * MAX_COUNTED;
  uint32_t* row = s.cv_traj + (size_t)(it % s.cv_traj_cap) * nq;
  for (uint32_t q = threadIdx.x; q < nq; q += blockDim.x) {
    const uint32_t v = s.cv_count[q];
    s.cv_now[q] = v;
    if (to_ring) row[q] = v;
    s.cv_count[q] = 0;
  }
}

// after an upload's sort: the latest counted-volume counts (no ring row)
template <typename T>
__global__ void k_publish_cv(State<T> s) {
  publish_cv(s, 0, false);
}

// initial counted-volume membership of staged molecules (uploads): the reference's
// ray-parity test against each counted object
template <typename T>
__global__ void k_cv_init(State<T> s, uint32_t n_staged) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n_staged; k += gridDim.x * blockDim.x) {
    Product<T> p = s.prod[k];
    const uint32_t m = meta_of(p.pos);
    const Geo<T>& g = geo_of(s, m);
    if (!g.n_cv) continue;
    const V3<double> x = v3<double>((double)p.pos.x, (double)p.pos.y, (double)p.pos.z);
    uint32_t cv = counted_volume_bits(g, x);
    if (cv == NONE) {
      // the ray met an edge, where the reference stops: counted outside every object
      atomicAdd(&s.cnt->warn_inside_redo, 1ull);
      cv = 0;
    }
    set_meta(p.pos, (m & ~(0x7Fu << META_CV_SHIFT)) | (cv << META_CV_SHIFT));
    s.prod[k].pos = p.pos;
  }
}

// bookkeeping at the end of an iteration (one block)
template <typename T>
__global__ void k_end(State<T> s) {
  Counters* c = s.cnt;
  const uint32_t it = c->iteration;
  count_species(s, it % s.traj_cap);
  publish_cv(s, it, true);
  __syncthreads();
  if (threadIdx.x != 0) return;
  if (c->n_prod > c->n_prod_done) atomicOr(&c->status, ST_WATCHDOG);  // product chain deeper than the passes
  c->n_live = min(c->n_live_next, s.cap);
  c->n_props = 0;
  for (int r = 0; r <= GRID_REDO_ROUNDS; r++) c->redo_n[r] = 0;
  for (int r = 0; r < GRID_REDO_ROUNDS; r++) c->redo_np[r] = 0;
  c->n_prod = 0;
  c->n_prod_done = 0;
  c->prod_hi = 0;
  c->work = 0;
  c->iteration = it + 1;
}

// ---- uploads: bin freshly added molecules (staged in the product list) into the first arrays

// re-binning (uploads): existing molecules keep their position (b = a, status
// survivor) and staged ones sit in the product list; both are counted here and
// moved by k_scatter
// remove: molecules (by index) that leave with this re-binning (a vacuum release), or
// null; staged_status: the staged molecules' status was written by their producer (a
// release whose single draws may place nothing), else every staged molecule is placed
template <typename T>
__global__ void k_rebin_count(State<T> s, uint32_t n_staged, const uint8_t* remove, int staged_status) {
  const uint32_t n = s.cnt->n_live;
  for (uint32_t base = blockIdx.x * TPB; base < n; base += gridDim.x * TPB) {
    uint32_t i = base + threadIdx.x;
    bool active = i < n;
    uint32_t key = 0;
    if (active) {
      P4<T> p = s.a_pos[i];
      s.b_pos[i] = p;
      // molecules of a dropped replica leave with this re-binning
      active = geo_of(s, meta_of(p)).mode != REP_DROP && !(remove && remove[i]);
      s.st[i] = active ? 0 : 2;
      if (active) key = key_of_rec(s, p);
    }
    warp_count(s.counts, key, active);
  }
  for (uint32_t base = blockIdx.x * TPB; base < n_staged; base += gridDim.x * TPB) {
    uint32_t k = base + threadIdx.x;
    bool active = k < n_staged;
    uint32_t key = 0;
    if (active) {
      if (staged_status) {
        active = s.pst[k] == 0;
      } else {
        s.pst[k] = 0;
      }
      if (active) key = key_of_rec(s, s.prod[k].pos);
    }
    warp_count(s.counts, key, active);
  }
}


// ---- volume releases on the device (ReleaseEvent::release_ellipsoid_or_rectcuboid,
// release_inside_regions; release_event.cpp:904-1006): new molecules written into
// the staging (product) list, then binned like an upload

constexpr int REL_SPHERE = 0, REL_CUBOID = 1, REL_SHELL = 2, REL_INSIDE = 3;

constexpr int REGION_EXPR_MAX = 15;  // tokens of a region expression
struct ReleaseDesc {
  uint32_t rep, species, n, object;
  int shape;
  double center[3], diameter[3];  // ellipsoid / cuboid / shell
  double llf[3], urb[3];          // sampling box of a release inside a region
  uint64_t seed, uid0;
  // REL_INSIDE: the region, a postfix program of objects (>= 0) and operators (-1
  // union, -2 intersection, -3 difference); the low corner of each leaf object's box
  int32_t expr[REGION_EXPR_MAX];
  uint32_t n_expr;
  double leaf_llf[REGION_EXPR_MAX][3];
  // each molecule's point is drawn once and kept only if inside (the reference's
  // approximate count of a concentration release into an expression)
  int single_draw;
};

// one molecule of ReleaseEvent::release_ellipsoid_or_rectcuboid (release_event.cpp:953-
// 1000): a point of the unit cube around 0, kept (spheroidal shapes) inside the ball of
// radius 0.5, on a shell moved onto the sphere, scaled by the diameter and moved to the
// center; fp64 without fused multiply-adds, so that injected draws give the
// reference's positions. False when 1024 tries gave no point.
template <class D>
__device__ bool release_point(int shape, const double* center, const double* diameter, D& d, V3<double>& out) {
  const bool spheroidal = shape == REL_SPHERE || shape == REL_SHELL;
  V3<double> q = v3<double>(0, 0, 0);
  bool ok = false;
  for (int attempt = 0; attempt < 1024 && !ok; attempt++) {
    q.x = __dsub_rn(draw_dbl(d), 0.5);
    q.y = __dsub_rn(draw_dbl(d), 0.5);
    q.z = __dsub_rn(draw_dbl(d), 0.5);
    ok = !spheroidal || rn_dot3(q.x, q.y, q.z, q.x, q.y, q.z) < 0.25;
  }
  if (shape == REL_SHELL) {
    const double r = __dmul_rn(sqrt(rn_dot3(q.x, q.y, q.z, q.x, q.y, q.z)), 2.0);
    q = r == 0 ? v3<double>(0, 0, 0.5) : v3<double>(q.x / r, q.y / r, q.z / r);
  }
  out = v3<double>(__dadd_rn(__dmul_rn(q.x, diameter[0]), center[0]), __dadd_rn(__dmul_rn(q.y, diameter[1]), center[1]),
                   __dadd_rn(__dmul_rn(q.z, diameter[2]), center[2]));
  return ok;
}

// is_point_inside_region_expr_recursively (release_event.cpp:785-810) over the postfix
// program: every leaf's inside test (the reference evaluates both operands of every
// operator), combined by union, intersection or difference; NONE when a leaf's ray met
// a wall edge
template <typename T>
__device__ uint32_t inside_expr(const Geo<T>& g, V3<double> p, const ReleaseDesc& r) {
  uint32_t st = 0;  // results, the last one in bit 0
  for (uint32_t k = 0; k < r.n_expr; k++) {
    const int32_t t = r.expr[k];
    if (t >= 0) {
      const uint32_t in = inside_region(g, p, (uint32_t)t, r.leaf_llf[k]);
      if (in == NONE) return NONE;
      st = (st << 1) | in;
    } else {
      const uint32_t b = st & 1u, a = (st >> 1) & 1u;
      const uint32_t v = t == -1 ? (a | b) : (t == -2 ? (a & b) : (a & (b ^ 1u)));
      st = ((st >> 2) << 1) | v;
    }
  }
  return st & 1u;
}

// a point of the region's bounding box (release_inside_regions, release_event.cpp:923-926)
template <class D>
__device__ __forceinline__ V3<double> box_point(const double* llf, const double* urb, D& d) {
  V3<double> out;
  out.x = __dadd_rn(llf[0], __dmul_rn(__dsub_rn(urb[0], llf[0]), draw_dbl(d)));
  out.y = __dadd_rn(llf[1], __dmul_rn(__dsub_rn(urb[1], llf[1]), draw_dbl(d)));
  out.z = __dadd_rn(llf[2], __dmul_rn(__dsub_rn(urb[2], llf[2]), draw_dbl(d)));
  return out;
}

// one molecule of ReleaseEvent::release_inside_regions (release_event.cpp:904-952): a
// point of the region's bounding box, kept if inside the region (the reference's ray
// tests; a ray through an edge, where the reference's test would fail, draws again).
// single_draw: one point only, kept if inside (false when it is not)
template <typename T, class D>
__device__ bool release_inside_point(const Geo<T>& g, const ReleaseDesc& r, D& d, V3<double>& out, uint32_t& redo) {
  for (int attempt = 0; attempt < 1024; attempt++) {
    out = box_point(r.llf, r.urb, d);
    const uint32_t in = inside_expr(g, out, r);
    if (in == NONE) {
      redo++;
      continue;
    }
    if (in || r.single_draw) return in != 0;
  }
  return false;
}

template <typename T>
__global__ void k_release(State<T> s, ReleaseDesc r) {
  const Geo<T>& g = s.geos[r.rep];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < r.n; i += gridDim.x * blockDim.x) {
    PhiloxDraws d;
    d.ph.init(r.seed, i, 0, 7);
    V3<double> p = v3<double>(0, 0, 0);
    uint32_t redo = 0;
    const bool ok = r.shape == REL_INSIDE ? release_inside_point(g, r, d, p, redo)
                                          : release_point(r.shape, r.center, r.diameter, d, p);
    // a single draw outside the region places nothing; else no point in 1024 tries
    s.pst[i] = ok ? 0 : 2;
    if (!ok && !r.single_draw) atomicOr(&s.cnt->status, ST_WATCHDOG);
    Product<T> m;
    m.pos.x = (T)p.x;
    m.pos.y = (T)p.y;
    m.pos.z = (T)p.z;
    uint32_t cv = g.n_cv ? counted_volume_bits(g, p) : 0u;
    if (cv == NONE) {
      redo++;
      cv = 0;
    }
    if (redo) atomicAdd(&s.cnt->warn_inside_redo, (unsigned long long)redo);
    set_meta(m.pos, make_meta(r.species, r.rep, META_SCHEDULE_UNIMOL | (cv << META_CV_SHIFT)));
    m.birth = 0;
    m.uid = r.uid0 + i;
    m.tuni = TIME_FOREVER;
    s.prod[i] = m;
  }
}

// Molecules uploaded from host arrays (positions in fp64, species), staged into the
// product list at `offset` for the re-binning: checked (species, inside the partition),
// and in fp32 moved off any wall plane of their subpartition they lie within
// max(1e-4, 8 fp32 ulps of the coordinates) of, to that distance on their own side
// (twice, for edges and corners), in fp64 without fused multiply-adds. err bit 0: a
// species out of range, bit 1: a molecule outside the partition.
template <typename T>
__global__ void k_stage_upload(State<T> s, uint32_t rep, uint32_t n, const double* pos, const uint32_t* species,
                               uint64_t uid0, uint32_t offset, uint32_t nsp, uint32_t* err) {
  const Geo<T>& g = s.geos[rep];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t sp = species[i];
    double p[3] = {pos[3 * (size_t)i], pos[3 * (size_t)i + 1], pos[3 * (size_t)i + 2]};
    if (sp >= nsp) {
      atomicOr(err, 1u);
      continue;
    }
    if (!(p[0] >= (double)g.origin.x && p[1] >= (double)g.origin.y && p[2] >= (double)g.origin.z &&
          p[0] < (double)g.opposite.x && p[1] < (double)g.opposite.y && p[2] < (double)g.opposite.z)) {
      atomicOr(err, 2u);
      continue;
    }
    if (sizeof(T) == 4 && g.w64) {
      int ix[3];
      for (int a = 0; a < 3; a++)
        ix[a] = min(max((int)__dmul_rn(__dsub_rn(p[a], g.origin64[a]), g.sp_rcp64), 0), g.nsub - 1);
      const uint32_t c = (uint32_t)ix[0] + (uint32_t)ix[1] * (uint32_t)g.nsub + (uint32_t)ix[2] * (uint32_t)g.nsub2;
      const double mag = fmax(fabs(p[0]), fmax(fabs(p[1]), fabs(p[2])));
      const double margin = fmax(1e-4, __dmul_rn(__dmul_rn(8.0, mag), 1.1920928955078125e-07));
      // fp32 screen first (GB300's FP64 rate is low): the fp32 distance is within
      // 1e-4 + 1e-6 * |p| of the fp64 one, so a wall farther than that beyond the margin
      // cannot be within it
      const float screen = (float)(margin + 1e-3 + 1e-5 * mag);
      for (int pass = 0; pass < 2; pass++) {
        bool moved = false;
        float px = (float)p[0], py = (float)p[1], pz = (float)p[2];
        for (uint32_t k = g.wsp_off[c]; k < g.wsp_off[c + 1]; k++) {
          const uint32_t wi = g.wsp_list[k];
          const P4<T> rj = g.wrej[wi];
          if (fabsf((float)rj.x * px + (float)rj.y * py + (float)rj.z * pz - (float)rj.w) > screen) continue;
          const double* pl = g.w64 + 16 * (size_t)wi;
          const double dd = __dsub_rn(
              __dadd_rn(__dadd_rn(__dmul_rn(pl[0], p[0]), __dmul_rn(pl[1], p[1])), __dmul_rn(pl[2], p[2])), pl[3]);
          if (fabs(dd) >= margin) continue;
          const double shift = __dsub_rn(dd >= 0 ? margin : -margin, dd);
          for (int a = 0; a < 3; a++) p[a] = __dadd_rn(p[a], __dmul_rn(shift, pl[a]));
          px = (float)p[0];
          py = (float)p[1];
          pz = (float)p[2];
          moved = true;
        }
        if (!moved) break;
      }
    }
    Product<T> m;
    m.pos.x = (T)p[0];
    m.pos.y = (T)p[1];
    m.pos.z = (T)p[2];
    set_meta(m.pos, make_meta(sp, rep, META_SCHEDULE_UNIMOL));
    m.birth = 0;
    m.uid = uid0 + i;
    m.tuni = TIME_FOREVER;
    s.prod[offset + i] = m;
  }
}

// the molecules of a species of replica rep inside a region (vacuum_inside_regions,
// release_event.cpp:864-896: the species, the region's bounding box, then the region's
// inside tests): their ids and indices, in no particular order
template <typename T>
__global__ void k_vacuum_candidates(State<T> s, ReleaseDesc r, uint64_t* ids, uint32_t* idx, uint32_t* count) {
  const Geo<T>& g = s.geos[r.rep];
  const uint32_t n = s.cnt->n_live;
  uint32_t redo = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const P4<T> p = s.a_pos[i];
    const uint32_t meta = meta_of(p);
    if (meta_rep(meta) != r.rep || (meta & META_SPECIES_MASK) != r.species) continue;
    const V3<double> q = v3<double>((double)p.x, (double)p.y, (double)p.z);
    if (!(q.x >= r.llf[0] && q.x <= r.urb[0] && q.y >= r.llf[1] && q.y <= r.urb[1] && q.z >= r.llf[2] &&
          q.z <= r.urb[2]))
      continue;
    const uint32_t in = inside_expr(g, q, r);
    if (in == NONE) {
      redo++;  // counted outside
      continue;
    }
    if (!in) continue;
    const uint32_t k = warp_slot(count);
    ids[k] = s.a_uid[i];
    idx[k] = i;
  }
  if (redo) atomicAdd(&s.cnt->warn_inside_redo, (unsigned long long)redo);
}

// Parity harness of release_inside_regions (release_event.cpp:904-952), one thread:
// `n` molecules drawn in turn from one injected stream; with single_draw each draw is
// one of the n (kept if inside), else draws repeat until inside. NONE (a ray through an
// edge) draws again. out: positions; *n_out placed; *used draws (0xFFFFFFFF overrun)
template <typename T>
__global__ void k_release_region_harness(State<T> s, ReleaseDesc r, const uint32_t* draws, uint32_t ndraws,
                                         double* out, uint32_t cap, uint32_t* n_out, uint32_t* used) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const Geo<T>& g = s.geos[r.rep];
  InjectedDraws d;
  d.d = draws;
  d.n = ndraws;
  d.used = 0;
  d.over = false;
  uint32_t placed = 0;
  int64_t left = r.n;
  uint32_t guard = 0;
  while (left > 0 && !d.over && ++guard < (1u << 22)) {
    const V3<double> p = box_point(r.llf, r.urb, d);
    const uint32_t in = d.over ? 0u : inside_expr(g, p, r);
    if (in == NONE) continue;
    if (!in) {
      if (r.single_draw) left--;
      continue;
    }
    if (placed < cap) {
      out[3 * placed] = p.x;
      out[3 * placed + 1] = p.y;
      out[3 * placed + 2] = p.z;
    }
    placed++;
    left--;
  }
  *n_out = placed;
  *used = d.over ? 0xFFFFFFFFu : d.used;
}

// inside tests on given points (parity harness): kind 0 the counted-volume bits, kind 1
// inside object obj (bounding box low corner llf); NONE where the ray met an edge
template <typename T>
__global__ void k_inside_tests(State<T> s, uint32_t rep, uint32_t n, const double* pos, int kind, uint32_t obj,
                               const double* llf, uint32_t* out) {
  const Geo<T>& g = s.geos[rep];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const V3<double> p = v3<double>(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    out[i] = kind == 0 ? counted_volume_bits(g, p) : inside_region(g, p, obj, llf);
  }
}

// ---- per-routine parity harness: injected displacement and draws

template <typename T>
__global__ void k_trace_cases(State<T> s, uint32_t ncases, const uint32_t* idx, const double* disp,
                              const uint32_t* draws, uint32_t ndraws, const double* rrf, const double* tst,
                              double* out) {
  uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncases) return;
  double* o = out + (size_t)c * 265;
  for (int k = 0; k < 265; k++) o[k] = 0;
  const uint32_t i = idx[c];
  P4<T> rec = s.a_pos[i];
  const int species = (int)(meta_of(rec) & META_SPECIES_MASK);
  const Geo<T>& g = geo_of(s, meta_of(rec));
  InjectedDraws d;
  d.d = draws + (size_t)c * ndraws;
  d.n = ndraws;
  d.used = 0;
  d.over = false;
  EventLog ev;
  ev.out = o;
  Cells<T> cells;
  cells.pos = s.a_pos;
  cells.uid = s.a_uid;
  cells.start = s.start;
  cells.dead = nullptr;
  cells.maxc = s.maxc;
  cells.maxset = s.maxset;
  V3<T> dv = v3<T>((T)disp[3 * c], (T)disp[3 * c + 1], (T)disp[3 * c + 2]);
  TraceOut<T> r =
      trace_molecule<T>(g, cells, i, v3<T>(rec.x, rec.y, rec.z), species, dv, (T)rrf[c], (T)tst[c], (T)0, d, ev);
  count_fallbacks(s, r.err);
  int status = r.status;
  if (d.over) status = 3;
  o[0] = status;
  o[1] = (double)r.pos.x;
  o[2] = (double)r.pos.y;
  o[3] = (double)r.pos.z;
  o[4] = r.subpart;
  o[5] = d.used;
  o[7] = r.elapsed;
  o[8] = r.t_steps;
}

}  // namespace mcg
