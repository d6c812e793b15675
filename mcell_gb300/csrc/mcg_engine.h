// Device engine interface shared by the fp64 and fp32 translation units and the C ABI.
//
// One engine holds any number of replicas (independent models: own mesh,
// partition grid, reactions, seed and molecules) in one set of device arrays;
// every kernel of an iteration covers all of them. The plain C ABI drives an
// engine with a single replica (slot 0).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "mcg_setup.h"

namespace mcg {

// Reaction classes of a model (BNG::RxnClass as test_bimolecular and
// which_unimolecular use it, src4/rxn_utils.inl:336-414, :774-783): per reactant pair
// and per unimolecular reactant, up to MAX_PATHWAYS pathways in the order they were
// added, their cumulative probabilities (bimolecular) or rates times the time step
// (unimolecular), and up to two products each (-1 = none).
constexpr int MAX_PATHWAYS = 4;
struct ChemHost {
  uint32_t nsp = 0;
  double space_step[16] = {0};
  double unimol_k[16];                    // k_tot = last cumulative rate, < 0: none
  int uni_npw[16];
  double uni_cum[16][MAX_PATHWAYS];
  int uni_prod[16][MAX_PATHWAYS][2];
  double bimol_p[16][16];                 // max_fixed_p = last cumulative probability, < 0: none
  int bimol_npw[16][16];
  double bimol_cum[16][16][MAX_PATHWAYS];
  int bimol_prod[16][16][MAX_PATHWAYS][2];
  ChemHost() {
    for (int a = 0; a < 16; a++) {
      unimol_k[a] = -1;
      uni_npw[a] = 0;
      for (int k = 0; k < MAX_PATHWAYS; k++) {
        uni_cum[a][k] = 0;
        uni_prod[a][k][0] = uni_prod[a][k][1] = -1;
      }
      for (int b = 0; b < 16; b++) {
        bimol_p[a][b] = -1;
        bimol_npw[a][b] = 0;
        for (int k = 0; k < MAX_PATHWAYS; k++) {
          bimol_cum[a][b][k] = 0;
          bimol_prod[a][b][k][0] = bimol_prod[a][b][k][1] = -1;
        }
      }
    }
  }
  // appends a pathway; false if the class is full
  bool add_bimol(int a, int b, double p, int p0, int p1) {
    const int k = bimol_npw[a][b];
    if (k >= MAX_PATHWAYS) return false;
    const double c = (k ? bimol_cum[a][b][k - 1] : 0.0) + p;
    for (int pass = 0; pass < (a == b ? 1 : 2); pass++) {
      const int x = pass ? b : a, y = pass ? a : b;
      bimol_cum[x][y][k] = c;
      bimol_prod[x][y][k][0] = p0;
      bimol_prod[x][y][k][1] = p1;
      bimol_npw[x][y] = k + 1;
      bimol_p[x][y] = c;
    }
    return true;
  }
  bool add_unimol(int a, double k_tot, int p0, int p1) {
    const int k = uni_npw[a];
    if (k >= MAX_PATHWAYS) return false;
    uni_cum[a][k] = (k ? uni_cum[a][k - 1] : 0.0) + k_tot;
    uni_prod[a][k][0] = p0;
    uni_prod[a][k][1] = p1;
    uni_npw[a] = k + 1;
    unimol_k[a] = uni_cum[a][k];
    return true;
  }
  // species that are products of some reaction and reactants of a bimolecular one
  // (their same-step reactions are outside the GPU path); returns a bit mask
  uint32_t reactive_products() const {
    uint32_t prod = 0, react = 0;
    for (uint32_t a = 0; a < nsp; a++) {
      for (int k = 0; k < uni_npw[a]; k++)
        for (int q = 0; q < 2; q++)
          if (uni_prod[a][k][q] >= 0) prod |= 1u << uni_prod[a][k][q];
      for (uint32_t b = 0; b < nsp; b++) {
        if (bimol_npw[a][b]) react |= 1u << a;
        for (int k = 0; k < bimol_npw[a][b]; k++)
          for (int q = 0; q < 2; q++)
            if (bimol_prod[a][b][k][q] >= 0) prod |= 1u << bimol_prod[a][b][k][q];
      }
    }
    return prod & react;
  }
};

// one model to add as a replica
struct ReplicaSpec {
  const HostSetup* hs = nullptr;
  const ChemHost* chem = nullptr;
  const std::vector<uint8_t>* wall_class = nullptr;  // [wall][species]
  uint64_t seed = 1;
  uint64_t n_mol = 0;
  const double* pos = nullptr;       // [n_mol][3]
  const uint32_t* species = nullptr;  // [n_mol]
  const std::vector<uint16_t>* wall_obj = nullptr;  // geometry object of each wall (optional)
  std::vector<uint16_t> counted;     // objects whose contents are counted (at most 7)
  uint32_t n_iterations = 0;         // iterations to run, then the replica freezes; 0 = unlimited
  bool octants = true;               // bin occupants per subpartition octant when the key space allows
};

class DeviceEngine {
 public:
  virtual ~DeviceEngine() {}
  // engine with max_replicas replica slots of nsp species each
  virtual int create(uint32_t nsp, uint32_t max_replicas, uint64_t capacity, std::string& err) = 0;
  // adds replicas (one re-sort of all molecules); slots written to reps[]
  virtual int add_replicas(const ReplicaSpec* specs, uint32_t n, uint32_t* reps, std::string& err) = 0;
  // frees replica slots; their molecules leave with one re-sort
  virtual int remove_replicas(const uint32_t* reps, uint32_t n, std::string& err) = 0;
  virtual int add_molecules(uint32_t rep, uint64_t n, const double* pos, const uint32_t* species, uint64_t uid0,
                            std::string& err) = 0;
  virtual int step(uint32_t n, std::string& err) = 0;
  virtual int sync(std::string& err) = 0;
  virtual int counts(uint32_t rep, uint64_t* out, std::string& err) = 0;
  // non-blocking counts: a copy queued after the work queued so far, read by ticket
  virtual int request_counts(uint32_t rep, uint64_t* ticket, std::string& err) = 0;
  virtual int wait_counts(uint64_t ticket, uint64_t* out, std::string& err) = 0;
  virtual int trajectory(uint32_t rep, uint32_t n, uint64_t* out, std::string& err) = 0;
  virtual int download(uint32_t rep, uint64_t cap, double* pos, uint32_t* species, uint64_t* ids, uint64_t* n_out,
                       std::string& err) = 0;
  // checkpoints: molecules with ids, unimolecular times (relative to the next
  // iteration) and flags (bit 0: time not drawn yet), and the replica's iteration
  virtual int export_state(uint32_t rep, uint64_t cap, double* pos, uint32_t* species, uint64_t* ids, double* tuni,
                           uint8_t* flags, uint64_t* n_out, uint64_t* iteration, std::string& err) = 0;
  virtual int import_state(uint32_t rep, uint64_t n, const double* pos, const uint32_t* species, const uint64_t* ids,
                           const double* tuni, const uint8_t* flags, uint64_t iteration, std::string& err) = 0;
  // volume release on the device (shape: 0 ellipsoid, 1 cuboid, 2 ellipsoid shell, 3
  // inside geometry object `object`); ids continue the replica's
  virtual int release(uint32_t rep, uint32_t species, uint64_t n, int shape, const double* center,
                      const double* diameter, uint32_t object, uint64_t seed, std::string& err) = 0;
  // release into / vacuum from a region expression (mcg_release_region); draws != null:
  // the parity harness (nothing changes; positions or removed ids are returned)
  virtual int release_region(uint32_t rep, uint32_t species, int method, int64_t number, double concentration,
                             double length_unit, const int32_t* expr, uint32_t n_expr, uint64_t seed,
                             int64_t* done, std::string& err) = 0;
  // the id the replica's next new molecule gets
  virtual uint64_t next_molecule_id(uint32_t rep) = 0;
  virtual int release_region_harness(uint32_t rep, uint32_t species, int method, int64_t number,
                                     double concentration, double length_unit, const int32_t* expr, uint32_t n_expr,
                                     const uint32_t* draws, uint32_t n_draws, double* pos, uint32_t cap,
                                     uint32_t* n_pos, uint64_t* removed, uint32_t* n_removed, uint32_t* used,
                                     std::string& err) = 0;
  // counted volumes: molecules of each species inside each counted object after the
  // last iteration or upload ([nsp][n_counted]), and their trajectory
  virtual int counted_counts(uint32_t rep, uint64_t* out, std::string& err) = 0;
  virtual int counted_trajectory(uint32_t rep, uint32_t n, uint64_t* out, std::string& err) = 0;
  // counts before the replica's first iteration: world[nsp], and inside[nsp][n_counted]
  // (may be null) for its counted objects
  virtual int initial_counts(uint32_t rep, uint64_t* world, uint64_t* inside, std::string& err) = 0;
  // iterations the replica has run (it freezes after its n_iterations)
  virtual int replica_iterations(uint32_t rep, uint64_t* done, std::string& err) = 0;
  // the replica's counted objects and the engine iterations since it was added (the
  // rows of its count trajectories, frozen ones included)
  virtual int replica_rows(uint32_t rep, uint32_t* n_counted, uint64_t* since_added, std::string& err) = 0;
  // device bytes held for the replica (mesh, grid, its share of the molecule arrays)
  virtual uint64_t replica_bytes(uint32_t rep) = 0;
  virtual uint64_t device_bytes() = 0;
  virtual int trace(uint32_t n, const uint64_t* ids, const double* disp, const uint32_t* draws, uint32_t ndraws,
                    const double* rrf, const double* tst, double* out, std::string& err) = 0;
  // trace() on the fixed scratch of mcg_trace_static.cu (no device allocation)
  virtual int trace_static(uint32_t n, const uint64_t* ids, const double* disp, const uint32_t* draws,
                           uint32_t ndraws, const double* rrf, const double* tst, double* out, std::string& err) = 0;
  virtual void stats(uint64_t* iterations, uint64_t* mol_steps, uint64_t* launches) = 0;
  // exact fallbacks taken: [0] traces that refilled a full candidate page, [1] traces
  // whose partner list overflowed (partners scanned along the walk); [2] inside tests
  // whose ray met a wall edge
  virtual int fallbacks(uint64_t* out, std::string& err) = 0;
  // inside tests on points (parity harness): kind 0 counted-volume bits, 1 inside
  // object obj; 0xFFFFFFFF where the ray met an edge
  virtual int inside_tests(uint32_t rep, uint32_t n, const double* pos, int kind, uint32_t obj, uint32_t* out,
                           std::string& err) = 0;
  // test hook: capacities of a candidate page (<= 16) and of the partner list (<= 48)
  virtual int set_trace_limits(int maxc, int maxset, std::string& err) = 0;
  virtual void set_options(int use_graphs, int profile) = 0;
  // diffuse-kernel shape: resident blocks per SM of the persistent grid (0 = as many as fit)
  virtual int set_diffuse_blocks_per_sm(int blocks, std::string& err) = 0;
  virtual int max_diffuse_blocks_per_sm() = 0;
  virtual int profile(double* out, std::string& err) = 0;
  virtual int debug_molecule(uint64_t uid, std::string& err) = 0;
  virtual int debug_log(double* out, std::string& err) = 0;
  virtual int escapes(double* out, uint32_t cap, uint32_t* n, std::string& err) = 0;
};

// test hook: the device allocation after `after` more successful ones fails as if the
// device were out of memory (once); negative: off (mcg_inject_device_alloc_failure)
void set_alloc_failure(long long after);

// reaction decisions on injected draws (parity harness; kind 0 test_bimolecular, 1
// which_unimolecular): cum[n][MAX_PATHWAYS], npw[n], scaling[n] (kind 0), draws[n]
int rxn_decisions(int kind, uint32_t n, const double* cum, const uint32_t* npw, const double* scaling,
                  const uint32_t* draws, int32_t* out, std::string& err);

// release positions on an injected stream (parity harness of release_point): shape 0
// ellipsoid, 1 cuboid, 2 ellipsoid shell; one stream for the whole release; *used = the
// draws consumed (0xFFFFFFFF if they ran out)
int release_positions(int shape, uint32_t n, const double* center, const double* diameter, const uint32_t* draws,
                      uint32_t ndraws, double* out, uint32_t* used, std::string& err);

DeviceEngine* make_engine_f64();
DeviceEngine* make_engine_f32();

// maps device status bits to the ABI error codes (0 if clean)
int status_to_error(uint32_t status, std::string& err);

}  // namespace mcg
