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

struct ChemHost {
  uint32_t nsp = 0;
  double space_step[16] = {0};
  double unimol_k[16];
  int uni_prod[16][2];
  double bimol_p[16][16];
  int bimol_prod[16][16][2];
  ChemHost() {
    for (int a = 0; a < 16; a++) {
      unimol_k[a] = -1;
      uni_prod[a][0] = uni_prod[a][1] = -1;
      for (int b = 0; b < 16; b++) {
        bimol_p[a][b] = -1;
        bimol_prod[a][b][0] = bimol_prod[a][b][1] = -1;
      }
    }
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
  // counted volumes: molecules of each species inside each counted object after the
  // last iteration or upload ([nsp][n_counted]), and their trajectory
  virtual int counted_counts(uint32_t rep, uint64_t* out, std::string& err) = 0;
  virtual int counted_trajectory(uint32_t rep, uint32_t n, uint64_t* out, std::string& err) = 0;
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

DeviceEngine* make_engine_f64();
DeviceEngine* make_engine_f32();

// maps device status bits to the ABI error codes (0 if clean)
int status_to_error(uint32_t status, std::string& err);

}  // namespace mcg
