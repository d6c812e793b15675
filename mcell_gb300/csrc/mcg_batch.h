// Host-side state behind an mcg_batch handle (shared by the batch C ABI and the
// serving loop, which drives a batch from its worker thread).
#pragma once

#include <string>
#include <vector>

#include "mcg_model.h"

struct mcg_batch {
  mcg_batch_config cfg;
  std::string err;
  mcg::DeviceEngine* dev = nullptr;
  std::vector<uint32_t> nsub;  // subpartitions per edge of each replica slot
  bool tune_pending = false;
  int diffuse_blocks = 0;
};

// The host half of admitting a model as a replica: the model's checks, its
// subpartition grid (the autotuner's choice when `autotune`) and its setup (wall
// constants and lists). It only reads the model, so a server runs it at
// submission, in the submitting thread, and its worker does the device half alone.
struct ReplicaPrep {
  mcg::HostSetup hs;
  uint32_t nsub = 0;
  bool octants = true;
};
int batch_prepare_replica(const mcg_engine* m, bool autotune, ReplicaPrep& out, std::string& err);  // MCG code
// The device half: the prepared models become replicas (ids out), as mcg_batch_add.
int batch_add_prepared(mcg_batch* b, uint32_t n, mcg_engine* const* models, ReplicaPrep* const* preps,
                       const uint32_t* n_iterations, uint32_t* ids);
