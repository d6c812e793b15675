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
