// Host-side model description behind an mcg_engine handle (shared by the C ABI
// of single models and of batches, which take models as replica descriptions).
#pragma once

#include <string>
#include <vector>

#include "../../include/mcell_gb300.h"
#include "mcg_engine.h"

struct mcg_engine {
  mcg_config cfg;
  std::string err;
  mcg::ChemHost chem;
  bool species_set = false;
  std::vector<double> verts;
  std::vector<uint32_t> walls;
  std::vector<uint8_t> wclass;
  std::vector<uint16_t> wall_obj;     // geometry object of each wall (optional)
  std::vector<uint16_t> counted;      // counted objects (at most 7)
  std::vector<double> pend_pos;       // molecules added before the device engine exists
  std::vector<uint32_t> pend_species;
  uint64_t next_uid = 0;
  mcg::DeviceEngine* dev = nullptr;   // created on first use (mcg_prepare / mcg_step)
};
