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

namespace mcg {

// Model features outside the GPU path are refused, with no fallback. A product of
// any reaction that is also a reactant of a bimolecular reaction would, in the
// reference, diffuse the rest of its birth step with vol-vol reaction tests (the
// queue of new diffuse actions, src4/diffuse_react_event.cpp:116-129, :2883-2886);
// the GPU's products diffuse the rest of that step without them, so such models
// are refused (MCG_ERR_UNSUPPORTED) rather than run with other semantics.
inline int check_model_supported(const mcg_engine& m, std::string& why) {
  const uint32_t rp = m.chem.reactive_products();
  if (rp) {
    uint32_t s = 0;
    while (!((rp >> s) & 1u)) s++;
    why = "species " + std::to_string(s) +
          " is a reaction product and a bimolecular reactant: same-step reactions of products are not on the "
          "GPU path";
    return MCG_ERR_UNSUPPORTED;
  }
  return MCG_OK;
}

}  // namespace mcg
