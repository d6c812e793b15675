// GpuDiffuseReactEvent: C++ host-side event that runs MCell4's volume diffuse-react
// step on the GB300 engine through the C ABI in mcell_gb300.h.
//
// It has the scheduling interface of DiffuseReactEvent (src4/diffuse_react_event.h:100-160,
// BaseEvent src4/base_event.h:63-135): one step() per iteration, rescheduled every
// periodicity_interval, blocked by barriers (count / viz events), with the time up to
// the next barrier set by the scheduler before each step. In MCell4 it derives from
// BaseEvent; World::init_simulation (src4/world.cpp:280-282) creates it instead of
// DiffuseReactEvent when the model selects the GPU engine. This header does not
// depend on MCell4's headers: the members below mirror BaseEvent's so the class can
// be dropped into the reference with "class GpuDiffuseReactEvent : public BaseEvent".
#ifndef MCELL_GB300_EVENT_HPP
#define MCELL_GB300_EVENT_HPP

#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "mcell_gb300.h"

namespace mcg {

class GpuDiffuseReactEvent {
 public:
  // DIFFUSE_REACT_EVENT_PERIODICITY and DIFFUSION_TIME_UPPER_LIMIT of the reference
  static constexpr double PERIODICITY = 1.0;
  static constexpr double MAX_TIME_UP_TO_NEXT_BARRIER = 100.0;

  explicit GpuDiffuseReactEvent(const mcg_config& cfg) : event_time(0.0), periodicity_interval(PERIODICITY) {
    check(mcg_create(&cfg, &engine_), "mcg_create");
  }
  ~GpuDiffuseReactEvent() { mcg_destroy(engine_); }
  GpuDiffuseReactEvent(const GpuDiffuseReactEvent&) = delete;
  GpuDiffuseReactEvent& operator=(const GpuDiffuseReactEvent&) = delete;

  // ---- model setup (what MCell4Converter hands the World: species, walls, rxns, releases)
  void set_species(const std::vector<double>& space_steps) {
    check(mcg_set_species(engine_, (uint32_t)space_steps.size(), space_steps.data()), "mcg_set_species");
  }
  void upload_mesh(const std::vector<double>& vertices, const std::vector<uint32_t>& walls,
                   const std::vector<uint8_t>& wall_class) {
    check(mcg_upload_mesh(engine_, (uint32_t)(vertices.size() / 3), vertices.data(), (uint32_t)(walls.size() / 3),
                          walls.data(), wall_class.data()),
          "mcg_upload_mesh");
  }
  void add_bimol_rxn(uint32_t a, uint32_t b, double max_fixed_p, int32_t p0, int32_t p1 = -1) {
    check(mcg_add_bimol_rxn(engine_, a, b, max_fixed_p, p0, p1), "mcg_add_bimol_rxn");
  }
  void add_unimol_rxn(uint32_t a, double k_tot, int32_t p0 = -1, int32_t p1 = -1) {
    check(mcg_add_unimol_rxn(engine_, a, k_tot, p0, p1), "mcg_add_unimol_rxn");
  }
  void release(const std::vector<double>& pos, const std::vector<uint32_t>& species) {
    check(mcg_add_molecules(engine_, species.size(), pos.data(), species.data()), "mcg_add_molecules");
  }

  // ---- BaseEvent interface
  void step() {
    // time_up_to_next_barrier is a whole number of iterations (>= 1); run them all
    const uint32_t n = (uint32_t)std::lround(std::fmin(time_up_to_next_barrier_, periodicity_interval));
    check(mcg_step(engine_, n < 1 ? 1 : n), "mcg_step");
  }
  bool update_event_time_for_next_scheduled_time() {
    event_time += (time_up_to_next_barrier_ < periodicity_interval) ? time_up_to_next_barrier_ : periodicity_interval;
    return true;
  }
  bool may_be_blocked_by_barrier_and_needs_set_time_step() const { return true; }
  double get_max_time_up_to_next_barrier() const { return MAX_TIME_UP_TO_NEXT_BARRIER; }
  void set_barrier_time_for_next_execution(double t) {
    if (!(t > 0)) throw std::runtime_error("Diffusion must advance even if a little bit");
    time_up_to_next_barrier_ = t;
  }

  // ---- what barrier events read (MolOrRxnCountEvent, checkpoints, viz)
  std::vector<uint64_t> counts(uint32_t n_species) {
    std::vector<uint64_t> c(n_species);
    check(mcg_get_counts(engine_, c.data()), "mcg_get_counts");
    return c;
  }
  // the same counts without waiting now: a ticket for a copy queued behind the
  // iterations run so far, redeemed later (a count buffer's flush)
  uint64_t request_counts() {
    uint64_t t = 0;
    check(mcg_request_counts(engine_, &t), "mcg_request_counts");
    return t;
  }
  std::vector<uint64_t> wait_counts(uint64_t ticket, uint32_t n_species) {
    std::vector<uint64_t> c(n_species);
    check(mcg_wait_counts(engine_, ticket, c.data()), "mcg_wait_counts");
    return c;
  }
  void molecules(std::vector<double>& pos, std::vector<uint32_t>& species, std::vector<uint64_t>& ids) {
    uint64_t n = 0;
    check(mcg_download_molecules(engine_, 0, nullptr, nullptr, nullptr, &n), "mcg_download_molecules");
    pos.resize(3 * n);
    species.resize(n);
    ids.resize(n);
    check(mcg_download_molecules(engine_, n, pos.data(), species.data(), ids.data(), &n), "mcg_download_molecules");
  }
  void sync() { check(mcg_sync(engine_), "mcg_sync"); }
  mcg_engine* engine() { return engine_; }

  double event_time;
  double periodicity_interval;

 private:
  void check(int rc, const char* what) {
    if (rc != MCG_OK) {
      // the caller maps this to World::fatal_error / API::RuntimeError
      throw std::runtime_error(std::string(what) + " failed (" + std::to_string(rc) +
                               "): " + (engine_ ? mcg_last_error(engine_) : ""));
    }
  }
  mcg_engine* engine_ = nullptr;
  double time_up_to_next_barrier_ = PERIODICITY;
};

}  // namespace mcg

#endif
