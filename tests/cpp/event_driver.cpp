// C++ host driver: runs the GPU diffuse-react event the way MCell4's scheduler does
// (barrier-limited steps, count barrier every iteration) on a closed reflective cube
// with A + B -> C, and checks conservation and confinement. Exit code 0 = pass.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "mcell_gb300_event.hpp"

int main() {
  mcg_config cfg{};
  cfg.precision = MCG_PRECISION_FP64;
  cfg.partition_origin[0] = cfg.partition_origin[1] = cfg.partition_origin[2] = -60.0;
  cfg.partition_edge = 120.0;
  cfg.subparts_per_edge = 12;
  cfg.rxn_radius = 0.5641895835477563;
  cfg.seed = 3;
  cfg.n_species = 3;
  try {
    mcg::GpuDiffuseReactEvent ev(cfg);
    ev.set_species({2.0, 2.0, 1.4142135623730951});
    // the Model API's create_box(edge_dimension=1 um) in internal units
    const double h = 50.0;
    std::vector<double> v = {-h, -h, -h, -h, -h, h, -h, h, -h, -h, h, h, h, -h, -h, h, -h, h, h, h, -h, h, h, h};
    std::vector<uint32_t> w = {1, 2, 0, 3, 6, 2, 7, 4, 6, 5, 0, 4, 6, 0, 2, 3, 5, 7,
                               1, 3, 2, 3, 7, 6, 7, 5, 4, 5, 1, 0, 6, 4, 0, 3, 1, 5};
    ev.upload_mesh(v, w, std::vector<uint8_t>(12 * 3, 0));
    ev.add_bimol_rxn(0, 1, 0.0368, 2);
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> U(-h, h);
    const int n = 10000;
    std::vector<double> pos(3 * n);
    std::vector<uint32_t> sp(n);
    for (int i = 0; i < n; i++) {
      for (int k = 0; k < 3; k++) pos[3 * i + k] = U(rng);
      sp[i] = i % 2;
    }
    ev.release(pos, sp);
    // scheduler loop: a count barrier at every iteration
    for (int it = 0; it < 100; it++) {
      ev.set_barrier_time_for_next_execution(1.0);
      ev.step();
      ev.update_event_time_for_next_scheduled_time();
      std::vector<uint64_t> c = ev.counts(3);
      if (c[0] + c[2] != (uint64_t)n / 2 || c[1] + c[2] != (uint64_t)n / 2) {
        std::printf("mass balance broken at iteration %d: %llu %llu %llu\n", it, (unsigned long long)c[0],
                    (unsigned long long)c[1], (unsigned long long)c[2]);
        return 1;
      }
    }
    // a count buffer that takes a ticket at each barrier and reads it one barrier later
    uint64_t prev = 0;
    for (int it = 0; it < 20; it++) {
      ev.set_barrier_time_for_next_execution(1.0);
      ev.step();
      ev.update_event_time_for_next_scheduled_time();
      const uint64_t t = ev.request_counts();
      if (prev) {
        std::vector<uint64_t> c = ev.wait_counts(prev, 3);
        if (c[0] + c[2] != (uint64_t)n / 2 || c[1] + c[2] != (uint64_t)n / 2) {
          std::printf("mass balance broken in the counts read late at iteration %d\n", it);
          return 1;
        }
      }
      prev = t;
    }
    if (ev.wait_counts(prev, 3) != ev.counts(3)) {
      std::printf("the last ticket's counts differ from the counts now\n");
      return 1;
    }
    std::vector<double> p;
    std::vector<uint32_t> s;
    std::vector<uint64_t> ids;
    ev.molecules(p, s, ids);
    for (double x : p)
      if (std::fabs(x) > h) {
        std::printf("molecule outside the box\n");
        return 1;
      }
    std::vector<uint64_t> c = ev.counts(3);
    std::printf("event driver ok: t=%.0f A=%llu B=%llu C=%llu\n", ev.event_time, (unsigned long long)c[0],
                (unsigned long long)c[1], (unsigned long long)c[2]);
    return c[2] > 0 ? 0 : 1;
  } catch (const std::exception& ex) {
    std::printf("error: %s\n", ex.what());
    return 1;
  }
}
