// Host side of releases into regions and by concentration, and of vacuum releases:
// volumes of closed objects, bounding boxes of region expressions, the number of
// molecules a concentration gives, and the random choice of the molecules a vacuum
// removes. Compiled with -ffp-contract=off: the arithmetic is the reference's, in its
// order, so the numbers are the reference's bit for bit.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/mcell_gb300.h"
#include "mcg_region.h"

namespace mcg {

namespace {
constexpr double kAvogadro = 6.0221417930e23;  // N_AV (src/mcell_structs_shared.h:19)
constexpr double kPi = 3.14159265358979323846;   // MY_PI (src/mcell_structs_shared.h:18)

// tetrahedral_volume (src4/geometry.cpp:835-846): signed volume of the tetrahedron
// a, b, c, d, the reference's terms in its order
double tetrahedral_volume(const double* a, const double* b, const double* c, const double* d) {
  return (double)1 / (double)6 *
         (-1 * (a[2] - d[2]) * (b[1] - d[1]) * (c[0] - d[0]) + (a[1] - d[1]) * (b[2] - d[2]) * (c[0] - d[0]) +
          (a[2] - d[2]) * (b[0] - d[0]) * (c[1] - d[1]) - (a[0] - d[0]) * (b[2] - d[2]) * (c[1] - d[1]) -
          (a[1] - d[1]) * (b[0] - d[0]) * (c[2] - d[2]) + (a[0] - d[0]) * (b[1] - d[1]) * (c[2] - d[2]));
}
}  // namespace

bool object_boxes(const MeshView& m, std::vector<double>& llf, std::vector<double>& urb) {
  uint32_t nobj = 0;
  for (uint32_t w = 0; w < m.n_walls; w++) nobj = std::max<uint32_t>(nobj, (uint32_t)m.object_of_wall[w] + 1);
  llf.assign(3 * (size_t)nobj, 0);
  urb.assign(3 * (size_t)nobj, 0);
  std::vector<char> seen(nobj, 0);
  // Region::compute_bounding_box (src4/wall.cpp:416-460): from the first vertex of the
  // first wall, widened by every vertex
  for (uint32_t w = 0; w < m.n_walls; w++) {
    const uint32_t o = m.object_of_wall[w];
    for (int k = 0; k < 3; k++) {
      const uint32_t vi = m.walls[3 * (size_t)w + k];
      if (vi >= m.n_verts) return false;
      const double* v = m.verts + 3 * (size_t)vi;
      if (!seen[o]) {
        for (int a = 0; a < 3; a++) llf[3 * o + a] = urb[3 * o + a] = v[a];
        seen[o] = 1;
      }
      for (int a = 0; a < 3; a++) {
        if (llf[3 * o + a] > v[a])
          llf[3 * o + a] = v[a];
        else if (urb[3 * o + a] < v[a])
          urb[3 * o + a] = v[a];
      }
    }
  }
  for (uint32_t o = 0; o < nobj; o++)
    if (!seen[o]) llf[3 * o] = 1, urb[3 * o] = 0;  // no walls: an empty box
  return true;
}

bool object_volume(const MeshView& m, uint32_t obj, double* volume) {
  std::vector<double> llf, urb;
  if (!object_boxes(m, llf, urb) || obj >= llf.size() / 3 || llf[3 * obj] > urb[3 * obj]) return false;
  // Region::initialize_volume_info_if_needed (src4/geometry.cpp:860-897): the region's
  // walls in index order, each face's tetrahedron with the center of the bounding box
  double d[3];
  for (int a = 0; a < 3; a++) d[a] = (llf[3 * obj + a] + urb[3 * obj + a]) * 0.5;
  double v = 0;
  for (uint32_t w = 0; w < m.n_walls; w++) {
    if (m.object_of_wall[w] != obj) continue;
    const uint32_t* t = m.walls + 3 * (size_t)w;
    v += tetrahedral_volume(m.verts + 3 * (size_t)t[0], m.verts + 3 * (size_t)t[1], m.verts + 3 * (size_t)t[2], d);
  }
  *volume = v;
  return true;
}

bool region_expr_valid(const int32_t* expr, uint32_t n, uint32_t n_objects) {
  if (!expr || n == 0 || n > MAX_REGION_EXPR) return false;
  int depth = 0;
  for (uint32_t k = 0; k < n; k++) {
    if (expr[k] >= 0) {
      if ((uint32_t)expr[k] >= n_objects) return false;
      depth++;
    } else {
      if (expr[k] < MCG_REGION_DIFFERENCE || depth < 2) return false;
      depth--;
    }
  }
  return depth == 1;
}

void region_expr_bbox(const int32_t* expr, uint32_t n, const double* obj_llf, const double* obj_urb, double* llf,
                      double* urb) {
  // compute_region_expr_bounding_box (src4/geometry.cpp:1180-1265) over the postfix
  // program: union widens, intersection narrows, difference keeps the left box
  std::vector<double> st;
  for (uint32_t k = 0; k < n; k++) {
    if (expr[k] >= 0) {
      for (int a = 0; a < 3; a++) st.push_back(obj_llf[3 * expr[k] + a]);
      for (int a = 0; a < 3; a++) st.push_back(obj_urb[3 * expr[k] + a]);
      continue;
    }
    double r[6], l[6];
    for (int q = 5; q >= 0; q--) r[q] = st.back(), st.pop_back();
    for (int q = 5; q >= 0; q--) l[q] = st.back(), st.pop_back();
    if (expr[k] == MCG_REGION_UNION) {
      for (int a = 0; a < 3; a++) {
        if (l[a] > r[a]) l[a] = r[a];
        if (l[3 + a] < r[3 + a]) l[3 + a] = r[3 + a];
      }
    } else if (expr[k] == MCG_REGION_INTERSECT) {
      for (int a = 0; a < 3; a++) {
        if (l[a] < r[a]) l[a] = r[a];
        if (l[3 + a] > r[3 + a]) l[3 + a] = r[3 + a];
      }
    }
    for (int q = 0; q < 6; q++) st.push_back(l[q]);
  }
  for (int a = 0; a < 3; a++) {
    llf[a] = st[a];
    urb[a] = st[3 + a];
  }
}

double concentration_number(double concentration, double volume, double length_unit) {
  // num_vol_mols_from_conc (src4/release_event.cpp:826-856) and
  // calculate_number_to_release (:509-553): molar concentration times the volume in
  // litres, rounded to the nearest count
  return kAvogadro * 1e-15 * concentration * volume * std::pow(length_unit, 3.0) + 0.5;
}

double sphere_volume(const double* diameter) {
  // calculate_number_to_release, SPHERICAL (src4/release_event.cpp:523-526)
  return (1.0 / 6.0) * kPi * diameter[0] * diameter[1] * diameter[2];
}

int select_for_removal(uint32_t m, uint32_t n_remove, const std::function<double()>& draw, uint8_t* removed) {
  // randomly_remove_molecules (src4/release_event.cpp:578-597): each candidate in turn
  // goes with the probability of the removals still to make over the candidates left
  int k = (int)n_remove, done = 0;
  for (uint32_t i = 0; i < m; i++) {
    const int remaining = (int)(m - i);
    removed[i] = 0;
    if (draw() < ((double)(k)) / ((double)remaining)) {
      removed[i] = 1;
      done++;
      k--;
    }
  }
  return done;
}

}  // namespace mcg

extern "C" {

int mcg_object_volume(uint32_t n_verts, const double* verts, uint32_t n_walls, const uint32_t* walls,
                      const uint16_t* object_of_wall, uint32_t object, double* volume) {
  if (!verts || !walls || !object_of_wall || !volume || n_walls == 0) return MCG_ERR_ARG;
  const mcg::MeshView m{n_verts, verts, n_walls, walls, object_of_wall};
  return mcg::object_volume(m, object, volume) ? MCG_OK : MCG_ERR_ARG;
}

int mcg_region_expr_bbox(uint32_t n_verts, const double* verts, uint32_t n_walls, const uint32_t* walls,
                         const uint16_t* object_of_wall, const int32_t* expr, uint32_t n_expr, double* llf,
                         double* urb) {
  if (!verts || !walls || !object_of_wall || !llf || !urb || n_walls == 0) return MCG_ERR_ARG;
  const mcg::MeshView m{n_verts, verts, n_walls, walls, object_of_wall};
  std::vector<double> ol, ou;
  if (!mcg::object_boxes(m, ol, ou) || !mcg::region_expr_valid(expr, n_expr, (uint32_t)(ol.size() / 3)))
    return MCG_ERR_ARG;
  mcg::region_expr_bbox(expr, n_expr, ol.data(), ou.data(), llf, urb);
  return MCG_OK;
}

int mcg_release_number_from_concentration(const double* diameter, double concentration_molar, double length_unit_um,
                                          uint64_t* n) {
  if (!diameter || !n || !(concentration_molar >= 0) || !(length_unit_um > 0)) return MCG_ERR_ARG;
  const double num =
      mcg::concentration_number(concentration_molar, mcg::sphere_volume(diameter), length_unit_um);
  if (!(num >= 0) || num > 2147483647.0) return MCG_ERR_ARG;  // check_max_release_count (:497-506)
  *n = (uint64_t)(uint32_t)num;
  return MCG_OK;
}

int mcg_vacuum_select(uint32_t m, uint32_t n_remove, const uint32_t* draws, uint32_t n_draws, uint8_t* removed,
                      uint32_t* draws_used) {
  if ((m && (!draws || !removed)) || !draws_used) return MCG_ERR_ARG;
  uint32_t used = 0;
  bool over = false;
  mcg::select_for_removal(m, n_remove, [&]() {
    if (used >= n_draws) {
      over = true;
      return 0.0;
    }
    return (double)draws[used++] * (1.0 / 4294967296.0);
  }, removed);
  *draws_used = over ? 0xFFFFFFFFu : used;
  return MCG_OK;
}

}  // extern "C"
