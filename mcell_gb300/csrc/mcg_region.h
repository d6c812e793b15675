// Host helpers of the region releases (mcg_region.cpp): closed-object volumes and
// boxes, region-expression boxes, concentration counts and the vacuum's choice.
#pragma once

#include <cstdint>
#include <functional>
#include <vector>

namespace mcg {

// tokens of a region expression's postfix program
constexpr uint32_t MAX_REGION_EXPR = 15;

struct MeshView {
  uint32_t n_verts;
  const double* verts;  // [n_verts][3]
  uint32_t n_walls;
  const uint32_t* walls;  // [n_walls][3] vertex indices
  const uint16_t* object_of_wall;
};

// bounding box of each object's walls (an object without walls gets llf.x > urb.x)
bool object_boxes(const MeshView& m, std::vector<double>& llf, std::vector<double>& urb);
bool object_volume(const MeshView& m, uint32_t obj, double* volume);
// a postfix program of objects (< n_objects) and MCG_REGION_* operators with one result
bool region_expr_valid(const int32_t* expr, uint32_t n, uint32_t n_objects);
void region_expr_bbox(const int32_t* expr, uint32_t n, const double* obj_llf, const double* obj_urb, double* llf,
                      double* urb);
// molecules for a molar concentration in a volume (internal units), before truncation
double concentration_number(double concentration, double volume, double length_unit);
double sphere_volume(const double* diameter);
// the vacuum's choice of n_remove of m candidates in order; returns how many it removed
int select_for_removal(uint32_t m, uint32_t n_remove, const std::function<double()>& draw, uint8_t* removed);

}  // namespace mcg
