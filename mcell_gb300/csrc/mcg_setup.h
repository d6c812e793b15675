// Host-side model setup shared by both precisions (see mcg_setup.cpp).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace mcg {

struct HostSetup {
  double origin[3], opposite[3];
  double part_edge, sp_edge, sp_rcp, R;
  uint32_t nsub, nw;
  // per wall, 24 doubles: normal xyz, d, unit_u xyz, unit_v xyz, uv_vert1_u, uv_vert2 u v,
  // v0 xyz, v1 xyz, v2 xyz, 2 spare
  std::vector<double> wall;
  std::vector<uint32_t> wsp_off, wsp_list;  // walls per subpartition, ascending
  // per list entry: cells of the subpartition's 4x4x4 grid (bit x + 4y + 16z quarters)
  // whose box, grown by the same leeway as the subpartition's, the wall intersects
  std::vector<uint64_t> wsp_cells;
};

int compute_setup(const double* origin, double partition_edge, uint32_t nsub, double rxn_radius, uint32_t nv,
                  const double* verts, uint32_t nw, const uint32_t* tris, HostSetup& hs, std::string& err);

}  // namespace mcg
