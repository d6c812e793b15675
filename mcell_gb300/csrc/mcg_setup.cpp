// Host-side setup of the engine (runs once per model, not on the step path):
// subpartition grid, wall constants and the wall lists per subpartition.
//
//   SimulationConfig::init_subpartition_edge_length  src4/simulation_config.cpp:45-70
//   Partition ctor (origin, opposite corner)          src4/partition.cpp:36-60
//   Wall::initialize_wall_constants                   src4/wall.cpp:281-342
//   get_wall_bounding_box / wall_subparts_collision_test  src4/geometry_utils.inl:66-200
//   wall_in_box                                       src4/wall_utils.inl:326-516
//   Partition::finalize_walls                         src4/partition.cpp:91-116
// Computed in fp64 with the reference's operation order (this file is built
// with -ffp-contract=off) so that the device's wall data and wall lists are the
// ones the reference would build.
#include "mcg_setup.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

namespace mcg {

namespace {

struct D3 {
  double x, y, z;
};
inline D3 d3(double x, double y, double z) { return D3{x, y, z}; }
inline D3 operator+(D3 a, D3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline D3 operator-(D3 a, D3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline D3 mulc(D3 a, D3 b) { return d3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline double dotp(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 crossp(D3 a, D3 b) { return d3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }

inline bool distinguishable_d(double a, double b, double eps) {
  double c = std::fabs(a - b);
  a = std::fabs(a);
  if (a < 1) a = 1;
  b = std::fabs(b);
  if (b < a)
    eps *= a;
  else
    eps *= b;
  return c > eps;
}

struct Grid {
  D3 origin;
  double sp_edge, sp_rcp, part_edge, R;
  int nsub;
  void idx3(D3 p, int& x, int& y, int& z) const {
    D3 r = p - origin;
    x = (int)(r.x * sp_rcp);
    y = (int)(r.y * sp_rcp);
    z = (int)(r.z * sp_rcp);
  }
};

// one face of the box: the triangle edge v1->v2 crosses the plane axis=c inside the face
inline bool edge_face(double v1a, double v2a, double c, double v1b, double v2b, double v1d, double v2d, double lob,
                      double hib, double lod, double hid) {
  if ((v1a <= c && c < v2a) || (v1a > c && c >= v2a)) {
    double r = (c - v1a) / (v2a - v1a);
    double a3 = v1b + r * (v2b - v1b);
    double a4 = v1d + r * (v2d - v1d);
    if (lob <= a3 && a3 <= hib && lod <= a4 && a4 <= hid) return true;
  }
  return false;
}

inline bool point_in_box(D3 p, D3 l, D3 u) {
  return p.x >= l.x && p.x <= u.x && p.y >= l.y && p.y <= u.y && p.z >= l.z && p.z <= u.z;
}

// does triangle (vert, normal n, plane offset d) intersect the box [l, u]?
bool wall_in_box(const D3* vert, D3 n, double d, D3 l, D3 u) {
  for (int i = 0; i < 3; i++)
    if (point_in_box(vert[i], l, u)) return true;
  for (int i = 0; i < 3; i++) {
    const D3& b = vert[i];
    const D3& a = (i == 0) ? vert[2] : vert[i - 1];
    if (edge_face(a.x, b.x, l.x, a.y, b.y, a.z, b.z, l.y, u.y, l.z, u.z)) return true;
    if (edge_face(a.x, b.x, u.x, a.y, b.y, a.z, b.z, l.y, u.y, l.z, u.z)) return true;
    if (edge_face(a.y, b.y, l.y, a.x, b.x, a.z, b.z, l.x, u.x, l.z, u.z)) return true;
    if (edge_face(a.y, b.y, u.y, a.x, b.x, a.z, b.z, l.x, u.x, l.z, u.z)) return true;
    if (edge_face(a.z, b.z, l.z, a.y, b.y, a.x, b.x, l.y, u.y, l.x, u.x)) return true;
    if (edge_face(a.z, b.z, u.z, a.y, b.y, a.x, b.x, l.y, u.y, l.x, u.x)) return true;
  }
  // box edges against the triangle. The 12 edges of the box are walked as a path
  // through its 8 corners (7 edges) plus the 5 remaining edges; corner bits give
  // which of l/u each coordinate takes.
  static const int c1x[12] = {0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 0, 1};
  static const int c1y[12] = {0, 0, 1, 1, 1, 1, 0, 0, 0, 0, 1, 0};
  static const int c1z[12] = {0, 1, 1, 0, 0, 1, 1, 0, 0, 1, 1, 0};
  static const int c2x[12] = {0, 0, 0, 1, 1, 1, 1, 0, 0, 1, 1, 0};
  static const int c2y[12] = {0, 1, 1, 1, 1, 0, 0, 0, 1, 0, 1, 1};
  static const int c2z[12] = {1, 1, 0, 0, 1, 1, 0, 0, 0, 1, 1, 0};
  static const int e1[12] = {0, 1, 3, 2, 6, 7, 5, 4, 0, 1, 3, 4};
  static const int e2[12] = {1, 3, 2, 6, 7, 5, 4, 0, 2, 5, 7, 2};
  D3 uu = vert[1] - vert[0];
  double ru = 1 / std::sqrt(uu.x * uu.x + uu.y * uu.y + uu.z * uu.z);
  uu = mulc(uu, d3(ru, ru, ru));
  D3 vv = crossp(n, uu);
  double vu[3], vvv[3];
  for (int j = 0; j < 3; j++) {
    vu[j] = dotp(vert[j], uu);
    vvv[j] = dotp(vert[j], vv);
  }
  D3 bb = l, ba = l;
  double dbox[8];
  dbox[0] = dotp(bb, n);
  for (int i = 0; i < 12; i++) {
    double a1, a2;
    if (i < 7) {
      ba = bb;
      bb = d3(c2x[i] ? u.x : l.x, c2y[i] ? u.y : l.y, c2z[i] ? u.z : l.z);
      a2 = dbox[e2[i]] = dotp(bb, n);
      a1 = dbox[e1[i]];
      if ((a1 - d < 0 && a2 - d < 0) || (a1 - d > 0 && a2 - d > 0)) continue;
    } else {
      a1 = dbox[e1[i]];
      a2 = dbox[e2[i]];
      if ((a1 - d < 0 && a2 - d < 0) || (a1 - d > 0 && a2 - d > 0)) continue;
      ba = d3(c1x[i] ? u.x : l.x, c1y[i] ? u.y : l.y, c1z[i] ? u.z : l.z);
      bb = d3(c2x[i] ? u.x : l.x, c2y[i] ? u.y : l.y, c2z[i] ? u.z : l.z);
    }
    double r = (d - a1) / (a2 - a1);
    D3 c = ba + mulc(d3(r, r, r), bb - ba);
    double cu = dotp(c, uu), cv = dotp(c, vv);
    int crossings = 0;
    for (int j = 0; j < 3; j++) {
      int k = (j == 0) ? 2 : j - 1;
      if ((vu[k] < cu && cu <= vu[j]) || (vu[k] >= cu && cu > vu[j])) {
        double rr = (cu - vu[k]) / (vu[j] - vu[k]);
        if ((vvv[k] + rr * (vvv[j] - vvv[k])) > cv) crossings++;
      }
    }
    if (crossings & 1) return true;
  }
  return false;
}

}  // namespace

int compute_setup(const double* origin, double partition_edge, uint32_t nsub, double rxn_radius, uint32_t nv,
                  const double* verts, uint32_t nw, const uint32_t* tris, HostSetup& hs, std::string& err) {
  if (nsub == 0 || nsub > 300 || !(partition_edge > 0)) {
    err = "subparts_per_edge must be in 1..300 and partition_edge > 0";
    return -1;
  }
  // the neighbour collection reaches one subpartition across a face, edge or corner,
  // so R * sqrt(2) must stay below half an edge (mcell4_converter.cpp:121-127)
  if (!(rxn_radius * 1.41421356238 < partition_edge / (double)nsub / 2.0)) {
    err = "reaction radius times sqrt(2) must be less than half of the subpartition edge";
    return -1;
  }
  hs.nsub = nsub;
  hs.sp_edge = partition_edge / (double)nsub;
  hs.sp_rcp = 1.0 / hs.sp_edge;
  hs.part_edge = hs.sp_edge * nsub;
  for (int k = 0; k < 3; k++) {
    hs.origin[k] = origin[k];
    hs.opposite[k] = origin[k] + hs.part_edge;
  }
  hs.R = rxn_radius;
  hs.nw = nw;
  hs.wall.assign((size_t)nw * 24, 0.0);
  std::vector<D3> V(nv);
  for (uint32_t i = 0; i < nv; i++) V[i] = d3(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
  for (uint32_t w = 0; w < nw; w++) {
    for (int k = 0; k < 3; k++) {
      if (tris[3 * w + k] >= nv) {
        err = "wall vertex index out of range";
        return -1;
      }
    }
  }
  Grid g{d3(origin[0], origin[1], origin[2]), hs.sp_edge, hs.sp_rcp, hs.part_edge, rxn_radius, (int)nsub};
  // incidences (subpartition, wall, cell mask) in wall order; bucketed by subpartition
  // below (a stable counting sort keeps each list in ascending wall order)
  std::vector<uint32_t> inc_sp, inc_w;
  std::vector<uint64_t> inc_mask;
  for (uint32_t w = 0; w < nw; w++) {
    D3 v0 = V[tris[3 * w]], v1 = V[tris[3 * w + 1]], v2 = V[tris[3 * w + 2]];
    double* o = &hs.wall[(size_t)w * 24];
    // Wall::initialize_wall_constants
    D3 vX = crossp(v1 - v0, v2 - v0);
    double area = 0.5 * std::sqrt(vX.x * vX.x + vX.y * vX.y + vX.z * vX.z);
    D3 n = d3(0, 0, 0), uu = d3(0, 0, 0), vv = d3(0, 0, 0);
    double dist = 0, uv1u = 0, uv2u = 0, uv2v = 0;
    if (distinguishable_d(area, 0, 1e-12)) {
      D3 f1 = v1 - v0;
      double inv_f1 = 1 / std::sqrt(f1.x * f1.x + f1.y * f1.y + f1.z * f1.z);
      uu = mulc(f1, d3(inv_f1, inv_f1, inv_f1));
      D3 f2 = v2 - v0;
      D3 nn = crossp(uu, f2);
      double inv_n = 1 / std::sqrt(nn.x * nn.x + nn.y * nn.y + nn.z * nn.z);
      n = mulc(nn, d3(inv_n, inv_n, inv_n));
      vv = crossp(n, uu);
      dist = dotp(v0, n);
      uv1u = dotp(f1, uu);
      uv2u = dotp(f2, uu);
      uv2v = dotp(f2, vv);
    }
    const double vals[24] = {n.x,  n.y,  n.z,  dist, uu.x, uu.y, uu.z, vv.x, vv.y, vv.z, uv1u, uv2u,
                             uv2v, v0.x, v0.y, v0.z, v1.x, v1.y, v1.z, v2.x, v2.y, v2.z, 0,    0};
    std::memcpy(o, vals, sizeof(vals));
    // wall_subparts_collision_test
    D3 vert[3] = {v0, v1, v2};
    D3 llf, urb;
    llf = urb = v0;
    if (v1.x < llf.x) llf.x = v1.x; else if (v1.x > urb.x) urb.x = v1.x;
    if (v2.x < llf.x) llf.x = v2.x; else if (v2.x > urb.x) urb.x = v2.x;
    if (v1.y < llf.y) llf.y = v1.y; else if (v1.y > urb.y) urb.y = v1.y;
    if (v2.y < llf.y) llf.y = v2.y; else if (v2.y > urb.y) urb.y = v2.y;
    if (v1.z < llf.z) llf.z = v1.z; else if (v1.z > urb.z) urb.z = v1.z;
    if (v2.z < llf.z) llf.z = v2.z; else if (v2.z > urb.z) urb.z = v2.z;
    double leeway = 1;
    if (llf.x < -leeway) leeway = -llf.x;
    if (llf.y < -leeway) leeway = -llf.y;
    if (llf.z < -leeway) leeway = -llf.z;
    if (urb.x > leeway) leeway = urb.x;
    if (urb.y > leeway) leeway = urb.y;
    if (urb.z > leeway) leeway = urb.z;
    leeway = 1e-12 + leeway * 1e-12;
    leeway += rxn_radius;
    D3 l3 = d3(leeway, leeway, leeway);
    llf = llf - l3;
    urb = urb + l3;
    int x0, y0, z0, x1, y1, z1;
    g.idx3(llf, x0, y0, z0);
    g.idx3(urb, x1, y1, z1);
    auto clampi = [&](int v) { return v < 0 ? 0 : (v >= (int)nsub ? (int)nsub - 1 : v); };
    x0 = clampi(x0); y0 = clampi(y0); z0 = clampi(z0);
    x1 = clampi(x1); y1 = clampi(y1); z1 = clampi(z1);
    D3 e3 = d3(hs.sp_edge, hs.sp_edge, hs.sp_edge);
    for (int x = x0; x <= x1; x++)
      for (int y = y0; y <= y1; y++)
        for (int z = z0; z <= z1; z++) {
          D3 sl = g.origin + mulc(d3(x, y, z), e3);
          D3 su = sl + e3;
          if (wall_in_box(vert, n, dist, sl - l3, su + l3)) {
            const size_t s = (size_t)x + (size_t)y * nsub + (size_t)z * nsub * nsub;
            inc_sp.push_back((uint32_t)s);
            inc_w.push_back(w);
            // cells of the subpartition's 4x4x4 grid the wall reaches (same leeway); only
            // the cells the wall's grown box overlaps are tested
            const double q = 0.25 * hs.sp_edge;
            int c0[3], c1[3];
            const double lo_[3] = {llf.x, llf.y, llf.z}, hi_[3] = {urb.x, urb.y, urb.z};
            const double sl_[3] = {sl.x, sl.y, sl.z};
            for (int a = 0; a < 3; a++) {
              c0[a] = std::max(0, std::min(3, (int)std::floor((lo_[a] - sl_[a]) / q)));  // llf, urb are grown
              c1[a] = std::max(0, std::min(3, (int)std::floor((hi_[a] - sl_[a]) / q)));
            }
            // a box of at most 8 cells is taken whole (a superset; small walls), larger
            // ones cell by cell
            const bool exact = (c1[0] - c0[0] + 1) * (c1[1] - c0[1] + 1) * (c1[2] - c0[2] + 1) > 8;
            uint64_t mask = 0;
            for (int cz = c0[2]; cz <= c1[2]; cz++)
              for (int cy = c0[1]; cy <= c1[1]; cy++)
                for (int cx = c0[0]; cx <= c1[0]; cx++) {
                  D3 ol = sl + d3(cx * q, cy * q, cz * q);
                  D3 ou = ol + d3(q, q, q);
                  if (!exact || wall_in_box(vert, n, dist, ol - l3, ou + l3)) mask |= 1ull << (cx + 4 * cy + 16 * cz);
                }
            inc_mask.push_back(mask ? mask : ~0ull);
          }
        }
  }
  const size_t n3 = (size_t)nsub * nsub * nsub;
  hs.wsp_off.assign(n3 + 1, 0);
  for (uint32_t sp : inc_sp) hs.wsp_off[sp + 1]++;
  for (size_t s = 0; s < n3; s++) hs.wsp_off[s + 1] += hs.wsp_off[s];
  hs.wsp_list.resize(inc_sp.size());
  hs.wsp_cells.resize(inc_sp.size());
  std::vector<uint32_t> fill(hs.wsp_off.begin(), hs.wsp_off.end() - 1);
  for (size_t k = 0; k < inc_sp.size(); k++) {
    const uint32_t at = fill[inc_sp[k]]++;
    hs.wsp_list[at] = inc_w[k];
    hs.wsp_cells[at] = inc_mask[k];
  }
  if (nw >= (1u << 24)) {
    err = "more than 16,777,215 walls";
    return -1;
  }
  return 0;
}

}  // namespace mcg
