/*
 * Minimal project-written stand-ins for the MCell4 classes that the reference's
 * hot-path routines touch (Partition, Molecule, Wall, Collision, RxnClass,
 * SimulationConfig, SimulationStats). The reference's own headers for these
 * classes pull in libbng, boost, sparsehash and the whole World, none of which
 * exist here, so the routines are compiled against these classes instead.
 *
 * Member names and signatures are the ones the routines call (they must match
 * for the routines to compile unchanged):
 *   Partition          src4/partition.h:198 (accessors :248-298, :641, :889)
 *   Molecule           src4/molecule.h:52
 *   Wall / rejection   src4/wall.h:200-350
 *   Collision          src4/collision_structs.h:29-140
 *   SimulationConfig   src4/simulation_config.h:28-135
 *   CountedVolume, GeometryObject, Region   src4/geometry.h:39-320
 * The bodies are this project's own. Test infrastructure only: this header is
 * compiled into oracle/_ref and is never part of the product.
 */
#ifndef ORACLE_REF_SHIM_H
#define ORACLE_REF_SHIM_H

#include <map>
#include <set>
#include <vector>
#include <cstring>
#include <cstdint>

#include "defines.h"

// ---- injected random numbers (replaces the single ISAAC64 stream) ----
struct ShimRng {
  const uint32_t* draws = nullptr;
  size_t n = 0;
  size_t used = 0;
  bool overrun = false;
  unsigned int next_uint() {
    if (used >= n) {
      overrun = true;
      return 0;
    }
    return draws[used++];
  }
  double next_dbl() {
    // rng_dbl is a 32-bit draw scaled by 2^-32 (src/isaac64.h isaac64_dbl32)
    return (double)next_uint() * (1.0 / 4294967296.0);
  }
};
#undef rng_state
#undef rng_uint
#undef rng_dbl
#define rng_state ShimRng
#define rng_uint(x) ((x)->next_uint())
#define rng_dbl(x) ((x)->next_dbl())

namespace BNG {

const int PATHWAY_INDEX_NO_RXN = -2;
const int PATHWAY_INDEX_LEAST_VALID = 0;
typedef int rxn_class_pathway_index_t;
const species_id_t SPECIES_FLAG_CAN_VOLWALL = 1u << 4;

enum class RxnType { Invalid, Standard, Transparent, Reflect, AbsorbRegionBorder };

// reaction class for one reactant pair: max_fixed_p and cumulative pathway probabilities
class RxnClass {
public:
  RxnType type = RxnType::Standard;
  std::vector<double> cum_probs;
  size_t get_num_reactions() const { return cum_probs.size(); }
  double get_max_fixed_p() const { return cum_probs.empty() ? 0.0 : cum_probs.back(); }
  void update_rxn_rates_if_needed(const double) { }
  double get_next_time_of_rxn_rate_update() const { return 1e20; }
  bool is_transparent_type() const { return type == RxnType::Transparent; }
  // pathway lookup; MCell3 uses binary_search_double over cum_probs (src/react_cond.c)
  int get_pathway_index_for_probability(const double prob, const double local_prob_factor) const;
};

typedef std::vector<RxnClass*> RxnClassesVector;

class Species {
public:
  uint flags = 0;
  double space_step = 0;
  double time_step = 1;
  bool has_flag(uint f) const { return (flags & f) != 0; }
  bool can_diffuse() const { return space_step != 0; }
};

} // namespace BNG

namespace MCell {

using std::map;  // the reference's headers bring std names into MCell

const uint MOLECULE_FLAG_DEFUNCT = 1u << 31;
const uint MOLECULE_FLAG_VOL = 1u << 1;
const uint MOLECULE_FLAG_SCHEDULE_UNIMOL_RXN = 1u << 8;

class Molecule {
public:
  Molecule() = default;
  Molecule(const molecule_id_t id_, const species_id_t species_id_, const Vec3& pos_, const double time_)
    : id(id_), species_id(species_id_), birthday(time_) {
    v.pos = pos_;
  }
  molecule_id_t id = MOLECULE_ID_INVALID;
  species_id_t species_id = BNG::SPECIES_ID_INVALID;
  uint flags = 0;
  double birthday = 0;
  struct {
    Vec3 pos;
    subpart_index_t subpart_index = SUBPART_INDEX_INVALID;
  } v;
  void set_flag(const uint f) { flags |= f; }
  bool is_defunct() const { return (flags & MOLECULE_FLAG_DEFUNCT) != 0; }
  bool is_vol() const { return true; }
  bool is_surf() const { return false; }
};

class WallCollisionRejectionData {
public:
  Vec3 normal;
  pos_t distance_to_origin = 0;
};

class Partition;

class Wall: public WallCollisionRejectionData {
public:
  wall_index_t index = WALL_INDEX_INVALID;
  wall_id_t id = 0;
  vertex_index_t vertex_indices[3];
  pos_t area = 0;
  bool wall_constants_initialized = false;
  pos_t uv_vert1_u = 0;
  Vec2 uv_vert2;
  Vec3 unit_u, unit_v;
  uint surf_class_of_species_mask = 0; // unused by the routines
  geometry_object_index_t object_index = 0;
  geometry_object_id_t object_id = 0;
  bool exists_in_partition() const { return id != WALL_ID_NOT_IN_PARTITION; }
  bool is_overlapped_wall() const { return false; }
  void initialize_wall_constants(const Partition& p);
};

class WallWithVertices: public Wall {
public:
  Vec3 vertices[3];
};

typedef uint_set<wall_index_t> WallsInSubpart;

enum class CollisionType {
  INVALID, WALL_REDO, WALL_MISS, WALL_FRONT, WALL_BACK,
  VOLMOL_VOLMOL, SURFMOL_SURFMOL, VOLMOL_SURFMOL, UNIMOLECULAR, INTERMEMBRANE_SURFMOL_SURFMOL
};

enum class RayTraceState { UNDEFINED, HIT_SUBPARTITION, RAY_TRACE_HIT_WALL, FINISHED };

class Collision {
public:
  Collision() : type(CollisionType::INVALID), partition(nullptr), diffused_molecule_id(0),
      time(0), pos(0), colliding_molecule_id(0), rxn_class(nullptr), colliding_wall_index(0) { }
  Collision(const CollisionType type_, Partition* p_, const molecule_id_t dm, const double time_,
      const Vec3& pos_, const molecule_id_t cm, BNG::RxnClass* rc)
    : type(type_), partition(p_), diffused_molecule_id(dm), time(time_), pos(pos_),
      colliding_molecule_id(cm), rxn_class(rc), colliding_wall_index(WALL_INDEX_INVALID) { }
  Collision(const CollisionType type_, Partition* p_, const molecule_id_t dm, const double time_,
      const Vec3& pos_, const wall_index_t wi)
    : type(type_), partition(p_), diffused_molecule_id(dm), time(time_), pos(pos_),
      colliding_molecule_id(MOLECULE_ID_INVALID), rxn_class(nullptr), colliding_wall_index(wi) { }
  bool is_vol_mol_vol_mol_collision() const { return type == CollisionType::VOLMOL_VOLMOL; }
  bool is_wall_collision() const { return type == CollisionType::WALL_FRONT || type == CollisionType::WALL_BACK; }

  CollisionType type;
  Partition* partition;
  molecule_id_t diffused_molecule_id;
  double time;
  Vec3 pos;
  molecule_id_t colliding_molecule_id;
  BNG::RxnClass* rxn_class;
  wall_index_t colliding_wall_index;
};

typedef std::vector<Collision> CollisionsVector;

class SimulationConfig {
public:
  pos_t partition_edge_length = 0;
  uint num_subparts_per_partition_edge = 0;
  uint num_subparts_per_partition_edge_squared = 0;
  uint num_subparts = 0;
  pos_t subpart_edge_length = 0;
  pos_t subpart_edge_length_rcp = 0;
  pos_t rxn_radius_3d = 0;
  bool use_expanded_list = true;
  double length_unit = 0.01;
  double rcp_length_unit = 100;
  double grid_density = 10000;
  void init_subpartition_edge_length();
};

// the set of geometry objects a position is inside (src4/geometry.h:39)
class CountedVolume {
public:
  counted_volume_index_t index = COUNTED_VOLUME_INDEX_INVALID;
  uint_set<geometry_object_index_t> contained_in_objects;
};

class GeometryObject {
public:
  geometry_object_index_t index = 0;
  geometry_object_id_t id = 0;
  bool counted = false;  // a counted volume (is_counted_volume_or_compartment)
  region_id_t encompassing_region_id = 0;
  bool is_counted_volume_or_compartment() const { return counted; }
};

template<typename T> using small_vector = boost::container::small_vector<T, BASE_CONTAINER_ALLOC>;
typedef std::map<subpart_index_t, small_vector<wall_index_t>> WallsPerSubpartMap;

// a closed region made of the walls of one geometry object (src4/geometry.h:186-320)
class Region {
public:
  std::string name;
  std::map<wall_index_t, std::set<edge_index_t>> walls_and_edges;
  WallsPerSubpartMap walls_per_subpart;
  Vec3 bounding_box_llf, bounding_box_urb;
  pos_t volume = 0;
  bool volume_info_initialized = false;
  bool region_is_manifold = true;
  // the reference's (geometry.cpp:860), compiled from its source
  void initialize_volume_info_if_needed(const Partition& p);
  bool is_manifold() const { return region_is_manifold; }
  pos_t get_volume() const { return volume; }
  // the reference's waypoint test falls back to is_point_inside_region_no_waypoints
  // where its ray meets an edge (geometry.cpp:1048-1090); the stand-in is that test,
  // which decides the same for points that are not on the region's walls
  bool is_point_inside(Partition& p, const Vec3& pos);
  const Vec3& get_bounding_box_llf() const { return bounding_box_llf; }
  const WallsPerSubpartMap& get_walls_per_subpart() const { return walls_per_subpart; }
  void compute_bounding_box(const Partition& p, Vec3& llf, Vec3& urb);
};

class SimulationStats {
public:
  void inc_ray_voxel_tests() const { }
  void inc_ray_polygon_tests() const { }
  void inc_ray_polygon_colls() const { }
  void inc_diffuse_3d_calls() const { }
  void inc_mol_wall_reflections() const { }
  void inc_vol_mol_vol_mol_collisions() const { }
  template<typename A, typename B> void inc_rxn_skipped(const A&, const B*, double) const { }
};

class RxnContainerShim {
public:
  std::map<std::pair<uint, uint>, BNG::RxnClass*> bimol;
  BNG::RxnClass* get_bimol_rxn_class(const species_id_t a, const species_id_t b) const {
    auto it = bimol.find(std::make_pair(a, b));
    return it == bimol.end() ? nullptr : it->second;
  }
};

class SpeciesContainerShim {
public:
  std::vector<BNG::Species> species;
  const BNG::Species& get(const species_id_t id) const { return species[id]; }
};

class Partition {
public:
  SimulationConfig config;
  SimulationStats stats;
  Vec3 origin_corner, opposite_corner;
  std::vector<Vec3> vertices;
  std::vector<Wall> walls;
  std::vector<WallCollisionRejectionData> wall_collision_rejection_data;
  std::vector<WallsInSubpart> walls_per_subpart;
  std::vector<Molecule> molecules;
  // reactants of species s in subpart p: molecules there that have a bimolecular rxn with s
  std::map<std::pair<subpart_index_t, species_id_t>, uint_set<molecule_id_t>> reactants;
  uint_set<molecule_id_t> empty_set;
  RxnContainerShim rxns;
  SpeciesContainerShim all_species;
  // surface class kind per (wall, species): 0 reflect, 1 transparent, 2 absorptive
  std::map<std::pair<wall_index_t, species_id_t>, int> wall_class;
  std::vector<GeometryObject> geometry_objects;
  std::vector<CountedVolume> counted_volumes;
  mutable ShimRng aux_rng;  // no draws: the routines that use it return on a re-try

  const GeometryObject& get_geometry_object(const geometry_object_index_t i) const { return geometry_objects[i]; }
  GeometryObject& get_geometry_object(const geometry_object_index_t i) { return geometry_objects[i]; }
  GeometryObject& get_geometry_object_by_id(const geometry_object_id_t id) { return geometry_objects[id]; }
  std::map<region_id_t, Region> regions_by_id;
  Region& get_region_by_id(const region_id_t id) { return regions_by_id.at(id); }
  std::vector<Molecule>& get_molecules() { return molecules; }
  void set_molecule_as_defunct(Molecule& m) { m.set_flag(MOLECULE_FLAG_DEFUNCT); }
  Molecule& add_volume_molecule(const Molecule& vm, const double) {
    molecules.push_back(vm);
    molecules.back().id = (molecule_id_t)(molecules.size() - 1);
    return molecules.back();
  }
  counted_volume_index_t find_or_add_counted_volume(const CountedVolume& cv) {
    for (size_t k = 0; k < counted_volumes.size(); k++) {
      if (counted_volumes[k].contained_in_objects == cv.contained_in_objects) {
        return (counted_volume_index_t)k;
      }
    }
    counted_volumes.push_back(cv);
    counted_volumes.back().index = (counted_volume_index_t)(counted_volumes.size() - 1);
    return counted_volumes.back().index;
  }

  const Vec3& get_origin_corner() const { return origin_corner; }
  bool in_this_partition(const Vec3& pos) const {
    return pos.x >= origin_corner.x && pos.y >= origin_corner.y && pos.z >= origin_corner.z &&
           pos.x < opposite_corner.x && pos.y < opposite_corner.y && pos.z < opposite_corner.z;
  }
  bool is_subpart_index_in_range(const int index) const {
    return index >= 0 && index < (int)config.num_subparts_per_partition_edge;
  }
  void get_subpart_3d_indices(const Vec3& pos, IVec3& res) const {
    Vec3 rel = pos - origin_corner;
    res = rel * config.subpart_edge_length_rcp;
  }
  subpart_index_t get_subpart_index_from_3d_indices_allow_outside(const IVec3& i) const {
    return i.x + i.y * config.num_subparts_per_partition_edge +
        i.z * config.num_subparts_per_partition_edge_squared;
  }
  subpart_index_t get_subpart_index_from_3d_indices(const IVec3& i) const {
    return get_subpart_index_from_3d_indices_allow_outside(i);
  }
  subpart_index_t get_subpart_index_from_3d_indices(const int x, const int y, const int z) const {
    return get_subpart_index_from_3d_indices(IVec3(x, y, z));
  }
  void get_subpart_3d_indices_from_index(const subpart_index_t index, IVec3& i) const {
    uint32_t n = config.num_subparts_per_partition_edge;
    i.x = index % n;
    i.y = (index / n) % n;
    i.z = (index / config.num_subparts_per_partition_edge_squared) % n;
  }
  subpart_index_t get_subpart_index(const Vec3& pos) const {
    IVec3 i;
    get_subpart_3d_indices(pos, i);
    return get_subpart_index_from_3d_indices(i);
  }
  void get_subpart_llf_point(const subpart_index_t s, Vec3& llf) const {
    IVec3 i;
    get_subpart_3d_indices_from_index(s, i);
    llf = origin_corner + Vec3(i) * Vec3(config.subpart_edge_length);
  }
  void get_subpart_urb_point_from_llf(const Vec3& llf, Vec3& urb) const {
    urb = llf + Vec3(config.subpart_edge_length);
  }
  const Vec3& get_geometry_vertex(const vertex_index_t i) const { return vertices[i]; }
  const Vec3& get_wall_vertex(const Wall& w, const uint k) const { return vertices[w.vertex_indices[k]]; }
  Wall& get_wall(const wall_index_t i) { return walls[i]; }
  const Wall& get_wall(const wall_index_t i) const { return walls[i]; }
  const WallCollisionRejectionData& get_wall_collision_rejection_data(const wall_index_t i) const {
    return wall_collision_rejection_data[i];
  }
  const WallsInSubpart& get_subpart_wall_indices(const subpart_index_t s) const {
    return walls_per_subpart[s];
  }
  Molecule& get_m(const molecule_id_t id) { return molecules[id]; }
  const Molecule& get_m(const molecule_id_t id) const { return molecules[id]; }
  const uint_set<molecule_id_t>& get_volume_molecule_reactants(const subpart_index_t s, const species_id_t sp) const {
    auto it = reactants.find(std::make_pair(s, sp));
    return it == reactants.end() ? empty_set : it->second;
  }
  const RxnContainerShim& get_all_rxns() const { return rxns; }
  const SpeciesContainerShim& get_all_species() const { return all_species; }
  const BNG::Species& get_species(const species_id_t id) const { return all_species.get(id); }
};

// the parts of the World and of ReleaseEvent (src4/release_event.h:35-260) that
// ReleaseEvent::release_ellipsoid_or_rectcuboid uses
enum class ReleaseShape { UNDEFINED = -1, SPHERICAL, SPHERICAL_SHELL, REGION, LIST, INITIAL_SURF_REGION };


class World {
public:
  Partition partition;
  Partition* outer = nullptr;  // a scene's partition instead of the own one
  SpeciesContainerShim species;
  ShimRng rng;
  SimulationConfig config;
  Partition& get_partition(const int) { return outer ? *outer : partition; }
  const SpeciesContainerShim& get_all_species() const { return species; }
};

// boolean expressions of closed objects for releases (src4/region_expr.h:23-90)
enum class RegionExprOperator { INVALID, UNION, INTERSECT, DIFFERENCE, LEAF_SURFACE_REGION, LEAF_GEOMETRY_OBJECT };
class RegionExprNode {
public:
  RegionExprOperator op = RegionExprOperator::INVALID;
  region_id_t region_id = 0;
  geometry_object_id_t geometry_object_id = 0;
  RegionExprNode* left = nullptr;
  RegionExprNode* right = nullptr;
};
class RegionExpr {
public:
  RegionExprNode* root = nullptr;
};

enum class ReleaseNumberMethod { INVALID, CONST_NUM, GAUSS_NUM, VOL_NUM, CONCENTRATION_NUM, DENSITY_NUM };

class ReleaseEvent {
public:
  World* world = nullptr;
  std::string release_site_name = "release";
  ReleaseShape release_shape = ReleaseShape::SPHERICAL;
  ReleaseNumberMethod release_number_method = ReleaseNumberMethod::CONST_NUM;
  uint release_number = 0;
  double concentration = 0;
  std::vector<CummAreaPWallIndexPair> cumm_area_and_pwall_index_pairs;
  RegionExpr region_expr;
  Vec3 region_llf, region_urb;
  Vec3 location, diameter;
  species_id_t species_id = 0;
  double event_time = 0;
  double get_release_delay_time() const { return 0; }
  void schedule_for_immediate_diffusion_if_needed(const molecule_id_t) { }
  void release_ellipsoid_or_rectcuboid(int computed_release_number);
  uint calculate_number_to_release();
  uint num_vol_mols_from_conc(bool& exact_number);
  int randomly_remove_molecules(Partition& p, const MoleculeIdsVector& mol_ids_in_region, int number_to_remove);
  int vacuum_inside_regions(int number_to_remove);
  bool is_point_inside_region_expr_recursively(Partition& p, const Vec3& pos, const RegionExprNode* region_expr_node);
  void release_inside_regions(int& computed_release_number);
};

} // namespace MCell

#endif
