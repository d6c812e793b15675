/*
 * C entry points over the reference's own hot-path routines (compiled in by
 * oracle/ref/build_ref.py). Project-written driver code; the routines it calls
 * (ray_trace_vol, sort_collisions_by_time, get_closest_wall_collision,
 * collide_wall, reflect_from_wall, exact_disk, test_bimolecular, test_intersect,
 * wall_subparts_collision_test, Wall::initialize_wall_constants,
 * SimulationConfig::init_subpartition_edge_length) are the reference's.
 *
 * ref_diffuse_case restates the volume branch of
 * DiffuseReactEvent::diffuse_vol_molecule (src4/diffuse_react_event.cpp:367-618)
 * around those routines, with the displacement and the random stream injected:
 *   - collide_and_react_with_vol_mol (:786-829): exact_disk, scaling, test_bimolecular
 *   - collide_and_react_with_walls (:991-1067): reflect / transparent / absorptive
 *   - cross_transparent_wall (:3007-3099), non-compartment branch
 * Result layout (doubles), shared with the oracle port and the GPU harness:
 *   [0] status (0 finished, 1 reacted with a partner, 2 absorbed by a wall, 3 draws ran out)
 *   [1..3] final position, [4] final subpartition, [5] draws used, [6] number of events,
 *   [7] elapsed time, [8] remaining t_steps,
 *   then 32 events of 8 doubles: kind, index, side, t_rel, t_abs, x, y, z
 *   kinds: 1 reflect, 2 transparent, 3 absorbed, 4 partner tested (no rxn),
 *          5 partner rxn fired, 6 partner occluded by a wall (exact_disk < 0)
 *   side: the wall side (1 front, 2 back) of wall events; the pathway of the
 *   pair's reaction class for kind 5 (reactions given for one pair in
 *   ref_scene_new are the pathways of its class, in that order)
 */
#include <cstdio>

using namespace MCell;

namespace {

const int RES_HDR = 9;
const int EV_SIZE = 8;
const int EV_MAX = 32;

struct Scene {
  Partition p;
  std::vector<BNG::RxnClass> rxn_store;
  std::vector<int> can_vol_react;
};

void put_event(double* out, int kind, int index, int side, double t_rel, double t_abs, const Vec3& pos) {
  int n = (int)out[6];
  if (n < EV_MAX) {
    double* e = out + RES_HDR + n * EV_SIZE;
    e[0] = kind; e[1] = index; e[2] = side; e[3] = t_rel; e[4] = t_abs;
    e[5] = pos.x; e[6] = pos.y; e[7] = pos.z;
  }
  out[6] = n + 1;
}

} // namespace

extern "C" {

int ref_pos_bytes() { return POS_T_BYTES; }

void* ref_scene_new(
    const double* origin, double partition_edge, unsigned nsub, double rxn_radius,
    unsigned nv, const double* verts, unsigned nw, const unsigned* tris,
    unsigned nspecies, const double* space_steps, const unsigned char* wall_class,
    unsigned nrxn, const unsigned* rxn_ab, const double* rxn_p,
    unsigned nmol, const double* mol_pos, const unsigned* mol_species) {
  Scene* s = new Scene();
  Partition& p = s->p;
  // SimulationConfig::init (simulation_config.cpp:45) and Partition ctor (partition.cpp:36)
  p.config.partition_edge_length = (pos_t)partition_edge;
  p.config.num_subparts_per_partition_edge = nsub;
  p.config.init_subpartition_edge_length();
  p.config.rxn_radius_3d = (pos_t)rxn_radius;
  p.config.use_expanded_list = true;
  p.origin_corner = Vec3((pos_t)origin[0], (pos_t)origin[1], (pos_t)origin[2]);
#if POS_T_BYTES == 4
  for (int k = 0; k < 3; k++) {
    float* f = &p.origin_corner[k];
    uint tmp;
    memcpy(&tmp, f, sizeof(uint));
    tmp &= 0xFFFFF000;
    memcpy(f, &tmp, sizeof(uint));
  }
#endif
  p.opposite_corner = p.origin_corner + Vec3(p.config.partition_edge_length);
  p.walls_per_subpart.resize(p.config.num_subparts);

  for (unsigned i = 0; i < nv; i++) {
    p.vertices.push_back(Vec3((pos_t)verts[3 * i], (pos_t)verts[3 * i + 1], (pos_t)verts[3 * i + 2]));
  }
  // walls: constants (wall.cpp:281) then subpartition binning as in Partition::finalize_walls (partition.cpp:91)
  for (unsigned i = 0; i < nw; i++) {
    Wall w;
    w.index = i;
    w.id = i;
    for (int k = 0; k < 3; k++) {
      w.vertex_indices[k] = tris[3 * i + k];
    }
    p.walls.push_back(w);
  }
  for (unsigned i = 0; i < nw; i++) {
    p.walls[i].initialize_wall_constants(p);
  }
  for (unsigned i = 0; i < nw; i++) {
    SubpartIndicesVector colliding;
    GeometryUtils::wall_subparts_collision_test(p, p.walls[i], colliding);
    for (subpart_index_t sp: colliding) {
      p.walls_per_subpart[sp].insert(i);
    }
    WallCollisionRejectionData r;
    r.normal = p.walls[i].normal;
    r.distance_to_origin = p.walls[i].distance_to_origin;
    p.wall_collision_rejection_data.push_back(r);
  }

  s->can_vol_react.assign(nspecies, 0);
  // one reaction class per reactant pair; the reactions of a pair are its pathways,
  // with cumulative probabilities (BNG::RxnClass::cum_probs)
  s->rxn_store.reserve(nrxn);
  for (unsigned r = 0; r < nrxn; r++) {
    unsigned a = rxn_ab[2 * r], b = rxn_ab[2 * r + 1];
    auto it = p.rxns.bimol.find(std::make_pair(a, b));
    if (it == p.rxns.bimol.end()) {
      s->rxn_store.emplace_back();
      BNG::RxnClass* rc = &s->rxn_store.back();
      rc->type = BNG::RxnType::Standard;
      rc->cum_probs.push_back(rxn_p[r]);
      p.rxns.bimol[std::make_pair(a, b)] = rc;
      p.rxns.bimol[std::make_pair(b, a)] = rc;
    }
    else {
      it->second->cum_probs.push_back(it->second->cum_probs.back() + rxn_p[r]);
    }
    s->can_vol_react[a] = 1;
    s->can_vol_react[b] = 1;
  }
  for (unsigned i = 0; i < nspecies; i++) {
    BNG::Species sp;
    sp.space_step = space_steps[i];
    for (unsigned w = 0; w < nw; w++) {
      int c = wall_class[(size_t)w * nspecies + i];
      if (c != 0) {
        p.wall_class[std::make_pair(w, i)] = c;
        sp.flags |= BNG::SPECIES_FLAG_CAN_VOLWALL;
      }
    }
    p.all_species.species.push_back(sp);
  }
  for (unsigned m = 0; m < nmol; m++) {
    Molecule mol;
    mol.id = m;
    mol.species_id = mol_species[m];
    mol.v.pos = Vec3((pos_t)mol_pos[3 * m], (pos_t)mol_pos[3 * m + 1], (pos_t)mol_pos[3 * m + 2]);
    mol.v.subpart_index = p.get_subpart_index(mol.v.pos);
    p.molecules.push_back(mol);
  }
  // per-subpartition reactant sets (Partition::update_molecule_reactants_map, partition.h:406)
  for (unsigned m = 0; m < nmol; m++) {
    const Molecule& mol = p.molecules[m];
    for (unsigned a = 0; a < nspecies; a++) {
      if (p.rxns.get_bimol_rxn_class(a, mol.species_id) != nullptr) {
        p.reactants[std::make_pair(mol.v.subpart_index, a)].insert(mol.id);
      }
    }
  }
  return s;
}

void ref_scene_free(void* sp) { delete (Scene*)sp; }

// subpart_edge, rcp, partition_edge, origin xyz, nsub
void ref_scene_info(void* sp, double* out) {
  Partition& p = ((Scene*)sp)->p;
  out[0] = p.config.subpart_edge_length;
  out[1] = p.config.subpart_edge_length_rcp;
  out[2] = p.config.partition_edge_length;
  out[3] = p.origin_corner.x; out[4] = p.origin_corner.y; out[5] = p.origin_corner.z;
  out[6] = p.config.num_subparts_per_partition_edge;
}

// per wall: normal xyz, d, unit_u xyz, unit_v xyz, uv_vert1_u, uv_vert2 u v  (14 doubles)
void ref_scene_wall_consts(void* sp, double* out) {
  Partition& p = ((Scene*)sp)->p;
  for (size_t i = 0; i < p.walls.size(); i++) {
    const Wall& w = p.walls[i];
    double* o = out + 14 * i;
    o[0] = w.normal.x; o[1] = w.normal.y; o[2] = w.normal.z; o[3] = w.distance_to_origin;
    o[4] = w.unit_u.x; o[5] = w.unit_u.y; o[6] = w.unit_u.z;
    o[7] = w.unit_v.x; o[8] = w.unit_v.y; o[9] = w.unit_v.z;
    o[10] = w.uv_vert1_u; o[11] = w.uv_vert2.u; o[12] = w.uv_vert2.v;
    o[13] = 0;
  }
}

// CSR of walls per subpartition: counts[nsub^3], list (ascending wall index); returns total
unsigned ref_scene_walls_in_subparts(void* sp, unsigned* counts, unsigned* list, unsigned cap) {
  Partition& p = ((Scene*)sp)->p;
  unsigned total = 0;
  for (size_t s = 0; s < p.walls_per_subpart.size(); s++) {
    counts[s] = (unsigned)p.walls_per_subpart[s].size();
    for (wall_index_t w: p.walls_per_subpart[s]) {
      if (total < cap) {
        list[total] = w;
      }
      total++;
    }
  }
  return total;
}

// ExactDiskUtils::exact_disk (exact_disk_utils.inl:840-1145) at one collision point:
// the molecule `moving` moving by mv from loc, the molecule `target` as the partner
double ref_exact_disk(void* sp, const double* loc, const double* mv, unsigned moving, unsigned target) {
  Partition& p = ((Scene*)sp)->p;
  Molecule& diffused = p.get_m(moving);
  Molecule& colliding = p.get_m(target);
  const Vec3 at((pos_t)loc[0], (pos_t)loc[1], (pos_t)loc[2]);
  Vec3 move((pos_t)mv[0], (pos_t)mv[1], (pos_t)mv[2]);
  return ExactDiskUtils::exact_disk(p, at, move, p.config.rxn_radius_3d, diffused, colliding,
                                    p.config.use_expanded_list);
}

unsigned ref_subpart_index(void* sp, const double* pos) {
  Partition& p = ((Scene*)sp)->p;
  return p.get_subpart_index(Vec3((pos_t)pos[0], (pos_t)pos[1], (pos_t)pos[2]));
}

void ref_diffuse_case(
    void* sp, unsigned mol, const double* disp, const unsigned* draws, unsigned ndraws,
    double r_rate_factor, double t_steps, double* out) {
  Scene* s = (Scene*)sp;
  Partition& p = s->p;
  Molecule saved = p.molecules[mol];
  memset(out, 0, sizeof(double) * (RES_HDR + EV_MAX * EV_SIZE));

  ShimRng rng;
  rng.draws = draws;
  rng.n = ndraws;

  Vec3 remaining_displacement((pos_t)disp[0], (pos_t)disp[1], (pos_t)disp[2]);
  const species_id_t species_id = p.molecules[mol].species_id;
  const bool can_vol_react = s->can_vol_react[species_id] != 0;
  RayTraceState state;
  CollisionsVector molecule_collisions;
  bool was_defunct = false;
  int status = 0;
  wall_index_t last_hit_wall_index = WALL_INDEX_INVALID;
  double elapsed_molecule_time = 0;
  int guard = 0;

  do {
    state = ray_trace_vol(p, rng, mol, can_vol_react, last_hit_wall_index,
                          remaining_displacement, molecule_collisions);
    if (molecule_collisions.size() > 1) {
      sort_collisions_by_time(molecule_collisions);
    }
    for (Collision& collision: molecule_collisions) {
      if (collision.is_vol_mol_vol_mol_collision()) {
        if (CollisionUtils::is_immediate_collision(collision.time)) {
          continue;
        }
        Molecule& colliding = p.get_m(collision.colliding_molecule_id);
        Molecule& diffused = p.get_m(collision.diffused_molecule_id);
        double factor = ExactDiskUtils::exact_disk(
            p, collision.pos, remaining_displacement, p.config.rxn_radius_3d,
            diffused, colliding, p.config.use_expanded_list);
        double t_abs = elapsed_molecule_time + t_steps * collision.time;
        if (factor < 0) {
          put_event(out, 6, collision.colliding_molecule_id, 0, collision.time, t_abs, collision.pos);
          continue;
        }
        double scaling = factor * r_rate_factor;
        int i = RxnUtils::test_bimolecular(
            p, collision.rxn_class, rng, colliding, diffused, scaling, 0, t_abs);
        if (i < BNG::PATHWAY_INDEX_LEAST_VALID) {
          put_event(out, 4, collision.colliding_molecule_id, 0, collision.time, t_abs, collision.pos);
          continue;
        }
        put_event(out, 5, collision.colliding_molecule_id, i, collision.time, t_abs, collision.pos);
        was_defunct = true;
        status = 1;
        break;
      }
      else if (collision.is_wall_collision()) {
        Molecule& vm = p.get_m(mol);
        int side = collision.type == CollisionType::WALL_FRONT ? 1 : 2;
        auto it = p.wall_class.find(std::make_pair(collision.colliding_wall_index, species_id));
        int kind = (it == p.wall_class.end()) ? 0 : it->second;
        double t_abs = elapsed_molecule_time + t_steps * collision.time;
        if (kind == 1) {
          // cross_transparent_wall, non-compartment branch (diffuse_react_event.cpp:3062-3094)
          vm.v.pos = collision.pos;
          vm.v.subpart_index = p.get_subpart_index(vm.v.pos);
          double t_smash = collision.time;
          remaining_displacement = remaining_displacement * Vec3(1.0 - t_smash);
          elapsed_molecule_time += t_steps * t_smash;
          t_steps *= (1.0 - t_smash);
          if (t_steps < EPS) {
            t_steps = EPS;
          }
          last_hit_wall_index = collision.colliding_wall_index;
          put_event(out, 2, collision.colliding_wall_index, side, collision.time, t_abs, collision.pos);
          break;
        }
        if (kind == 2) {
          int pw = RxnUtils::test_intersect(&RxnUtils::g_absorb_class, r_rate_factor, t_abs, rng);
          if (pw >= BNG::PATHWAY_INDEX_LEAST_VALID) {
            put_event(out, 3, collision.colliding_wall_index, side, collision.time, t_abs, collision.pos);
            was_defunct = true;
            status = 2;
            break;
          }
        }
        elapsed_molecule_time += t_steps * collision.time;
        CollisionUtils::reflect_from_wall(p, collision, vm, remaining_displacement, t_steps, last_hit_wall_index);
        put_event(out, 1, collision.colliding_wall_index, side, collision.time, t_abs, collision.pos);
        break;
      }
    }
    if (++guard > 100000) {
      status = 3;
      break;
    }
  } while (state != RayTraceState::FINISHED && !was_defunct);

  if (rng.overrun) {
    status = 3;
  }
  const Molecule& m = p.get_m(mol);
  out[0] = status;
  out[1] = m.v.pos.x; out[2] = m.v.pos.y; out[3] = m.v.pos.z;
  out[4] = m.v.subpart_index;
  out[5] = (double)rng.used;
  out[7] = elapsed_molecule_time;
  out[8] = t_steps;
  p.molecules[mol] = saved;
}

// geometry objects: the object of each wall and which objects are counted volumes
void ref_scene_set_objects(void* sp, unsigned nobj, const unsigned* object_of_wall, const unsigned char* counted) {
  Scene* s = (Scene*)sp;
  Partition& p = s->p;
  p.geometry_objects.assign(nobj, GeometryObject());
  for (unsigned k = 0; k < nobj; k++) {
    p.geometry_objects[k].index = k;
    p.geometry_objects[k].id = k;
    p.geometry_objects[k].counted = counted[k] != 0;
  }
  for (size_t w = 0; w < p.walls.size(); w++) {
    p.walls[w].object_index = object_of_wall[w];
    p.walls[w].object_id = object_of_wall[w];
  }
  p.regions_by_id.clear();
}

// compute_counted_volume_for_pos (collision_utils.inl:1515-1545): bit k set when pos is
// inside counted object k; bit 31 when the ray met a wall edge (the reference's
// release_assert on must_redo_test), tested with the same ray through
// get_num_crossed_walls_per_object
unsigned ref_counted_volume_for_pos(void* sp, const double* pos) {
  Partition& p = ((Scene*)sp)->p;
  const Vec3 v((pos_t)pos[0], (pos_t)pos[1], (pos_t)pos[2]);
  const counted_volume_index_t i = CollisionUtils::compute_counted_volume_for_pos(p, v);
  unsigned mask = 0;
  for (geometry_object_index_t o: p.counted_volumes[i].contained_in_objects) {
    mask |= 1u << o;
  }
  Vec3 dst = p.get_origin_corner();
  dst.x += p.config.subpart_edge_length / (pos_t)11;
  dst.y += p.config.subpart_edge_length / (pos_t)21;
  std::map<geometry_object_index_t, uint> crossed;
  bool redo = false;
  CollisionUtils::get_num_crossed_walls_per_object(p, v, dst, true, crossed, redo);
  return redo ? (mask | (1u << 31)) : mask;
}

// the closed region made of object obj's walls (walls_and_edges ordered by wall index,
// walls per subpartition as Region::initialize_wall_subpart_mapping_if_needed makes
// them), registered as the object's encompassing region
static Region& region_of(Scene* s, unsigned obj) {
  Partition& p = s->p;
  auto it = p.regions_by_id.find(obj);
  if (it == p.regions_by_id.end()) {
    Region reg;
    for (size_t w = 0; w < p.walls.size(); w++) {
      if (p.walls[w].object_index == obj) {
        reg.walls_and_edges[(wall_index_t)w];
      }
    }
    for (size_t sub = 0; sub < p.walls_per_subpart.size(); sub++) {
      for (wall_index_t w: p.walls_per_subpart[sub]) {
        if (p.walls[w].object_index == obj) {
          reg.walls_per_subpart[(subpart_index_t)sub].push_back(w);
        }
      }
    }
    reg.compute_bounding_box(p, reg.bounding_box_llf, reg.bounding_box_urb);
    it = p.regions_by_id.emplace(obj, reg).first;
    if (obj < p.geometry_objects.size()) {
      p.geometry_objects[obj].encompassing_region_id = obj;
    }
  }
  return it->second;
}

bool Region::is_point_inside(Partition& p, const Vec3& pos) {
  bool redo = false;
  return CollisionUtils::is_point_inside_region_no_waypoints(p, pos, *this, redo);
}

// is_point_inside_region_no_waypoints (collision_utils.inl:1484-1510) for the closed
// region made of object obj's walls: 0 outside, 1 inside, 2 the ray met a wall edge
int ref_inside_region(void* sp, unsigned obj, const double* pos) {
  Scene* s = (Scene*)sp;
  Region& reg = region_of(s, obj);
  const Vec3 v((pos_t)pos[0], (pos_t)pos[1], (pos_t)pos[2]);
  bool redo = false;
  const bool in = CollisionUtils::is_point_inside_region_no_waypoints(s->p, v, reg, redo);
  return redo ? 2 : (in ? 1 : 0);
}

// Region::initialize_volume_info_if_needed (geometry.cpp:860-897): object obj's volume
double ref_region_volume(void* sp, unsigned obj) {
  Scene* s = (Scene*)sp;
  Region& reg = region_of(s, obj);
  reg.volume_info_initialized = false;
  reg.initialize_volume_info_if_needed(s->p);
  return reg.get_volume();
}

// A region expression from a postfix program: tokens >= 0 are objects, -1 union,
// -2 intersection, -3 difference (the node pool lives as long as the call)
static RegionExprNode* expr_from_postfix(Scene* s, const int* tok, unsigned n, std::vector<RegionExprNode>& pool) {
  pool.assign(n, RegionExprNode());
  std::vector<RegionExprNode*> st;
  for (unsigned k = 0; k < n; k++) {
    RegionExprNode* e = &pool[k];
    if (tok[k] >= 0) {
      region_of(s, (unsigned)tok[k]);
      e->op = RegionExprOperator::LEAF_GEOMETRY_OBJECT;
      e->geometry_object_id = (geometry_object_id_t)tok[k];
    } else {
      e->op = tok[k] == -1 ? RegionExprOperator::UNION
                           : (tok[k] == -2 ? RegionExprOperator::INTERSECT : RegionExprOperator::DIFFERENCE);
      e->right = st.back();
      st.pop_back();
      e->left = st.back();
      st.pop_back();
    }
    st.push_back(e);
  }
  return st.empty() ? nullptr : st.back();
}

// compute_region_expr_bounding_box (geometry.cpp:1180-1265)
void ref_region_expr_bbox(void* sp, const int* tok, unsigned n, double* llf, double* urb) {
  Scene* s = (Scene*)sp;
  std::vector<RegionExprNode> pool;
  RegionExprNode* root = expr_from_postfix(s, tok, n, pool);
  World world;
  world.outer = &s->p;
  Vec3 lo, hi;
  compute_region_expr_bounding_box(&world, root, lo, hi);
  llf[0] = lo.x; llf[1] = lo.y; llf[2] = lo.z;
  urb[0] = hi.x; urb[1] = hi.y; urb[2] = hi.z;
}

// ReleaseEvent::calculate_number_to_release (release_event.cpp:509-575) by
// concentration (molar) for a spherical release of the given diameter
unsigned ref_number_from_concentration(const double* diameter, double concentration, double length_unit) {
  World world;
  world.config.length_unit = length_unit;
  ReleaseEvent ev;
  ev.world = &world;
  ev.release_shape = ReleaseShape::SPHERICAL;
  ev.release_number_method = ReleaseNumberMethod::CONCENTRATION_NUM;
  ev.concentration = concentration;
  ev.diameter = Vec3((pos_t)diameter[0], (pos_t)diameter[1], (pos_t)diameter[2]);
  return ev.calculate_number_to_release();
}

// ReleaseEvent::release_inside_regions (release_event.cpp:904-952) into the region
// expression `tok` with the random stream injected. method 0: `number` molecules
// (CONST_NUM; a negative number removes molecules of `species`, vacuum_inside_regions
// :864-896); method 1: by concentration (num_vol_mols_from_conc :826-856). Released
// positions go to pos (up to cap), removed molecule indices to removed; the scene's
// molecules are left as they were. Returns the computed release number; draws_used =
// draws taken (0xFFFFFFFF if the stream ran out).
int ref_release_inside_regions(void* sp, const int* tok, unsigned ntok, int method, int number, unsigned species,
                               double concentration, double length_unit, const unsigned* draws, unsigned ndraws,
                               double* pos, unsigned cap, unsigned* n_pos, unsigned* removed, unsigned* n_removed,
                               unsigned* draws_used) {
  Scene* s = (Scene*)sp;
  Partition& p = s->p;
  std::vector<RegionExprNode> pool;
  World world;
  world.outer = &p;
  world.config.length_unit = length_unit;
  world.rng.draws = draws;
  world.rng.n = ndraws;
  ReleaseEvent ev;
  ev.world = &world;
  ev.release_shape = ReleaseShape::REGION;
  ev.release_number_method = method == 1 ? ReleaseNumberMethod::CONCENTRATION_NUM : ReleaseNumberMethod::CONST_NUM;
  ev.release_number = (uint)(number < 0 ? 0 : number);
  ev.concentration = concentration;
  ev.species_id = species;
  ev.region_expr.root = expr_from_postfix(s, tok, ntok, pool);
  compute_region_expr_bounding_box(&world, ev.region_expr.root, ev.region_llf, ev.region_urb);
  const std::vector<Molecule> saved = p.molecules;
  int computed = number;
  ev.release_inside_regions(computed);
  unsigned np = 0, nr = 0;
  for (size_t i = saved.size(); i < p.molecules.size() && np < cap; i++, np++) {
    pos[3 * np] = p.molecules[i].v.pos.x;
    pos[3 * np + 1] = p.molecules[i].v.pos.y;
    pos[3 * np + 2] = p.molecules[i].v.pos.z;
  }
  for (size_t i = 0; i < saved.size(); i++) {
    if (p.molecules[i].is_defunct() && !saved[i].is_defunct()) {
      removed[nr++] = (unsigned)i;
    }
  }
  p.molecules = saved;
  *n_pos = np;
  *n_removed = nr;
  *draws_used = world.rng.overrun ? 0xFFFFFFFFu : (unsigned)world.rng.used;
  return computed;
}

// ReleaseEvent::release_ellipsoid_or_rectcuboid (release_event.cpp:953-1000) with the
// random stream injected: shape 0 sphere (ellipsoid), 1 cuboid, 2 spherical shell; the
// positions of the n molecules in release order; returns the draws used
unsigned ref_release_ellipsoid_or_rectcuboid(int shape, unsigned n, const double* location, const double* diameter,
                                              const unsigned* draws, unsigned ndraws, double* out) {
  World world;
  world.species.species.resize(1);
  world.rng.draws = draws;
  world.rng.n = ndraws;
  ReleaseEvent ev;
  ev.world = &world;
  ev.release_shape = shape == 0 ? ReleaseShape::SPHERICAL
                                : (shape == 2 ? ReleaseShape::SPHERICAL_SHELL : ReleaseShape::REGION);
  ev.location = Vec3((pos_t)location[0], (pos_t)location[1], (pos_t)location[2]);
  ev.diameter = Vec3((pos_t)diameter[0], (pos_t)diameter[1], (pos_t)diameter[2]);
  ev.release_ellipsoid_or_rectcuboid((int)n);
  const std::vector<Molecule>& m = world.partition.molecules;
  for (size_t i = 0; i < m.size() && i < n; i++) {
    out[3 * i] = m[i].v.pos.x;
    out[3 * i + 1] = m[i].v.pos.y;
    out[3 * i + 2] = m[i].v.pos.z;
  }
  return world.rng.overrun ? 0xFFFFFFFFu : (unsigned)world.rng.used;
}

// reaction tests on injected uniforms
int ref_test_bimolecular(double max_fixed_p, double scaling, unsigned draw) {
  Partition p;
  BNG::RxnClass rc;
  rc.cum_probs.push_back(max_fixed_p);
  Molecule a, b;
  ShimRng rng;
  rng.draws = &draw;
  rng.n = 1;
  return RxnUtils::test_bimolecular(p, &rc, rng, a, b, scaling, 0, 0);
}

// test_bimolecular over a class of n pathways (cumulative probabilities): pathway or < 0
int ref_test_bimolecular_pw(const double* cum, unsigned n, double scaling, unsigned draw) {
  Partition p;
  BNG::RxnClass rc;
  rc.cum_probs.assign(cum, cum + n);
  Molecule a, b;
  ShimRng rng;
  rng.draws = &draw;
  rng.n = 1;
  return RxnUtils::test_bimolecular(p, &rc, rng, a, b, scaling, 0, 0);
}

// which_unimolecular over a class of n pathways (cumulative rates)
int ref_which_unimolecular(const double* cum, unsigned n, unsigned draw) {
  BNG::RxnClass rc;
  rc.cum_probs.assign(cum, cum + n);
  Molecule m;
  ShimRng rng;
  rng.draws = &draw;
  rng.n = 1;
  return RxnUtils::which_unimolecular(m, &rc, rng);
}

double ref_time_of_unimol(double k_tot, unsigned draw) {
  BNG::RxnClass rc;
  rc.cum_probs.push_back(k_tot);
  ShimRng rng;
  rng.draws = &draw;
  rng.n = 1;
  return RxnUtils::time_of_unimol(&rc, rng);
}

// the reference's ISAAC64 stream (src/isaac64.c) and ziggurat Gaussian (src/rng.c)
void ref_rng_uint32(unsigned long long seed, unsigned n, unsigned* out) {
  isaac64_state st;
  isaac64_init(&st, (unsigned int)seed);
  for (unsigned i = 0; i < n; i++) {
    out[i] = isaac64_uint32(&st);
  }
}

void ref_rng_gauss(unsigned long long seed, unsigned n, double* out) {
  isaac64_state st;
  isaac64_init(&st, (unsigned int)seed);
  for (unsigned i = 0; i < n; i++) {
    out[i] = rng_gauss(&st);
  }
}

} // extern "C"
