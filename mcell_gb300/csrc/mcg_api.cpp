// C ABI of the engine (declared in include/mcell_gb300.h).
#include "../../include/mcell_gb300.h"

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "mcg_model.h"

namespace mcg {
int status_to_error(uint32_t status, std::string& err) {
  if (status & (1u << 1)) {
    err = "a molecule escaped the partition (enlarge the partition or enclose the model in a reflective box)";
    return MCG_ERR_ESCAPE;
  }
  if (status & (1u << 0)) {
    err = "capacity exceeded (molecules, products or proposals)";
    return MCG_ERR_CAPACITY;
  }
  if (status & (1u << 2)) {
    err = "a bounded device loop gave up (edge re-tries, wall bounces, reaction rounds or product chain)";
    return MCG_ERR_WATCHDOG;
  }
  return MCG_OK;
}
}  // namespace mcg

static int fail(mcg_engine* e, int code, const std::string& msg) {
  if (e) e->err = msg;
  return code;
}

static int prepare(mcg_engine* e) {
  if (e->dev) return MCG_OK;
  if (!e->species_set) return fail(e, MCG_ERR_ARG, "mcg_set_species must be called first");
  {
    std::string why;
    if (int rc = mcg::check_model_supported(*e, why)) return fail(e, rc, why);
  }
  if (e->wclass.empty() && !e->walls.empty()) return fail(e, MCG_ERR_ARG, "mesh without wall classes");
  mcg::HostSetup hs;
  std::string err;
  if (mcg::compute_setup(e->cfg.partition_origin, e->cfg.partition_edge, e->cfg.subparts_per_edge, e->cfg.rxn_radius,
                         (uint32_t)(e->verts.size() / 3), e->verts.data(), (uint32_t)(e->walls.size() / 3),
                         e->walls.data(), hs, err))
    return fail(e, MCG_ERR_ARG, err);
  mcg::DeviceEngine* d = e->cfg.precision == MCG_PRECISION_FP64 ? mcg::make_engine_f64() : mcg::make_engine_f32();
  uint64_t cap = e->cfg.capacity;
  if (cap == 0) cap = std::max<uint64_t>(1024, e->pend_species.size() * 3 / 2);
  int rc = d->create(e->cfg.n_species, 1, cap, err);
  if (rc) {
    delete d;
    return fail(e, rc, err);
  }
  // the model is replica 0 of a one-replica engine
  mcg::ReplicaSpec sp;
  sp.hs = &hs;
  sp.chem = &e->chem;
  sp.wall_class = &e->wclass;
  sp.wall_obj = e->wall_obj.empty() ? nullptr : &e->wall_obj;
  sp.counted = e->counted;
  sp.seed = e->cfg.seed;
  sp.n_mol = e->pend_species.size();
  sp.pos = e->pend_pos.data();
  sp.species = e->pend_species.data();
  uint32_t rep = 0;
  rc = d->add_replicas(&sp, 1, &rep, err);
  e->pend_pos.clear();
  e->pend_species.clear();
  if (rc) {
    delete d;
    return fail(e, rc, err);
  }
  e->dev = d;
  return MCG_OK;
}

extern "C" {

int mcg_create(const mcg_config* cfg, mcg_engine** out) {
  if (!cfg || !out) return MCG_ERR_ARG;
  *out = nullptr;
  if (cfg->precision != MCG_PRECISION_FP64 && cfg->precision != MCG_PRECISION_FP32) return MCG_ERR_ARG;
  if (cfg->n_species == 0 || cfg->n_species > MCG_MAX_SPECIES) return MCG_ERR_ARG;
  if (cfg->subparts_per_edge == 0 || cfg->subparts_per_edge > 300) return MCG_ERR_ARG;
  if (!(cfg->partition_edge > 0) || !(cfg->rxn_radius > 0)) return MCG_ERR_ARG;
  mcg_engine* e = new mcg_engine();
  e->cfg = *cfg;
  e->chem.nsp = cfg->n_species;
  *out = e;
  return MCG_OK;
}

void mcg_destroy(mcg_engine* e) {
  if (!e) return;
  delete e->dev;
  delete e;
}

const char* mcg_last_error(const mcg_engine* e) { return e ? e->err.c_str() : "null engine"; }

int mcg_set_species(mcg_engine* e, uint32_t n, const double* space_step) {
  if (!e || !space_step) return MCG_ERR_ARG;
  if (e->dev) return fail(e, MCG_ERR_ARG, "species must be set before the first step");
  if (n != e->cfg.n_species) return fail(e, MCG_ERR_ARG, "species count differs from mcg_config.n_species");
  for (uint32_t i = 0; i < n; i++) {
    if (!(space_step[i] >= 0)) return fail(e, MCG_ERR_ARG, "space step must be >= 0");
    e->chem.space_step[i] = space_step[i];
  }
  e->species_set = true;
  return MCG_OK;
}

int mcg_upload_mesh(mcg_engine* e, uint32_t nv, const double* vertices, uint32_t nw, const uint32_t* walls,
                    const uint8_t* wall_class) {
  if (!e || (nv && !vertices) || (nw && (!walls || !wall_class))) return MCG_ERR_ARG;
  if (e->dev) return fail(e, MCG_ERR_ARG, "the mesh must be uploaded before the first step (static geometry only)");
  const uint32_t ns = e->cfg.n_species;
  for (uint64_t k = 0; k < (uint64_t)nw * ns; k++)
    if (wall_class[k] > 2) return fail(e, MCG_ERR_ARG, "wall class must be 0, 1 or 2");
  e->verts.assign(vertices, vertices + 3 * (size_t)nv);
  e->walls.assign(walls, walls + 3 * (size_t)nw);
  e->wclass.assign(wall_class, wall_class + (size_t)nw * ns);
  return MCG_OK;
}

int mcg_add_bimol_rxn(mcg_engine* e, uint32_t a, uint32_t b, double p, int32_t p0, int32_t p1) {
  if (!e) return MCG_ERR_ARG;
  const int ns = (int)e->cfg.n_species;
  if (e->dev) return fail(e, MCG_ERR_ARG, "reactions must be added before the first step");
  if (a >= (uint32_t)ns || b >= (uint32_t)ns || p0 >= ns || p1 >= ns || p0 < -1 || p1 < -1 || !(p >= 0))
    return fail(e, MCG_ERR_ARG, "invalid bimolecular reaction");
  // a further reaction of the same reactant pair is a further pathway of its class
  if (!e->chem.add_bimol((int)a, (int)b, p, p0, p1))
    return fail(e, MCG_ERR_UNSUPPORTED, "more than MCG_MAX_PATHWAYS reactions for one reactant pair");
  return MCG_OK;
}

int mcg_add_unimol_rxn(mcg_engine* e, uint32_t a, double k, int32_t p0, int32_t p1) {
  if (!e) return MCG_ERR_ARG;
  const int ns = (int)e->cfg.n_species;
  if (e->dev) return fail(e, MCG_ERR_ARG, "reactions must be added before the first step");
  if (a >= (uint32_t)ns || p0 >= ns || p1 >= ns || p0 < -1 || p1 < -1 || !(k >= 0))
    return fail(e, MCG_ERR_ARG, "invalid unimolecular reaction");
  if (!e->chem.add_unimol((int)a, k, p0, p1))
    return fail(e, MCG_ERR_UNSUPPORTED, "more than MCG_MAX_PATHWAYS unimolecular reactions for one species");
  return MCG_OK;
}

int mcg_add_molecules(mcg_engine* e, uint64_t n, const double* pos, const uint32_t* species) {
  if (!e || (n && (!pos || !species))) return MCG_ERR_ARG;
  for (uint64_t i = 0; i < n; i++)
    if (species[i] >= e->cfg.n_species) return fail(e, MCG_ERR_ARG, "species index out of range");
  if (!e->dev) {
    e->pend_pos.insert(e->pend_pos.end(), pos, pos + 3 * n);
    e->pend_species.insert(e->pend_species.end(), species, species + n);
    e->next_uid += n;
    return MCG_OK;
  }
  std::string err;
  int rc = e->dev->add_molecules(0, n, pos, species, e->next_uid, err);
  if (rc) return fail(e, rc, err);
  e->next_uid += n;
  return MCG_OK;
}

int mcg_prepare(mcg_engine* e) {
  if (!e) return MCG_ERR_ARG;
  return prepare(e);
}

int mcg_step(mcg_engine* e, uint32_t n) {
  if (!e) return MCG_ERR_ARG;
  int rc = prepare(e);
  if (rc) return rc;
  std::string err;
  rc = e->dev->step(n, err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_sync(mcg_engine* e) {
  if (!e) return MCG_ERR_ARG;
  if (!e->dev) return MCG_OK;
  std::string err;
  int rc = e->dev->sync(err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_get_counts(mcg_engine* e, uint64_t* counts) {
  if (!e || !counts) return MCG_ERR_ARG;
  int rc = prepare(e);
  if (rc) return rc;
  std::string err;
  rc = e->dev->counts(0, counts, err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_request_counts(mcg_engine* e, uint64_t* ticket) {
  if (!e || !ticket) return MCG_ERR_ARG;
  int rc = prepare(e);
  if (rc) return rc;
  std::string err;
  rc = e->dev->request_counts(0, ticket, err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_wait_counts(mcg_engine* e, uint64_t ticket, uint64_t* counts) {
  if (!e || !counts || !e->dev) return MCG_ERR_ARG;
  std::string err;
  int rc = e->dev->wait_counts(ticket, counts, err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_get_count_trajectory(mcg_engine* e, uint32_t n, uint64_t* counts) {
  if (!e || !counts || !e->dev) return MCG_ERR_ARG;
  std::string err;
  int rc = e->dev->trajectory(0, n, counts, err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_download_molecules(mcg_engine* e, uint64_t cap, double* pos, uint32_t* species, uint64_t* ids,
                           uint64_t* n_out) {
  if (!e || !n_out) return MCG_ERR_ARG;
  int rc = prepare(e);
  if (rc) return rc;
  std::string err;
  rc = e->dev->download(0, cap, pos, species, ids, n_out, err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_get_stats(mcg_engine* e, uint64_t* iterations, uint64_t* mol_steps, uint64_t* launches) {
  if (!e) return MCG_ERR_ARG;
  if (!e->dev) {
    if (iterations) *iterations = 0;
    if (mol_steps) *mol_steps = 0;
    if (launches) *launches = 0;
    return MCG_OK;
  }
  e->dev->stats(iterations, mol_steps, launches);
  return MCG_OK;
}

int mcg_reaction_decisions(int kind, uint32_t n, const double* cum, const uint32_t* npw, const double* scaling,
                           const uint32_t* draws, int32_t* out) {
  if ((kind != 0 && kind != 1) || (n && (!cum || !npw || !draws || !out || (kind == 0 && !scaling))))
    return MCG_ERR_ARG;
  for (uint32_t c = 0; c < n; c++)
    if (npw[c] < 1 || npw[c] > MCG_MAX_PATHWAYS) return MCG_ERR_ARG;
  std::vector<double> sc;
  if (kind == 1) sc.assign(n, 0.0);
  std::string err;
  return mcg::rxn_decisions(kind, n, cum, npw, kind == 0 ? scaling : sc.data(), draws, out, err);
}

int mcg_get_fallbacks(mcg_engine* e, uint64_t* out) {
  if (!e || !out) return MCG_ERR_ARG;
  if (!e->dev) {
    out[0] = out[1] = out[2] = 0;
    return MCG_OK;
  }
  std::string err;
  int rc = e->dev->fallbacks(out, err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_inside_tests(mcg_engine* e, uint32_t n, const double* pos, int kind, uint32_t object, uint32_t* out) {
  if (!e || (n && (!pos || !out)) || (kind != 0 && kind != 1)) return MCG_ERR_ARG;
  int rc = prepare(e);
  if (rc) return rc;
  std::string err;
  rc = e->dev->inside_tests(0, n, pos, kind, object, out, err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_release_positions(int shape, uint32_t n, const double* center, const double* diameter, const uint32_t* draws,
                          uint32_t n_draws, double* pos, uint32_t* draws_used) {
  if (shape < MCG_RELEASE_SPHERE || shape > MCG_RELEASE_SHELL || !center || !diameter || !draws_used ||
      (n && !pos) || (n_draws && !draws))
    return MCG_ERR_ARG;
  std::string err;
  return mcg::release_positions(shape, n, center, diameter, draws, n_draws, pos, draws_used, err);
}

int mcg_set_trace_limits(mcg_engine* e, uint32_t max_candidates, uint32_t max_subparts) {
  if (!e) return MCG_ERR_ARG;
  int rc = prepare(e);
  if (rc) return rc;
  std::string err;
  rc = e->dev->set_trace_limits((int)std::min<uint32_t>(max_candidates, 1u << 30),
                                (int)std::min<uint32_t>(max_subparts, 1u << 30), err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_set_options(mcg_engine* e, int use_graphs, int profile) {
  if (!e) return MCG_ERR_ARG;
  int rc = prepare(e);
  if (rc) return rc;
  e->dev->set_options(use_graphs, profile);
  return MCG_OK;
}

int mcg_inject_device_alloc_failure(int64_t after) {
  mcg::set_alloc_failure((long long)after);
  return MCG_OK;
}

int mcg_get_profile(mcg_engine* e, double* out) {
  if (!e || !out || !e->dev) return MCG_ERR_ARG;
  std::string err;
  int rc = e->dev->profile(out, err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_debug_molecule(mcg_engine* e, uint64_t id) {
  if (!e) return MCG_ERR_ARG;
  int rc = prepare(e);
  if (rc) return rc;
  std::string err;
  rc = e->dev->debug_molecule(id, err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_get_debug_log(mcg_engine* e, double* out) {
  if (!e || !out || !e->dev) return MCG_ERR_ARG;
  std::string err;
  int rc = e->dev->debug_log(out, err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_get_escapes(mcg_engine* e, uint32_t cap, double* out, uint32_t* n) {
  if (!e || !n || (cap && !out) || !e->dev) return MCG_ERR_ARG;
  std::string err;
  double rec[8 * 13];
  int rc = e->dev->escapes(rec, 8, n, err);
  if (rc) return fail(e, rc, err);
  for (uint32_t k = 0; k < std::min<uint32_t>(std::min<uint32_t>(cap, *n), 8); k++)
    std::memcpy(out + 12 * k, rec + 13 * k, 12 * sizeof(double));  // the replica field is always 0 here
  return MCG_OK;
}

int mcg_trace_cases(mcg_engine* e, uint32_t n, const uint64_t* ids, const double* disp, const uint32_t* draws,
                    uint32_t draws_per_case, const double* rrf, const double* tst, double* out) {
  if (!e || (n && (!ids || !disp || !rrf || !tst || !out))) return MCG_ERR_ARG;
  int rc = prepare(e);
  if (rc) return rc;
  std::string err;
  rc = e->dev->trace(n, ids, disp, draws, draws_per_case, rrf, tst, out, err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_trace_cases_static(mcg_engine* e, uint32_t n, const uint64_t* ids, const double* disp,
                           const uint32_t* draws, uint32_t draws_per_case, const double* rrf, const double* tst,
                           double* out) {
  if (!e || (n && (!ids || !disp || !rrf || !tst || !out))) return MCG_ERR_ARG;
  // preparing would allocate: this entry point only runs on an engine that is ready
  if (!e->dev || !e->pend_species.empty())
    return fail(e, MCG_ERR_ARG, "mcg_trace_cases_static: call mcg_prepare first (no molecules may be pending)");
  if (n > MCG_TRACE_STATIC_MAX_CASES)
    return fail(e, MCG_ERR_ARG, "mcg_trace_cases_static: n_cases " + std::to_string(n) + " exceeds the maximum " +
                                    std::to_string(MCG_TRACE_STATIC_MAX_CASES));
  if ((uint64_t)n * draws_per_case > MCG_TRACE_STATIC_MAX_DRAWS)
    return fail(e, MCG_ERR_ARG, "mcg_trace_cases_static: n_cases x draws_per_case " +
                                    std::to_string((uint64_t)n * draws_per_case) + " exceeds the maximum " +
                                    std::to_string(MCG_TRACE_STATIC_MAX_DRAWS));
  if (n && draws_per_case && !draws) return MCG_ERR_ARG;
  std::string err;
  int rc = e->dev->trace_static(n, ids, disp, draws, draws_per_case, rrf, tst, out, err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_set_wall_objects(mcg_engine* e, uint32_t n_walls, const uint16_t* object_of_wall) {
  if (!e || (n_walls && !object_of_wall)) return MCG_ERR_ARG;
  if (e->dev) return fail(e, MCG_ERR_ARG, "wall objects must be set before the first step");
  if (n_walls != e->walls.size() / 3) return fail(e, MCG_ERR_ARG, "wall count differs from the uploaded mesh");
  e->wall_obj.assign(object_of_wall, object_of_wall + n_walls);
  return MCG_OK;
}

int mcg_set_counted_objects(mcg_engine* e, uint32_t n, const uint16_t* objects) {
  if (!e || (n && !objects)) return MCG_ERR_ARG;
  if (e->dev) return fail(e, MCG_ERR_ARG, "counted objects must be set before the first step");
  if (n > 7) return fail(e, MCG_ERR_UNSUPPORTED, "at most 7 counted objects per model on the GPU path");
  if (n && e->wall_obj.empty()) return fail(e, MCG_ERR_ARG, "counted objects need mcg_set_wall_objects first");
  e->counted.assign(objects, objects + n);
  return MCG_OK;
}

int mcg_get_counted_volume_counts(mcg_engine* e, uint64_t* counts) {
  if (!e || !counts) return MCG_ERR_ARG;
  int rc = prepare(e);
  if (rc) return rc;
  std::string err;
  rc = e->dev->counted_counts(0, counts, err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_get_counted_volume_trajectory(mcg_engine* e, uint32_t n, uint64_t* counts) {
  if (!e || (n && !counts)) return MCG_ERR_ARG;
  int rc = prepare(e);
  if (rc) return rc;
  std::string err;
  rc = e->dev->counted_trajectory(0, n, counts, err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_release(mcg_engine* e, uint32_t species, uint64_t n, int shape, const double* center,
                const double* diameter, uint32_t object, uint64_t release_seed) {
  if (!e || (shape != MCG_RELEASE_INSIDE_OBJECT && (!center || !diameter))) return MCG_ERR_ARG;
  if (!e->pend_species.empty() || !e->dev) {
    int rc = prepare(e);  // pending host molecules are uploaded first
    if (rc) return rc;
  }
  std::string err;
  int rc = e->dev->release(0, species, n, shape, center, diameter, object, release_seed, err);
  if (rc) return fail(e, rc, err);
  e->next_uid += n;
  return MCG_OK;
}

int mcg_release_region(mcg_engine* e, uint32_t species, int method, int64_t number, double concentration_molar,
                       double length_unit_um, const int32_t* expr, uint32_t n_expr, uint64_t release_seed,
                       int64_t* done) {
  if (!e || !expr || !done) return MCG_ERR_ARG;
  if (!e->pend_species.empty() || !e->dev) {
    int rc = prepare(e);  // pending host molecules are uploaded first
    if (rc) return rc;
  }
  std::string err;
  int rc = e->dev->release_region(0, species, method, number, concentration_molar, length_unit_um, expr, n_expr,
                                  release_seed, done, err);
  if (rc) return fail(e, rc, err);
  // the ids the release gave out (one per draw of a single-draw release, placed or not)
  e->next_uid = std::max<uint64_t>(e->next_uid, e->dev->next_molecule_id(0));
  return MCG_OK;
}

int mcg_release_region_harness(mcg_engine* e, uint32_t species, int method, int64_t number,
                               double concentration_molar, double length_unit_um, const int32_t* expr,
                               uint32_t n_expr, const uint32_t* draws, uint32_t n_draws, double* pos, uint32_t cap,
                               uint32_t* n_pos, uint64_t* removed, uint32_t* n_removed, uint32_t* draws_used) {
  if (!e || !expr || !n_pos || !n_removed || !draws_used || (n_draws && !draws) || (cap && (!pos || !removed)))
    return MCG_ERR_ARG;
  int rc = prepare(e);
  if (rc) return rc;
  std::string err;
  rc = e->dev->release_region_harness(0, species, method, number, concentration_molar, length_unit_um, expr, n_expr,
                                      draws, n_draws, pos, cap, n_pos, removed, n_removed, draws_used, err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_export_state(mcg_engine* e, uint64_t cap, double* pos, uint32_t* species, uint64_t* ids, double* tuni,
                     uint8_t* flags, uint64_t* n_out, uint64_t* iteration) {
  if (!e || !n_out || !iteration || (cap && (!pos || !species || !ids || !tuni || !flags))) return MCG_ERR_ARG;
  int rc = prepare(e);
  if (rc) return rc;
  std::string err;
  rc = e->dev->export_state(0, cap, pos, species, ids, tuni, flags, n_out, iteration, err);
  return rc ? fail(e, rc, err) : MCG_OK;
}

int mcg_import_state(mcg_engine* e, uint64_t n, const double* pos, const uint32_t* species, const uint64_t* ids,
                     const double* tuni, const uint8_t* flags, uint64_t iteration) {
  if (!e || (n && (!pos || !species || !ids || !tuni || !flags))) return MCG_ERR_ARG;
  if (!e->pend_species.empty()) return fail(e, MCG_ERR_ARG, "mcg_import_state: the handle already has molecules");
  for (uint64_t i = 0; i < n; i++)
    if (species[i] >= e->cfg.n_species) return fail(e, MCG_ERR_ARG, "species index out of range");
  int rc = prepare(e);
  if (rc) return rc;
  std::string err;
  rc = e->dev->import_state(0, n, pos, species, ids, tuni, flags, iteration, err);
  if (rc) return fail(e, rc, err);
  for (uint64_t i = 0; i < n; i++) e->next_uid = std::max<uint64_t>(e->next_uid, ids[i] + 1);
  return MCG_OK;
}

int mcg_wall_consts(mcg_engine* e, double* out) {
  if (!e || !out) return MCG_ERR_ARG;
  mcg::HostSetup hs;
  std::string err;
  if (mcg::compute_setup(e->cfg.partition_origin, e->cfg.partition_edge, e->cfg.subparts_per_edge, e->cfg.rxn_radius,
                         (uint32_t)(e->verts.size() / 3), e->verts.data(), (uint32_t)(e->walls.size() / 3),
                         e->walls.data(), hs, err))
    return fail(e, MCG_ERR_ARG, err);
  for (uint32_t w = 0; w < hs.nw; w++) {
    std::memcpy(out + 14 * (size_t)w, &hs.wall[24 * (size_t)w], 13 * sizeof(double));
    out[14 * (size_t)w + 13] = 0;
  }
  return MCG_OK;
}

int mcg_walls_in_subparts(mcg_engine* e, uint32_t* counts, uint32_t* list, uint64_t cap, uint64_t* total) {
  if (!e || !counts || !total) return MCG_ERR_ARG;
  mcg::HostSetup hs;
  std::string err;
  if (mcg::compute_setup(e->cfg.partition_origin, e->cfg.partition_edge, e->cfg.subparts_per_edge, e->cfg.rxn_radius,
                         (uint32_t)(e->verts.size() / 3), e->verts.data(), (uint32_t)(e->walls.size() / 3),
                         e->walls.data(), hs, err))
    return fail(e, MCG_ERR_ARG, err);
  const size_t n3 = hs.wsp_off.size() - 1;
  for (size_t s = 0; s < n3; s++) counts[s] = hs.wsp_off[s + 1] - hs.wsp_off[s];
  *total = hs.wsp_list.size();
  if (list)
    for (uint64_t k = 0; k < std::min<uint64_t>(cap, hs.wsp_list.size()); k++) list[k] = hs.wsp_list[k];
  return MCG_OK;
}

}  // extern "C"
