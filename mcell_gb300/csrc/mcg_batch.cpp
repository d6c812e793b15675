// C ABI of batches (declared in include/mcell_gb300.h): many independent models
// as replicas of one device engine, plus the batch autotuner.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "mcg_batch.h"

namespace {

int bfail(mcg_batch* b, int code, const std::string& msg) {
  if (b) b->err = msg;
  return code;
}

// Autotuner, part 1: subpartitions per edge of one replica, from a cost model of
// the per-molecule work of an iteration, in units of one partner test, evaluated
// on a sample of the model's molecules (e = subpartition edge, d = mean absolute
// displacement per axis, R = reaction radius):
//   partner tests     local partner density * volume scanned: with octant bins
//                     prod(e/2 + d + 2R), without prod(e + d + 2R*sqrt(2))
//   subpartitions     3.6 per subpartition collected, prod(1 + (d + 2R*sqrt(2))/e)
//   wall tests        2 * walls listed for the molecule's
//                     subpartition (walls binned by bounding box grown by R)
//   key-space sweep   0.07 * sort keys / molecules (scan and scatter touch every key)
// The constants were fitted to measured k_diffuse times of the 1M-molecule sphere
// model and of batch replicas at several grids. Candidates run over a geometric
// ladder around the model's own count, with edges of at least 4 reaction radii
// (the converter needs 2*sqrt(2)): dense meshes get finer subpartitions, sparse
// models coarser ones.
uint32_t choose_subparts(const mcg_engine* m, bool* octants) {
  const double L = m->cfg.partition_edge;
  const double* O = m->cfg.partition_origin;
  const uint32_t n_user = m->cfg.subparts_per_edge;
  const size_t N = m->pend_species.size();
  const uint32_t nsp = m->cfg.n_species;
  const double R = m->cfg.rxn_radius;
  const size_t nw = m->walls.size() / 3;
  if (N == 0) {
    *octants = true;
    return n_user;
  }
  // sampled molecules and triangle boxes (grown by R, the binning leeway)
  double d = 0;  // mean absolute displacement per axis: space_step / sqrt(2) * sqrt(2 / pi)
  for (uint32_t a = 0; a < nsp; a++) d = std::max(d, 0.5641896 * m->chem.space_step[a]);
  const size_t stride = std::max<size_t>(1, N / 8192);
  std::vector<const double*> smp;
  for (size_t i = 0; i < N; i += stride) smp.push_back(&m->pend_pos[3 * i]);
  const double S = (double)smp.size();
  std::vector<double> box(6 * nw);
  for (size_t w = 0; w < nw; w++) {
    double* bx = &box[6 * w];
    for (int a = 0; a < 3; a++) {
      bx[a] = 1e300;
      bx[3 + a] = -1e300;
    }
    for (int k = 0; k < 3; k++) {
      const double* v = &m->verts[3 * (size_t)m->walls[3 * w + k]];
      for (int a = 0; a < 3; a++) {
        bx[a] = std::min(bx[a], v[a] - R);
        bx[3 + a] = std::max(bx[3 + a], v[a] + R);
      }
    }
  }
  const uint32_t n_max = (uint32_t)std::max(1.0, std::min(300.0, std::floor(L / (4.0 * R))));
  std::vector<uint32_t> cand;
  for (int k = -16; k <= 12; k++) {
    const uint32_t n = (uint32_t)std::lround(n_user * std::pow(2.0, k / 4.0));
    if (n >= 1 && n <= n_max && std::find(cand.begin(), cand.end(), n) == cand.end()) cand.push_back(n);
  }
  if (std::find(cand.begin(), cand.end(), n_user) == cand.end()) cand.push_back(n_user);
  uint32_t best_n = n_user;
  bool best_oct = true;
  double best = 1e300;
  std::vector<uint32_t> dense;  // samples per subpartition (dense grids)
  std::vector<uint64_t> cell;   // subpartition of each sample
  for (uint32_t n : cand) {
    const double e = L / n;
    auto idx = [&](double x, int a) {
      long i = (long)std::floor((x - O[a]) / e);
      return (uint32_t)std::min<long>(std::max<long>(i, 0), (long)n - 1);
    };
    // molecule-weighted molecules and walls per subpartition: sum over sampled
    // molecules of the samples in their subpartition, and over walls of the samples
    // in the subpartitions their grown box covers (integer sums, exact in any order)
    double mates = 0, walls = 0;
    const uint64_t n3c = (uint64_t)n * n * n;
    if (n3c <= (1ull << 21)) {
      // dense counts for grids of up to 128 per edge (cleared after use)
      if (dense.size() < n3c) dense.resize(n3c, 0);
      cell.resize(smp.size());
      for (size_t i = 0; i < smp.size(); i++) {
        const double* p = smp[i];
        cell[i] = idx(p[0], 0) + (uint64_t)n * (idx(p[1], 1) + (uint64_t)n * idx(p[2], 2));
        dense[cell[i]]++;
      }
      uint64_t m2 = 0, ws = 0;
      for (uint64_t c : cell) m2 += dense[c];
      for (size_t w = 0; w < nw; w++) {
        const double* bx = &box[6 * w];
        const uint32_t x0 = idx(bx[0], 0), y0 = idx(bx[1], 1), z0 = idx(bx[2], 2);
        const uint32_t x1 = idx(bx[3], 0), y1 = idx(bx[4], 1), z1 = idx(bx[5], 2);
        if ((uint64_t)(x1 - x0 + 1) * (y1 - y0 + 1) * (z1 - z0 + 1) > 4096) continue;  // huge walls: any n sees them
        for (uint32_t z = z0; z <= z1; z++)
          for (uint32_t y = y0; y <= y1; y++)
            for (uint32_t x = x0; x <= x1; x++) ws += dense[x + (uint64_t)n * (y + (uint64_t)n * z)];
      }
      for (uint64_t c : cell) dense[c] = 0;
      mates = (double)m2;
      walls = (double)ws;
    } else {
      std::unordered_map<uint64_t, std::pair<double, double>> occ;  // subpartition -> (molecules, walls)
      for (const double* p : smp) {
        const uint64_t s = idx(p[0], 0) + (uint64_t)n * (idx(p[1], 1) + (uint64_t)n * idx(p[2], 2));
        occ[s].first += 1.0;
      }
      for (size_t w = 0; w < nw; w++) {
        const double* bx = &box[6 * w];
        const uint32_t x0 = idx(bx[0], 0), y0 = idx(bx[1], 1), z0 = idx(bx[2], 2);
        const uint32_t x1 = idx(bx[3], 0), y1 = idx(bx[4], 1), z1 = idx(bx[5], 2);
        if ((uint64_t)(x1 - x0 + 1) * (y1 - y0 + 1) * (z1 - z0 + 1) > 4096) continue;
        for (uint32_t z = z0; z <= z1; z++)
          for (uint32_t y = y0; y <= y1; y++)
            for (uint32_t x = x0; x <= x1; x++) {
              auto it = occ.find(x + (uint64_t)n * (y + (uint64_t)n * z));
              if (it != occ.end()) it->second.second += 1.0;
            }
      }
      for (const auto& kv : occ) {
        mates += kv.second.first * kv.second.first;
        walls += kv.second.first * kv.second.second;
      }
    }
    mates *= (double)N / (S * S);  // molecule-weighted molecules per subpartition
    walls /= S;                    // molecule-weighted walls per subpartition
    const double rho_p = 0.5 * mates / (e * e * e);  // local density of partners
    const double a_oct = d + 2.0 * R, a_col = d + 2.0 * R * 1.41421356;
    const double collected = std::pow(1.0 + a_col / e, 3.0);
    const double n3 = (double)n * n * n;
    for (int oct = 1; oct >= 0; oct--) {
      const double keys = nsp * n3 * (oct ? 8.0 : 1.0);
      if (oct && keys > (double)(1u << 26)) continue;
      const double scanned = oct ? std::pow(0.5 * e + a_oct, 3.0) : std::pow(e + a_col, 3.0);
      const double cost = rho_p * scanned + 3.6 * collected + 2.0 * walls + 0.07 * keys / (double)N;
      if (cost < best) {
        best = cost;
        best_n = n;
        best_oct = oct != 0;
      }
    }
  }
  *octants = best_oct;
  return best_n;
}

// Autotuner, part 2: resident blocks per SM of the persistent diffuse kernel,
// timed on the first iterations (two per candidate, CUDA events around the
// kernel). The simulation advances meanwhile; the grid shape does not change
// results.
int tune_diffuse(mcg_batch* b, uint32_t* used, uint32_t budget, std::string& err) {
  const int mx = b->dev->max_diffuse_blocks_per_sm();
  std::vector<int> cand;
  for (int c : {mx, mx - 1, mx - 2, (mx * 2) / 3, mx / 2, 2})
    if (c >= 1 && c <= mx && std::find(cand.begin(), cand.end(), c) == cand.end()) cand.push_back(c);
  if (budget < 2 * cand.size()) return 0;  // not enough iterations yet: tune on a later call
  b->dev->set_options(0, 1);
  double prof[6];
  if (b->dev->profile(prof, err)) return -2;  // discard earlier records
  double best = 1e300;
  int best_c = mx;
  for (int c : cand) {
    int rc = b->dev->set_diffuse_blocks_per_sm(c, err);
    if (!rc) rc = b->dev->step(2, err);
    if (!rc) rc = b->dev->profile(prof, err);
    if (rc) return rc;
    *used += 2;
    if (prof[1] < best) {
      best = prof[1];
      best_c = c;
    }
  }
  b->dev->set_options(1, 0);
  int rc = b->dev->set_diffuse_blocks_per_sm(best_c, err);
  if (rc) return rc;
  b->diffuse_blocks = best_c;
  b->tune_pending = false;
  return 0;
}

}  // namespace

int batch_prepare_replica(const mcg_engine* m, bool autotune, ReplicaPrep& out, std::string& err) {
  if (!m) {
    err = "null model";
    return MCG_ERR_ARG;
  }
  if (m->dev) {
    err = "a model added to a batch must not have been prepared or stepped";
    return MCG_ERR_ARG;
  }
  if (!m->species_set) {
    err = "model without mcg_set_species";
    return MCG_ERR_ARG;
  }
  if (m->wclass.empty() && !m->walls.empty()) {
    err = "mesh without wall classes";
    return MCG_ERR_ARG;
  }
  if (int rc = mcg::check_model_supported(*m, err)) return rc;
  out.octants = true;
  out.nsub = autotune ? choose_subparts(m, &out.octants) : m->cfg.subparts_per_edge;
  if (mcg::compute_setup(m->cfg.partition_origin, m->cfg.partition_edge, out.nsub, m->cfg.rxn_radius,
                         (uint32_t)(m->verts.size() / 3), m->verts.data(), (uint32_t)(m->walls.size() / 3),
                         m->walls.data(), out.hs, err))
    return MCG_ERR_ARG;
  return MCG_OK;
}

int batch_add_prepared(mcg_batch* b, uint32_t n, mcg_engine* const* models, ReplicaPrep* const* preps,
                       const uint32_t* n_iterations, uint32_t* ids) {
  if (!b || (n && (!models || !preps || !ids))) return MCG_ERR_ARG;
  if (!b->dev) return bfail(b, MCG_ERR_CUDA, "batch has no device engine");
  std::vector<mcg::ReplicaSpec> specs(n);
  for (uint32_t k = 0; k < n; k++) {
    const mcg_engine* m = models[k];
    if (!m || !preps[k]) return bfail(b, MCG_ERR_ARG, "null model");
    if (m->cfg.n_species != b->cfg.n_species) return bfail(b, MCG_ERR_ARG, "model species count differs from the batch");
    mcg::ReplicaSpec& sp = specs[k];
    sp.hs = &preps[k]->hs;
    sp.chem = &m->chem;
    sp.wall_class = &m->wclass;
    sp.wall_obj = m->wall_obj.empty() ? nullptr : &m->wall_obj;
    sp.counted = m->counted;
    sp.seed = m->cfg.seed;
    sp.n_mol = m->pend_species.size();
    sp.pos = m->pend_pos.data();
    sp.species = m->pend_species.data();
    sp.n_iterations = n_iterations ? n_iterations[k] : 0;
    sp.octants = preps[k]->octants;
  }
  std::string err;
  int rc = b->dev->add_replicas(specs.data(), n, ids, err);
  if (rc) return bfail(b, rc, err);
  for (uint32_t k = 0; k < n; k++) b->nsub[ids[k]] = preps[k]->nsub;
  return MCG_OK;
}

extern "C" {

int mcg_batch_create(const mcg_batch_config* cfg, mcg_batch** out) {
  if (!cfg || !out) return MCG_ERR_ARG;
  *out = nullptr;
  if (cfg->precision != MCG_PRECISION_FP64 && cfg->precision != MCG_PRECISION_FP32) return MCG_ERR_ARG;
  if (cfg->n_species == 0 || cfg->n_species > MCG_MAX_SPECIES) return MCG_ERR_ARG;
  if (cfg->max_replicas == 0 || cfg->max_replicas > 65536) return MCG_ERR_ARG;
  mcg_batch* b = new mcg_batch();
  b->cfg = *cfg;
  b->dev = cfg->precision == MCG_PRECISION_FP64 ? mcg::make_engine_f64() : mcg::make_engine_f32();
  std::string err;
  int rc = b->dev->create(cfg->n_species, cfg->max_replicas, cfg->capacity, err);
  if (rc) {
    delete b->dev;
    b->dev = nullptr;
    *out = b;  // the message stays readable through mcg_batch_last_error
    b->err = err;
    return rc;
  }
  b->nsub.assign(cfg->max_replicas, 0);
  b->tune_pending = cfg->autotune != 0;
  b->diffuse_blocks = b->dev->max_diffuse_blocks_per_sm();
  *out = b;
  return MCG_OK;
}

void mcg_batch_destroy(mcg_batch* b) {
  if (!b) return;
  delete b->dev;
  delete b;
}

const char* mcg_batch_last_error(const mcg_batch* b) { return b ? b->err.c_str() : "null batch"; }

int mcg_batch_add(mcg_batch* b, uint32_t n, mcg_engine* const* models, const uint32_t* n_iterations,
                  uint32_t* ids) {
  if (!b || (n && (!models || !ids))) return MCG_ERR_ARG;
  if (!b->dev) return bfail(b, MCG_ERR_CUDA, "batch has no device engine");
  // the host halves only read their models: prepared on several threads (a replica of
  // the batching workload takes about 20 ms on one core, most of it the wall setup)
  std::vector<ReplicaPrep> prep(n);
  std::vector<ReplicaPrep*> pp(n);
  std::vector<int> rcs(n, MCG_OK);
  std::vector<std::string> errs(n);
  const bool tune = b->cfg.autotune != 0;
  const uint32_t nt = std::min<uint32_t>(n, std::max(1u, std::min(16u, std::thread::hardware_concurrency())));
  std::atomic<uint32_t> next{0};
  auto work = [&] {
    for (uint32_t k; (k = next.fetch_add(1)) < n;) rcs[k] = batch_prepare_replica(models[k], tune, prep[k], errs[k]);
  };
  if (nt <= 1) {
    work();
  } else {
    std::vector<std::thread> th;
    for (uint32_t t = 0; t < nt; t++) th.emplace_back(work);
    for (auto& x : th) x.join();
  }
  for (uint32_t k = 0; k < n; k++) {
    if (rcs[k]) return bfail(b, rcs[k], errs[k]);
    pp[k] = &prep[k];
  }
  return batch_add_prepared(b, n, models, pp.data(), n_iterations, ids);
}

int mcg_batch_remove(mcg_batch* b, uint32_t n, const uint32_t* ids) {
  if (!b || (n && !ids)) return MCG_ERR_ARG;
  if (!b->dev) return bfail(b, MCG_ERR_CUDA, "batch has no device engine");
  std::string err;
  int rc = b->dev->remove_replicas(ids, n, err);
  if (rc) return bfail(b, rc, err);
  for (uint32_t k = 0; k < n; k++) b->nsub[ids[k]] = 0;
  return MCG_OK;
}

int mcg_batch_step(mcg_batch* b, uint32_t n) {
  if (!b) return MCG_ERR_ARG;
  if (!b->dev) return bfail(b, MCG_ERR_CUDA, "batch has no device engine");
  std::string err;
  uint32_t used = 0;
  if (b->tune_pending) {
    int rc = tune_diffuse(b, &used, n, err);
    if (rc) return bfail(b, rc, err);
  }
  if (n > used) {
    int rc = b->dev->step(n - used, err);
    if (rc) return bfail(b, rc, err);
  }
  return MCG_OK;
}

int mcg_batch_sync(mcg_batch* b) {
  if (!b) return MCG_ERR_ARG;
  if (!b->dev) return bfail(b, MCG_ERR_CUDA, "batch has no device engine");
  std::string err;
  int rc = b->dev->sync(err);
  return rc ? bfail(b, rc, err) : MCG_OK;
}

int mcg_batch_replica_info(mcg_batch* b, uint32_t rep, uint64_t* done, uint32_t* nsub) {
  if (!b || !done) return MCG_ERR_ARG;
  if (!b->dev) return bfail(b, MCG_ERR_CUDA, "batch has no device engine");
  std::string err;
  int rc = b->dev->replica_iterations(rep, done, err);
  if (rc) return bfail(b, rc, err);
  if (nsub) *nsub = b->nsub[rep];
  return MCG_OK;
}

int mcg_batch_get_counts(mcg_batch* b, uint32_t rep, uint64_t* counts) {
  if (!b || !counts) return MCG_ERR_ARG;
  if (!b->dev) return bfail(b, MCG_ERR_CUDA, "batch has no device engine");
  std::string err;
  int rc = b->dev->counts(rep, counts, err);
  return rc ? bfail(b, rc, err) : MCG_OK;
}

int mcg_batch_get_count_trajectory(mcg_batch* b, uint32_t rep, uint32_t n, uint64_t* counts) {
  if (!b || (n && !counts)) return MCG_ERR_ARG;
  if (!b->dev) return bfail(b, MCG_ERR_CUDA, "batch has no device engine");
  std::string err;
  int rc = b->dev->trajectory(rep, n, counts, err);
  return rc ? bfail(b, rc, err) : MCG_OK;
}

int mcg_batch_download_molecules(mcg_batch* b, uint32_t rep, uint64_t cap, double* pos, uint32_t* species,
                                 uint64_t* ids, uint64_t* n_out) {
  if (!b || !n_out) return MCG_ERR_ARG;
  if (!b->dev) return bfail(b, MCG_ERR_CUDA, "batch has no device engine");
  std::string err;
  int rc = b->dev->download(rep, cap, pos, species, ids, n_out, err);
  return rc ? bfail(b, rc, err) : MCG_OK;
}

int mcg_batch_get_stats(mcg_batch* b, uint64_t* iterations, uint64_t* mol_steps, uint64_t* launches) {
  if (!b) return MCG_ERR_ARG;
  if (!b->dev) return bfail(b, MCG_ERR_CUDA, "batch has no device engine");
  b->dev->stats(iterations, mol_steps, launches);
  return MCG_OK;
}

int mcg_batch_get_fallbacks(mcg_batch* b, uint64_t* out) {
  if (!b || !out) return MCG_ERR_ARG;
  if (!b->dev) return bfail(b, MCG_ERR_CUDA, "batch has no device engine");
  std::string err;
  int rc = b->dev->fallbacks(out, err);
  return rc ? bfail(b, rc, err) : MCG_OK;
}

int mcg_batch_set_options(mcg_batch* b, int use_graphs, int profile) {
  if (!b) return MCG_ERR_ARG;
  if (!b->dev) return bfail(b, MCG_ERR_CUDA, "batch has no device engine");
  b->dev->set_options(use_graphs, profile);
  return MCG_OK;
}

int mcg_batch_get_profile(mcg_batch* b, double* out) {
  if (!b || !out) return MCG_ERR_ARG;
  if (!b->dev) return bfail(b, MCG_ERR_CUDA, "batch has no device engine");
  std::string err;
  int rc = b->dev->profile(out, err);
  return rc ? bfail(b, rc, err) : MCG_OK;
}

int mcg_batch_get_memory(mcg_batch* b, uint64_t* bytes) {
  if (!b || !bytes) return MCG_ERR_ARG;
  if (!b->dev) return bfail(b, MCG_ERR_CUDA, "batch has no device engine");
  *bytes = b->dev->device_bytes();
  return MCG_OK;
}

int mcg_batch_release(mcg_batch* b, uint32_t replica, uint32_t species, uint64_t n, int shape, const double* center,
                      const double* diameter, uint32_t object, uint64_t release_seed) {
  if (!b || (shape != MCG_RELEASE_INSIDE_OBJECT && (!center || !diameter))) return MCG_ERR_ARG;
  if (!b->dev) return bfail(b, MCG_ERR_CUDA, "batch has no device engine");
  std::string err;
  int rc = b->dev->release(replica, species, n, shape, center, diameter, object, release_seed, err);
  return rc ? bfail(b, rc, err) : MCG_OK;
}

int mcg_batch_release_region(mcg_batch* b, uint32_t replica, uint32_t species, int method, int64_t number,
                             double concentration_molar, double length_unit_um, const int32_t* expr, uint32_t n_expr,
                             uint64_t release_seed, int64_t* done) {
  if (!b || !expr || !done) return MCG_ERR_ARG;
  if (!b->dev) return bfail(b, MCG_ERR_CUDA, "batch has no device engine");
  std::string err;
  int rc = b->dev->release_region(replica, species, method, number, concentration_molar, length_unit_um, expr, n_expr,
                                  release_seed, done, err);
  return rc ? bfail(b, rc, err) : MCG_OK;
}

int mcg_batch_get_escapes(mcg_batch* b, uint32_t cap, double* out, uint32_t* n) {
  if (!b || !n || (cap && !out)) return MCG_ERR_ARG;
  if (!b->dev) return bfail(b, MCG_ERR_CUDA, "batch has no device engine");
  std::string err;
  double rec[8 * 13];
  int rc = b->dev->escapes(rec, 8, n, err);
  if (rc) return bfail(b, rc, err);
  std::memcpy(out, rec, sizeof(double) * 13 * std::min<uint32_t>(std::min<uint32_t>(cap, *n), 8));
  return MCG_OK;
}

int mcg_autotune_subparts(const mcg_engine* m, uint32_t* nsub, int* octants) {
  if (!m || !nsub || !octants) return MCG_ERR_ARG;
  bool oct = true;
  *nsub = choose_subparts(m, &oct);
  *octants = oct ? 1 : 0;
  return MCG_OK;
}

int mcg_batch_get_tuning(mcg_batch* b, int* blocks) {
  if (!b || !blocks) return MCG_ERR_ARG;
  *blocks = b->diffuse_blocks;
  return MCG_OK;
}

}  // extern "C"
