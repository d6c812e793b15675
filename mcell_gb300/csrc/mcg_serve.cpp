// Serving loop (declared in include/mcell_gb300.h): simulation requests arrive
// at any time and are continuously batched. One worker thread owns a batch on
// the device; between blocks of iterations it admits queued requests as replica
// slots and the device-memory budget allow (first come, first served), runs the
// block for every admitted request at once, collects the requests that reached
// their iteration count and frees their slots. A request's state stays resident
// on the device from admission to its last iteration. The host half of an
// admission (grid, wall constants and lists) is done at submission, in the
// submitting thread: in the worker it held the device idle (20-30 ms a request).
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>

#include <cuda_runtime.h>

#include "mcg_batch.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  mcg_engine model;             // copy of the description given at submission
  uint32_t n_iterations = 0;
  int state = MCG_REQ_QUEUED;
  uint32_t rep = 0;             // replica slot while running
  uint64_t done = 0;            // iterations run
  uint64_t est_bytes = 0;       // device bytes reserved against the budget
  Clock::time_point t_submit, t_done;
  std::vector<uint64_t> traj;   // [iterations][n_species], harvested block by block
  std::string err;              // why the request failed
  // host half of the admission (grid, wall constants and lists), made at submission
  // so that the worker, which the device waits on, only does the device half
  std::unique_ptr<ReplicaPrep> prep;
};

}  // namespace

struct mcg_server {
  mcg_server_config cfg;
  std::string err;
  mcg_batch* batch = nullptr;
  int device = 0;
  std::thread worker;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stop = false;
  bool failed = false;
  uint64_t next_ticket = 1;
  std::deque<uint64_t> queue;
  std::unordered_map<uint64_t, Request> reqs;
  std::vector<uint64_t> running;
  uint64_t reserved = 0;        // estimated device bytes of the running requests
  uint64_t completed = 0, mol_steps = 0;
  double busy_s = 0;
};

namespace {

int sfail(mcg_server* s, int code, const std::string& msg) {
  if (s) s->err = msg;
  return code;
}

// device bytes a request needs while resident: its mesh and wall lists, its sort
// keys, and its molecules (both sorted copies and per-iteration scratch, with
// room for products)
uint64_t estimate_bytes(const mcg_engine& m, int precision, uint32_t subparts_per_edge) {
  const uint64_t nw = m.walls.size() / 3;
  const uint64_t n = subparts_per_edge;
  const uint64_t keys = (uint64_t)m.cfg.n_species * n * n * n * 8;
  const uint64_t per_wall = precision == MCG_PRECISION_FP64 ? 232 : 120;
  const uint64_t per_mol = precision == MCG_PRECISION_FP64 ? 330 : 240;
  const uint64_t mol = (uint64_t)(m.pend_species.size() * 3 / 2 + 1024);
  return nw * (per_wall + 8 + m.cfg.n_species) + keys * 16 + mol * per_mol + (1u << 20);
}

// one pass of the worker: admit, run a block, collect. Returns an MCG code.
int serve_once(mcg_server* s, std::unique_lock<std::mutex>& lk) {
  // admission (first come, first served; the head waits until it fits)
  std::vector<uint64_t> admit;
  uint64_t extra = 0;
  while (!s->queue.empty()) {
    Request& r = s->reqs[s->queue.front()];
    if (s->running.size() + admit.size() >= s->cfg.max_slots) break;
    if (s->reserved + extra + r.est_bytes > s->cfg.hbm_budget_bytes && !(s->running.empty() && admit.empty())) break;
    extra += r.est_bytes;
    admit.push_back(s->queue.front());
    s->queue.pop_front();
  }
  if (admit.empty() && s->running.empty()) return MCG_OK;
  std::vector<mcg_engine*> models;
  std::vector<ReplicaPrep*> preps;
  std::vector<uint32_t> iters;
  for (uint64_t t : admit) {
    models.push_back(&s->reqs[t].model);
    preps.push_back(s->reqs[t].prep.get());
    iters.push_back(s->reqs[t].n_iterations);
  }
  lk.unlock();
  std::vector<uint32_t> ids(admit.size());
  int rc = admit.empty() ? MCG_OK
                         : batch_add_prepared(s->batch, (uint32_t)admit.size(), models.data(), preps.data(),
                                              iters.data(), ids.data());
  if (rc && mcg_batch_sync(s->batch) == MCG_OK) {
    // the admission failed (device memory, a model the batch rejects) but left the
    // batch as it was: those requests fail, the running ones go on
    lk.lock();
    const std::string why = std::string("admission: ") + s->batch->err;
    for (uint64_t t : admit) {
      Request& r = s->reqs[t];
      r.state = MCG_REQ_FAILED;
      r.err = why;
      r.t_done = Clock::now();
    }
    s->cv_done.notify_all();
    return MCG_OK;
  }
  lk.lock();
  if (rc) return sfail(s, rc, std::string("admission: ") + s->batch->err);
  for (size_t k = 0; k < admit.size(); k++) {
    Request& r = s->reqs[admit[k]];
    r.state = MCG_REQ_RUNNING;
    r.rep = ids[k];
    r.model.pend_pos.clear();  // the device holds the molecules now
    r.model.pend_pos.shrink_to_fit();
    r.model.pend_species.clear();
    r.model.pend_species.shrink_to_fit();
    r.prep.reset();
    s->running.push_back(admit[k]);
  }
  s->reserved += extra;
  // block length: until the first running request is due, between 1 and 64 iterations
  uint64_t block = 64;
  for (uint64_t t : s->running) {
    const Request& r = s->reqs[t];
    block = std::min<uint64_t>(block, r.n_iterations - r.done);
  }
  block = std::max<uint64_t>(block, 1);
  std::vector<std::pair<uint64_t, uint32_t>> run;
  for (uint64_t t : s->running) run.emplace_back(t, s->reqs[t].rep);
  lk.unlock();
  const auto t0 = Clock::now();
  uint64_t steps0 = 0, steps1 = 0;
  rc = mcg_batch_get_stats(s->batch, nullptr, &steps0, nullptr);
  if (!rc) rc = mcg_batch_step(s->batch, (uint32_t)block);
  if (!rc) rc = mcg_batch_sync(s->batch);
  if (!rc) rc = mcg_batch_get_stats(s->batch, nullptr, &steps1, nullptr);
  const auto t1 = Clock::now();
  // harvest this block's count rows of every running request
  std::vector<std::vector<uint64_t>> rows(run.size());
  std::vector<uint64_t> done(run.size(), 0);
  const uint32_t nsp = s->cfg.n_species;
  for (size_t k = 0; k < run.size() && !rc; k++) {
    rc = mcg_batch_replica_info(s->batch, run[k].second, &done[k], nullptr);
    if (rc) break;
    rows[k].resize((size_t)block * nsp);
    rc = mcg_batch_get_count_trajectory(s->batch, run[k].second, (uint32_t)block, rows[k].data());
  }
  lk.lock();
  if (rc) return sfail(s, rc, std::string("step: ") + s->batch->err);
  s->busy_s += std::chrono::duration<double>(t1 - t0).count();
  s->mol_steps += steps1 - steps0;
  std::vector<uint32_t> finished_reps;
  std::vector<uint64_t> still;
  for (size_t k = 0; k < run.size(); k++) {
    Request& r = s->reqs[run[k].first];
    const uint64_t fresh = std::min<uint64_t>(block, r.n_iterations - r.done);
    r.traj.insert(r.traj.end(), rows[k].begin(), rows[k].begin() + fresh * nsp);
    r.done = done[k];
    if (r.state == MCG_REQ_CANCELLED || r.done >= r.n_iterations) {
      if (r.state != MCG_REQ_CANCELLED) {
        r.state = MCG_REQ_DONE;
        s->completed++;
      }
      r.t_done = t1;
      finished_reps.push_back(r.rep);
      s->reserved -= std::min(s->reserved, r.est_bytes);
    } else {
      still.push_back(run[k].first);
    }
  }
  s->running = still;
  if (!finished_reps.empty()) {
    lk.unlock();
    rc = mcg_batch_remove(s->batch, (uint32_t)finished_reps.size(), finished_reps.data());
    lk.lock();
    if (rc) return sfail(s, rc, std::string("collect: ") + s->batch->err);
    s->cv_done.notify_all();
  }
  return MCG_OK;
}

void worker_main(mcg_server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (!s->stop) {
    if (s->queue.empty() && s->running.empty()) {
      s->cv_work.wait(lk, [s] { return s->stop || !s->queue.empty(); });
      continue;
    }
    int rc = serve_once(s, lk);
    if (rc) {
      // a device error ends the server: every open request fails with the message
      s->failed = true;
      for (auto& kv : s->reqs)
        if (kv.second.state == MCG_REQ_QUEUED || kv.second.state == MCG_REQ_RUNNING) kv.second.state = MCG_REQ_FAILED;
      s->queue.clear();
      s->running.clear();
      s->cv_done.notify_all();
      break;
    }
  }
}

}  // namespace

extern "C" {

int mcg_serve_create(const mcg_server_config* cfg, mcg_server** out) {
  if (!cfg || !out) return MCG_ERR_ARG;
  *out = nullptr;
  if (cfg->max_slots == 0 || cfg->max_slots > 65536 || cfg->hbm_budget_bytes == 0) return MCG_ERR_ARG;
  mcg_batch_config bc;
  std::memset(&bc, 0, sizeof(bc));
  bc.precision = cfg->precision;
  bc.n_species = cfg->n_species;
  bc.max_replicas = cfg->max_slots;
  bc.autotune = cfg->autotune;
  mcg_server* s = new mcg_server();
  s->cfg = *cfg;
  int rc = mcg_batch_create(&bc, &s->batch);
  if (rc) {
    s->err = s->batch ? s->batch->err : "invalid batch configuration";
    mcg_batch_destroy(s->batch);
    s->batch = nullptr;
    *out = s;  // readable through mcg_serve_last_error
    return rc;
  }
  cudaGetDevice(&s->device);
  s->worker = std::thread(worker_main, s);
  *out = s;
  return MCG_OK;
}

void mcg_serve_destroy(mcg_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  mcg_batch_destroy(s->batch);
  delete s;
}

const char* mcg_serve_last_error(const mcg_server* s) { return s ? s->err.c_str() : "null server"; }

int mcg_serve_submit(mcg_server* s, const mcg_engine* model, uint32_t n_iterations, uint64_t* ticket) {
  if (!s || !model || !ticket || n_iterations == 0) return MCG_ERR_ARG;
  if (!s->batch) return sfail(s, MCG_ERR_CUDA, "server has no device engine");
  if (model->dev) return sfail(s, MCG_ERR_ARG, "a submitted model must not have been prepared or stepped");
  if (model->cfg.n_species != s->cfg.n_species) return sfail(s, MCG_ERR_ARG, "model species count differs");
  if (!model->species_set) return sfail(s, MCG_ERR_ARG, "model without mcg_set_species");
  Request r;
  r.t_submit = Clock::now();  // the time to result includes the preparation below
  r.prep.reset(new ReplicaPrep());
  {
    std::string why;
    if (int rc = batch_prepare_replica(model, s->cfg.autotune != 0, *r.prep, why)) return sfail(s, rc, why);
  }
  r.model = *model;
  r.model.err.clear();
  r.n_iterations = n_iterations;
  r.est_bytes = estimate_bytes(*model, s->cfg.precision, r.prep->nsub);
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->failed) return sfail(s, MCG_ERR_CUDA, "server stopped after a device error: " + s->err);
  if (r.est_bytes > s->cfg.hbm_budget_bytes)
    return sfail(s, MCG_ERR_CAPACITY, "request needs more device memory than the whole budget");
  const uint64_t t = s->next_ticket++;
  s->reqs.emplace(t, std::move(r));
  s->queue.push_back(t);
  *ticket = t;
  s->cv_work.notify_all();
  return MCG_OK;
}

int mcg_serve_poll(mcg_server* s, uint64_t ticket, int* state, double* seconds) {
  if (!s || !state) return MCG_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return sfail(s, MCG_ERR_ARG, "unknown ticket");
  *state = it->second.state;
  if (seconds) {
    const bool over = it->second.state == MCG_REQ_DONE || it->second.state == MCG_REQ_CANCELLED;
    const auto end = over ? it->second.t_done : Clock::now();
    *seconds = std::chrono::duration<double>(end - it->second.t_submit).count();
  }
  return MCG_OK;
}

int mcg_serve_wait(mcg_server* s, uint64_t ticket, double timeout_s, int* state) {
  if (!s || !state) return MCG_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return sfail(s, MCG_ERR_ARG, "unknown ticket");
  auto open = [&] {
    const int st = s->reqs[ticket].state;
    return st == MCG_REQ_QUEUED || st == MCG_REQ_RUNNING;
  };
  s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return !open(); });
  *state = s->reqs[ticket].state;
  return MCG_OK;
}

int mcg_serve_result(mcg_server* s, uint64_t ticket, uint64_t* final_counts, uint32_t cap_rows, uint64_t* trajectory,
                     uint32_t* n_rows) {
  if (!s || !n_rows) return MCG_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return sfail(s, MCG_ERR_ARG, "unknown ticket");
  const Request& r = it->second;
  if (r.state == MCG_REQ_FAILED && !r.err.empty()) return sfail(s, MCG_ERR_CUDA, "request failed: " + r.err);
  if (r.state != MCG_REQ_DONE) return sfail(s, MCG_ERR_ARG, "request has no result (not done)");
  const uint32_t nsp = s->cfg.n_species;
  const uint32_t rows = (uint32_t)(r.traj.size() / nsp);
  *n_rows = rows;
  if (final_counts && rows) std::memcpy(final_counts, &r.traj[(size_t)(rows - 1) * nsp], sizeof(uint64_t) * nsp);
  if (trajectory) std::memcpy(trajectory, r.traj.data(), sizeof(uint64_t) * nsp * std::min(rows, cap_rows));
  return MCG_OK;
}

int mcg_serve_cancel(mcg_server* s, uint64_t ticket) {
  if (!s) return MCG_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return sfail(s, MCG_ERR_ARG, "unknown ticket");
  Request& r = it->second;
  if (r.state == MCG_REQ_QUEUED) {
    for (auto q = s->queue.begin(); q != s->queue.end(); ++q)
      if (*q == ticket) {
        s->queue.erase(q);
        break;
      }
    r.state = MCG_REQ_CANCELLED;
    r.t_done = Clock::now();
    s->cv_done.notify_all();
  } else if (r.state == MCG_REQ_RUNNING) {
    r.state = MCG_REQ_CANCELLED;  // collected at the end of the current block
  }
  return MCG_OK;
}

int mcg_serve_release(mcg_server* s, uint64_t ticket) {
  if (!s) return MCG_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return sfail(s, MCG_ERR_ARG, "unknown ticket");
  if (it->second.state == MCG_REQ_QUEUED || it->second.state == MCG_REQ_RUNNING)
    return sfail(s, MCG_ERR_ARG, "request still open (cancel it first)");
  s->reqs.erase(it);
  return MCG_OK;
}

int mcg_serve_get_stats(mcg_server* s, mcg_serve_stats* out) {
  if (!s || !out) return MCG_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  out->queued = s->queue.size();
  out->running = s->running.size();
  out->completed = s->completed;
  out->mol_steps = s->mol_steps;
  out->reserved_bytes = s->reserved;
  out->busy_seconds = s->busy_s;
  out->failed = s->failed ? 1 : 0;
  return MCG_OK;
}

}  // extern "C"
