/*
 * mcell_gb300: GB300 (sm_103a) engine for MCell4's volume-molecule
 * diffuse-react step, behind a C ABI.
 *
 * The engine replaces DiffuseReactEvent::step for volume molecules
 * (src4/diffuse_react_event.cpp:53-64) together with SortMolsBySubpartEvent::step
 * (src4/sort_mols_by_subpart_event.cpp:62-97) and the per-subpartition reactant
 * maps (src4/partition.h:354-418). The host World/Scheduler keeps calling one
 * event per iteration; a GpuDiffuseReactEvent (include/mcell_gb300_event.hpp)
 * forwards it here.
 *
 * Units are MCell4's internal ones: lengths in length_unit (1/sqrt(surface
 * grid density) um, 0.01 um by default), time in time steps (one per
 * iteration). Setup conversions (space steps, reaction probabilities,
 * partition layout) happen on the host before these calls.
 *
 * Conventions: every call returns 0 (MCG_OK) or a negative MCG_ERR_* code;
 * mcg_last_error() gives a message. Handles are not thread-safe; each owns
 * its CUDA stream. No call falls back to a CPU path.
 */
#ifndef MCELL_GB300_H
#define MCELL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCG_OK 0
#define MCG_ERR_ARG (-1)          /* invalid argument or call order */
#define MCG_ERR_CUDA (-2)         /* CUDA runtime error (message has details) */
#define MCG_ERR_CAPACITY (-3)     /* molecule / product / list capacity exceeded */
#define MCG_ERR_ESCAPE (-4)       /* a molecule left the partition (diffuse_react_event.cpp:592-612) */
#define MCG_ERR_WATCHDOG (-5)     /* a bounded device loop gave up (REDO / DDA / resolve rounds) */
#define MCG_ERR_UNSUPPORTED (-6)  /* model feature outside the GPU path (no fallback) */

#define MCG_PRECISION_FP64 0
#define MCG_PRECISION_FP32 1

#define MCG_MAX_SPECIES 16
#define MCG_TRACE_RESULT_SIZE 265 /* doubles per traced case: 9 header + 32 events x 8 */

typedef struct mcg_engine mcg_engine;

/* Replaces the SimulationConfig fields the step reads (src4/simulation_config.h:59-107)
   plus the partition placement of Partition's ctor (src4/partition.cpp:36-60). */
typedef struct mcg_config {
  int precision;                /* MCG_PRECISION_FP64 / MCG_PRECISION_FP32 */
  double partition_origin[3];   /* internal units */
  double partition_edge;        /* internal units */
  uint32_t subparts_per_edge;   /* num_subparts_per_partition_edge (<= 300) */
  double rxn_radius;            /* rxn_radius_3d, internal units */
  uint64_t seed;                /* Config.seed */
  uint64_t capacity;            /* maximum live molecules (0 = 1.5 x first upload) */
  uint32_t n_species;           /* <= MCG_MAX_SPECIES */
} mcg_config;

/* Engine lifetime (World::init_simulation creating the event, src4/world.cpp:280-282). */
int mcg_create(const mcg_config* cfg, mcg_engine** out);
void mcg_destroy(mcg_engine* e);
const char* mcg_last_error(const mcg_engine* e);

/* Species: space step per time step in internal units (Species::space_step as
   set by src/mcell_species.c:270-274); 0 = does not diffuse. */
int mcg_set_species(mcg_engine* e, uint32_t n, const double* space_step);

/* Static mesh (Partition::finalize_walls, src4/partition.cpp:91; wall constants
   src4/wall.cpp:281). wall_class[w * n_species + s]: 0 reflective,
   1 transparent, 2 absorptive for species s at wall w (surface classes,
   libmcell/api/mcell4_converter.cpp:515-575). */
int mcg_upload_mesh(mcg_engine* e, uint32_t n_vertices, const double* vertices, uint32_t n_walls,
                    const uint32_t* walls, const uint8_t* wall_class);

/* Bimolecular vol+vol reaction a+b -> products (-1 = none) with probability p
   (k * pb_factor). The reactions of one reactant pair form its reaction class
   (BNG::RxnClass): each call adds a pathway, in call order, up to MCG_MAX_PATHWAYS;
   the class's cumulative probabilities are what test_bimolecular
   (src4/rxn_utils.inl:336-414) compares with and selects the pathway from
   (max_fixed_p = their sum). A product species that is also a bimolecular
   reactant makes the model unsupported (MCG_ERR_UNSUPPORTED at mcg_prepare,
   mcg_batch_add or mcg_serve_submit): its same-step reactions are not on the path. */
#define MCG_MAX_PATHWAYS 4
int mcg_add_bimol_rxn(mcg_engine* e, uint32_t a, uint32_t b, double p, int32_t product0, int32_t product1);
/* Unimolecular reaction a -> products with k = rate * time_step. Each call adds a
   pathway of a's unimolecular class (up to MCG_MAX_PATHWAYS): the lifetime is drawn
   from their sum (time_of_unimol, src4/rxn_utils.inl:721) and the pathway by
   which_unimolecular (src4/rxn_utils.inl:774-783). */
int mcg_add_unimol_rxn(mcg_engine* e, uint32_t a, double k_tot, int32_t product0, int32_t product1);

/* Volume molecules released before the first iteration (ReleaseEvent::step,
   src4/release_event.cpp:1255). Their ids are given in call order from 0. */
int mcg_add_molecules(mcg_engine* e, uint64_t n, const double* pos, const uint32_t* species);

/* Runs n iterations of the diffuse-react step (DiffuseReactEvent::step, once per
   iteration) without synchronising the host. */
int mcg_step(mcg_engine* e, uint32_t n_iterations);
/* Waits for queued work and reports device-side errors. */
int mcg_sync(mcg_engine* e);

/* Live molecule count per species after the last iteration
   (replaces counting molecules for MolOrRxnCountEvent, src4/mol_or_rxn_count_event.cpp:707). */
int mcg_get_counts(mcg_engine* e, uint64_t* counts /* [n_species] */);
/* Non-blocking counts (no reference counterpart: MolOrRxnCountEvent counts the
   molecules in place). mcg_request_counts queues, after the work queued so far, a
   copy of the counts mcg_get_counts would return now and returns a ticket at once;
   mcg_wait_counts waits for that copy alone, not for iterations queued after the
   request, and returns the counts (device-side errors as mcg_sync reports them).
   A host that requests after each mcg_step and waits for the previous ticket reads
   every iteration's counts while the device runs the next one. Eight tickets can be
   outstanding: a request takes the slot of the ticket eight before it, whose wait
   then fails with MCG_ERR_ARG. */
int mcg_request_counts(mcg_engine* e, uint64_t* ticket);
int mcg_wait_counts(mcg_engine* e, uint64_t ticket, uint64_t* counts /* [n_species] */);
/* Count trajectory: counts after each of the last n iterations run, oldest first
   ([n * n_species]); n <= iterations run since the last mcg_create. */
int mcg_get_count_trajectory(mcg_engine* e, uint32_t n, uint64_t* counts);
/* Copies live molecules out (in subpartition order). Returns the number in *n_out. */
int mcg_download_molecules(mcg_engine* e, uint64_t cap, double* pos, uint32_t* species, uint64_t* ids,
                           uint64_t* n_out);
/* Iterations run, molecule-steps run, and a device status word. */
int mcg_get_stats(mcg_engine* e, uint64_t* iterations, uint64_t* mol_steps, uint64_t* launches);

/* Execution options: use_graphs (replay blocks of two iterations from CUDA graphs,
   default on) and profile (record CUDA events around the kernel groups of each
   iteration; implies no graphs). */
int mcg_set_options(mcg_engine* e, int use_graphs, int profile);
/* Test hook (no counterpart in the reference): the device allocation that follows
   `after` more successful ones, in any engine of the process, fails as if the device
   were out of memory (once; the call returns MCG_ERR_CUDA); a negative value turns it
   off. Lets tests run the out-of-memory paths (no leak, the engine left as it was)
   without exhausting HBM. */
int mcg_inject_device_alloc_failure(int64_t after);
/* Exact fallbacks taken since the engine was prepared (the step's results do not
   depend on them; they cost time): out[0] ray traces with more vol-vol collision
   candidates than one fixed-size page holds (16; the reference's list grows), whose
   later candidates were collected again in time order, page by page; out[1] traces
   whose partner subpartitions overflowed the fixed-size list (48), whose partners
   were then scanned along the walk with repeated candidates dropped. Both restate the
   growable lists of ray_trace_vol / collect_crossed_subparts
   (src4/diffuse_react_event.cpp:627-780, src4/collision_utils_subparts.inl:127-300).
   out[2]: inside tests (counted-volume membership, releases into an object) whose ray
   met a wall edge, where the reference's test stops (its must_redo_test); such a
   molecule is counted outside, such a release point drawn again. */
int mcg_get_fallbacks(mcg_engine* e, uint64_t* out /* [3] */);
/* Test hook (no counterpart in the reference): smaller page and list capacities
   (1..16 candidates, 1..48 subpartitions) so that tests can drive the fallbacks. */
int mcg_set_trace_limits(mcg_engine* e, uint32_t max_candidates, uint32_t max_subparts);
/* Profile since the last call: out[0] iteration ms, [1] diffuse kernel ms, [2] reaction
   resolution ms, [3] products ms, [4] sort (scan + scatter) ms, [5] iterations profiled. */
int mcg_get_profile(mcg_engine* e, double* out);

/* Molecules that left the partition (MCG_ERR_ESCAPE): total in *n and up to
   min(cap, 8) records of 12 doubles: id, species, iteration, start xyz,
   displacement xyz, final xyz. */
int mcg_get_escapes(mcg_engine* e, uint32_t cap, double* out, uint32_t* n);

/* Diagnostics: log every step of one molecule (by id) into a ring of the last 64
   iterations; each record is 271 doubles: the trace result layout of
   mcg_trace_cases (slot 5 holds the iteration), then start xyz and displacement xyz. */
int mcg_debug_molecule(mcg_engine* e, uint64_t id);
int mcg_get_debug_log(mcg_engine* e, double* out /* [64 * 271] */);

/* Per-routine parity harness: one diffusion of a chosen molecule per case with
   the displacement and the random draws injected, through the same device
   functions the step uses (ray_trace_vol + the collision loop of
   diffuse_vol_molecule, src4/diffuse_react_event.cpp:367-780). Molecules
   must have been added and at least mcg_prepare() called. out: n_cases x
   MCG_TRACE_RESULT_SIZE doubles (layout in mcell_gb300/csrc/mcg_device.cuh). */
int mcg_prepare(mcg_engine* e);
int mcg_trace_cases(mcg_engine* e, uint32_t n_cases, const uint64_t* mol_ids, const double* disp,
                    const uint32_t* draws, uint32_t draws_per_case, const double* r_rate_factor,
                    const double* t_steps, double* out);

/* Parity harness of the reaction decisions (no engine; test infrastructure): for
   case c, the device's test_bimolecular (kind 0: a class of n_pathways[c]
   pathways with cumulative probabilities cum_probs[c * MCG_MAX_PATHWAYS ...],
   scaling[c], one injected 32-bit draw; src4/rxn_utils.inl:336-414) or
   which_unimolecular (kind 1: cumulative rates, the draw used only for several
   pathways; src4/rxn_utils.inl:774-783). pathway[c] = the pathway index, or -1
   for no reaction. */
int mcg_reaction_decisions(int kind, uint32_t n, const double* cum_probs, const uint32_t* n_pathways,
                           const double* scaling, const uint32_t* draws, int32_t* pathway);

/* mcg_trace_cases without device allocation. It has no counterpart in the
   reference: it exists for callers that must not allocate device memory while
   they check a model, for example a loop that keeps other engines running on
   the same device (cudaFree waits for the whole device and would stall them)
   or a process whose device memory is fully committed to resident models (an
   allocation could fail half-way). Inputs, results and the id lookup use one
   fixed scratch array per device, built into the library (about 0.6 MB).
   Limits: n_cases <= MCG_TRACE_STATIC_MAX_CASES and
   n_cases * draws_per_case <= MCG_TRACE_STATIC_MAX_DRAWS; larger requests
   return MCG_ERR_ARG without running anything. The engine must be prepared
   (mcg_prepare) with no molecules pending, else MCG_ERR_ARG. The scratch's
   device memory is taken, and its address looked up, when the engine is
   prepared (mcg_prepare or the first mcg_step), not by this call; call it from
   a thread whose current device is the one the engine was prepared on (else
   MCG_ERR_ARG). After a cudaDeviceReset in the process, engines prepared before
   it are invalid, this call included. All handles of a process on one device
   share the one scratch: calls that overlap in time (from several threads)
   race on it and must be serialised by the caller. Same arguments, results and
   errors as mcg_trace_cases. */
#define MCG_TRACE_STATIC_MAX_CASES 256
#define MCG_TRACE_STATIC_MAX_DRAWS 16384
int mcg_trace_cases_static(mcg_engine* e, uint32_t n_cases, const uint64_t* mol_ids, const double* disp,
                           const uint32_t* draws, uint32_t draws_per_case, const double* r_rate_factor,
                           const double* t_steps, double* out);

/* ---- Batching: many independent models (replicas) advanced together.
   The reference runs one model per process; these calls have no counterpart
   there. Each replica is described by an mcg_engine handle that was set up
   with the calls above but never prepared or stepped (mcg_create,
   mcg_set_species, mcg_upload_mesh, mcg_add_*_rxn, mcg_add_molecules); the
   batch copies the description, so the handle may be destroyed afterwards.
   All replicas' molecules live in one set of device arrays: every kernel of an
   iteration runs once over all of them (one persistent diffuse kernel per
   iteration), and blocks of iterations replay from CUDA graphs. A replica's
   random stream depends only on its own seed, molecule ids and iteration
   count, so its results are the same alone and in any mix. */
typedef struct mcg_batch mcg_batch;

typedef struct mcg_batch_config {
  int precision;          /* MCG_PRECISION_FP64 / MCG_PRECISION_FP32 */
  uint32_t n_species;     /* species of every replica (<= MCG_MAX_SPECIES) */
  uint32_t max_replicas;  /* replica slots (<= 65536) */
  uint64_t capacity;      /* molecules over all replicas (0 = grow as needed) */
  int autotune;           /* 1: subpartitions per edge chosen per replica from its density and mesh
                             (a cost model; never finer than the model asks), and the resident
                             blocks of the diffuse kernel timed on the first iterations */
} mcg_batch_config;

/* On MCG_ERR_CUDA (no usable device) *out still receives a handle whose only
   uses are mcg_batch_last_error and mcg_batch_destroy. */
int mcg_batch_create(const mcg_batch_config* cfg, mcg_batch** out);
void mcg_batch_destroy(mcg_batch* b);
const char* mcg_batch_last_error(const mcg_batch* b);
/* Adds n models as replicas; replica k runs n_iterations[k] iterations and then
   freezes (0 = until removed). Slots are written to replica_ids. */
int mcg_batch_add(mcg_batch* b, uint32_t n, mcg_engine* const* models, const uint32_t* n_iterations,
                  uint32_t* replica_ids);
/* Frees replica slots; their molecules are dropped. */
int mcg_batch_remove(mcg_batch* b, uint32_t n, const uint32_t* replica_ids);
/* Runs n iterations of every running replica. */
int mcg_batch_step(mcg_batch* b, uint32_t n_iterations);
int mcg_batch_sync(mcg_batch* b);
/* Iterations a replica has run and the subpartitions per edge it runs with. */
int mcg_batch_replica_info(mcg_batch* b, uint32_t replica, uint64_t* iterations_done, uint32_t* subparts_per_edge);
int mcg_batch_get_counts(mcg_batch* b, uint32_t replica, uint64_t* counts);
int mcg_batch_get_count_trajectory(mcg_batch* b, uint32_t replica, uint32_t n, uint64_t* counts);
int mcg_batch_download_molecules(mcg_batch* b, uint32_t replica, uint64_t cap, double* pos, uint32_t* species,
                                 uint64_t* ids, uint64_t* n_out);
int mcg_batch_get_stats(mcg_batch* b, uint64_t* iterations, uint64_t* mol_steps, uint64_t* launches);
int mcg_batch_set_options(mcg_batch* b, int use_graphs, int profile);
/* As mcg_get_fallbacks, over all replicas. */
int mcg_batch_get_fallbacks(mcg_batch* b, uint64_t* out /* [3] */);
int mcg_batch_get_profile(mcg_batch* b, double* out);
/* Device bytes held by the batch, and the resident blocks per SM the diffuse
   kernel runs with (the autotuner's choice, or the maximum). */
int mcg_batch_get_memory(mcg_batch* b, uint64_t* device_bytes);
int mcg_batch_get_tuning(mcg_batch* b, int* diffuse_blocks_per_sm);
/* As mcg_get_escapes, with a 13th double per record: the replica. */
int mcg_batch_get_escapes(mcg_batch* b, uint32_t cap, double* out, uint32_t* n);
/* The autotuner's subpartition choice for a model (host only, no device):
   subpartitions per edge and whether occupants are binned per octant. */
int mcg_autotune_subparts(const mcg_engine* model, uint32_t* subparts_per_edge, int* octants);

/* ---- Serving: simulation requests that arrive at any time, continuously
   batched on one device (no counterpart in the reference). A worker thread
   owns a batch; between blocks of iterations it admits queued requests, first
   come first served, as replica slots and the device-memory budget allow, runs
   every admitted request in the same kernels, and collects the requests that
   reached their iteration count. A request's molecules, mesh and partition stay
   resident on the device from admission to its last iteration. Results (the
   species-count trajectory) are the same as the model run alone. The model
   handle is copied at submission and may be destroyed afterwards. */
typedef struct mcg_server mcg_server;

typedef struct mcg_server_config {
  int precision;              /* MCG_PRECISION_FP64 / MCG_PRECISION_FP32 */
  uint32_t n_species;         /* species of every request */
  uint32_t max_slots;         /* requests on the device at once (<= 65536) */
  uint64_t hbm_budget_bytes;  /* device memory the admitted requests may hold (estimated per request) */
  int autotune;               /* as mcg_batch_config.autotune */
} mcg_server_config;

#define MCG_REQ_QUEUED 0
#define MCG_REQ_RUNNING 1
#define MCG_REQ_DONE 2
#define MCG_REQ_CANCELLED 3
#define MCG_REQ_FAILED 4

typedef struct mcg_serve_stats {
  uint64_t queued, running, completed;
  uint64_t mol_steps;       /* molecule-steps run by the server */
  uint64_t reserved_bytes;  /* budget held by running requests */
  double busy_seconds;      /* wall time spent in blocks of iterations */
  int failed;               /* 1 after a device error (every open request failed) */
} mcg_serve_stats;

/* On MCG_ERR_CUDA *out still receives a handle for mcg_serve_last_error /
   mcg_serve_destroy. */
int mcg_serve_create(const mcg_server_config* cfg, mcg_server** out);
/* Stops the worker (open requests are abandoned) and frees everything. */
void mcg_serve_destroy(mcg_server* s);
const char* mcg_serve_last_error(const mcg_server* s);
/* Queues a copy of the model for n_iterations. The host half of its admission (its
   subpartition grid, autotuned when the server autotunes, and its wall constants
   and lists: milliseconds for a mesh of thousands of walls) is done here, in the
   caller's thread, so that the worker keeps the device busy; a request's time to
   result starts at this call. */
int mcg_serve_submit(mcg_server* s, const mcg_engine* model, uint32_t n_iterations, uint64_t* ticket);
/* State of a request and seconds from submission to its result (or until now). */
int mcg_serve_poll(mcg_server* s, uint64_t ticket, int* state, double* seconds);
/* Blocks until the request is no longer queued or running, or timeout_s passes. */
int mcg_serve_wait(mcg_server* s, uint64_t ticket, double timeout_s, int* state);
/* Result of a finished request: counts after its last iteration ([n_species]) and
   its count trajectory (up to cap_rows rows of n_species, one per iteration);
   *n_rows = its iteration count. */
int mcg_serve_result(mcg_server* s, uint64_t ticket, uint64_t* final_counts, uint32_t cap_rows, uint64_t* trajectory,
                     uint32_t* n_rows);
/* Queued requests leave the queue; running ones stop at the end of the current block. */
int mcg_serve_cancel(mcg_server* s, uint64_t ticket);
/* Forgets a finished, cancelled or failed request (frees its host result). */
int mcg_serve_release(mcg_server* s, uint64_t ticket);
int mcg_serve_get_stats(mcg_server* s, mcg_serve_stats* out);

/* ---- Volume releases generated on the device (ReleaseEvent::
   release_ellipsoid_or_rectcuboid and release_inside_regions,
   src4/release_event.cpp:904-1006): n molecules of a species, uniform in an
   ellipsoid, a cuboid or on an ellipsoid shell (center and diameter, internal
   units), or inside a closed geometry object (rejection in the object's bounding
   box with the reference's ray-parity inside test). The random numbers come from
   the counter-based generator keyed by release_seed, so positions are not the
   reference's; their distribution is. Molecule ids continue the model's. The
   region must lie inside the partition. Walls are assigned to objects with
   mcg_set_wall_objects (before the first step). The positions follow the reference's
   arithmetic from the draws (mcg_release_positions gives them on injected draws); the
   inside test is the reference's (mcg_inside_tests). */
#define MCG_RELEASE_SPHERE 0
#define MCG_RELEASE_CUBOID 1
#define MCG_RELEASE_SHELL 2
#define MCG_RELEASE_INSIDE_OBJECT 3
int mcg_set_wall_objects(mcg_engine* e, uint32_t n_walls, const uint16_t* object_of_wall);
int mcg_release(mcg_engine* e, uint32_t species, uint64_t n, int shape, const double* center, const double* diameter,
                uint32_t object, uint64_t release_seed);
int mcg_batch_release(mcg_batch* b, uint32_t replica, uint32_t species, uint64_t n, int shape, const double* center,
                      const double* diameter, uint32_t object, uint64_t release_seed);

/* Parity harness of the inside tests (test infrastructure; the engine must have its
   wall objects, and for kind 0 its counted objects): for each point, kind 0 the
   counted-volume bits (bit q: inside counted object q; compute_counted_volume_for_pos,
   src4/collision_utils.inl:1515-1545), kind 1 whether it lies inside geometry object
   `object` (is_point_inside_region_no_waypoints, src4/collision_utils.inl:1484-1510);
   0xFFFFFFFF where the ray met a wall edge. */
int mcg_inside_tests(mcg_engine* e, uint32_t n, const double* pos, int kind, uint32_t object, uint32_t* out);
/* Parity harness of the volume releases (no engine; test infrastructure): n positions
   of ReleaseEvent::release_ellipsoid_or_rectcuboid (src4/release_event.cpp:953-1000)
   for shape MCG_RELEASE_SPHERE / _CUBOID / _SHELL, drawing from one injected stream
   of 32-bit draws as the reference's generator would; *draws_used = the draws it took
   (0xFFFFFFFF if the stream ran out). */
int mcg_release_positions(int shape, uint32_t n, const double* center, const double* diameter, const uint32_t* draws,
                          uint32_t n_draws, double* pos, uint32_t* draws_used);

/* ---- Releases into region expressions, by concentration, and vacuum releases
   (ReleaseEvent::release_inside_regions, src4/release_event.cpp:904-952, with
   is_point_inside_region_expr_recursively :785-810, num_vol_mols_from_conc :826-856,
   vacuum_inside_regions :864-896, randomly_remove_molecules :578-597).
   A region expression is a postfix program of at most 15 tokens: a geometry object
   index (>= 0, objects as given to mcg_set_wall_objects) or one of the operators
   below, which combine the two results before it; e.g. {1, 0, MCG_REGION_DIFFERENCE}
   is "inside object 1 and not inside object 0". */
#define MCG_REGION_UNION (-1)
#define MCG_REGION_INTERSECT (-2)
#define MCG_REGION_DIFFERENCE (-3)
#define MCG_RELEASE_BY_NUMBER 0
#define MCG_RELEASE_BY_CONCENTRATION 1
/* Volume of the closed object `object` of a mesh (Region::initialize_volume_info_if_needed,
   src4/geometry.cpp:860-897: tetrahedra of its faces, in wall order, with the center of
   its bounding box; internal units cubed). Host only. */
int mcg_object_volume(uint32_t n_verts, const double* verts, uint32_t n_walls, const uint32_t* walls,
                      const uint16_t* object_of_wall, uint32_t object, double* volume);
/* Bounding box of a region expression (compute_region_expr_bounding_box,
   src4/geometry.cpp:1180-1265): union widens, intersection narrows, difference keeps the
   left operand's box. Host only. */
int mcg_region_expr_bbox(uint32_t n_verts, const double* verts, uint32_t n_walls, const uint32_t* walls,
                         const uint16_t* object_of_wall, const int32_t* expr, uint32_t n_expr, double* llf,
                         double* urb);
/* Molecules a release of a molar concentration into a sphere of the given diameter
   (internal units) places (calculate_number_to_release, src4/release_event.cpp:509-553);
   length_unit_um = microns per internal unit. Host only. */
int mcg_release_number_from_concentration(const double* diameter, double concentration_molar, double length_unit_um,
                                          uint64_t* n);
/* The vacuum's choice (randomly_remove_molecules) of n_remove of m candidates, in
   candidate order, drawing from an injected stream of 32-bit draws (one per candidate);
   removed[i] = 1 for the chosen. Parity harness and host logic; host only. */
int mcg_vacuum_select(uint32_t m, uint32_t n_remove, const uint32_t* draws, uint32_t n_draws, uint8_t* removed,
                      uint32_t* draws_used);
/* Release into, or vacuum from, a region expression of the model's closed objects.
   method MCG_RELEASE_BY_NUMBER: number > 0 places that many molecules of the species,
   uniform in the expression (rejection in its bounding box with the reference's inside
   tests, a point whose ray meets a wall edge drawn again); number < 0 removes up to
   -number molecules of the species that lie inside (candidates in id order, the
   reference's choice; the draws come from a generator keyed by release_seed).
   method MCG_RELEASE_BY_CONCENTRATION: the count is the reference's from the molar
   concentration: for a single object from its volume, and all those molecules are
   placed; for an expression from its bounding box's volume, each of those draws placing
   a molecule only if it falls inside (as the reference's approximate count does).
   *done = molecules placed, or removed (negative). Molecule ids continue the model's. */
int mcg_release_region(mcg_engine* e, uint32_t species, int method, int64_t number, double concentration_molar,
                       double length_unit_um, const int32_t* expr, uint32_t n_expr, uint64_t release_seed,
                       int64_t* done);
/* The same for one replica of a batch (the objects of that replica's model). */
int mcg_batch_release_region(mcg_batch* b, uint32_t replica, uint32_t species, int method, int64_t number,
                             double concentration_molar, double length_unit_um, const int32_t* expr, uint32_t n_expr,
                             uint64_t release_seed, int64_t* done);
/* Parity harness of release_inside_regions (test infrastructure): the positions the
   release above would place, computed in one device thread from one injected stream of
   32-bit draws as the reference's generator would be consumed (number < 0: the indices,
   in id order, of the molecules the vacuum removes, in `removed`, nothing changed).
   *n_pos / *n_removed = how many were written; *draws_used (0xFFFFFFFF if the stream
   ran out). */
int mcg_release_region_harness(mcg_engine* e, uint32_t species, int method, int64_t number,
                               double concentration_molar, double length_unit_um, const int32_t* expr,
                               uint32_t n_expr, const uint32_t* draws, uint32_t n_draws, double* pos, uint32_t cap,
                               uint32_t* n_pos, uint64_t* removed, uint32_t* n_removed, uint32_t* draws_used);

/* ---- Counted volumes: molecules inside closed geometry objects, per species, for
   MolOrRxnCountEvent (src4/mol_or_rxn_count_event.cpp:707). As MCell4's counted-
   volume index, each molecule carries its membership (up to 7 counted objects per
   model), set at upload or release by the reference's ray-parity test
   (compute_counted_volume_for_pos, src4/collision_utils.inl:1515-1545) and set at
   every crossing of a (transparent) wall of a counted object: inside after a hit on
   its front face, outside after a hit on its back face
   (update_counted_volume_id_when_crossing_wall, src4/collision_utils.inl:1637-1694);
   products inherit their reactant's. Objects are named by the ids of mcg_set_wall_objects; set
   before the first step. Counts: [n_species][n_counted] after the last iteration
   or upload; trajectory: [n][n_species][n_counted] for the last n iterations. */
int mcg_set_counted_objects(mcg_engine* e, uint32_t n, const uint16_t* objects);
int mcg_get_counted_volume_counts(mcg_engine* e, uint64_t* counts);
int mcg_get_counted_volume_trajectory(mcg_engine* e, uint32_t n_iterations, uint64_t* counts);

/* ---- Checkpoints (the device side of ChkptVolMol, libmcell/api/model.cpp:591-650).
   A checkpoint is the live molecules — position, species, id, unimolecular time
   relative to the next iteration (1e20 = none), flags (bit 0: the unimolecular time
   is not drawn yet; bits 1-7: inside counted object k) — and the iteration counter. With the same model definition and
   seed, a run continued from it repeats the uninterrupted run (the random streams
   are counter based: seed, molecule id, iteration). mcg_export_state: call with
   cap = 0 for the count, then with arrays of that size. mcg_import_state: on a
   handle that has no molecules and has not run an iteration; it prepares the
   engine. */
int mcg_export_state(mcg_engine* e, uint64_t cap, double* pos, uint32_t* species, uint64_t* ids,
                     double* unimol_time, uint8_t* flags, uint64_t* n_out, uint64_t* iteration);
int mcg_import_state(mcg_engine* e, uint64_t n, const double* pos, const uint32_t* species, const uint64_t* ids,
                     const double* unimol_time, const uint8_t* flags, uint64_t iteration);

/* ---- Visualisation output from device state (VizOutputEvent,
   src4/viz_output_event.cpp:48-279): writes
   "<prefix>.ascii.<iteration>.dat" (lines "name id x y z nx ny nz") or
   "<prefix>.cellbin.<iteration>.dat" (CellBlender binary, version 1 or 2), with
   positions in um (internal units x length_unit_um) and the iteration zero-padded
   to the digits of total_iterations. species_names: n_species strings. */
#define MCG_VIZ_ASCII 0
#define MCG_VIZ_CELLBLENDER_V1 1
#define MCG_VIZ_CELLBLENDER_V2 2
int mcg_write_viz(mcg_engine* e, const char* prefix, int mode, const char* const* species_names, uint64_t iteration,
                  uint64_t total_iterations, double length_unit_um);
int mcg_batch_write_viz(mcg_batch* b, uint32_t replica, const char* prefix, int mode,
                        const char* const* species_names, uint64_t iteration, uint64_t total_iterations,
                        double length_unit_um);

/* ---- Count output from device counts (MolOrRxnCountEvent::compute_counts and
   CountBuffer, src4/mol_or_rxn_count_event.cpp:607-700, src4/count_buffer.cpp:30-128):
   for the last n_iterations iterations, those whose number of iterations run is a
   multiple of `every`, the counts at time (iterations run) x time_step_s, as DAT files
   ("<prefix>.<name>.dat", lines "time value", C++ stream defaults) or one GDAT file
   ("<prefix>.gdat": a '#' header of right-aligned names, then per row the time and the
   values in scientific notation, 8 decimals, two-digit exponents). Column k counts
   species[k] in the whole world (objects[k] = -1) or inside counted object objects[k]
   (an index into the list given to mcg_set_counted_objects), named names[k]. A window
   that reaches back to the model's first iteration (n_iterations = all iterations
   run) starts with a row at time 0: the counts before the first iteration, after the
   uploads and releases, as the reference's count event runs before the diffusion
   event in iteration 0. */
#define MCG_COUNTS_DAT 0
#define MCG_COUNTS_GDAT 1
int mcg_write_counts(mcg_engine* e, const char* prefix, int format, uint32_t n_iterations, uint32_t every,
                     double time_step_s, uint32_t n_columns, const uint32_t* species, const int32_t* objects,
                     const char* const* names);
/* The same for one replica of a batch; a replica frozen after its iteration budget
   keeps its last counts in the later rows (times count from its admission). */
int mcg_batch_write_counts(mcg_batch* b, uint32_t replica, const char* prefix, int format, uint32_t n_iterations,
                           uint32_t every, double time_step_s, uint32_t n_columns, const uint32_t* species,
                           const int32_t* objects, const char* const* names);

/* Setup queries for parity tests: wall constants (14 doubles per wall, same
   layout as the oracle) and the wall lists per subpartition. */
int mcg_wall_consts(mcg_engine* e, double* out);
int mcg_walls_in_subparts(mcg_engine* e, uint32_t* counts, uint32_t* list, uint64_t cap, uint64_t* total);

#ifdef __cplusplus
}
#endif
#endif
