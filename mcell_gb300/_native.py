"""ctypes binding of the engine's C ABI (include/mcell_gb300.h).

The library is built in-tree by mcell_gb300.build into mcell_gb300/_lib/. There is
no CPU fallback: if the library is missing or cannot be loaded, every call
raises.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libmcell_gb300.so"

MCG_OK = 0
ERRORS = {-1: "MCG_ERR_ARG", -2: "MCG_ERR_CUDA", -3: "MCG_ERR_CAPACITY", -4: "MCG_ERR_ESCAPE",
          -5: "MCG_ERR_WATCHDOG", -6: "MCG_ERR_UNSUPPORTED"}
PRECISION = {"fp64": 0, "fp32": 1}
TRACE_RESULT_SIZE = 265

# every entry point declared in include/mcell_gb300.h
EXPORTS = [
    "mcg_create", "mcg_destroy", "mcg_last_error", "mcg_set_species", "mcg_upload_mesh", "mcg_add_bimol_rxn",
    "mcg_add_unimol_rxn", "mcg_add_molecules", "mcg_step", "mcg_sync", "mcg_get_counts",
    "mcg_request_counts", "mcg_wait_counts", "mcg_get_count_trajectory", "mcg_download_molecules", "mcg_get_stats", "mcg_prepare", "mcg_trace_cases",
    "mcg_wall_consts", "mcg_walls_in_subparts", "mcg_set_options", "mcg_inject_device_alloc_failure", "mcg_get_profile",
    "mcg_get_escapes", "mcg_debug_molecule", "mcg_get_debug_log", "mcg_trace_cases_static",
    "mcg_batch_create", "mcg_batch_destroy", "mcg_batch_last_error", "mcg_batch_add", "mcg_batch_remove",
    "mcg_batch_step", "mcg_batch_sync", "mcg_batch_replica_info", "mcg_batch_get_counts",
    "mcg_batch_get_count_trajectory", "mcg_batch_download_molecules", "mcg_batch_get_stats",
    "mcg_batch_set_options", "mcg_batch_get_profile", "mcg_batch_get_memory", "mcg_batch_get_tuning",
    "mcg_autotune_subparts", "mcg_batch_get_escapes",
    "mcg_serve_create", "mcg_serve_destroy", "mcg_serve_last_error", "mcg_serve_submit", "mcg_serve_poll",
    "mcg_serve_wait", "mcg_serve_result", "mcg_serve_cancel", "mcg_serve_release", "mcg_serve_get_stats",
    "mcg_export_state", "mcg_import_state", "mcg_write_viz", "mcg_batch_write_viz", "mcg_write_counts", "mcg_batch_write_counts",
    "mcg_set_wall_objects", "mcg_release", "mcg_batch_release", "mcg_set_counted_objects",
    "mcg_get_counted_volume_counts", "mcg_get_counted_volume_trajectory",
    "mcg_get_fallbacks", "mcg_set_trace_limits", "mcg_batch_get_fallbacks", "mcg_reaction_decisions",
    "mcg_inside_tests", "mcg_release_positions",
    "mcg_object_volume", "mcg_region_expr_bbox", "mcg_release_number_from_concentration", "mcg_vacuum_select",
    "mcg_release_region", "mcg_release_region_harness", "mcg_batch_release_region",
]
REGION_OPS = {"union": -1, "intersect": -2, "difference": -3}
MAX_PATHWAYS = 4


class McgConfig(ctypes.Structure):
    _fields_ = [
        ("precision", ctypes.c_int),
        ("partition_origin", ctypes.c_double * 3),
        ("partition_edge", ctypes.c_double),
        ("subparts_per_edge", ctypes.c_uint32),
        ("rxn_radius", ctypes.c_double),
        ("seed", ctypes.c_uint64),
        ("capacity", ctypes.c_uint64),
        ("n_species", ctypes.c_uint32),
    ]


class McgBatchConfig(ctypes.Structure):
    _fields_ = [
        ("precision", ctypes.c_int),
        ("n_species", ctypes.c_uint32),
        ("max_replicas", ctypes.c_uint32),
        ("capacity", ctypes.c_uint64),
        ("autotune", ctypes.c_int),
    ]


class McgServerConfig(ctypes.Structure):
    _fields_ = [
        ("precision", ctypes.c_int),
        ("n_species", ctypes.c_uint32),
        ("max_slots", ctypes.c_uint32),
        ("hbm_budget_bytes", ctypes.c_uint64),
        ("autotune", ctypes.c_int),
    ]


class McgServeStats(ctypes.Structure):
    _fields_ = [
        ("queued", ctypes.c_uint64),
        ("running", ctypes.c_uint64),
        ("completed", ctypes.c_uint64),
        ("mol_steps", ctypes.c_uint64),
        ("reserved_bytes", ctypes.c_uint64),
        ("busy_seconds", ctypes.c_double),
        ("failed", ctypes.c_int),
    ]


REQ_STATES = {0: "queued", 1: "running", 2: "done", 3: "cancelled", 4: "failed"}


class EngineError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run mcell_gb300.build (nvcc, sm_103a) first")
        L = ctypes.CDLL(str(LIB_PATH))
        vp = ctypes.c_void_p
        L.mcg_create.argtypes = [ctypes.POINTER(McgConfig), ctypes.POINTER(vp)]
        L.mcg_destroy.argtypes = [vp]
        L.mcg_destroy.restype = None
        L.mcg_last_error.argtypes = [vp]
        L.mcg_last_error.restype = ctypes.c_char_p
        L.mcg_batch_create.argtypes = [ctypes.POINTER(McgBatchConfig), ctypes.POINTER(vp)]
        L.mcg_batch_destroy.argtypes = [vp]
        L.mcg_batch_destroy.restype = None
        L.mcg_batch_last_error.argtypes = [vp]
        L.mcg_batch_last_error.restype = ctypes.c_char_p
        L.mcg_serve_create.argtypes = [ctypes.POINTER(McgServerConfig), ctypes.POINTER(vp)]
        L.mcg_serve_destroy.argtypes = [vp]
        L.mcg_serve_destroy.restype = None
        L.mcg_serve_last_error.argtypes = [vp]
        L.mcg_serve_last_error.restype = ctypes.c_char_p
        L.mcg_serve_wait.argtypes = [vp, ctypes.c_uint64, ctypes.c_double, ctypes.POINTER(ctypes.c_int)]
        for name in EXPORTS:
            getattr(L, name)
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def inject_device_alloc_failure(after):
    """Test hook: the device allocation after `after` more successful ones fails as if
    out of memory (once); None or a negative value turns it off."""
    lib().mcg_inject_device_alloc_failure(ctypes.c_int64(-1 if after is None else int(after)))


def reaction_decisions(kind, cum, scaling, draws):
    """Device reaction decisions on injected draws (mcg_reaction_decisions): kind
    "bimol" (test_bimolecular) or "unimol" (which_unimolecular); cum: one list of
    cumulative pathway values per case. Returns the pathway per case, -1 = none."""
    n = len(cum)
    c = np.zeros((n, MAX_PATHWAYS))
    npw = np.zeros(n, np.uint32)
    for i, row in enumerate(cum):
        c[i, :len(row)] = row
        npw[i] = len(row)
    sc = np.ascontiguousarray(np.zeros(n) if scaling is None else scaling, np.float64)
    dr = np.ascontiguousarray(draws, np.uint32)
    out = np.zeros(n, np.int32)
    rc = lib().mcg_reaction_decisions(ctypes.c_int({"bimol": 0, "unimol": 1}[kind]), ctypes.c_uint32(n), _p(c),
                                      _p(npw), _p(sc), _p(dr), _p(out))
    if rc:
        raise EngineError(rc, "mcg_reaction_decisions failed")
    return out


def release_positions(shape, n, center, diameter, draws):
    """Device release positions on an injected stream (mcg_release_positions): shape
    "sphere", "cuboid" or "shell". Returns (positions [n, 3], draws used or None)."""
    out = np.zeros((n, 3))
    c = np.ascontiguousarray(center, np.float64)
    d = np.ascontiguousarray(diameter, np.float64)
    dr = np.ascontiguousarray(draws, np.uint32)
    used = ctypes.c_uint32()
    rc = lib().mcg_release_positions(ctypes.c_int({"sphere": 0, "cuboid": 1, "shell": 2}[shape]), ctypes.c_uint32(n),
                                     _p(c), _p(d), _p(dr), ctypes.c_uint32(len(dr)), _p(out), ctypes.byref(used))
    if rc:
        raise EngineError(rc, "mcg_release_positions failed")
    return out, (None if used.value == 0xFFFFFFFF else int(used.value))


def _mesh_args(verts, walls, object_of_wall):
    v = np.ascontiguousarray(verts, np.float64)
    w = np.ascontiguousarray(walls, np.uint32)
    o = np.ascontiguousarray(object_of_wall, np.uint16)
    return (v, w, o), (ctypes.c_uint32(len(v)), _p(v), ctypes.c_uint32(len(w)), _p(w), _p(o))


def region_expr(tokens):
    """A region expression as the C ABI's postfix program: object indices and the
    operator names "union", "intersect", "difference"."""
    return np.array([REGION_OPS[t] if isinstance(t, str) else int(t) for t in tokens], np.int32)


def object_volume(verts, walls, object_of_wall, obj):
    """Volume of a closed object of a mesh (mcg_object_volume; host only)."""
    keep, args = _mesh_args(verts, walls, object_of_wall)
    out = ctypes.c_double()
    rc = lib().mcg_object_volume(*args, ctypes.c_uint32(obj), ctypes.byref(out))
    if rc:
        raise EngineError(rc, "mcg_object_volume failed")
    return out.value


def region_expr_bbox(verts, walls, object_of_wall, tokens):
    """(llf, urb) of a region expression (mcg_region_expr_bbox; host only)."""
    keep, args = _mesh_args(verts, walls, object_of_wall)
    ex = region_expr(tokens)
    lo, hi = np.zeros(3), np.zeros(3)
    rc = lib().mcg_region_expr_bbox(*args, _p(ex), ctypes.c_uint32(len(ex)), _p(lo), _p(hi))
    if rc:
        raise EngineError(rc, "mcg_region_expr_bbox failed")
    return lo, hi


def release_number_from_concentration(diameter, concentration, length_unit_um):
    """Molecules a molar concentration places in a sphere (mcg_release_number_from_concentration)."""
    d = np.ascontiguousarray(diameter, np.float64)
    n = ctypes.c_uint64()
    rc = lib().mcg_release_number_from_concentration(_p(d), ctypes.c_double(concentration),
                                                     ctypes.c_double(length_unit_um), ctypes.byref(n))
    if rc:
        raise EngineError(rc, "mcg_release_number_from_concentration failed")
    return n.value


def vacuum_select(m, n_remove, draws):
    """The vacuum's choice of n_remove of m candidates on injected draws (mcg_vacuum_select):
    (0/1 per candidate, draws used or None)."""
    dr = np.ascontiguousarray(draws, np.uint32)
    out = np.zeros(max(m, 1), np.uint8)
    used = ctypes.c_uint32()
    rc = lib().mcg_vacuum_select(ctypes.c_uint32(m), ctypes.c_uint32(n_remove), _p(dr), ctypes.c_uint32(len(dr)),
                                 _p(out), ctypes.byref(used))
    if rc:
        raise EngineError(rc, "mcg_vacuum_select failed")
    return out[:m], (None if used.value == 0xFFFFFFFF else int(used.value))


class Engine:
    """One GPU model: thin object over the C ABI (same calls a C++ host makes)."""

    def __init__(self, precision, origin, partition_edge, nsub, rxn_radius, n_species, seed=1, capacity=0):
        L = lib()
        cfg = McgConfig()
        cfg.precision = PRECISION[precision] if isinstance(precision, str) else int(precision)
        for k in range(3):
            cfg.partition_origin[k] = float(origin[k])
        cfg.partition_edge = float(partition_edge)
        cfg.subparts_per_edge = int(nsub)
        cfg.rxn_radius = float(rxn_radius)
        cfg.seed = int(seed)
        cfg.capacity = int(capacity)
        cfg.n_species = int(n_species)
        h = ctypes.c_void_p()
        rc = L.mcg_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != MCG_OK:
            raise EngineError(rc, "mcg_create rejected the configuration")
        self.h = h
        self.n_species = int(n_species)

    def close(self):
        if getattr(self, "h", None):
            lib().mcg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc):
        if rc != MCG_OK:
            msg = lib().mcg_last_error(self.h)
            raise EngineError(rc, msg.decode() if msg else "")

    def set_species(self, space_steps):
        a = np.ascontiguousarray(space_steps, np.float64)
        self._chk(lib().mcg_set_species(self.h, ctypes.c_uint32(len(a)), _p(a)))

    def upload_mesh(self, verts, walls, wall_class):
        v = np.ascontiguousarray(verts, np.float64)
        w = np.ascontiguousarray(walls, np.uint32)
        c = np.ascontiguousarray(wall_class, np.uint8)
        self._chk(lib().mcg_upload_mesh(self.h, ctypes.c_uint32(len(v)), _p(v), ctypes.c_uint32(len(w)), _p(w), _p(c)))

    def add_bimol_rxn(self, a, b, p, products=(-1, -1)):
        pr = list(products) + [-1] * (2 - len(products))
        self._chk(lib().mcg_add_bimol_rxn(self.h, ctypes.c_uint32(a), ctypes.c_uint32(b), ctypes.c_double(p),
                                          ctypes.c_int32(pr[0]), ctypes.c_int32(pr[1])))

    def add_unimol_rxn(self, a, k, products=(-1, -1)):
        pr = list(products) + [-1] * (2 - len(products))
        self._chk(lib().mcg_add_unimol_rxn(self.h, ctypes.c_uint32(a), ctypes.c_double(k), ctypes.c_int32(pr[0]),
                                           ctypes.c_int32(pr[1])))

    def add_molecules(self, pos, species):
        p = np.ascontiguousarray(pos, np.float64)
        s = np.ascontiguousarray(species, np.uint32)
        self._chk(lib().mcg_add_molecules(self.h, ctypes.c_uint64(len(s)), _p(p), _p(s)))

    def prepare(self):
        self._chk(lib().mcg_prepare(self.h))

    def step(self, n=1):
        self._chk(lib().mcg_step(self.h, ctypes.c_uint32(n)))

    def sync(self):
        self._chk(lib().mcg_sync(self.h))

    def counts(self):
        out = np.zeros(self.n_species, np.uint64)
        self._chk(lib().mcg_get_counts(self.h, _p(out)))
        return out

    def trajectory(self, n):
        out = np.zeros((n, self.n_species), np.uint64)
        self._chk(lib().mcg_get_count_trajectory(self.h, ctypes.c_uint32(n), _p(out)))
        return out

    def request_counts(self):
        """Queue a copy of the counts after the work queued so far; returns a ticket at once."""
        t = ctypes.c_uint64()
        self._chk(lib().mcg_request_counts(self.h, ctypes.byref(t)))
        return t.value

    def wait_counts(self, ticket):
        """The counts of a request, waiting for its copy only (not for later iterations)."""
        out = np.zeros(self.n_species, np.uint64)
        self._chk(lib().mcg_wait_counts(self.h, ctypes.c_uint64(ticket), _p(out)))
        return out

    def molecules(self, cap=None):
        n = ctypes.c_uint64()
        self._chk(lib().mcg_download_molecules(self.h, ctypes.c_uint64(0), None, None, None, ctypes.byref(n)))
        m = n.value if cap is None else min(cap, n.value)
        pos = np.zeros((m, 3))
        sp = np.zeros(m, np.uint32)
        ids = np.zeros(m, np.uint64)
        self._chk(lib().mcg_download_molecules(self.h, ctypes.c_uint64(m), _p(pos), _p(sp), _p(ids), ctypes.byref(n)))
        return pos, sp, ids

    def stats(self):
        it, ms, ln = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        self._chk(lib().mcg_get_stats(self.h, ctypes.byref(it), ctypes.byref(ms), ctypes.byref(ln)))
        return it.value, ms.value, ln.value

    def set_options(self, use_graphs=True, profile=False):
        self._chk(lib().mcg_set_options(self.h, ctypes.c_int(int(use_graphs)), ctypes.c_int(int(profile))))

    def fallbacks(self):
        """(traces that refilled a full candidate page, traces that scanned partners along the
        walk, inside tests whose ray met a wall edge)."""
        out = np.zeros(3, np.uint64)
        self._chk(lib().mcg_get_fallbacks(self.h, _p(out)))
        return int(out[0]), int(out[1]), int(out[2])

    def inside_tests(self, pos, kind, obj=0):
        """mcg_inside_tests: kind "counted" (counted-volume bits) or "object" (inside obj)."""
        p = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        out = np.zeros(len(p), np.uint32)
        self._chk(lib().mcg_inside_tests(self.h, ctypes.c_uint32(len(p)), _p(p),
                                         ctypes.c_int({"counted": 0, "object": 1}[kind]), ctypes.c_uint32(obj),
                                         _p(out)))
        return out

    def set_trace_limits(self, max_candidates, max_subparts):
        """Test hook: smaller candidate page / partner list capacities (drives the fallbacks)."""
        self._chk(lib().mcg_set_trace_limits(self.h, ctypes.c_uint32(max_candidates), ctypes.c_uint32(max_subparts)))

    def profile(self):
        """ms since the last call: iteration, diffuse, reactions, products, sort; iterations profiled"""
        out = np.zeros(6)
        self._chk(lib().mcg_get_profile(self.h, _p(out)))
        return out

    def escapes(self):
        out = np.zeros((8, 12))
        n = ctypes.c_uint32()
        rc = lib().mcg_get_escapes(self.h, ctypes.c_uint32(8), _p(out), ctypes.byref(n))
        self._chk(rc)
        return n.value, out[:min(8, n.value)]

    def debug_molecule(self, uid):
        self._chk(lib().mcg_debug_molecule(self.h, ctypes.c_uint64(uid)))

    def debug_log(self):
        out = np.zeros((64, 271))
        self._chk(lib().mcg_get_debug_log(self.h, _p(out)))
        return out

    def trace_cases(self, ids, disp, draws, r_rate_factor=None, t_steps=None):
        ids = np.ascontiguousarray(ids, np.uint64)
        n = len(ids)
        disp = np.ascontiguousarray(disp, np.float64).reshape(n, 3)
        draws = np.ascontiguousarray(draws, np.uint32).reshape(n, -1)
        rrf = np.ascontiguousarray(np.ones(n) if r_rate_factor is None else r_rate_factor, np.float64)
        tst = np.ascontiguousarray(np.ones(n) if t_steps is None else t_steps, np.float64)
        out = np.zeros((n, TRACE_RESULT_SIZE))
        self._chk(lib().mcg_trace_cases(self.h, ctypes.c_uint32(n), _p(ids), _p(disp), _p(draws),
                                        ctypes.c_uint32(draws.shape[1]), _p(rrf), _p(tst), _p(out)))
        return out

    def set_wall_objects(self, object_of_wall):
        o = np.ascontiguousarray(object_of_wall, np.uint16)
        self._chk(lib().mcg_set_wall_objects(self.h, ctypes.c_uint32(len(o)), _p(o)))

    def set_counted_objects(self, objects):
        o = np.ascontiguousarray(objects, np.uint16)
        self.n_counted = len(o)
        self._chk(lib().mcg_set_counted_objects(self.h, ctypes.c_uint32(len(o)), _p(o)))

    def counted_counts(self):
        out = np.zeros((self.n_species, self.n_counted), np.uint64)
        self._chk(lib().mcg_get_counted_volume_counts(self.h, _p(out)))
        return out

    def counted_trajectory(self, n):
        out = np.zeros((n, self.n_species, self.n_counted), np.uint64)
        self._chk(lib().mcg_get_counted_volume_trajectory(self.h, ctypes.c_uint32(n), _p(out)))
        return out

    def release(self, species, n, shape="sphere", center=(0, 0, 0), diameter=(1, 1, 1), obj=0, seed=1):
        shapes = {"sphere": 0, "cuboid": 1, "shell": 2, "inside": 3}
        c = np.ascontiguousarray(center, np.float64)
        d = np.ascontiguousarray(diameter, np.float64)
        self._chk(lib().mcg_release(self.h, ctypes.c_uint32(species), ctypes.c_uint64(n), ctypes.c_int(shapes[shape]),
                                    _p(c), _p(d), ctypes.c_uint32(obj), ctypes.c_uint64(seed)))

    def release_region(self, species, tokens, number=0, concentration=None, length_unit_um=0.01, seed=1):
        """Release into (number > 0, or a molar concentration) or vacuum from (number < 0)
        a region expression (mcg_release_region). Returns molecules placed (removed < 0)."""
        ex = region_expr(tokens)
        method = 0 if concentration is None else 1
        done = ctypes.c_int64()
        self._chk(lib().mcg_release_region(self.h, ctypes.c_uint32(species), ctypes.c_int(method),
                                           ctypes.c_int64(number), ctypes.c_double(concentration or 0.0),
                                           ctypes.c_double(length_unit_um), _p(ex), ctypes.c_uint32(len(ex)),
                                           ctypes.c_uint64(seed), ctypes.byref(done)))
        return done.value

    def release_region_harness(self, species, tokens, draws, number=0, concentration=None, length_unit_um=0.01,
                               cap=100000):
        """Parity harness (mcg_release_region_harness): (positions [k, 3], removed ids, draws used or None)."""
        ex = region_expr(tokens)
        dr = np.ascontiguousarray(draws, np.uint32)
        pos = np.zeros((cap, 3))
        rem = np.zeros(cap, np.uint64)
        n_pos, n_rem, used = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        method = 0 if concentration is None else 1
        self._chk(lib().mcg_release_region_harness(
            self.h, ctypes.c_uint32(species), ctypes.c_int(method), ctypes.c_int64(number),
            ctypes.c_double(concentration or 0.0), ctypes.c_double(length_unit_um), _p(ex), ctypes.c_uint32(len(ex)),
            _p(dr), ctypes.c_uint32(len(dr)), _p(pos), ctypes.c_uint32(cap), ctypes.byref(n_pos), _p(rem),
            ctypes.byref(n_rem), ctypes.byref(used)))
        return (pos[:min(cap, n_pos.value)], rem[:min(cap, n_rem.value)],
                None if used.value == 0xFFFFFFFF else int(used.value))

    def export_state(self):
        """Checkpoint: dict of pos, species, ids, unimol_time, flags and the iteration."""
        n = ctypes.c_uint64()
        it = ctypes.c_uint64()
        self._chk(lib().mcg_export_state(self.h, ctypes.c_uint64(0), None, None, None, None, None, ctypes.byref(n),
                                         ctypes.byref(it)))
        m = n.value
        st = {"pos": np.zeros((m, 3)), "species": np.zeros(m, np.uint32), "ids": np.zeros(m, np.uint64),
              "unimol_time": np.zeros(m), "flags": np.zeros(m, np.uint8)}
        self._chk(lib().mcg_export_state(self.h, ctypes.c_uint64(m), _p(st["pos"]), _p(st["species"]), _p(st["ids"]),
                                         _p(st["unimol_time"]), _p(st["flags"]), ctypes.byref(n), ctypes.byref(it)))
        st["iteration"] = it.value
        return st

    def import_state(self, st):
        pos = np.ascontiguousarray(st["pos"], np.float64)
        sp = np.ascontiguousarray(st["species"], np.uint32)
        ids = np.ascontiguousarray(st["ids"], np.uint64)
        tu = np.ascontiguousarray(st["unimol_time"], np.float64)
        fl = np.ascontiguousarray(st["flags"], np.uint8)
        self._chk(lib().mcg_import_state(self.h, ctypes.c_uint64(len(sp)), _p(pos), _p(sp), _p(ids), _p(tu), _p(fl),
                                         ctypes.c_uint64(int(st["iteration"]))))

    def write_viz(self, prefix, species_names, iteration, total_iterations, mode="ascii", length_unit_um=0.01):
        modes = {"ascii": 0, "cellblender_v1": 1, "cellblender_v2": 2}
        names = (ctypes.c_char_p * len(species_names))(*[n.encode() for n in species_names])
        self._chk(lib().mcg_write_viz(self.h, str(prefix).encode(), ctypes.c_int(modes[mode]), names,
                                      ctypes.c_uint64(iteration), ctypes.c_uint64(total_iterations),
                                      ctypes.c_double(length_unit_um)))

    def write_counts(self, prefix, columns, n_iterations, every=1, time_step_s=1e-6, fmt="dat"):
        """Count files (DAT or GDAT) of the last n_iterations iterations; columns:
        [(species, counted object index or -1 for the world, name)]."""
        sp = np.ascontiguousarray([c[0] for c in columns], np.uint32)
        ob = np.ascontiguousarray([c[1] for c in columns], np.int32)
        names = (ctypes.c_char_p * len(columns))(*[c[2].encode() for c in columns])
        self._chk(lib().mcg_write_counts(self.h, str(prefix).encode(), ctypes.c_int({"dat": 0, "gdat": 1}[fmt]),
                                         ctypes.c_uint32(n_iterations), ctypes.c_uint32(every),
                                         ctypes.c_double(time_step_s), ctypes.c_uint32(len(columns)), _p(sp), _p(ob),
                                         names))

    def autotune_subparts(self):
        """The batch autotuner's (subpartitions per edge, octant bins) for this model."""
        n = ctypes.c_uint32()
        o = ctypes.c_int()
        self._chk(lib().mcg_autotune_subparts(self.h, ctypes.byref(n), ctypes.byref(o)))
        return n.value, bool(o.value)

    def trace_cases_static(self, ids, disp, draws, r_rate_factor=None, t_steps=None):
        """trace_cases through mcg_trace_cases_static (fixed device scratch, no allocation)."""
        ids = np.ascontiguousarray(ids, np.uint64)
        n = len(ids)
        disp = np.ascontiguousarray(disp, np.float64).reshape(n, 3)
        draws = np.ascontiguousarray(draws, np.uint32).reshape(n, -1)
        rrf = np.ascontiguousarray(np.ones(n) if r_rate_factor is None else r_rate_factor, np.float64)
        tst = np.ascontiguousarray(np.ones(n) if t_steps is None else t_steps, np.float64)
        out = np.zeros((n, TRACE_RESULT_SIZE))
        self._chk(lib().mcg_trace_cases_static(self.h, ctypes.c_uint32(n), _p(ids), _p(disp), _p(draws),
                                               ctypes.c_uint32(draws.shape[1]), _p(rrf), _p(tst), _p(out)))
        return out

    def wall_consts(self, nw):
        out = np.zeros((nw, 14))
        self._chk(lib().mcg_wall_consts(self.h, _p(out)))
        return out

    def walls_in_subparts(self, nsub3, cap=1 << 22):
        counts = np.zeros(nsub3, np.uint32)
        lst = np.zeros(cap, np.uint32)
        tot = ctypes.c_uint64()
        self._chk(lib().mcg_walls_in_subparts(self.h, _p(counts), _p(lst), ctypes.c_uint64(cap), ctypes.byref(tot)))
        return counts, lst[:tot.value]


class Batch:
    """Many models advanced together as replicas of one device engine (mcg_batch_*).

    Models are unprepared Engine objects (set up, never stepped); the batch
    copies them, so they may be closed after add()."""

    def __init__(self, precision, n_species, max_replicas, capacity=0, autotune=False):
        L = lib()
        cfg = McgBatchConfig()
        cfg.precision = PRECISION[precision] if isinstance(precision, str) else int(precision)
        cfg.n_species = int(n_species)
        cfg.max_replicas = int(max_replicas)
        cfg.capacity = int(capacity)
        cfg.autotune = 1 if autotune else 0
        h = ctypes.c_void_p()
        rc = L.mcg_batch_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != MCG_OK:
            msg = L.mcg_batch_last_error(h) if h.value else b"mcg_batch_create rejected the configuration"
            if h.value:
                L.mcg_batch_destroy(h)
            raise EngineError(rc, msg.decode() if msg else "")
        self.h = h
        self.n_species = int(n_species)

    def close(self):
        if getattr(self, "h", None):
            lib().mcg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc):
        if rc != MCG_OK:
            msg = lib().mcg_batch_last_error(self.h)
            raise EngineError(rc, msg.decode() if msg else "")

    def add(self, models, n_iterations=None):
        n = len(models)
        arr = (ctypes.c_void_p * n)(*[m.h.value for m in models])
        its = np.ascontiguousarray(np.zeros(n) if n_iterations is None else n_iterations, np.uint32)
        ids = np.zeros(n, np.uint32)
        self._chk(lib().mcg_batch_add(self.h, ctypes.c_uint32(n), arr, _p(its), _p(ids)))
        return ids

    def remove(self, ids):
        ids = np.ascontiguousarray(ids, np.uint32)
        self._chk(lib().mcg_batch_remove(self.h, ctypes.c_uint32(len(ids)), _p(ids)))

    def step(self, n=1):
        self._chk(lib().mcg_batch_step(self.h, ctypes.c_uint32(n)))

    def sync(self):
        self._chk(lib().mcg_batch_sync(self.h))

    def replica_info(self, rep):
        done = ctypes.c_uint64()
        nsub = ctypes.c_uint32()
        self._chk(lib().mcg_batch_replica_info(self.h, ctypes.c_uint32(rep), ctypes.byref(done), ctypes.byref(nsub)))
        return done.value, nsub.value

    def counts(self, rep):
        out = np.zeros(self.n_species, np.uint64)
        self._chk(lib().mcg_batch_get_counts(self.h, ctypes.c_uint32(rep), _p(out)))
        return out

    def trajectory(self, rep, n):
        out = np.zeros((n, self.n_species), np.uint64)
        self._chk(lib().mcg_batch_get_count_trajectory(self.h, ctypes.c_uint32(rep), ctypes.c_uint32(n), _p(out)))
        return out

    def molecules(self, rep):
        n = ctypes.c_uint64()
        self._chk(lib().mcg_batch_download_molecules(self.h, ctypes.c_uint32(rep), ctypes.c_uint64(0), None, None,
                                                     None, ctypes.byref(n)))
        pos = np.zeros((n.value, 3))
        sp = np.zeros(n.value, np.uint32)
        ids = np.zeros(n.value, np.uint64)
        self._chk(lib().mcg_batch_download_molecules(self.h, ctypes.c_uint32(rep), ctypes.c_uint64(n.value), _p(pos),
                                                     _p(sp), _p(ids), ctypes.byref(n)))
        return pos, sp, ids

    def stats(self):
        it, ms, la = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        self._chk(lib().mcg_batch_get_stats(self.h, ctypes.byref(it), ctypes.byref(ms), ctypes.byref(la)))
        return it.value, ms.value, la.value

    def set_options(self, use_graphs=True, profile=False):
        self._chk(lib().mcg_batch_set_options(self.h, int(use_graphs), int(profile)))

    def fallbacks(self):
        out = np.zeros(3, np.uint64)
        self._chk(lib().mcg_batch_get_fallbacks(self.h, _p(out)))
        return int(out[0]), int(out[1]), int(out[2])

    def profile(self):
        out = np.zeros(6)
        self._chk(lib().mcg_batch_get_profile(self.h, _p(out)))
        return out

    def device_bytes(self):
        b = ctypes.c_uint64()
        self._chk(lib().mcg_batch_get_memory(self.h, ctypes.byref(b)))
        return b.value

    def write_counts(self, rep, prefix, columns, n_iterations, every=1, time_step_s=1e-6, fmt="dat"):
        """Count files of one replica (as Engine.write_counts)."""
        sp = np.ascontiguousarray([c[0] for c in columns], np.uint32)
        ob = np.ascontiguousarray([c[1] for c in columns], np.int32)
        names = (ctypes.c_char_p * len(columns))(*[c[2].encode() for c in columns])
        self._chk(lib().mcg_batch_write_counts(self.h, ctypes.c_uint32(rep), str(prefix).encode(),
                                               ctypes.c_int({"dat": 0, "gdat": 1}[fmt]), ctypes.c_uint32(n_iterations),
                                               ctypes.c_uint32(every), ctypes.c_double(time_step_s),
                                               ctypes.c_uint32(len(columns)), _p(sp), _p(ob), names))

    def write_viz(self, rep, prefix, species_names, iteration, total_iterations, mode="ascii", length_unit_um=0.01):
        modes = {"ascii": 0, "cellblender_v1": 1, "cellblender_v2": 2}
        names = (ctypes.c_char_p * len(species_names))(*[n.encode() for n in species_names])
        self._chk(lib().mcg_batch_write_viz(self.h, ctypes.c_uint32(rep), str(prefix).encode(),
                                            ctypes.c_int(modes[mode]), names, ctypes.c_uint64(iteration),
                                            ctypes.c_uint64(total_iterations), ctypes.c_double(length_unit_um)))

    def escapes(self):
        """Molecules that left their partition: rows of uid, species + 1000 * kind, iteration, start xyz,
        displacement xyz, final xyz, replica (kind 1 escape, 2 watchdog)."""
        out = np.zeros((8, 13))
        n = ctypes.c_uint32()
        self._chk(lib().mcg_batch_get_escapes(self.h, ctypes.c_uint32(8), _p(out), ctypes.byref(n)))
        return out[:min(n.value, 8)], n.value

    def release(self, rep, species, n, shape="sphere", center=(0, 0, 0), diameter=(1, 1, 1), obj=0, seed=1):
        """mcg_batch_release into replica rep."""
        shapes = {"sphere": 0, "cuboid": 1, "shell": 2, "inside": 3}
        c = np.ascontiguousarray(center, np.float64)
        d = np.ascontiguousarray(diameter, np.float64)
        self._chk(lib().mcg_batch_release(self.h, ctypes.c_uint32(rep), ctypes.c_uint32(species), ctypes.c_uint64(n),
                                          ctypes.c_int(shapes[shape]), _p(c), _p(d), ctypes.c_uint32(obj),
                                          ctypes.c_uint64(seed)))

    def release_region(self, rep, species, tokens, number=0, concentration=None, length_unit_um=0.01, seed=1):
        """mcg_batch_release_region into (or a vacuum from) replica rep's region expression."""
        ex = region_expr(tokens)
        done = ctypes.c_int64()
        self._chk(lib().mcg_batch_release_region(
            self.h, ctypes.c_uint32(rep), ctypes.c_uint32(species), ctypes.c_int(0 if concentration is None else 1),
            ctypes.c_int64(number), ctypes.c_double(concentration or 0.0), ctypes.c_double(length_unit_um), _p(ex),
            ctypes.c_uint32(len(ex)), ctypes.c_uint64(seed), ctypes.byref(done)))
        return done.value

    def diffuse_blocks_per_sm(self):
        v = ctypes.c_int()
        self._chk(lib().mcg_batch_get_tuning(self.h, ctypes.byref(v)))
        return v.value


class Server:
    """Serving loop (mcg_serve_*): requests are continuously batched on the device
    by a worker thread inside the library. Models are unprepared Engine objects,
    copied at submission."""

    def __init__(self, precision, n_species, max_slots=256, hbm_budget_bytes=150 << 30, autotune=True):
        L = lib()
        cfg = McgServerConfig()
        cfg.precision = PRECISION[precision] if isinstance(precision, str) else int(precision)
        cfg.n_species = int(n_species)
        cfg.max_slots = int(max_slots)
        cfg.hbm_budget_bytes = int(hbm_budget_bytes)
        cfg.autotune = 1 if autotune else 0
        h = ctypes.c_void_p()
        rc = L.mcg_serve_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != MCG_OK:
            msg = L.mcg_serve_last_error(h) if h.value else b"mcg_serve_create rejected the configuration"
            if h.value:
                L.mcg_serve_destroy(h)
            raise EngineError(rc, msg.decode() if msg else "")
        self.h = h
        self.n_species = int(n_species)

    def close(self):
        if getattr(self, "h", None):
            lib().mcg_serve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc):
        if rc != MCG_OK:
            msg = lib().mcg_serve_last_error(self.h)
            raise EngineError(rc, msg.decode() if msg else "")

    def submit(self, model, n_iterations):
        t = ctypes.c_uint64()
        self._chk(lib().mcg_serve_submit(self.h, model.h, ctypes.c_uint32(n_iterations), ctypes.byref(t)))
        return t.value

    def poll(self, ticket):
        st = ctypes.c_int()
        sec = ctypes.c_double()
        self._chk(lib().mcg_serve_poll(self.h, ctypes.c_uint64(ticket), ctypes.byref(st), ctypes.byref(sec)))
        return REQ_STATES[st.value], sec.value

    def wait(self, ticket, timeout_s=600.0):
        st = ctypes.c_int()
        self._chk(lib().mcg_serve_wait(self.h, ctypes.c_uint64(ticket), ctypes.c_double(timeout_s), ctypes.byref(st)))
        return REQ_STATES[st.value]

    def result(self, ticket):
        n = ctypes.c_uint32()
        self._chk(lib().mcg_serve_result(self.h, ctypes.c_uint64(ticket), None, ctypes.c_uint32(0), None,
                                         ctypes.byref(n)))
        traj = np.zeros((n.value, self.n_species), np.uint64)
        final = np.zeros(self.n_species, np.uint64)
        self._chk(lib().mcg_serve_result(self.h, ctypes.c_uint64(ticket), _p(final), ctypes.c_uint32(n.value),
                                         _p(traj), ctypes.byref(n)))
        return final, traj

    def cancel(self, ticket):
        self._chk(lib().mcg_serve_cancel(self.h, ctypes.c_uint64(ticket)))

    def release(self, ticket):
        self._chk(lib().mcg_serve_release(self.h, ctypes.c_uint64(ticket)))

    def stats(self):
        st = McgServeStats()
        self._chk(lib().mcg_serve_get_stats(self.h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in McgServeStats._fields_}
