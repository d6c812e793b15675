"""ctypes binding of the oracle's serial engine (oracle/mcell_oracle.c).

TEST INFRASTRUCTURE: used by tests/ and by bench.py's CPU baseline / reference
leg only; the product never imports it.
"""
import ctypes
from pathlib import Path

import numpy as np

LIB = Path(__file__).resolve().parent / "_build" / "libmcell_oracle.so"
_lib = None


def oracle_lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(LIB))
    return _lib


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleEngine:
    def __init__(self, **kw):
        self.lib = oracle_lib()
        self.lib.orc_engine_new.restype = ctypes.c_void_p
        self.lib.orc_engine_num_live.restype = ctypes.c_uint64
        self.lib.orc_engine_mol_steps.restype = ctypes.c_uint64
        self.lib.orc_engine_molecules.restype = ctypes.c_uint64
        self.keep = []
        d = OrcDesc()
        for k, v in kw.items():
            if isinstance(v, np.ndarray):
                self.keep.append(v)
                setattr(d, k, v.ctypes.data_as(ctypes.c_void_p))
            else:
                setattr(d, k, v)
        self.d = d
        self.h = ctypes.c_void_p(self.lib.orc_engine_new(ctypes.byref(d)))
        self.nsp = kw["nspecies"]

    def run(self, n):
        out = np.zeros((n, self.nsp), np.uint64)
        rc = self.lib.orc_engine_run(self.h, ctypes.c_uint(n), ptr(out))
        assert rc == 0
        return out

    def molecules(self):
        n = self.lib.orc_engine_num_live(self.h)
        pos = np.zeros((n, 3))
        sp = np.zeros(n, np.uint32)
        self.lib.orc_engine_molecules(self.h, ctypes.c_uint64(n), ptr(pos), ptr(sp))
        return pos, sp

    def __del__(self):
        self.lib.orc_engine_free(self.h)


vp = ctypes.c_void_p


class OrcDesc(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_double * 3), ("partition_edge", ctypes.c_double), ("nsub", ctypes.c_uint),
                ("rxn_radius", ctypes.c_double), ("nv", ctypes.c_uint), ("verts", vp), ("nw", ctypes.c_uint),
                ("tris", vp), ("nspecies", ctypes.c_uint), ("space_steps", vp), ("wall_class", vp),
                ("nbimol", ctypes.c_uint), ("bimol_reactants", vp), ("bimol_p", vp), ("bimol_products", vp),
                ("nunimol", ctypes.c_uint), ("unimol_reactant", vp), ("unimol_k", vp), ("unimol_products", vp),
                ("nmol", ctypes.c_uint), ("mol_pos", vp), ("mol_species", vp), ("seed", ctypes.c_uint64)]


def make_oracle_engine(sc, bimol=(), unimol=(), seed=1):
    """bimol: [(a, b, p, (p0, p1))], unimol: [(a, k, (p0, p1))]"""
    nsp = len(sc.space_steps)
    kw = dict(origin=(ctypes.c_double * 3)(*sc.origin), partition_edge=sc.partition_edge, nsub=sc.nsub,
              rxn_radius=sc.rxn_radius, nv=len(sc.verts), verts=np.ascontiguousarray(sc.verts, np.float64),
              nw=len(sc.tris), tris=np.ascontiguousarray(sc.tris, np.uint32), nspecies=nsp,
              space_steps=np.ascontiguousarray(sc.space_steps, np.float64),
              wall_class=np.ascontiguousarray(sc.wall_class, np.uint8),
              nbimol=len(bimol),
              bimol_reactants=np.array([[b[0], b[1]] for b in bimol] or [[0, 0]], np.uint32),
              bimol_p=np.array([b[2] for b in bimol] or [0.0]),
              bimol_products=np.array([list(b[3]) for b in bimol] or [[-1, -1]], np.int32),
              nunimol=len(unimol),
              unimol_reactant=np.array([u[0] for u in unimol] or [0], np.uint32),
              unimol_k=np.array([u[1] for u in unimol] or [0.0]),
              unimol_products=np.array([list(u[2]) for u in unimol] or [[-1, -1]], np.int32),
              nmol=len(sc.mol_species), mol_pos=np.ascontiguousarray(sc.mol_pos, np.float64),
              mol_species=np.ascontiguousarray(sc.mol_species, np.uint32), seed=seed)
    return OracleEngine(**kw)






def oracle_engine_for_model(m, seed=1, n_mol=None):
    """Oracle serial engine of a mcell_gb300.workloads.Model (first n_mol molecules)."""
    class _S:
        pass
    s = _S()
    s.space_steps, s.origin, s.partition_edge, s.nsub = m.space_steps, m.origin, m.partition_edge, m.nsub
    s.rxn_radius, s.verts, s.tris, s.wall_class = m.rxn_radius, m.verts, m.walls, m.wall_class
    n = len(m.species) if n_mol is None else n_mol
    s.mol_pos, s.mol_species = m.pos[:n], m.species[:n]
    return make_oracle_engine(s, bimol=m.bimol, unimol=m.unimol, seed=seed)
