"""Checkpoint files of a GPU engine: the state mcg_export_state returns (live
molecules with ids, unimolecular times and flags, and the iteration) in one .npz
file. Restoring needs the same model definition and seed on a fresh handle
(mcg_import_state); the run then continues as if it had not stopped."""
from __future__ import annotations

import numpy as np

FIELDS = ("pos", "species", "ids", "unimol_time", "flags", "iteration")


def save(engine, path):
    st = engine.export_state()
    np.savez(path, **{k: np.asarray(st[k]) for k in FIELDS})
    return st


def load(engine, path):
    z = np.load(path)
    st = {k: z[k] for k in FIELDS}
    st["iteration"] = int(st["iteration"])
    engine.import_state(st)
    return st
