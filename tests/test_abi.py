"""CPU tests of the drop-in boundary: the library builds, loads and exports every
entry point include/mcell_gb300.h declares; host-side argument checks work
without a GPU; and the product path fails loudly (no CPU fallback) when no
device is present."""
import re

import numpy as np
import pytest

from tests import harness as H
from mcell_gb300 import _native


def declared_symbols():
    text = (H.ROOT / "include" / "mcell_gb300.h").read_text()
    return sorted(set(re.findall(r"\b(mcg_[a-z_]+)\s*\(", text)))


def test_header_and_binding_agree():
    assert declared_symbols() == sorted(_native.EXPORTS)


def test_headers_compile_as_c_and_cpp():
    import shutil
    import subprocess
    if not shutil.which("gcc") or not shutil.which("g++"):
        pytest.skip("no host compiler")
    inc = H.ROOT / "include"
    subprocess.run(["gcc", "-fsyntax-only", "-std=c99", "-Wall", "-Werror", "-x", "c", str(inc / "mcell_gb300.h")],
                   check=True)
    subprocess.run(["g++", "-fsyntax-only", "-std=c++17", "-Wall", "-Werror", "-x", "c++", "-I", str(inc),
                    str(inc / "mcell_gb300_event.hpp")], check=True)


def test_library_exports_every_declared_symbol():
    L = _native.lib()
    for name in declared_symbols():
        assert hasattr(L, name), name


def test_config_validation():
    with pytest.raises(_native.EngineError):
        _native.Engine("fp64", (0, 0, 0), 100.0, 0, 0.56, 3)        # no subpartitions
    with pytest.raises(_native.EngineError):
        _native.Engine("fp64", (0, 0, 0), 100.0, 301, 0.56, 3)      # over MAX_SUBPARTS_PER_PARTITION
    with pytest.raises(_native.EngineError):
        _native.Engine("fp64", (0, 0, 0), 100.0, 10, 0.56, 17)      # too many species
    e = _native.Engine("fp64", (-60, -60, -60), 120.0, 12, 0.5642, 3)
    with pytest.raises(_native.EngineError):
        e.set_species([2.0, 2.0])                                   # count mismatch
    e.set_species([2.0, 2.0, 1.41])
    with pytest.raises(_native.EngineError):
        e.add_bimol_rxn(0, 5, 0.1)                                  # bad species
    e.add_bimol_rxn(0, 1, 0.0368, (2, -1))
    for _ in range(_native.MAX_PATHWAYS - 1):
        e.add_bimol_rxn(1, 0, 0.01)                                 # further pathways of the pair's class
    with pytest.raises(_native.EngineError) as ex:
        e.add_bimol_rxn(1, 0, 0.01)                                 # one pathway too many
    assert ex.value.code == -6
    with pytest.raises(_native.EngineError):
        e.add_molecules(np.zeros((1, 3)), np.array([7]))
    # R * sqrt(2) must stay below half a subpartition edge (mcell4_converter.cpp:121):
    # 120 / 100 = 1.2 units against 0.5642 * sqrt(2) = 0.798; refused before any device work
    f = _native.Engine("fp64", (-60, -60, -60), 120.0, 100, 0.5642, 3)
    f.set_species([2.0, 2.0, 1.41])
    with pytest.raises(_native.EngineError) as ex:
        f.prepare()
    assert ex.value.code == -1 and "subpartition edge" in str(ex.value)
    f.close()


def test_reactive_products_are_refused_without_a_device():
    """A product that is also a bimolecular reactant would react in its birth step in
    the reference; the GPU path refuses such models (MCG_ERR_UNSUPPORTED) before any
    device work, for single models and for batches."""
    def model(rxns):
        e = _native.Engine("fp64", (-60, -60, -60), 120.0, 12, 0.5642, 4)
        e.set_species([2.0, 2.0, 1.41, 1.0])
        for a, b, prods in rxns:
            e.add_bimol_rxn(a, b, 0.05, prods)
        e.add_unimol_rxn(3, 1e-3, (2, -1))
        return e
    for rxns in ([(0, 1, (2, -1)), (2, 0, (3, -1))],    # C = A + B is a reactant of C + A
                 [(0, 1, (3, -1)), (2, 1, (-1, -1))]):  # C = the product of D's decay reacts with B
        e = model(rxns)
        with pytest.raises(_native.EngineError) as ex:
            e.prepare()
        assert ex.value.code == -6 and "product" in str(ex.value)
        e.close()


def test_host_setup_matches_oracle_without_gpu():
    """Wall constants and wall lists come from host code and must equal the oracle's
    (which equal the reference's, see test_oracle)."""
    for name in H.GOLDEN_SCENES:
        sc, g = H.load_golden(name)
        nsp = len(sc.space_steps)
        e = _native.Engine("fp64", sc.origin, sc.partition_edge, sc.nsub, sc.rxn_radius, nsp)
        e.set_species(sc.space_steps)
        e.upload_mesh(sc.verts, sc.tris, sc.wall_class.reshape(len(sc.tris), nsp))
        assert np.array_equal(e.wall_consts(len(sc.tris)), g["wall_consts"]), name
        counts, lst = e.walls_in_subparts(sc.nsub ** 3)
        assert np.array_equal(counts, g["wsp_counts"]) and np.array_equal(lst, g["wsp_list"]), name


def test_fails_loudly_without_device():
    import torch  # only to ask whether a device exists
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    sc = H.cube_scene(np.random.default_rng(0), n_mol=10)
    with pytest.raises(_native.EngineError) as ei:
        H.engine_from_scene(sc)
    assert ei.value.code == -2  # MCG_ERR_CUDA, no silent fallback


def test_batch_config_validation_and_no_fallback():
    with pytest.raises(_native.EngineError) as ei:
        _native.Batch("fp32", 3, 0)                                 # no replica slots
    assert ei.value.code == -1
    with pytest.raises(_native.EngineError):
        _native.Batch("fp32", 17, 4)                                # too many species
    import torch
    if torch.cuda.is_available():
        return
    with pytest.raises(_native.EngineError) as ei:
        _native.Batch("fp32", 3, 4)
    assert ei.value.code == -2  # MCG_ERR_CUDA: a batch needs the device, no CPU path


def test_batch_subpartition_autotuner_choices():
    """The cost model keeps the dense 1M-molecule model's grid and coarsens sparse replicas."""
    from mcell_gb300 import workloads as W
    dense = W.sphere_in_cube(n_mol=1_000_000)
    n, octants = W.model_handle(dense).autotune_subparts()
    assert dense.nsub <= n <= 2 * dense.nsub and octants  # measured optimum 34-44 of 26
    sparse = W.replica_models(1, seed=1, n_range=(1000, 1001), edge_range_um=(3.0, 3.0), sphere_fraction=0.0)[0]
    n, octants = W.model_handle(sparse).autotune_subparts()
    assert n <= sparse.nsub // 2 and not octants


# (model grid, chosen grid, octants) for replica_models(24, seed=7) and
# replica_models(8, seed=3, n_range=(1e5, 2e6)): the cost model's choices, kept
# when its sums are computed another way
AUTOTUNE_PINS = [(18, 21, 1), (28, 17, 0), (10, 24, 1), (12, 20, 0), (8, 13, 1), (14, 20, 1), (10, 10, 1),
                 (28, 12, 1), (24, 29, 0), (20, 14, 1), (8, 16, 1), (12, 20, 1), (8, 27, 1), (28, 12, 1),
                 (28, 20, 1), (30, 21, 1), (18, 8, 1), (12, 29, 0), (12, 20, 1), (10, 14, 1), (22, 18, 1),
                 (24, 17, 1), (10, 10, 1), (8, 10, 1), (8, 19, 1), (14, 20, 1), (30, 25, 1), (8, 23, 1),
                 (10, 24, 1), (24, 29, 1), (30, 30, 1), (26, 26, 1)]


def test_batch_autotuner_choices_are_pinned():
    from mcell_gb300 import workloads as W
    ms = W.replica_models(24, seed=7) + W.replica_models(8, seed=3, n_range=(100_000, 2_000_000))
    got = []
    for m in ms:
        h = W.model_handle(m, "fp32")
        n, octants = h.autotune_subparts()
        h.close()
        got.append((m.nsub, n, int(octants)))
    assert got == AUTOTUNE_PINS


def test_server_needs_the_device():
    with pytest.raises(_native.EngineError) as ei:
        _native.Server("fp32", 3, max_slots=0)
    assert ei.value.code == -1
    import torch
    if torch.cuda.is_available():
        return
    with pytest.raises(_native.EngineError) as ei:
        _native.Server("fp32", 3, max_slots=4)
    assert ei.value.code == -2


def test_output_and_test_hook_entry_points_check_their_arguments():
    import ctypes
    L = _native.lib()
    null = ctypes.c_void_p(None)
    # count and viz writers refuse a missing handle or prefix without touching a device
    assert L.mcg_write_counts(null, b"x", 0, 1, 1, ctypes.c_double(1e-6), 1, null, null, null) == -1
    assert L.mcg_batch_write_counts(null, 0, b"x", 0, 1, 1, ctypes.c_double(1e-6), 1, null, null, null) == -1
    assert L.mcg_write_viz(null, b"x", 0, null, ctypes.c_uint64(0), ctypes.c_uint64(1), ctypes.c_double(0.01)) == -1
    # the non-blocking counts refuse a missing handle, ticket output or engine without a device
    assert L.mcg_request_counts(null, null) == -1
    assert L.mcg_wait_counts(null, ctypes.c_uint64(1), null) == -1
    e = _native.Engine("fp64", (-60, -60, -60), 120.0, 12, 0.5642, 3)
    out = np.zeros(3, np.uint64)
    assert L.mcg_wait_counts(e.h, ctypes.c_uint64(1), out.ctypes.data_as(ctypes.c_void_p)) == -1
    e.close()
    # the out-of-memory hook arms and disarms without a device
    assert L.mcg_inject_device_alloc_failure(ctypes.c_int64(5)) == 0
    assert L.mcg_inject_device_alloc_failure(ctypes.c_int64(-1)) == 0
