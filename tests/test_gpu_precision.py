"""Precision form on a reduced bumpy tube (2 um long, 40,400 triangles, 200k
molecules, 5% within 1 nm of mesh edges and vertices, dt = 0.1 us, 100
subpartitions per edge: 0.022 um, above the 2 * sqrt(2) * R = 0.016 um the reaction
radius needs, and close to the full tube's 0.034 um): the fp32
engine against the fp64 engine (which follows the reference routines bit for bit).

Bars: wall-hit identity mismatch rate below 1e-3 (half of the cases start next
to edges) and below 2e-4 when both engines start from the fp32 engine's stored
positions, no molecule leaves the tube in either precision, and the product
count after 40 iterations within 3x the difference two fp64 seeds give."""
import numpy as np
import pytest

from mcell_gb300 import precision
from mcell_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tube():
    return W.bumpy_tube(n_mol=200_000, length_um=2.0, n_z=100, subparts_per_edge=100)


def test_fp32_wall_hits_match_fp64_near_edges(tube):
    n = len(tube.species)
    near = np.arange(n - int(round(0.05 * n)), n)
    r = precision.wall_hit_mismatch(tube, n_cases=40_000, near_ids=near)
    print("tube fp32 vs fp64:", r)
    assert r["cases_with_wall_events"] > 1000
    assert r["rate"] < 1e-3
    assert r["max_position_error"] < 0.1


def test_fp32_trace_arithmetic_matches_fp64_from_the_same_start(tube):
    # the fp64 engine holds the fp32 engine's stored positions: what remains is the
    # fp32 ray arithmetic with its fp64 tie-breaks
    n = len(tube.species)
    near = np.arange(n - int(round(0.05 * n)), n)
    r = precision.wall_hit_mismatch(tube, n_cases=40_000, near_ids=near, same_start=True)
    print("tube fp32 vs fp64, same start:", r)
    assert r["cases_with_wall_events"] > 1000
    assert r["rate"] < 2e-4


def test_fp32_counts_follow_fp64(tube):
    r = precision.count_error(tube, n_iter=40)
    print("tube counts:", r)
    c = r["final_counts"]
    for tag in c:
        assert c[tag][0] + c[tag][2] == 100_000  # A + C conserved (no escapes, no losses)
    assert r["max_rel_error_fp32_vs_fp64"] <= 3 * max(r["max_rel_difference_two_fp64_seeds"], 1e-3)
