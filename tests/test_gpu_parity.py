"""GPU parity of the per-molecule step: the per-routine harness with injected draws.

The CUDA device functions that the production kernel runs are driven through
the C ABI (mcg_trace_cases) with injected displacements and injected 32-bit
draws, and compared with
  - the golden fixtures recorded from the reference's own routines, and
  - the oracle port on fresh random cases.
fp64: wall-hit identity (wall, side, order), subpartitions, partners, reaction
fire / no-fire and the draws consumed are bit-exact; times and positions are
compared exactly too (tolerance 1e-6 relative is the stated bar; the
fp64 build has none because -fmad=false keeps the reference's rounding). The
only allowed deviation is exact_disk's transcendental functions (CUDA vs libm)
in the last bits: those cases are re-compared at 1e-9 relative.
fp32: reported as a mismatch rate against the fp64 oracle.
"""
import numpy as np
import pytest

from tests import harness as H

pytestmark = pytest.mark.gpu


def _trace(e, sc, mols, disps, draws):
    return e.trace_cases(np.asarray(mols, np.uint64), disps, draws)


@pytest.mark.parametrize("name", H.GOLDEN_SCENES)
def test_fp64_matches_reference_golden(name):
    sc, g = H.load_golden(name)
    e = H.engine_from_scene(sc, "fp64")
    got = _trace(e, sc, g["mols"], g["disps"], g["draws"])
    bad = H.compare_results(got, g["results"], rel=0.0, scene=sc)
    hard = [c for c in bad if H.compare_results(got[c:c + 1], g["results"][c:c + 1], rel=1e-9, scene=sc)]
    for c in hard[:3]:
        w = g["results"][c]
        n = int(w[6])
        print("case", c, "mol", g["mols"][c], "disp", g["disps"][c])
        print(" want", w[:9], w[9:9 + 8 * min(n, 4)].reshape(-1, 8))
        print(" got ", got[c, :9], got[c, 9:9 + 8 * min(int(got[c, 6]), 4)].reshape(-1, 8))
    assert not hard, f"{len(hard)} of {len(got)} cases differ from the reference routines: {hard[:5]}"
    assert len(bad) <= len(got) // 100


@pytest.mark.parametrize("seed", [5, 6])
def test_fp64_matches_oracle_random(seed):
    rng = np.random.default_rng(seed)
    star = H.star_scene(rng, n_mol=3000)
    star.rxn_p = np.array([0.4])
    for sc in [H.cube_scene(rng, n_mol=3000, p_rxn=0.4),
               H.sphere_in_cube_scene(rng, levels=3, n_mol=4000, radius_um=0.6, cube_um=1.5, p_rxn=0.4), star]:
        cases = H.random_cases(rng, sc, 3000, scale=3.0, near_wall_frac=0.5)
        mols = [c[0] for c in cases]
        disps = np.array([c[1] for c in cases])
        draws = np.array([c[2] for c in cases])
        draws[::2] >>= 5
        e = H.engine_from_scene(sc, "fp64")
        got = _trace(e, sc, mols, disps, draws)
        orc = H.oracle().scene(sc)
        want = np.array([orc.diffuse_case(m, d, dr) for m, d, dr in zip(mols, disps, draws)])
        bad = H.compare_results(got, want, rel=0.0, scene=sc)
        hard = [c for c in bad if H.compare_results(got[c:c + 1], want[c:c + 1], rel=1e-9, scene=sc)]
        assert not hard, f"{len(hard)} cases differ: {hard[:5]}"


def test_fp32_wall_hit_mismatch_rate():
    """fp32 geometry against the fp64 oracle: wall-hit identity must agree on nearly
    every case, and final positions closely. Bounds at about 3x what was measured here
    (0 of 4,000 mismatches; 9-12 per 100,000 on the 10M-molecule precision tube, i.e.
    1.1-1.4 expected at 3x that rate; largest position error 0.028 internal units)."""
    rng = np.random.default_rng(7)
    sc = H.sphere_in_cube_scene(rng, levels=3, n_mol=3000, radius_um=0.6, cube_um=1.5, p_rxn=0.0)
    cases = H.random_cases(rng, sc, 4000, scale=3.0, near_wall_frac=0.6)
    mols = [c[0] for c in cases]
    disps = np.array([c[1] for c in cases])
    draws = np.array([c[2] for c in cases])
    e = H.engine_from_scene(sc, "fp32")
    got = _trace(e, sc, mols, disps, draws)
    orc = H.oracle().scene(sc)
    want = np.array([orc.diffuse_case(m, d, dr) for m, d, dr in zip(mols, disps, draws)])
    walls_g = [tuple(got[c, 9 + 1:9 + 8 * int(got[c, 6]):8]) for c in range(len(got))]
    walls_w = [tuple(want[c, 9 + 1:9 + 8 * int(want[c, 6]):8]) for c in range(len(want))]
    mism = sum(a != b for a, b in zip(walls_g, walls_w))
    rate = mism / len(got)
    print(f"fp32 wall-hit identity mismatch rate: {rate:.5f} ({mism}/{len(got)})")
    assert mism <= 2
    same = [c for c in range(len(got)) if walls_g[c] == walls_w[c]]
    err = np.abs(got[same, 1:4] - want[same, 1:4]).max()
    print(f"fp32 max final-position error on matching cases: {err:.3g} internal units")
    assert err < 0.08  # internal units (0.8 nm); fp32 ulp at 150 internal units is 1.5e-5


@pytest.mark.parametrize("name", H.GOLDEN_SCENES)
def test_fallbacks_are_exact_with_small_pages(name):
    """The candidate page (16 in production) and the partner list (48) have fixed sizes
    where the reference's lists grow. With both cut to a few entries, the refilled
    pages and the partner scan along the walk must still reproduce the reference's
    routines on every golden case."""
    sc, g = H.load_golden(name)
    e = H.engine_from_scene(sc, "fp64")
    e.set_trace_limits(1, 2)
    got = _trace(e, sc, g["mols"], g["disps"], g["draws"])
    bad = H.compare_results(got, g["results"], rel=0.0, scene=sc)
    hard = [c for c in bad if H.compare_results(got[c:c + 1], g["results"][c:c + 1], rel=1e-9, scene=sc)]
    fb = e.fallbacks()
    print(name, "fallbacks (page refills, walk scans):", fb)
    assert not hard, f"{len(hard)} of {len(got)} cases differ with small pages: {hard[:5]}"
    assert fb[0] + fb[1] > 0
    e.close()


@pytest.mark.parametrize("dense", [False, True])
def test_fallbacks_are_exact_on_random_cases(dense):
    """Long steps on a fine grid (partner sets beyond the list), and in a crowded cube
    (150,000 molecules: several candidates per step, pages refilled), with pages of
    two candidates and lists of three subpartitions, against the oracle."""
    rng = np.random.default_rng(17)
    if dense:
        sc = H.cube_scene(rng, n_mol=150_000, p_rxn=0.3)
    else:
        sc = H.sphere_in_cube_scene(rng, levels=3, n_mol=6000, radius_um=0.6, cube_um=1.5, p_rxn=0.3, nsub=30)
    cases = H.random_cases(rng, sc, 3000, scale=6.0, near_wall_frac=0.5)
    mols = [c[0] for c in cases]
    disps = np.array([c[1] for c in cases])
    draws = np.array([c[2] for c in cases])
    draws[::4] >>= 4
    orc = H.oracle().scene(sc)
    want = np.array([orc.diffuse_case(m, d, dr) for m, d, dr in zip(mols, disps, draws)])
    e = H.engine_from_scene(sc, "fp64")
    full = _trace(e, sc, mols, disps, draws)
    e.set_trace_limits(2, 3)
    small = _trace(e, sc, mols, disps, draws)
    fb = e.fallbacks()
    print("fallbacks (page refills, walk scans):", fb)
    for got in (full, small):
        bad = H.compare_results(got, want, rel=0.0, scene=sc)
        hard = [c for c in bad if H.compare_results(got[c:c + 1], want[c:c + 1], rel=1e-9, scene=sc)]
        assert not hard, f"{len(hard)} cases differ: {hard[:5]}"
    assert fb[0] > 0 if dense else fb[1] > 0
    e.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_fallbacks_leave_the_trajectory_unchanged(precision):
    """A dense cube with long steps on a fine grid (many candidates per trace, partner
    sets larger than the 4x4x4 window): 20 iterations with the production capacities
    and with pages of one candidate and lists of four subpartitions give the same
    molecules, bit for bit."""
    rng = np.random.default_rng(21)
    sc = H.cube_scene(rng, n_mol=12000, nsub=24, p_rxn=0.2)
    sc.space_steps = np.array([20.0, 20.0, 14.0])
    runs = []
    for limits in (None, (1, 4)):
        e = H.make_gpu_engine(sc, precision, bimol=[(0, 1, 0.2, (2, -1))], seed=5)
        if limits:
            e.set_trace_limits(*limits)
        e.step(20)
        pos, sp, ids = e.molecules()
        o = np.argsort(ids)
        runs.append((pos[o], sp[o], ids[o], e.trajectory(20), e.fallbacks()))
        e.close()
    (p0, s0, i0, t0, f0), (p1, s1, i1, t1, f1) = runs
    print("fallbacks: production", f0, "small", f1)
    assert f1[0] > 0 and f1[1] > 0
    assert np.array_equal(i0, i1) and np.array_equal(s0, s1) and np.array_equal(p0, p1)
    assert np.array_equal(t0, t1)


def test_reaction_decisions_match_reference_golden():
    """The device's test_bimolecular and which_unimolecular on injected draws against
    the reference's routines: fire / no-fire and the pathway chosen, bit for bit, over
    classes of one (rxn_tests) and of 1-4 pathways (rxn_pathways), including the branch
    where the class's probability cannot be scaled enough."""
    from mcell_gb300 import _native
    z = np.load(H.GOLDEN / "rxn_tests.npz")
    got = _native.reaction_decisions("bimol", [[p] for p in z["P"]], z["S"], z["U"])
    assert np.array_equal(got >= 0, z["bimol"] >= 0)
    assert np.array_equal(got[got >= 0], z["bimol"][z["bimol"] >= 0])
    z = np.load(H.GOLDEN / "rxn_pathways.npz")
    cum = [z["cum"][i, :z["npw"][i]] for i in range(len(z["U"]))]
    got = _native.reaction_decisions("bimol", cum, z["scaling"], z["U"])
    assert np.array_equal(np.where(got < 0, -1, got), np.where(z["bimol"] < 0, -1, z["bimol"]))
    ucum = [z["ucum"][i, :z["unpw"][i]] for i in range(len(z["Uu"]))]
    got = _native.reaction_decisions("unimol", ucum, None, z["Uu"])
    assert np.array_equal(got, z["unimol"])
