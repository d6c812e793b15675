#!/usr/bin/env python3
"""Build oracle/_ref/libmcell_ref{64,32}.so: the reference's own hot-path routines.

The MCell4 engine cannot be built here: libbng (an un-vendored sibling repo),
boost, sparsehash, VTK, nfsim, bison/flex and swig are all absent. Its hot-path
routines are plain static functions, though, so this recipe compiles them from
the reference sources where they lie:

  1. read the named function definitions out of the reference files (brace
     matching, nothing edited),
  2. prepend oracle/ref/ref_shim.h (project-written stand-ins for Partition,
     Molecule, Wall, Collision, RxnClass and libbng's shared_defines.h) and
     append oracle/ref/ref_harness.cpp (project-written C entry points that
     drive the routines with injected displacements and random draws),
  3. pipe the translation unit straight into g++ (nothing of the reference is
     written into this repository; the only output is the .so in oracle/_ref/).

It also compiles the reference's ISAAC64 and ziggurat generator
(src/isaac64.c, src/rng.c through src/rng.h) into the same library.

Usage: python oracle/ref/build_ref.py [--ref <reference checkout>]
The checkout defaults to $MCELL_REFERENCE_ROOT, else a directory named
"reference" beside this repository.
Test infrastructure only; the product never loads oracle/_ref.
"""
import argparse
import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
OUT = ORACLE / "_ref"

# (file, name, namespace). Every routine on the volume diffuse-react path that
# does not need the World: see the citations in ref_harness.cpp.
FUNCS = [
    ("src4/simulation_config.cpp", "SimulationConfig::init_subpartition_edge_length", "MCell"),
    ("src4/wall.cpp", "Wall::initialize_wall_constants", "MCell"),
    ("src4/geometry_utils.inl", "get_wall_bounding_box", "MCell::GeometryUtils"),
    ("src4/wall_utils.inl", "wall_in_box", "MCell::WallUtils"),
    ("src4/geometry_utils.inl", "wall_subparts_collision_test", "MCell::GeometryUtils"),
    ("src4/collision_utils_subparts.inl", "collect_neighboring_subparts", "MCell::CollisionUtils"),
    ("src4/collision_utils_subparts.inl", "collect_crossed_subparts", "MCell::CollisionUtils"),
    ("src4/collision_utils.inl", "get_displacement_up_to_partition_boundary", "MCell::CollisionUtils"),
    ("src4/collision_utils.inl", "collide_mol", "MCell::CollisionUtils"),
    ("src4/collision_utils.inl", "collide_mol_loop_body", "MCell::CollisionUtils"),
    ("src4/collision_utils.inl", "jump_away_line", "MCell::CollisionUtils"),
    ("src4/collision_utils.inl", "collide_wall", "MCell::CollisionUtils"),
    ("src4/collision_utils.inl", "is_immediate_collision", "MCell::CollisionUtils"),
    ("src4/collision_utils.inl", "get_closest_wall_collision", "MCell::CollisionUtils"),
    ("src4/collision_utils.inl", "reflect_from_wall", "MCell::CollisionUtils"),
    ("src4/collision_utils.inl", "raycast_with_endpoints", "MCell::CollisionUtils"),
    ("src4/collision_utils.inl", "compute_inputs_for_raycast_with_endpoints", "MCell::CollisionUtils"),
    ("src4/collision_utils.inl", "get_crossed_subparts_for_walls", "MCell::CollisionUtils"),
    ("src4/collision_utils.inl", "get_num_crossed_region_walls", "MCell::CollisionUtils"),
    ("src4/collision_utils.inl", "get_num_crossed_walls_per_object", "MCell::CollisionUtils"),
    ("src4/collision_utils.inl", "is_point_inside_region_no_waypoints", "MCell::CollisionUtils"),
    ("src4/collision_utils.inl", "compute_counted_volume_for_pos", "MCell::CollisionUtils"),
    ("src4/wall.cpp", "Region::compute_bounding_box", "MCell"),
    ("src4/release_event.cpp", "ReleaseEvent::release_ellipsoid_or_rectcuboid", "MCell"),
    ("src4/geometry.cpp", "tetrahedral_volume", "MCell"),
    ("src4/geometry.cpp", "Region::initialize_volume_info_if_needed", "MCell"),
    ("src4/geometry.cpp", "compute_region_expr_bounding_box", "MCell"),
    ("src4/release_event.cpp", "check_max_release_count", "MCell"),
    ("src4/release_event.cpp", "ReleaseEvent::calculate_number_to_release", "MCell"),
    ("src4/release_event.cpp", "ReleaseEvent::num_vol_mols_from_conc", "MCell"),
    ("src4/release_event.cpp", "ReleaseEvent::randomly_remove_molecules", "MCell"),
    ("src4/release_event.cpp", "ReleaseEvent::is_point_inside_region_expr_recursively", "MCell"),
    ("src4/release_event.cpp", "ReleaseEvent::vacuum_inside_regions", "MCell"),
    ("src4/release_event.cpp", "ReleaseEvent::release_inside_regions", "MCell"),
    ("src4/rxn_utils.inl", "binary_search_double", "MCell::RxnUtils"),
    ("src4/rxn_utils.inl", "test_bimolecular", "MCell::RxnUtils"),
    ("src4/rxn_utils.inl", "test_intersect", "MCell::RxnUtils"),
    ("src4/rxn_utils.inl", "time_of_unimol", "MCell::RxnUtils"),
    ("src4/rxn_utils.inl", "which_unimolecular", "MCell::RxnUtils"),
    ("src4/diffuse_react_event.cpp", "sort_collisions_by_time", "MCell"),
    ("src4/diffuse_react_event.cpp", "ray_trace_vol", "MCell"),
]
# whole namespace body of the exact-disk file (types, helpers and exact_disk itself)
REGIONS = [
    ("src4/exact_disk_utils.inl", "namespace ExactDiskUtils {", "} // namespace exact_disk_util",
     "MCell::ExactDiskUtils"),
]


def _skip_comment_or_literal(text, i):
    """If text[i] starts a comment or literal, return the index after it, else None."""
    if text.startswith("//", i):
        j = text.find("\n", i)
        return len(text) if j < 0 else j
    if text.startswith("/*", i):
        j = text.find("*/", i + 2)
        return len(text) if j < 0 else j + 2
    if text[i] in "\"'":
        q = text[i]
        j = i + 1
        while j < len(text) and text[j] != q:
            j += 2 if text[j] == "\\" else 1
        return j + 1
    return None


def _match_brace(text, i):
    """text[i] == '{'; return the index just past its matching '}'."""
    depth = 0
    while i < len(text):
        k = _skip_comment_or_literal(text, i)
        if k is not None:
            i = k
            continue
        c = text[i]
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                return i + 1
        i += 1
    raise ValueError("unbalanced braces")


def extract_function(text, name):
    """Return the first column-0 definition of `name` (signature through body)."""
    pat = re.compile(r"^[A-Za-z_][^\n;{}]*?\b" + re.escape(name) + r"\s*\(", re.M)
    for m in pat.finditer(text):
        # find the end of the parameter list, then require a body
        i = m.end() - 1
        depth = 0
        while True:
            k = _skip_comment_or_literal(text, i)
            if k is not None:
                i = k
                continue
            if text[i] == "(":
                depth += 1
            elif text[i] == ")":
                depth -= 1
                if depth == 0:
                    break
            i += 1
        j = i + 1
        while j < len(text) and text[j] in " \t\r\n":
            j += 1
        if j < len(text) and text[j] == "{":
            end = _match_brace(text, j)
            return text[m.start():end]
    raise KeyError(f"definition of {name} not found")


def build_tu(ref: Path, pos_bytes: int) -> str:
    parts = [f"#define POS_T_BYTES {pos_bytes}\n", '#include "ref_shim.h"\n',
             '#include "ref_prelude.h"\n']
    for rel, name, ns in FUNCS:
        text = (ref / rel).read_text(errors="replace")
        body = extract_function(text, name)
        opens = "".join(f"namespace {n} {{ " for n in ns.split("::"))
        closes = "}" * len(ns.split("::"))
        parts.append(f"\n// ---- {rel}: {name}\n{opens}\n#line 1 \"{rel}:{name}\"\n{body}\n{closes}\n")
    for rel, start, end, ns in REGIONS:
        text = (ref / rel).read_text(errors="replace")
        a = text.index(start) + len(start)
        b = text.index(end, a)
        opens = "".join(f"namespace {n} {{ " for n in ns.split("::"))
        closes = "}" * len(ns.split("::"))
        parts.append(f"\n// ---- {rel}: region\n{opens}\n{text[a:b]}\n{closes}\n")
    parts.append('#include "ref_harness.cpp"\n')
    return "".join(parts)


def compile_lib(ref: Path, pos_bytes: int, out: Path, verbose=False):
    tu = build_tu(ref, pos_bytes)
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-DNDEBUG",
           "-w", "-x", "c++",
           "-I", str(HERE), "-I", str(HERE / "shim"),
           "-I", str(ref / "src4"), "-I", str(ref / "src"), "-I", str(ref / "include"),
           "-", "-o", str(out)]
    r = subprocess.run(cmd, input=tu, text=True, capture_output=True)
    if r.returncode != 0:
        sys.stderr.write(r.stderr[-6000:])
        raise SystemExit(f"compiling {out.name} failed")
    if verbose:
        print(f"built {out}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("MCELL_REFERENCE_ROOT", str(ORACLE.parent.parent / "reference")))
    ap.add_argument("-v", action="store_true")
    a = ap.parse_args()
    ref = Path(a.ref)
    if not (ref / "src4" / "collision_utils.inl").exists():
        print(f"reference sources not found under {ref}; oracle/_ref not built")
        return 0
    OUT.mkdir(exist_ok=True)
    compile_lib(ref, 8, OUT / "libmcell_ref64.so", a.v)
    compile_lib(ref, 4, OUT / "libmcell_ref32.so", a.v)
    return 0


if __name__ == "__main__":
    sys.exit(main())
