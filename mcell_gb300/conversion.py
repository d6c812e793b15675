"""Unit and setup conversions of the MCell4 Model API (host side, runs once).

Restates what MCell4Converter does before the first iteration so that a model
described in the reference's user units (um, s, cm^2/s, M^-1 s^-1) becomes the
engine's internal units (length_unit = 1/sqrt(surface_grid_density) um, one
time step per iteration):

- length unit and default reaction radius: libmcell/api/mcell4_converter.cpp:246-256,
  src/mcell_reactions.c:1302-1303
- partition origin, size and subpartition alignment: mcell4_converter.cpp:278-403
- subpartition edge and reciprocal: src4/simulation_config.cpp:45-70
- volume space step: src/mcell_species.c:270-274 (global time step case)
- vol-vol and unimolecular rate -> probability: src/react_util.c:45-184
  (compute_pb_factor); libbng, which holds MCell4's copy of this, is not in the
  reference tree, and MCell4's own MCell3 importer uses P = k * pb_factor
  (src4/mcell3_world_converter.cpp:1129-1135).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Optional, Sequence, Tuple

MY_PI = 3.14159265358979323846
N_AV = 6.0221417930e23
PARTITION_EDGE_EXTRA_MARGIN_UM = 0.01
MAX_SUBPARTS_PER_PARTITION = 300
DEFAULT_SURFACE_GRID_DENSITY = 10000.0
DEFAULT_PARTITION_DIMENSION_UM = 10.0
DEFAULT_SUBPARTITION_DIMENSION_UM = 0.5


def length_unit_um(surface_grid_density: float = DEFAULT_SURFACE_GRID_DENSITY) -> float:
    """length_unit = 1 / sqrt(grid density) um (mcell4_converter.cpp:246)."""
    return 1.0 / math.sqrt(surface_grid_density)


def default_rxn_radius_um(surface_grid_density: float = DEFAULT_SURFACE_GRID_DENSITY) -> float:
    """R = 1 / sqrt(pi * grid density) um (src/mcell_reactions.c:1302)."""
    return 1.0 / math.sqrt(MY_PI * surface_grid_density)


def space_step(d_cm2_s: float, time_step_s: float, length_unit: float) -> float:
    """Volume space step in internal units (src/mcell_species.c:270-274)."""
    if d_cm2_s == 0:
        return 0.0
    return math.sqrt(4.0 * 1.0e8 * d_cm2_s * time_step_s) * (1.0 / length_unit)


def bimol_probability(k_M_s: float, space_step_a: float, space_step_b: float,
                      rxn_radius_um: float, time_step_s: float, length_unit: float) -> float:
    """max_fixed_p of a vol+vol reaction: k * pb_factor (src/react_util.c:160-184)."""
    eff_vel = (space_step_a / 1.0 + space_step_b / 1.0) * length_unit / time_step_s  # um/s
    if eff_vel <= 0:
        return 0.0
    pb = 1.0 / (2.0 * math.sqrt(MY_PI) * rxn_radius_um * rxn_radius_um * eff_vel)
    pb *= 1.0e15 / N_AV
    return k_M_s * pb


def unimol_k_tot(k_s: float, time_step_s: float) -> float:
    """k_tot of a unimolecular reaction per iteration: k * time_unit (react_util.c:74)."""
    return k_s * time_step_s


def _floor_to_multiple_allow_negative(v: float, m: float) -> float:
    return math.floor(v / m) * m


def _ceil_to_multiple(v: float, m: float) -> float:
    return math.ceil(v / m) * m


@dataclass
class PartitionLayout:
    """Partition in internal units: origin corner, edge, subpartitions per edge."""
    origin: Tuple[float, float, float]
    edge: float
    nsub: int

    @property
    def subpart_edge(self) -> float:
        return self.edge / self.nsub


def partition_layout(bbox_llf_um: Sequence[float], bbox_urb_um: Sequence[float],
                     partition_dimension_um: float = DEFAULT_PARTITION_DIMENSION_UM,
                     subpartition_dimension_um: float = DEFAULT_SUBPARTITION_DIMENSION_UM,
                     initial_partition_origin_um: Optional[Sequence[float]] = None,
                     surface_grid_density: float = DEFAULT_SURFACE_GRID_DENSITY) -> PartitionLayout:
    """Partition sizing of MCell4Converter::convert_simulation_setup (mcell4_converter.cpp:278-403)."""
    lu = length_unit_um(surface_grid_density)
    llf = [c - PARTITION_EDGE_EXTRA_MARGIN_UM for c in bbox_llf_um]
    urb = [c + PARTITION_EDGE_EXTRA_MARGIN_UM for c in bbox_urb_um]
    auto_dim = max(urb) - min(llf)
    auto_origin = False
    llf_diff = 0.0
    if initial_partition_origin_um is None and auto_dim > partition_dimension_um:
        edge = auto_dim / lu
        origin = [(c - PARTITION_EDGE_EXTRA_MARGIN_UM) / lu for c in bbox_llf_um]
        auto_origin = True
    elif initial_partition_origin_um is not None and (
            any(o > l for o, l in zip(initial_partition_origin_um, llf)) or
            any(o + partition_dimension_um < u for o, u in zip(initial_partition_origin_um, urb))):
        o = list(initial_partition_origin_um)
        llf_diff = max(max(o[i] - llf[i], 0.0) for i in range(3))
        opp = [c + partition_dimension_um for c in o]
        urb_diff = max(max(urb[i] - opp[i], 0.0) for i in range(3))
        edge = (partition_dimension_um + llf_diff + urb_diff) / lu
    else:
        edge = partition_dimension_um / lu
    if initial_partition_origin_um is not None:
        origin = [(c - llf_diff) / lu for c in initial_partition_origin_um]
    elif not auto_origin:
        origin = [-edge / 2.0] * 3
    sp_len = subpartition_dimension_um / lu
    tentative = int(edge / sp_len)
    if tentative > MAX_SUBPARTS_PER_PARTITION:
        sp_len = edge / MAX_SUBPARTS_PER_PARTITION
    orig = list(origin)
    origin = [_floor_to_multiple_allow_negative(c, sp_len) for c in orig]
    moved = max(o - n for o, n in zip(orig, origin))
    edge = _ceil_to_multiple(edge + moved, sp_len)
    nsub = int(round(edge / sp_len))
    return PartitionLayout(origin=tuple(origin), edge=edge, nsub=nsub)
