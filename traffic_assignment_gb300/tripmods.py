"""Trip (OD demand) modifications as a scenario axis.

The reference reads modifications from a tab-separated file
(tap/parsetapfiles.c:573-638: ``id  P2P|UNIFORM|ALL  origin  dest
multiplier``, ``~`` comments) and applies one to the per-origin demand lists
(tap/tap_functions.c:521-598):

  P2P      origin, dest > 0: the first entry origin -> dest is multiplied
  UNIFORM  origin > 0, dest 0: every entry of that origin;
           origin 0, dest > 0: every entry towards that destination
  ALL      every entry

Here a list of modification sets becomes a [scenarios][OD entries] demand
matrix that ``Solver.set_scenario_demand`` hands to the batched solver, so
every set is solved in the same launches as capacity scenarios are.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import List, Sequence

import numpy as np

from .synth import Demand

__all__ = ["TripMod", "read_trip_mods", "write_trip_mods", "apply_trip_mod", "apply_trip_mods",
           "demand_entries", "demand_scenarios"]

_KINDS = ("P2P", "UNIFORM", "ALL")


@dataclass
class TripMod:
    change_id: str
    kind: str  # "P2P", "UNIFORM" or "ALL"
    origin: int
    dest: int
    multiplier: float


def _check(mod: TripMod) -> None:
    if mod.kind not in _KINDS:
        raise ValueError(f"invalid trip data change type '{mod.kind}'")
    if mod.kind == "P2P" and (mod.origin == 0 or mod.dest == 0):
        raise ValueError("origin and dest must be nonzero for point-to-point")
    if mod.kind != "ALL" and mod.origin == 0 and mod.dest == 0:
        raise ValueError("cannot have 0 for both origin and dest except type ALL")


def read_trip_mods(path: str) -> List[TripMod]:
    """Parse a trip modifications file (tap/parsetapfiles.c:573-638)."""
    out = []
    with open(path) as f:
        for line in f:
            if line.startswith("~") or not line.strip():
                continue
            tok = line.rstrip("\r\n").split("\t")
            mod = TripMod(tok[0], tok[1], int(float(tok[2])), int(float(tok[3])), float(tok[4]))
            _check(mod)
            out.append(mod)
    return out


def write_trip_mods(path: str, mods: Sequence[TripMod]) -> None:
    with open(path, "w") as f:
        f.write("~ id\ttype\torigin\tdest\tmultiplier\n")
        for m in mods:
            f.write(f"{m.change_id}\t{m.kind}\t{m.origin}\t{m.dest}\t{m.multiplier!r}\n")


def apply_trip_mod(dem: Demand, mod: TripMod) -> Demand:
    """A copy of `dem` with one modification applied (tap/tap_functions.c:521-598)."""
    _check(mod)
    z = dem.num_zones
    if mod.origin > z or mod.dest > z or mod.origin < 0 or mod.dest < 0:
        raise ValueError(f"bad origin {mod.origin} or dest {mod.dest} in trip modification")
    d = dem.od_demand.copy()
    ptr, dest = dem.od_ptr, dem.od_dest
    if mod.kind == "P2P":
        for i in range(ptr[mod.origin], ptr[mod.origin + 1]):
            if dest[i] == mod.dest:
                d[i] *= mod.multiplier
                break
    elif mod.kind == "UNIFORM":
        if mod.dest == 0 and mod.origin > 0:
            d[ptr[mod.origin]:ptr[mod.origin + 1]] *= mod.multiplier
        elif mod.origin == 0 and mod.dest > 0:
            sel = dest[ptr[1]:ptr[z + 1]] == mod.dest
            d[ptr[1]:ptr[z + 1]][sel] *= mod.multiplier
        else:
            raise ValueError("both origin and dest nonzero in uniform trip mod")
    else:
        d[ptr[1]:ptr[z + 1]] *= mod.multiplier
    return Demand(z, dem.od_ptr, dem.od_dest, d)


def apply_trip_mods(dem: Demand, mods: Sequence[TripMod]) -> Demand:
    for m in mods:
        dem = apply_trip_mod(dem, m)
    return dem


def demand_entries(dem: Demand) -> np.ndarray:
    """The OD entries of origins 1..Z in the order the solver stores them."""
    return dem.od_demand[dem.od_ptr[1]:dem.od_ptr[dem.num_zones + 1]]


def demand_scenarios(dem: Demand, mod_sets: Sequence[Sequence[TripMod]]) -> np.ndarray:
    """[len(mod_sets)][OD entries]: scenario s = `dem` with mod_sets[s] applied."""
    return np.stack([demand_entries(apply_trip_mods(dem, ms)) for ms in mod_sets])
