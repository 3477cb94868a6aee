"""Upgrade scenarios from a net-mods file, as the reference's MPI farm forms
them (tap/tap_mpi_main.c:201-240, 468-753), solved on the GPU.

Modes (the farm's flags):
  "single"   one scenario per distinct change id (default)
  "pairs"    every pair of distinct change ids, id "A_and_B" (-p, :491-522)
  "subsets"  every subset of size >= 3, at most 16 ids, id "A+B+C" (-s, :523-561)
  "list"     one scenario combining a comma-separated list of ids (-l, :562-597)

Change ids are ordered as the farm sorts them (strncmp, :477).  A CHANGE
record replaces the whole link record and an ADD record appends a link
(:201-240).  Scenarios that only change capacities share topology and costs
with the base network and are solved together by tapgpu_solve_scenarios;
any other scenario (added links, changed free-flow time or BPR parameters) is
solved on the GPU as its own network.
"""

from __future__ import annotations

import dataclasses
import itertools
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .solver import Solver
from .synth import Demand, Network, Scenario
from .tntp import read_net_mods

__all__ = ["NetMod", "group_mods", "enumerate_scenarios", "apply_mods", "solve_farm"]

MAX_SUBSET_MODS = 16  # tap/tap_mpi_main.c MAXBIT


@dataclasses.dataclass
class NetMod:
    change_id: str
    kind: str  # "ADD" or "CHANGE"
    link: Tuple  # init, term, capacity, length, fft, B, power, speed, toll, type
    project_cost: float = 0.0


def group_mods(mods: Sequence[NetMod]) -> Dict[str, List[NetMod]]:
    """Records grouped by change id, ids in the farm's sort order."""
    out: Dict[str, List[NetMod]] = {}
    for m in sorted(mods, key=lambda m: m.change_id.encode()):
        out.setdefault(m.change_id, []).append(m)
    return out


def enumerate_scenarios(ids: Sequence[str], mode: str = "single",
                        changelist: Optional[str] = None) -> List[Tuple[str, List[str]]]:
    """(scenario id, change ids applied) in the farm's order."""
    ids = list(ids)
    if mode == "single":
        return [(i, [i]) for i in ids]
    if mode == "pairs":
        return [(f"{a}_and_{b}", [a, b]) for a, b in itertools.combinations(ids, 2)]
    if mode == "subsets":
        if len(ids) > MAX_SUBSET_MODS:
            raise ValueError(f"maximum of {MAX_SUBSET_MODS} modifications allowed for subsets "
                             f"but {len(ids)} given")
        out = []
        for bits in range(7, 1 << len(ids)):
            if bin(bits).count("1") < 3:
                continue
            sel = [ids[k] for k in range(len(ids)) if bits >> k & 1]
            out.append(("+".join(sel), sel))
        return out
    if mode == "list":
        sel = [s for s in (changelist or "").split(",") if s]
        missing = [s for s in sel if s not in ids]
        if missing:
            raise KeyError(f"change {missing[0]} not found")
        return [("+".join(sel), sel)]
    raise ValueError(f"unknown mode {mode}")


def apply_mods(net: Network, mods: Sequence[NetMod]) -> Network:
    """The network with the records applied (tap/tap_mpi_main.c:201-240), links re-sorted."""
    n = net.copy()
    for m in mods:
        init, term, cap, length, fft, b, power, speed, toll, ltype = m.link
        if m.kind == "CHANGE":
            hit = np.nonzero((n.init == init) & (n.term == term))[0]
            if len(hit) == 0:
                raise KeyError(f"link not found for change {m.change_id}")
            k = hit[0]
            n.capacity[k], n.length[k], n.fft[k] = cap, length, fft
            n.alpha[k], n.beta[k], n.speed[k], n.toll[k], n.link_type[k] = b, power, speed, toll, ltype
        elif m.kind == "ADD":
            for f, v in (("init", init), ("term", term), ("capacity", cap), ("length", length),
                         ("fft", fft), ("alpha", b), ("beta", power), ("speed", speed),
                         ("toll", toll), ("link_type", ltype)):
                arr = getattr(n, f)
                setattr(n, f, np.append(arr, np.asarray(v, dtype=arr.dtype)))
        else:
            raise ValueError(f"bad modification type {m.kind}")
    return n.sort_links()


def _capacity_only(net: Network, mods: Sequence[NetMod]):
    """(link indices, new capacities) if the records only change capacities."""
    links, caps = [], []
    for m in mods:
        if m.kind != "CHANGE":
            return None
        init, term, cap, length, fft, b, power, speed, toll, ltype = m.link
        hit = np.nonzero((net.init == init) & (net.term == term))[0]
        if len(hit) == 0:
            raise KeyError(f"link not found for change {m.change_id}")
        k = int(hit[0])
        if (fft, b, power) != (net.fft[k], net.alpha[k], net.beta[k]):
            return None
        links.append(k)
        caps.append(cap)
    return np.asarray(links, np.int64), np.asarray(caps, np.float64)


def solve_farm(net: Network, dem: Demand, mods_path: str, mode: str = "single",
               changelist: Optional[str] = None, target_relgap: float = 1e-4,
               max_iters: int = 0, warm_start: bool = True, base_relgap: float = 1e-5,
               precision: str = "fp32", solver: Optional[Solver] = None):
    """Solve every scenario of a net-mods file; returns a list of dicts
    (id, total_cost = VHT, relgap, iterations, batched flag)."""
    raw = read_net_mods(mods_path)
    mods = [NetMod(c, k, l, p) for c, k, l, p in raw]
    groups = group_mods(mods)
    scen = enumerate_scenarios(list(groups), mode, changelist)
    own = solver is None
    s = solver or Solver(net, dem, precision=precision)
    try:
        x0 = None
        if warm_start:
            s.solve(target_relgap=base_relgap, max_iters=max_iters or 100000)
            x0 = s.flows()[0]
        batch, batch_ids, others = [], [], []
        for sid, sel in scen:
            recs = [m for c in sel for m in groups[c]]
            co = _capacity_only(net, recs)
            if co is None:
                others.append((sid, recs))
            else:
                batch.append(Scenario(sid, co[0], co[1]))
                batch_ids.append(sid)
        out = []
        if batch:
            res = s.solve_scenarios(batch, max_iters=max_iters, target_relgap=target_relgap,
                                    x0=x0)
            for sid, r in zip(batch_ids, res):
                out.append(dict(id=sid, batched=True, **r))
        for sid, recs in others:
            n2 = apply_mods(net, recs)
            with Solver(n2, dem, precision=precision) as s2:
                r = s2.solve(max_iters=max_iters, target_relgap=target_relgap)
            out.append(dict(id=sid, batched=False, **r))
        order = {sid: i for i, (sid, _) in enumerate(scen)}
        out.sort(key=lambda d: order[d["id"]])
        return out
    finally:
        if own:
            s.close()
