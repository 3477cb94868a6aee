"""Upgrade scenarios from a net-mods file, as the reference's MPI farm forms
them (tap/tap_mpi_main.c:201-240, 468-753), solved on the GPU.

Modes (the farm's flags):
  "single"   one scenario per distinct change id (default)
  "pairs"    every pair of distinct change ids, id "A_and_B" (-p, :491-522)
  "subsets"  every subset of size >= 3, at most 16 ids, id "A+B+C" (-s, :523-561)
  "list"     one scenario combining a comma-separated list of ids (-l, :562-597)

Change ids are ordered as the farm sorts them (strncmp, :477).  A CHANGE
record replaces the whole link record and an ADD record appends a link
(:201-240).  Every scenario, whatever its records, is solved in one batch
by tapgpu_solve_scenarios: the batch's network is the union of the base
links and each added link once (``build_link_batch``); a CHANGE becomes a
capacity edit plus, where free-flow time or BPR parameters change, a
per-scenario parameter edit (tapgpu_set_scenario_links); the added links of
other scenarios are absent from a scenario's network.  The warm start gives
added links zero flow, as tap/tap_frankwolfe_pthread.c:564-597 inserts them.
"""

from __future__ import annotations

import dataclasses
import itertools
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .solver import Solver
from .synth import Demand, Network, Scenario
from .tntp import read_net_mods

__all__ = ["NetMod", "group_mods", "enumerate_scenarios", "apply_mods", "LinkBatch",
           "build_link_batch", "solve_farm"]

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


@dataclasses.dataclass
class LinkBatch:
    """Scenarios of link records as one batch over the union network.

    union      base links (indices 0..num_base-1, base order) then each added
               link once, in order of first appearance
    scenarios  capacity edits per scenario (union link indices)
    edits      per scenario (links, fft, alpha, beta) of links whose free-flow
               time or BPR parameters differ from the union row
    absent     per scenario, the union links its network does not have
    members    per scenario, the union links of its network in the order the
               reference's link array holds them after the records
    """

    union: Network
    num_base: int
    scenarios: List[Scenario]
    edits: List[Tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]]
    absent: List[np.ndarray]
    members: List[np.ndarray]

    @property
    def needs_links(self) -> bool:
        """True when some scenario changes parameters or lacks a union link."""
        return any(len(e[0]) for e in self.edits) or any(len(a) for a in self.absent)

    def warm_start(self, x_base: np.ndarray) -> np.ndarray:
        """Base flows on the base links, zero on the added ones."""
        x = np.zeros(self.union.num_links)
        x[: self.num_base] = x_base
        return x

    def scenario_network(self, s: int) -> Network:
        """Scenario s's own network as the reference's farm solves it: its
        links with their capacity and cost parameters, sorted by (init, term)
        (the link order of scenario_order(s))."""
        u = self.union.copy()
        sc = self.scenarios[s]
        for k, c in zip(sc.links.tolist(), sc.new_capacity.tolist()):
            u.capacity[k] = c  # in record order: the last edit of a link wins
        el, f, a, b = self.edits[s]
        u.fft[el], u.alpha[el], u.beta[el] = f, a, b
        return u.take(self.scenario_order(s))

    def scenario_order(self, s: int) -> np.ndarray:
        """Union link index of each link of scenario_network(s), in its order."""
        mem = self.members[s]
        u = self.union
        return mem[np.lexsort((u.term[mem], u.init[mem]))]


_FIELDS = ("init", "term", "capacity", "length", "fft", "alpha", "beta", "speed", "toll",
           "link_type")


def build_link_batch(net: Network, scen_recs: Sequence[Tuple[str, Sequence[NetMod]]]
                     ) -> LinkBatch:
    """Union network and per-scenario edits for scenarios given as (id, records),
    the records applied in order as tap/tap_mpi_main.c:201-240 applies them:
    ADD appends a link, CHANGE replaces the record of the first link (in the
    scenario's link order) with the same end nodes."""
    M = net.num_links
    added: Dict[int, int] = {}  # id(record) -> union link
    add_rows: List[Tuple] = []
    for _, recs in scen_recs:
        for m in recs:
            if m.kind == "ADD" and id(m) not in added:
                added[id(m)] = M + len(add_rows)
                add_rows.append(m.link)
            elif m.kind not in ("ADD", "CHANGE"):
                raise ValueError(f"bad modification type {m.kind}")
    union = net.copy()
    if add_rows:
        cols = list(zip(*add_rows))
        for f, vals in zip(_FIELDS, cols):
            arr = getattr(union, f)
            setattr(union, f, np.concatenate([arr, np.asarray(vals, dtype=arr.dtype)]))
    U = union.num_links
    all_added = np.arange(M, U, dtype=np.int64)
    scen, edits, absent, members = [], [], [], []
    for sid, recs in scen_recs:
        links = list(range(M))  # this scenario's link array, in the reference's order
        cap_l, cap_v = [], []
        par: Dict[int, Tuple[float, float, float]] = {}
        mine = []
        for m in recs:
            init, term, cap, length, fft, b, power, speed, toll, ltype = m.link
            if m.kind == "ADD":
                u = added[id(m)]
                links.append(u)
                mine.append(u)
                par.pop(u, None)  # an added link starts from its own record
                continue
            u = next((k for k in links if union.init[k] == init and union.term[k] == term), None)
            if u is None:
                raise KeyError(f"link not found for change {m.change_id}")
            cap_l.append(u)
            cap_v.append(cap)
            par[u] = (fft, b, power)
        el = np.asarray([u for u, p in par.items()
                         if p != (union.fft[u], union.alpha[u], union.beta[u])], np.int64)
        edits.append((el, np.asarray([par[u][0] for u in el], np.float64),
                      np.asarray([par[u][1] for u in el], np.float64),
                      np.asarray([par[u][2] for u in el], np.float64)))
        scen.append(Scenario(sid, np.asarray(cap_l, np.int64), np.asarray(cap_v, np.float64)))
        absent.append(np.setdiff1d(all_added, np.asarray(mine, np.int64)))
        members.append(np.asarray(links, np.int64))
    return LinkBatch(union, M, scen, edits, absent, members)


def solve_farm(net: Network, dem: Demand, mods_path: str, mode: str = "single",
               changelist: Optional[str] = None, target_relgap: float = 1e-4,
               max_iters: int = 0, warm_start: bool = True, base_relgap: float = 1e-5,
               precision: str = "fp32", solver: Optional[Solver] = None):
    """Solve every scenario of a net-mods file in one batch; returns a list of
    dicts (id, total_cost = VHT, relgap, iterations, batched flag)."""
    raw = read_net_mods(mods_path)
    mods = [NetMod(c, k, l, p) for c, k, l, p in raw]
    groups = group_mods(mods)
    scen = enumerate_scenarios(list(groups), mode, changelist)
    batch = build_link_batch(net, [(sid, [m for c in sel for m in groups[c]])
                                   for sid, sel in scen])
    own = solver is None
    s = solver or Solver(net, dem, precision=precision)
    su = None
    try:
        x0 = None
        if warm_start:
            s.solve(target_relgap=base_relgap, max_iters=max_iters or 100000)
            x0 = batch.warm_start(s.flows()[0])
        # the union network differs from the base only when records add links
        if batch.union.num_links != net.num_links:
            su = Solver(batch.union, dem, precision=precision)
        sv = su or s
        if batch.needs_links:
            sv.set_scenario_links(batch.edits, batch.absent)
        try:
            res = sv.solve_scenarios(batch.scenarios, max_iters=max_iters,
                                     target_relgap=target_relgap, x0=x0)
        finally:
            if batch.needs_links:
                sv.set_scenario_links(None)
        return [dict(id=sid, batched=True, **r) for (sid, _), r in zip(scen, res)]
    finally:
        if su is not None:
            su.close()
        if own:
            s.close()
