"""Launch-shape autotuner for the batched Frank-Wolfe iteration.

The fastest shortest-path kernel depends on the network (node count, degree,
cost spread) and on how many tasks a launch holds.  ``tune`` sweeps

  * the shortest-path variant: bulk-synchronous rounds, asynchronous
    worklist, near-far, near-far with a FIFO ring (the default),
  * its block size (128 .. 1024 threads),
  * the near-far phase step, as a multiple of the mean free-flow time,
  * the all-or-nothing loading block size,

on a sample of the real workload: the network and its demand, a batch of
upgrade scenarios warm-started from a near-equilibrium flow, so that link
costs, label spreads and frontier sizes are those of the loop being tuned.
Each candidate runs a few FW iterations after one untimed iteration (graph
instantiation), timed per kernel with the solver's CUDA events; the
candidate with the smallest time per iteration wins.  Results are cached in
a JSON file keyed by a hash of the network's arrays, the precision, the
batch size and the GPU name, so a tuned deployment pays for the sweep once.
"""

from __future__ import annotations

import hashlib
import json
import os
import time
from dataclasses import asdict, dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np

from .solver import Solver
from .synth import Demand, Network, make_scenarios

__all__ = ["Candidate", "TuneResult", "candidates", "tune", "tuned_options", "cache_key"]

_VARIANTS = ("rounds", "async", "nearfar", "nearfar_queue")


@dataclass(frozen=True)
class Candidate:
    sssp_variant: str = "nearfar_queue"
    sssp_block: int = 256
    nf_scale: float = 16.0  # near-far step = nf_scale x mean free-flow time
    aon_block: int = 0  # 0: the library's choice for the precision and network size

    def solver_kwargs(self, net: Network) -> Dict:
        kw = dict(sssp_variant=self.sssp_variant, sssp_block=self.sssp_block,
                  aon_block=self.aon_block)
        if self.sssp_variant.startswith("nearfar"):
            kw["nf_delta"] = float(self.nf_scale * np.mean(net.fft))
        return kw


@dataclass
class TuneResult:
    best: Candidate
    ms_per_iteration: float
    table: List[Dict] = field(default_factory=list)
    key: str = ""
    from_cache: bool = False

    def solver_kwargs(self, net: Network) -> Dict:
        return self.best.solver_kwargs(net)


# networks up to this many nodes and links also try the edge-list sweeps
# (the library's default there)
SMALL_NET = 4096


def candidates(quick: bool = False, net: Optional[Network] = None) -> List[Candidate]:
    """The sweep: every variant x block, and near-far x step scale, with the
    library's loading shape; then the loading kernel's block at the library's
    shortest-path shape (block 0: the library's choice); with a small network
    (at most SMALL_NET nodes and links) the edge-list sweeps too."""
    out = []
    blocks = (256, 512) if quick else (128, 256, 512, 1024)
    scales = (8.0, 16.0, 32.0) if quick else (4.0, 8.0, 16.0, 32.0, 64.0)
    variants = _VARIANTS
    if net is not None and net.num_nodes + 1 <= SMALL_NET and net.num_links <= SMALL_NET:
        variants = variants + ("small",)
    for v in variants:
        for b in blocks:
            if v.startswith("nearfar"):
                out.extend(Candidate(v, b, s, 0) for s in scales)
            else:
                out.append(Candidate(v, b, 16.0, 0))
    # the loading kernel's block, at the default shortest-path shape
    out.extend(Candidate("nearfar_queue", 0, 16.0, a) for a in (256, 512, 1024))
    return out


def _device_name(device: int) -> str:
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(device)
    except Exception:  # pragma: no cover - torch is optional here
        pass
    return "cuda:%d" % device


def cache_key(net: Network, precision: str, scenarios: int, device_name: str) -> str:
    h = hashlib.sha1()
    for a in (net.init, net.term, net.fft, net.capacity):
        h.update(np.ascontiguousarray(a).tobytes())
    h.update(repr((net.num_nodes, net.num_zones, net.first_thru_node, precision, scenarios,
                   device_name)).encode())
    return h.hexdigest()


def _load_cache(path: Optional[str]) -> Dict:
    if not path or not os.path.exists(path):
        return {}
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store_cache(path: Optional[str], key: str, res: TuneResult) -> None:
    if not path:
        return
    data = _load_cache(path)
    data[key] = dict(best=asdict(res.best), ms_per_iteration=res.ms_per_iteration,
                     table=res.table)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1)
    os.replace(tmp, path)


def _time_candidate(net, dem, precision, cand, scen, x0, iters, device) -> Dict:
    t0 = time.perf_counter()
    with Solver(net, dem, precision=precision, device=device,
                **cand.solver_kwargs(net)) as s:
        s.solve_scenarios(scen, max_iters=1, x0=x0)
        s.run_iterations(1)  # graph instantiation, untimed
        s.set_timing(True)
        s.run_iterations(iters)
        tm = s.timing()
        s.set_timing(False)
    per = {k: tm[f"{k}_ms"] / iters for k in ("sssp", "aon", "line_search", "step")}
    return dict(candidate=asdict(cand), ms_per_iteration=sum(per.values()),
                kernels_ms=per, wall_s=time.perf_counter() - t0)


def tune(net: Network, dem: Demand, precision: str = "fp32", scenarios: int = 32,
         iters: int = 3, warm_iters: int = 40, cache: Optional[str] = None,
         cands: Optional[Sequence[Candidate]] = None, quick: bool = False, device: int = 0,
         scenario_list=None, verbose: bool = False) -> TuneResult:
    """Sweep launch shapes on `scenarios` upgrade scenarios of (net, dem)."""
    dev = _device_name(device)
    key = cache_key(net, precision, scenarios, dev)
    hit = _load_cache(cache).get(key)
    if hit:
        return TuneResult(Candidate(**hit["best"]), hit["ms_per_iteration"], hit["table"], key,
                          True)
    with Solver(net, dem, precision=precision, device=device) as base:
        base.solve(max_iters=warm_iters)
        x0, _ = base.flows()
    scen = scenario_list if scenario_list is not None else make_scenarios(net, scenarios,
                                                                          seed=4242)
    table = []
    for cand in (cands if cands is not None else candidates(quick, net)):
        try:
            row = _time_candidate(net, dem, precision, cand, scen, x0, iters, device)
        except RuntimeError as e:  # a shape that does not fit this network
            row = dict(candidate=asdict(cand), ms_per_iteration=float("inf"), error=str(e))
        table.append(row)
        if verbose:
            print("autotune", row["candidate"], "%.3f ms/it" % row["ms_per_iteration"],
                  flush=True)
    best_row = min(table, key=lambda r: r["ms_per_iteration"])
    if not np.isfinite(best_row["ms_per_iteration"]):
        raise RuntimeError("autotune: no candidate launch shape ran on this network")
    res = TuneResult(Candidate(**best_row["candidate"]), best_row["ms_per_iteration"], table, key)
    _store_cache(cache, key, res)
    return res


def tuned_options(net: Network, dem: Demand, precision: str = "fp32", scenarios: int = 32,
                  cache: Optional[str] = None, **kw) -> Dict:
    """Solver keyword arguments of the tuned launch shape (cached when `cache` is set)."""
    return tune(net, dem, precision, scenarios, cache=cache, **kw).solver_kwargs(net)
