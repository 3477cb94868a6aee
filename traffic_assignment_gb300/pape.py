"""Python 3 drop-in for the reference's ``pape`` extension module
(python_extension/pape_module.c:301-515), running on the GPU library.

Same three functions, arguments, module-level state and errors:

  build_adjlist(graph_dict, num_nodes, first_thru_node)
      graph_dict[u][v] = cost; nodes 0..num_nodes-1; edges are ordered by
      (u, v) as pape_module.c:121-146 orders them
  update_weights(weights)   new costs in that (u, v) order;
                            IndexError("list length != num edges") on mismatch
  pape(start_node)          list pred[v]: predecessor NODE of v on a shortest
                            path from start_node, -1 if none (v == start or
                            unreachable); IndexError("start_node >= num_nodes")

Nodes below first_thru_node are not passed through unless they are the
start node (pape_module.c:395).  Labels are those of the reference exactly;
among equal-cost predecessors the lowest-numbered link from a strictly closer
node is chosen, which can differ from the reference's visit order on ties.
"""

from __future__ import annotations

from typing import Dict, List

import numpy as np

from .solver import Solver
from .synth import Network

__all__ = ["build_adjlist", "update_weights", "pape"]

_S = {"solver": None, "num_nodes": 0, "first_thru": 0, "init": None, "weights": None}


def _network(init, term, num_nodes, first_thru):
    m = len(init)
    return Network(num_nodes=max(num_nodes - 1, 1), num_zones=0, first_thru_node=first_thru,
                   init=init, term=term, capacity=np.ones(m), length=np.ones(m),
                   fft=np.zeros(m), alpha=np.zeros(m), beta=np.ones(m), speed=np.zeros(m),
                   toll=np.zeros(m), link_type=np.ones(m, np.int16))


def _edges(graph_dict: Dict[int, Dict[int, float]]):
    rows = []
    for u, nbrs in graph_dict.items():
        if not nbrs:
            continue
        for v, c in nbrs.items():
            rows.append((int(u), int(v), float(c)))
    rows.sort(key=lambda r: (r[0], r[1]))
    init = np.array([r[0] for r in rows], np.int64)
    term = np.array([r[1] for r in rows], np.int64)
    w = np.array([r[2] for r in rows], np.float64)
    return init, term, w


def build_adjlist(graph_dict, num_nodes, first_thru_node):
    init, term, w = _edges(graph_dict)
    if _S["solver"] is not None:
        _S["solver"].close()
    _S["solver"] = Solver(_network(init, term, int(num_nodes), int(first_thru_node)), None)
    _S.update(num_nodes=int(num_nodes), first_thru=int(first_thru_node), init=init, weights=w)
    return None


def update_weights(weight_list):
    if _S["init"] is None or len(weight_list) != len(_S["init"]):
        raise IndexError("list length != num edges")
    _S["weights"] = np.asarray(weight_list, np.float64).copy()
    return None


def pape(start_node) -> List[int]:
    if _S["solver"] is None:
        raise RuntimeError("build_adjlist() has not been called")
    if int(start_node) >= _S["num_nodes"]:
        raise IndexError("start_node >= num_nodes")
    _, pred = _S["solver"].sssp(_S["weights"], [int(start_node)], want_dist=False)
    links = pred[0, : _S["num_nodes"]]
    out = np.where(links >= 0, _S["init"][np.maximum(links, 0)], -1)
    return [int(v) for v in out]
