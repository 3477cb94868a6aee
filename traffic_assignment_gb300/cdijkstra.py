"""Python 3 drop-in for the reference's ``cdijkstra`` extension module
(python_extension/dijkstra_module.c:79-201), running on the GPU library.

  dijkstra(graph, num_nodes, start_node) -> list pred[v]

graph[u][v] = cost with nodes 0..num_nodes-1; pred[v] is the predecessor node
of v on a shortest path from start_node, -1 if none.  Every node may be passed
through (the module has no first-thru-node rule).  IndexError
("start_node >= num_nodes") as in the reference.  On equal-cost paths the
predecessor can differ from the reference's heap order; labels are exact.
"""

from __future__ import annotations

import numpy as np

from .pape import _edges, _network
from .solver import Solver

__all__ = ["dijkstra"]


def dijkstra(graph, num_nodes, start_node):
    num_nodes = int(num_nodes)
    if int(start_node) >= num_nodes:
        raise IndexError("start_node >= num_nodes")
    init, term, w = _edges(graph)
    if len(init) == 0:
        return [-1] * num_nodes
    with Solver(_network(init, term, num_nodes, 0), None) as s:
        _, pred = s.sssp(w, [int(start_node)], want_dist=False)
    links = pred[0, :num_nodes]
    return [int(v) for v in np.where(links >= 0, init[np.maximum(links, 0)], -1)]
