"""The Python 3 drop-ins of the reference's extension modules (pape, cdijkstra)
against the oracle's Pape (tap/sssp_pape.c:120-220, the algorithm of
python_extension/pape_module.c) on tie-free random graphs: predecessor nodes
identical, first-thru-node rule honoured, the modules' IndexErrors kept."""

import numpy as np
import pytest

import oracle
from traffic_assignment_gb300 import cdijkstra, pape

pytestmark = pytest.mark.gpu


def _graph(seed, n=300, deg=4):
    rng = np.random.default_rng(seed)
    g = {u: {} for u in range(n)}
    for u in range(n):  # a ring keeps every node reachable, random chords add choice
        g[u][(u + 1) % n] = float(rng.uniform(1.0, 10.0))
        for v in rng.choice(n, deg - 1, replace=False):
            if int(v) != u:
                g[u][int(v)] = float(rng.uniform(1.0, 10.0))
    return g


def _oracle_pred_nodes(g, n, start, first_thru, weights=None):
    rows = sorted((u, v, c) for u, nb in g.items() for v, c in nb.items())
    init = np.array([r[0] for r in rows], np.int64)
    term = np.array([r[1] for r in rows], np.int64)
    w = np.array([r[2] for r in rows]) if weights is None else np.asarray(weights, float)
    va = np.zeros(n + 1, np.int64)
    np.add.at(va, init + 1, 1)
    va = np.cumsum(va)
    _, pred = oracle.sssp_all(va, term, w, n, [start], first_thru, lll=False)
    link = pred[0]
    return np.where(link >= 0, init[np.maximum(link, 0)], -1), w


@pytest.mark.parametrize("first_thru", [0, 7])
def test_pape_module(built_lib, first_thru):
    n = 300
    g = _graph(11)
    pape.build_adjlist(g, n, first_thru)
    _, w = _oracle_pred_nodes(g, n, 0, first_thru)
    pape.update_weights(list(w))
    for start in (0, 3, 150, 299):
        ref, _ = _oracle_pred_nodes(g, n, start, first_thru)
        assert pape.pape(start) == [int(v) for v in ref]
    # new weights through update_weights, same edge order
    w2 = w * np.random.default_rng(3).uniform(0.5, 2.0, w.size)
    pape.update_weights(list(w2))
    ref, _ = _oracle_pred_nodes(g, n, 42, first_thru, w2)
    assert pape.pape(42) == [int(v) for v in ref]
    with pytest.raises(IndexError, match="start_node >= num_nodes"):
        pape.pape(n)
    with pytest.raises(IndexError, match="list length != num edges"):
        pape.update_weights(list(w2[:-1]))


def test_cdijkstra_module(built_lib):
    n = 250
    g = _graph(12, n)
    for start in (0, 17, 249):
        ref, _ = _oracle_pred_nodes(g, n, start, 0)
        assert cdijkstra.dijkstra(g, n, start) == [int(v) for v in ref]
    with pytest.raises(IndexError, match="start_node >= num_nodes"):
        cdijkstra.dijkstra(g, n, n)
