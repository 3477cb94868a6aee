"""Seeded synthetic road networks and origin-destination demand.

The reference solver reads networks in the TNTP ``_net`` / ``_trips`` text
formats (tap/parsetapfiles.c:62-146, 181-311).  Its published runs use public
TNTP instances (SiouxFalls, Anaheim, ChicagoRegional) that are not shipped with
it, so every workload here is generated from a fixed seed with the shape, size
and value distributions of the named workload:

  ``small24``   24 nodes, 76 links, 24 zones (a 4 x 6 planar grid),
                fft U(2,10), capacity U(4000,26000), integer demand U(0,2000).
  ``grid416``   416 nodes, 914 links, 38 zones (16 x 26 grid spanning tree plus
                42 extra streets), fft lognormal(mean 1.5, sigma 0.6),
                capacity U(1000,8000), 30% of OD pairs nonzero U(1,500).
  ``grid10k``   100 x 100 perturbed grid plus 200 two-way long arterials
                (10,000 nodes, 40,000 links), 1,000 zones on random nodes,
                three capacity classes 1800/3600/7200, gravity demand of
                1.5M trips/h.
  ``grid100k``  316 x 316 grid plus arterials (99,856 nodes, ~400k links),
                4,000 zones, gravity demand.

Conventions match the reference: nodes are numbered 1..N, zones are nodes
1..Z, ``first_thru_node`` is 1 unless asked otherwise, BPR alpha = 0.15 and
beta = 4, and links are sorted by (init, term) as
tap/parsetapfiles.c:528-540 ``link_data_compar`` orders them.
"""

from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np

__all__ = [
    "Network",
    "Demand",
    "Scenario",
    "make_small24",
    "make_grid416",
    "make_grid10k",
    "make_grid100k",
    "make_workload",
    "make_scenarios",
    "make_integer_graph",
]


@dataclasses.dataclass
class Network:
    """Link table of a road network (tap/tap_types.h:20-44, one array per field)."""

    num_nodes: int
    num_zones: int
    first_thru_node: int
    init: np.ndarray  # int64 [M], 1-based
    term: np.ndarray  # int64 [M], 1-based
    capacity: np.ndarray  # float64 [M]
    length: np.ndarray
    fft: np.ndarray  # free-flow time (T_0 of BPR)
    alpha: np.ndarray  # BPR "B"
    beta: np.ndarray  # BPR "power"
    speed: np.ndarray
    toll: np.ndarray
    link_type: np.ndarray  # int16
    x: Optional[np.ndarray] = None  # node coordinates (0-based index node-1)
    y: Optional[np.ndarray] = None

    @property
    def num_links(self) -> int:
        return int(self.init.shape[0])

    def sort_links(self) -> "Network":
        """Return a copy with links ordered by (init, term)."""
        order = np.lexsort((self.term, self.init))
        return self.take(order)

    def take(self, order: np.ndarray) -> "Network":
        kw = {}
        for f in dataclasses.fields(self):
            v = getattr(self, f.name)
            if isinstance(v, np.ndarray) and f.name not in ("x", "y"):
                kw[f.name] = v[order].copy()
            else:
                kw[f.name] = v
        return Network(**kw)

    def copy(self) -> "Network":
        return self.take(np.arange(self.num_links))

    def csr(self):
        """Forward-star arrays (Va[N+2], Ea[M]) of tap/tap_functions.c:313-339."""
        va = np.zeros(self.num_nodes + 2, dtype=np.int64)
        np.add.at(va, self.init + 1, 1)
        va = np.cumsum(va)
        return va, self.term.astype(np.int64)


@dataclasses.dataclass
class Demand:
    """OD demand as a CSR over origins 1..Z (tap/tap_types.h:49-53 lists)."""

    num_zones: int
    od_ptr: np.ndarray  # int64 [Z+2]; entries of origin o are od_ptr[o]:od_ptr[o+1]
    od_dest: np.ndarray  # int64
    od_demand: np.ndarray  # float64

    @property
    def total(self) -> float:
        return float(self.od_demand.sum())

    def dense(self) -> np.ndarray:
        z = self.num_zones
        out = np.zeros((z + 1, z + 1))
        for o in range(1, z + 1):
            s, e = self.od_ptr[o], self.od_ptr[o + 1]
            out[o, self.od_dest[s:e]] += self.od_demand[s:e]
        return out

    @staticmethod
    def from_dense(mat: np.ndarray, keep_zeros: bool = False) -> "Demand":
        """``mat`` is (Z+1) x (Z+1) with row/column 0 unused."""
        z = mat.shape[0] - 1
        ptr = [0, 0]
        dests, vals = [], []
        for o in range(1, z + 1):
            row = mat[o, 1:]
            idx = np.arange(1, z + 1) if keep_zeros else np.nonzero(row)[0] + 1
            dests.append(idx.astype(np.int64))
            vals.append(mat[o, idx].astype(np.float64))
            ptr.append(ptr[-1] + len(idx))
        return Demand(
            num_zones=z,
            od_ptr=np.asarray(ptr, dtype=np.int64),
            od_dest=np.concatenate(dests) if dests else np.zeros(0, np.int64),
            od_demand=np.concatenate(vals) if vals else np.zeros(0),
        )


@dataclasses.dataclass
class Scenario:
    """One upgrade scenario: capacity multipliers on a subset of links."""

    change_id: str
    links: np.ndarray  # int64 link indices into the sorted link table
    new_capacity: np.ndarray  # float64


# ----------------------------------------------------------------------------
# graph construction helpers
# ----------------------------------------------------------------------------


def _grid_edges(rows: int, cols: int):
    idx = np.arange(rows * cols).reshape(rows, cols)
    h = np.stack([idx[:, :-1].ravel(), idx[:, 1:].ravel()], axis=1)
    v = np.stack([idx[:-1, :].ravel(), idx[1:, :].ravel()], axis=1)
    return np.concatenate([h, v], axis=0)


def _lognormal_mean(rng, mean, sigma, size):
    mu = math.log(mean) - 0.5 * sigma * sigma
    return rng.lognormal(mu, sigma, size)


def _spanning_tree(rng, n, edges):
    """Random spanning tree of the undirected ``edges`` (Kruskal, random order)."""
    parent = np.arange(n)

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    order = rng.permutation(len(edges))
    keep = np.zeros(len(edges), dtype=bool)
    for i in order:
        a, b = find(edges[i, 0]), find(edges[i, 1])
        if a != b:
            parent[a] = b
            keep[i] = True
    return keep


def _renumber_zones(rng, num_nodes, zone_nodes):
    """Map 0-based grid nodes to 1-based ids with the zones first (ids 1..Z).

    The other nodes keep their relative grid order, so the thru nodes stay
    spatially local in id order.
    """
    z = len(zone_nodes)
    new_id = np.zeros(num_nodes, dtype=np.int64)
    is_zone = np.zeros(num_nodes, dtype=bool)
    is_zone[zone_nodes] = True
    new_id[zone_nodes] = np.arange(1, z + 1)
    rest = np.nonzero(~is_zone)[0]
    new_id[rest] = np.arange(z + 1, num_nodes + 1)
    return new_id


def _build_network(num_nodes, num_zones, first_thru, u, v, cap, fft, length, ltype,
                   new_id, px, py) -> Network:
    m = len(u)
    init = new_id[u]
    term = new_id[v]
    xs = np.zeros(num_nodes)
    ys = np.zeros(num_nodes)
    xs[new_id - 1] = px
    ys[new_id - 1] = py
    net = Network(
        num_nodes=num_nodes,
        num_zones=num_zones,
        first_thru_node=first_thru,
        init=init.astype(np.int64),
        term=term.astype(np.int64),
        capacity=np.asarray(cap, dtype=np.float64),
        length=np.asarray(length, dtype=np.float64),
        fft=np.asarray(fft, dtype=np.float64),
        alpha=np.full(m, 0.15),
        beta=np.full(m, 4.0),
        speed=np.zeros(m),
        toll=np.zeros(m),
        link_type=np.asarray(ltype, dtype=np.int16),
        x=xs,
        y=ys,
    )
    return net.sort_links()


def _both_ways(e):
    return np.concatenate([e[:, 0], e[:, 1]]), np.concatenate([e[:, 1], e[:, 0]])


# ----------------------------------------------------------------------------
# the workloads
# ----------------------------------------------------------------------------


def make_small24(seed: int = 1001, integer_costs: bool = False):
    """24-node, 76-link planar network, every node a zone (SiouxFalls-sized)."""
    rng = np.random.default_rng(seed)
    rows, cols = 4, 6
    n = rows * cols
    e = _grid_edges(rows, cols)  # 38 undirected streets
    u, v = _both_ways(e)
    m = len(u)
    if integer_costs:
        fft = rng.integers(2, 11, m).astype(np.float64)
    else:
        fft = rng.uniform(2.0, 10.0, m)
    cap = rng.uniform(4000.0, 26000.0, m)
    px = (np.arange(n) % cols) + rng.uniform(-0.2, 0.2, n)
    py = (np.arange(n) // cols) + rng.uniform(-0.2, 0.2, n)
    length = np.hypot(px[u] - px[v], py[u] - py[v])
    zone_nodes = rng.permutation(n)
    new_id = _renumber_zones(rng, n, zone_nodes)
    net = _build_network(n, n, 1, u, v, cap, fft, length, np.ones(m), new_id, px, py)
    dem = rng.integers(0, 2001, (n + 1, n + 1)).astype(np.float64)
    dem[0, :] = 0
    dem[:, 0] = 0
    np.fill_diagonal(dem, 0)
    return net, Demand.from_dense(dem, keep_zeros=True)


def make_grid416(seed: int = 1002, integer_costs: bool = False, first_thru_node: int = 1):
    """416-node, 914-link street network with 38 zones (Anaheim-sized)."""
    rng = np.random.default_rng(seed)
    rows, cols = 16, 26
    n = rows * cols
    e = _grid_edges(rows, cols)
    keep = _spanning_tree(rng, n, e)
    extra = rng.choice(np.nonzero(~keep)[0], 42, replace=False)
    keep[extra] = True
    e = e[keep]  # 415 + 42 = 457 streets -> 914 links
    u, v = _both_ways(e)
    m = len(u)
    if integer_costs:
        fft = rng.integers(1, 6, m).astype(np.float64)
    else:
        fft = _lognormal_mean(rng, 1.5, 0.6, m)
    cap = rng.uniform(1000.0, 8000.0, m)
    px = (np.arange(n) % cols) + rng.uniform(-0.3, 0.3, n)
    py = (np.arange(n) // cols) + rng.uniform(-0.3, 0.3, n)
    length = np.hypot(px[u] - px[v], py[u] - py[v])
    z = 38
    zone_nodes = rng.choice(n, z, replace=False)
    new_id = _renumber_zones(rng, n, zone_nodes)
    net = _build_network(n, z, first_thru_node, u, v, cap, fft, length, np.ones(m),
                         new_id, px, py)
    dem = np.zeros((z + 1, z + 1))
    nz = rng.random((z, z)) < 0.30
    vals = rng.uniform(1.0, 500.0, (z, z))
    dem[1:, 1:] = np.where(nz, vals, 0.0)
    np.fill_diagonal(dem, 0)
    return net, Demand.from_dense(dem)


def make_grid416_centroids(seed: int = 1006):
    """The 416-node street network with its 38 zones as separate centroid nodes.

    Zones are nodes 1..38, each tied to a distinct street node by a two-way
    connector (fft 0.05, capacity 50000); street nodes are 39..454 and
    ``first_thru_node`` is 39, so no path passes through a zone (the layout of
    the TNTP instances whose zones are centroids).
    """
    rng = np.random.default_rng(seed)
    street, dem = make_grid416(seed=1002)
    z = street.num_zones
    n_st = street.num_nodes
    attach = rng.choice(n_st, z, replace=False) + 1  # street node ids (old numbering)
    shift = z  # street node i -> i + z
    init = np.concatenate([street.init + shift, np.arange(1, z + 1), attach + shift])
    term = np.concatenate([street.term + shift, attach + shift, np.arange(1, z + 1)])
    mc = 2 * z
    net = Network(
        num_nodes=n_st + z, num_zones=z, first_thru_node=z + 1,
        init=init.astype(np.int64), term=term.astype(np.int64),
        capacity=np.concatenate([street.capacity, np.full(mc, 50000.0)]),
        length=np.concatenate([street.length, np.full(mc, 0.1)]),
        fft=np.concatenate([street.fft, np.full(mc, 0.05)]),
        alpha=np.concatenate([street.alpha, np.full(mc, 0.15)]),
        beta=np.concatenate([street.beta, np.full(mc, 4.0)]),
        speed=np.zeros(street.num_links + mc), toll=np.zeros(street.num_links + mc),
        link_type=np.concatenate([street.link_type, np.full(mc, 3, np.int16)]))
    return net.sort_links(), dem


def _gravity(rng, zx, zy, total, scale):
    z = len(zx)
    prod = rng.lognormal(0.0, 0.5, z)
    attr = rng.lognormal(0.0, 0.5, z)
    d = np.hypot(zx[:, None] - zx[None, :], zy[:, None] - zy[None, :])
    t = prod[:, None] * attr[None, :] * np.exp(-d / scale)
    np.fill_diagonal(t, 0.0)
    t *= total / t.sum()
    dem = np.zeros((z + 1, z + 1))
    dem[1:, 1:] = t
    return dem


def _arterial_grid(seed, side, num_arterials, num_zones, total_demand, gravity_scale):
    rng = np.random.default_rng(seed)
    n = side * side
    e = _grid_edges(side, side)
    px = (np.arange(n) % side) + rng.uniform(-0.3, 0.3, n)
    py = (np.arange(n) // side) + rng.uniform(-0.3, 0.3, n)
    u, v = _both_ways(e)
    m_grid = len(u)
    fft = _lognormal_mean(rng, 1.5, 0.6, m_grid)
    cap = rng.choice([1800.0, 3600.0], m_grid, p=[0.7, 0.3])
    # long arterials: two-way links spanning 6-15 grid blocks, faster per block
    au = rng.integers(0, n, num_arterials)
    span_r = rng.integers(-15, 16, num_arterials)
    span_c = rng.integers(-15, 16, num_arterials)
    small = (np.abs(span_r) + np.abs(span_c)) < 6
    span_c[small] = 6 * np.sign(span_c[small] + 0.5).astype(np.int64)
    ar = np.clip(au // side + span_r, 0, side - 1)
    ac = np.clip(au % side + span_c, 0, side - 1)
    av = ar * side + ac
    ok = av != au
    pairs = np.stack([au[ok], av[ok]], axis=1)
    pairs = np.unique(np.sort(pairs, axis=1), axis=0)
    # drop any that duplicate a grid street
    grid_set = set(map(tuple, np.sort(e, axis=1).tolist()))
    pairs = np.asarray([p for p in pairs.tolist() if tuple(p) not in grid_set], dtype=np.int64)
    pairs = pairs[:num_arterials]
    blocks = np.abs(pairs[:, 0] // side - pairs[:, 1] // side) + np.abs(
        pairs[:, 0] % side - pairs[:, 1] % side)
    afft1 = 0.45 * 1.5 * blocks * rng.lognormal(0.0, 0.15, len(pairs))
    au2, av2 = _both_ways(pairs)
    afft = np.concatenate([afft1, afft1])
    u = np.concatenate([u, au2])
    v = np.concatenate([v, av2])
    fft = np.concatenate([fft, afft])
    cap = np.concatenate([cap, np.full(len(au2), 7200.0)])
    ltype = np.concatenate([np.ones(m_grid), np.full(len(au2), 2)])
    length = np.hypot(px[u] - px[v], py[u] - py[v])
    zone_nodes = rng.choice(n, num_zones, replace=False)
    new_id = _renumber_zones(rng, n, zone_nodes)
    net = _build_network(n, num_zones, 1, u, v, cap, fft, length, ltype, new_id, px, py)
    dem = _gravity(rng, px[zone_nodes], py[zone_nodes], total_demand, gravity_scale)
    return net, Demand.from_dense(dem)


def make_grid10k(seed: int = 1003):
    """100 x 100 grid + 200 two-way arterials: 10,000 nodes, 40,000 links, 1,000 zones."""
    return _arterial_grid(seed, 100, 200, 1000, 1.5e6, 25.0)


def make_grid3600(seed: int = 1007):
    """60 x 60 grid + 40 arterials, 100 zones: a mid-size test network whose
    per-origin shared-memory working set exceeds the 48 KB default."""
    return _arterial_grid(seed, 60, 40, 100, 1.5e5, 15.0)


def make_grid22k(seed: int = 1008):
    """150 x 150 grid + 300 arterials, 150 zones: 22,500 nodes (16-bit node
    ids) but ~90,000 links (beyond 16 bits), a test network for the compact
    loading layouts with plain link ids as predecessor words."""
    return _arterial_grid(seed, 150, 300, 150, 3.0e5, 30.0)


def make_grid100k(seed: int = 1005, num_zones: int = 4000):
    """316 x 316 grid + arterials: 99,856 nodes, ~400,000 links, 4,000 zones."""
    return _arterial_grid(seed, 316, 2000, num_zones, 15.0e6, 60.0)


def make_integer_graph(seed: int, rows: int = 12, cols: int = 12, max_w: int = 9):
    """Integer-weight grid for bit-exact distance checks (ties are frequent)."""
    rng = np.random.default_rng(seed)
    n = rows * cols
    e = _grid_edges(rows, cols)
    u, v = _both_ways(e)
    m = len(u)
    w = rng.integers(1, max_w + 1, m).astype(np.float64)
    px = (np.arange(n) % cols).astype(np.float64)
    py = (np.arange(n) // cols).astype(np.float64)
    new_id = np.arange(1, n + 1)
    z = n
    net = _build_network(n, z, 1, u, v, np.full(m, 1000.0), w, np.ones(m), np.ones(m),
                         new_id, px, py)
    return net


def make_scenarios(net: Network, count: int, seed: int = 1004, min_links: int = 1,
                   max_links: int = 20, min_gain: float = 0.25, max_gain: float = 1.0):
    """Upgrade scenarios: raise capacity by U(min_gain, max_gain) on 1-20 random links."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(count):
        k = int(rng.integers(min_links, max_links + 1))
        links = np.sort(rng.choice(net.num_links, k, replace=False)).astype(np.int64)
        gain = rng.uniform(min_gain, max_gain, k)
        out.append(Scenario(change_id=f"s{s:04d}", links=links,
                            new_capacity=net.capacity[links] * (1.0 + gain)))
    return out


def make_workload(name: str, seed: Optional[int] = None):
    """Build one of the named workloads (see the module docstring)."""
    table = {
        "small24": make_small24,
        "grid416": make_grid416,
        "grid3600": make_grid3600,
        "grid22k": make_grid22k,
        "grid10k": make_grid10k,
        "grid100k": make_grid100k,
    }
    fn = table[name]
    return fn() if seed is None else fn(seed)
