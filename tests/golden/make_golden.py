"""Generate the golden fixtures of tests/golden from the reference itself.

Runs the reference's own CPU solver, compiled from its sources into
oracle/_ref by oracle/build_oracle.py, on seeded synthetic inputs and on the
reference's shortest-path test graphs, and stores inputs and outputs as
compressed .npz files:

  fw_<case>.npz    network + demand, then the reference's flows / costs as
                   printed (%.15f), the flows-file header and every ``-v``
                   iteration line (objective, relgap, average excess, VHT)
  tripmods_<case>.npz  the same with a trip modifications file (-t): the
                   base demand and the modifications (kind, origin, dest,
                   multiplier, in file order)
  sssp_<case>.npz  forward star, weights, and for every source the labels and
                   predecessor links of sssp_pape_lll (tap/sssp_pape.c:284)

Run from the repository root where the reference tree exists:
    python tests/golden/make_golden.py
"""

from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from traffic_assignment_gb300 import synth, tntp  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
REF_SSSP_DIR = os.path.join(oracle.build_oracle.REF_TRUNK, "cuda_sssp")


def _save_fw(name, net, dem, r, extra=None, prefix="fw"):
    arrs = dict(
        num_nodes=net.num_nodes, num_zones=net.num_zones, first_thru_node=net.first_thru_node,
        init=net.init, term=net.term, capacity=net.capacity, length=net.length, fft=net.fft,
        alpha=net.alpha, beta=net.beta, od_ptr=dem.od_ptr, od_dest=dem.od_dest,
        od_demand=dem.od_demand, volume=r["volume"], cost=r["cost"], log=r["log"],
        hdr_iterations=r["header"].get("iterations", -1),
        hdr_objvalue=r["header"].get("objvalue", np.nan),
        hdr_relgap=r["header"].get("relgap", np.nan),
        hdr_totalcost=r["header"].get("totalcost", np.nan))
    if extra:
        arrs.update(extra)
    np.savez_compressed(os.path.join(OUT, f"{prefix}_{name}.npz"), **arrs)
    print("wrote", name, "iters", arrs["hdr_iterations"], "relgap", arrs["hdr_relgap"])


def fw_cases():
    net, dem = synth.make_small24()
    _save_fw("small24_i100", net, dem, oracle.run_reference(net, dem, threads=1, iters=100))

    net, dem = synth.make_grid416()
    _save_fw("grid416_i200", net, dem, oracle.run_reference(net, dem, threads=1, iters=200))
    _save_fw("grid416_r1e-3", net, dem, oracle.run_reference(net, dem, threads=1, relgap=1e-3))

    # warm start from the reference's own flows file after 30 iterations
    wd = tempfile.mkdtemp(prefix="golden_")
    first = oracle.run_reference(net, dem, threads=1, iters=30, workdir=wd)
    flows_path = os.path.join(wd, "flows30.txt")
    tntp.write_flows(flows_path, net, first["volume"], first["cost"])
    with open(flows_path) as f:
        txt = f.read()
    _, _, x0, _, _ = tntp.read_flows(txt, is_text=True)
    warm = oracle.run_reference(net, dem, threads=1, iters=20, warm_flows=flows_path, workdir=wd)
    _save_fw("grid416_warm", net, dem, warm, extra=dict(x0=x0))

    thru, dthru = synth.make_grid416_centroids()
    _save_fw("centroids454_i50", thru, dthru,
             oracle.run_reference(thru, dthru, threads=1, iters=50))


def tripmod_cases():
    """The reference's -t flag (tap/tap_main.c, tap/tap_functions.c:521-598):
    one modification of each kind, applied in file order, then 60 iterations."""
    from traffic_assignment_gb300 import tripmods
    net, dem = synth.make_grid416()
    o1 = 3
    d1 = int(dem.od_dest[dem.od_ptr[o1]])  # an OD pair that exists
    mods = [tripmods.TripMod("p2p", "P2P", o1, d1, 1.75),
            tripmods.TripMod("orig", "UNIFORM", 5, 0, 0.6),
            tripmods.TripMod("dest", "UNIFORM", 0, 12, 1.4),
            tripmods.TripMod("all", "ALL", 0, 0, 1.05)]
    wd = tempfile.mkdtemp(prefix="golden_")
    path = os.path.join(wd, "tripmods.txt")
    tripmods.write_trip_mods(path, mods)
    r = oracle.run_reference(net, dem, threads=1, iters=60, workdir=wd, trip_mods=path)
    _save_fw("grid416_i60", net, dem, r, extra=dict(
        mod_kind=np.array([m.kind for m in mods]), mod_origin=np.array([m.origin for m in mods]),
        mod_dest=np.array([m.dest for m in mods]),
        mod_mult=np.array([m.multiplier for m in mods])), prefix="tripmods")


def _read_rmat(path):
    with open(path) as f:
        n, _, m = (int(t) for t in f.readline().split())
        rows = [line.split() for line in f if line.strip()]
    a = np.array([int(r[0]) for r in rows], np.int64)
    b = np.array([int(r[1]) for r in rows], np.int64)
    w = np.array([float(r[2]) for r in rows])
    return n, a, b, w


def _save_sssp(name, num_nodes, init, term, w, first_thru=1):
    order = np.lexsort((term, init))
    init, term, w = init[order], term[order], w[order]
    n1 = num_nodes + 1
    va = np.zeros(n1 + 1, np.int64)
    np.add.at(va, init + 1, 1)
    va = np.cumsum(va)
    srcs = np.arange(1, n1)
    dist = np.zeros((len(srcs), n1))
    pred = np.zeros((len(srcs), n1), np.int64)
    for i, s in enumerate(srcs):
        dist[i], pred[i] = oracle.ref_sssp(va, term, w, n1, int(s), first_thru)
    np.savez_compressed(os.path.join(OUT, f"sssp_{name}.npz"), num_nodes=num_nodes, init=init,
                        term=term, weight=w, first_thru_node=first_thru, sources=srcs,
                        dist=dist, pred=pred)
    print("wrote sssp", name, num_nodes, len(w))


def sssp_cases():
    for tag in ("martin", "okuyama-example"):
        p = os.path.join(REF_SSSP_DIR, f"rmat.txt.{tag}")
        n, a, b, w = _read_rmat(p)
        _save_sssp(tag.replace("-", "_"), n, a, b, w)
    g = synth.make_integer_graph(11, rows=9, cols=11, max_w=5)
    _save_sssp("intgrid99", g.num_nodes, g.init, g.term, g.fft)


if __name__ == "__main__":
    if not oracle.reference_available():
        sys.exit("reference sources not available: cannot generate golden fixtures")
    fw_cases()
    tripmod_cases()
    sssp_cases()
