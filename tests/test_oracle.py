"""Pin the CPU oracle (oracle/oracle_tap.c) to the reference.

* against the golden fixtures made by the reference itself
  (tests/golden/make_golden.py): flows, costs and every -v log line must
  print identically with the reference's %.15f format;
* against the compiled reference (oracle/_ref) live, where its sources exist
  in this container (skipped elsewhere).
"""

import glob
import os

import numpy as np
import pytest

import oracle
from traffic_assignment_gb300.synth import Demand, Network


def load_fw_golden(path):
    z = np.load(path)
    m = len(z["init"])
    net = Network(num_nodes=int(z["num_nodes"]), num_zones=int(z["num_zones"]),
                  first_thru_node=int(z["first_thru_node"]), init=z["init"], term=z["term"],
                  capacity=z["capacity"], length=z["length"], fft=z["fft"], alpha=z["alpha"],
                  beta=z["beta"], speed=np.zeros(m), toll=np.zeros(m),
                  link_type=np.ones(m, np.int16))
    dem = Demand(num_zones=int(z["num_zones"]), od_ptr=z["od_ptr"], od_dest=z["od_dest"],
                 od_demand=z["od_demand"])
    return net, dem, z


def fmt(a):
    return np.array(["%.15f" % v for v in np.asarray(a).ravel()])


GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "fw_*.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_oracle_matches_reference_golden(path):
    net, dem, z = load_fw_golden(path)
    iters = int(z["hdr_iterations"])
    x0 = z["x0"] if "x0" in z.files else None
    name = os.path.basename(path)
    if "_r1e-3" in name:
        r = oracle.frankwolfe(net, dem, threads=1, target_relgap=1e-3)
    else:
        r = oracle.frankwolfe(net, dem, threads=1, max_iters=iters, x0=x0)
    assert r["iterations"] == iters
    np.testing.assert_array_equal(fmt(r["x"]), fmt(z["volume"]))
    np.testing.assert_array_equal(fmt(r["t"]), fmt(z["cost"]))
    log = z["log"]
    assert log.shape[0] == iters
    tr = r["trace"]
    for col_ref, col_port in ((1, 0), (2, 1), (3, 2), (4, 3)):
        np.testing.assert_array_equal(fmt(tr[:, col_port]), fmt(log[:, col_ref]))
    assert "%.15f" % r["relgap"] == "%.15f" % float(z["hdr_relgap"])
    assert "%.15f" % r["total_cost"] == "%.15f" % float(z["hdr_totalcost"])


SSSP = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "sssp_*.npz")))


@pytest.mark.parametrize("path", SSSP, ids=[os.path.basename(p) for p in SSSP])
def test_oracle_sssp_matches_reference_golden(path):
    z = np.load(path)
    n1 = int(z["num_nodes"]) + 1
    va = np.zeros(n1 + 1, np.int64)
    np.add.at(va, z["init"] + 1, 1)
    va = np.cumsum(va)
    d, p = oracle.sssp_all(va, z["term"], z["weight"], n1, z["sources"],
                           int(z["first_thru_node"]))
    np.testing.assert_array_equal(d, z["dist"])
    np.testing.assert_array_equal(p, z["pred"])


def test_oracle_threads_agree():
    from traffic_assignment_gb300 import synth
    net, dem = synth.make_grid416()
    a = oracle.frankwolfe(net, dem, threads=1, max_iters=30)
    b = oracle.frankwolfe(net, dem, threads=4, max_iters=30)
    assert np.abs(a["x"] - b["x"]).max() <= 1e-9 * np.abs(a["x"]).max()


needs_ref = pytest.mark.skipif(not oracle.reference_available(),
                               reason="reference sources not present")


@needs_ref
@pytest.mark.parametrize("threads", [1, 3])
def test_oracle_matches_live_reference(threads):
    from traffic_assignment_gb300 import synth
    net, dem = synth.make_grid416()
    ref = oracle.run_reference(net, dem, threads=threads, iters=40)
    port = oracle.frankwolfe(net, dem, threads=threads, max_iters=40)
    tol = 0 if threads == 1 else 1e-9
    assert np.abs(port["x"] - ref["volume"]).max() <= tol * np.abs(ref["volume"]).max() + 1e-9
    np.testing.assert_allclose(port["trace"][:, 1], ref["log"][:, 2], rtol=1e-12)


@needs_ref
def test_oracle_sssp_chicago_regional():
    """The reference's own ChicagoRegional graph (12,982 nodes): labels and
    predecessors of the port equal sssp_pape_lll's for a sample of sources."""
    from oracle import build_oracle as ob
    path = os.path.join(ob.REF_TRUNK, "cuda_sssp_double", "rmat.txt.chicagoregionalflows")
    if not os.path.exists(path):
        pytest.skip("graph file absent")
    with open(path) as f:
        n, _, _ = (int(t) for t in f.readline().split())
        rows = np.loadtxt(f)
    a = rows[:, 0].astype(np.int64)
    b = rows[:, 1].astype(np.int64)
    w = rows[:, 2]
    order = np.lexsort((b, a))
    a, b, w = a[order], b[order], w[order]
    n1 = n + 1
    va = np.zeros(n1 + 1, np.int64)
    np.add.at(va, a + 1, 1)
    va = np.cumsum(va)
    srcs = np.arange(1, 1791, 97)
    d, p = oracle.sssp_all(va, b, w, n1, srcs, 1)
    for i, s in enumerate(srcs):
        dr, pr = oracle.ref_sssp(va, b, w, n1, int(s), 1)
        np.testing.assert_array_equal(d[i], dr)
        np.testing.assert_array_equal(p[i], pr)


TRIPMODS = os.path.join(os.path.dirname(__file__), "golden", "tripmods_grid416_i60.npz")


def load_tripmods_golden(path=TRIPMODS):
    """Network, base demand, the trip modifications in file order, fixture."""
    from traffic_assignment_gb300 import tripmods
    net, dem, z = load_fw_golden(path)
    mods = [tripmods.TripMod(f"m{i}", str(k), int(o), int(d), float(m))
            for i, (k, o, d, m) in enumerate(zip(z["mod_kind"], z["mod_origin"], z["mod_dest"],
                                                  z["mod_mult"]))]
    return net, dem, mods, z


def test_oracle_with_trip_mods_matches_reference_golden():
    """The reference's -t run (one modification of each kind): the restated
    modifications (traffic_assignment_gb300/tripmods.py) and the oracle give
    the reference's printed flows, costs and log lines; without them the
    answer differs."""
    from traffic_assignment_gb300 import tripmods
    net, dem, mods, z = load_tripmods_golden()
    r = oracle.frankwolfe(net, tripmods.apply_trip_mods(dem, mods), threads=1, max_iters=60)
    assert r["iterations"] == int(z["hdr_iterations"]) == 60
    np.testing.assert_array_equal(fmt(r["x"]), fmt(z["volume"]))
    np.testing.assert_array_equal(fmt(r["t"]), fmt(z["cost"]))
    for col_ref, col_port in ((1, 0), (2, 1), (3, 2), (4, 3)):
        np.testing.assert_array_equal(fmt(r["trace"][:, col_port]), fmt(z["log"][:, col_ref]))
    assert "%.15f" % r["relgap"] == "%.15f" % float(z["hdr_relgap"])
    base = oracle.frankwolfe(net, dem, threads=1, max_iters=60)
    assert not np.array_equal(fmt(base["x"]), fmt(z["volume"]))
