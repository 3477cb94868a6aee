"""The drop-in entry points against the reference's golden outputs and the oracle.

* tap_frankwolfe_gpu (the CLI with tap/tap_main.c's flags) on the golden cases:
  flows and costs within 1e-6 relative (FP64), every -v log line's objective,
  relative gap and VHT within 1e-6, the same iteration count;
* tap_frankwolfe() called through the C ABI with parsed TNTP structures;
* pape_cuda / sssp_* / fw_assign: labels bit-exact against the reference's
  sssp_pape_lll labels, predecessors tight in-links;
* the tap_functions array operations against the oracle.
"""

import ctypes as C
import glob
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle
from test_abi import DemandData, LinkData, NetData, _libc
from test_oracle import load_fw_golden
from traffic_assignment_gb300 import build as B
from traffic_assignment_gb300 import synth, tntp

pytestmark = pytest.mark.gpu

GOLDEN_DIR = os.path.join(os.path.dirname(__file__), "golden")
FW_GOLDEN = sorted(glob.glob(os.path.join(GOLDEN_DIR, "fw_*.npz")))
SSSP_GOLDEN = sorted(glob.glob(os.path.join(GOLDEN_DIR, "sssp_*.npz")))
F64P = C.POINTER(C.c_double)
LP = C.POINTER(C.c_long)


def _rel(a, b):
    return np.abs(a - b).max() / max(1.0, np.abs(b).max())


def _bpr(net, x, cap=None):
    cap = net.capacity if cap is None else cap
    return net.fft * (1.0 + net.alpha * (x / cap) ** net.beta)


def _write_case(net, dem, wd):
    nf, tf = os.path.join(wd, "net.txt"), os.path.join(wd, "trips.txt")
    tntp.write_net(nf, net)
    tntp.write_trips(tf, dem)
    return nf, tf


def _run_cli(args, env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    res = subprocess.run([B.cli_path(), *args], capture_output=True, text=True, env=env,
                         timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    init, term, vol, cost, hdr = tntp.read_flows(res.stdout, is_text=True)
    return init, term, vol, cost, hdr, tntp.parse_iteration_log(res.stderr)


@pytest.mark.parametrize("path", FW_GOLDEN, ids=[os.path.basename(p) for p in FW_GOLDEN])
def test_cli_matches_reference_golden(built_lib, path, tmp_path):
    net, dem, z = load_fw_golden(path)
    nf, tf = _write_case(net, dem, str(tmp_path))
    iters = int(z["hdr_iterations"])
    args = ["-n", "4", "-v"]
    if "_r1e-3" in path:
        args += ["-r", "0.001"]
    else:
        args += ["-i", str(iters)]
    if "x0" in z.files:
        wf = os.path.join(str(tmp_path), "warm.txt")
        tntp.write_flows(wf, net, z["x0"], _bpr(net, z["x0"]))
        args += ["-w", wf]
    init, term, vol, cost, hdr, log = _run_cli(args + [nf, tf])
    np.testing.assert_array_equal(init, net.init)
    np.testing.assert_array_equal(term, net.term)
    assert _rel(vol, z["volume"]) < 1e-6
    assert _rel(cost, z["cost"]) < 1e-6
    assert int(hdr["iterations"]) == iters
    assert abs(hdr["relgap"] - float(z["hdr_relgap"])) <= 1e-6 * abs(float(z["hdr_relgap"]))
    assert abs(hdr["totalcost"] - float(z["hdr_totalcost"])) <= 1e-6 * float(z["hdr_totalcost"])
    ref = z["log"]
    assert log.shape == ref.shape
    np.testing.assert_array_equal(log[:, 0], ref[:, 0])
    for col in (1, 2, 4):  # objective, relative gap, VHT
        np.testing.assert_allclose(log[:, col], ref[:, col], rtol=1e-6)


def test_cli_fp32_paths(built_lib, tmp_path):
    net, dem, z = load_fw_golden(os.path.join(GOLDEN_DIR, "fw_grid416_i200.npz"))
    nf, tf = _write_case(net, dem, str(tmp_path))
    _, _, vol, _, hdr, _ = _run_cli(["-i", "200", nf, tf], {"TAPGPU_PRECISION": "fp32"})
    assert int(hdr["iterations"]) == 200
    assert _rel(vol, z["volume"]) < 1e-4


def _parse_case(lib, net, dem, wd):
    libc = _libc()
    nf, tf = _write_case(net, dem, wd)
    lib.parse_net_file.argtypes = [C.c_void_p, C.POINTER(NetData)]
    lib.parse_trips_file.argtypes = [C.c_void_p, C.POINTER(C.POINTER(C.POINTER(DemandData))),
                                     C.POINTER(C.c_long)]
    nd = NetData()
    fp = libc.fopen(nf.encode(), b"r")
    assert lib.parse_net_file(fp, C.byref(nd)) == 0
    libc.fclose(fp)
    dems = C.POINTER(C.POINTER(DemandData))()
    nz = C.c_long()
    fp = libc.fopen(tf.encode(), b"r")
    assert lib.parse_trips_file(fp, C.byref(dems), C.byref(nz)) == 0
    libc.fclose(fp)
    return nd, dems


def test_tap_frankwolfe_entry_point(built_lib, tmp_path):
    lib = built_lib
    net, dem, z = load_fw_golden(os.path.join(GOLDEN_DIR, "fw_small24_i100.npz"))
    nd, dems = _parse_case(lib, net, dem, str(tmp_path))
    libc = _libc()
    out = os.path.join(str(tmp_path), "flows.txt")
    fp = libc.fopen(out.encode(), b"w+")
    lib.tap_frankwolfe.argtypes = [C.POINTER(NetData), C.POINTER(C.POINTER(DemandData)), C.c_int,
                                   C.c_void_p, C.c_int, C.c_double, C.c_void_p, F64P, F64P,
                                   C.POINTER(C.c_int), F64P, C.c_int]
    lib.tap_frankwolfe.restype = C.c_int
    tc, ov, rg = C.c_double(), C.c_double(), C.c_double()
    it = C.c_int()
    rc = lib.tap_frankwolfe(C.byref(nd), dems, 0, None, 100, 0.0, fp, C.byref(tc), C.byref(ov),
                            C.byref(it), C.byref(rg), 0)
    libc.fclose(fp)
    assert rc == 0 and it.value == 100
    assert abs(tc.value - float(z["hdr_totalcost"])) <= 1e-6 * float(z["hdr_totalcost"])
    assert abs(rg.value - float(z["hdr_relgap"])) <= 1e-6 * abs(float(z["hdr_relgap"]))
    _, _, vol, cost, _ = tntp.read_flows(out)
    assert _rel(vol, z["volume"]) < 1e-6
    assert _rel(cost, z["cost"]) < 1e-6


def _forward_star(z):
    init, term, w = z["init"], z["term"], z["weight"]
    n1 = int(z["num_nodes"]) + 1
    va = np.zeros(n1 + 1, np.int64)
    np.add.at(va, init + 1, 1)
    return np.cumsum(va), np.ascontiguousarray(term, np.int64), np.ascontiguousarray(w), n1


def _check_tight(z, d, p, v_range, src):
    for v in v_range:
        k = p[v]
        if k < 0:
            assert v == src or d[v] == np.finfo(float).max
        else:
            assert z["term"][k] == v
            assert d[z["init"][k]] + z["weight"][k] == d[v]


@pytest.mark.parametrize("path", SSSP_GOLDEN, ids=[os.path.basename(p) for p in SSSP_GOLDEN])
def test_pape_cuda_labels_bit_exact(built_lib, path):
    lib = built_lib
    z = np.load(path)
    va, ea, wa, n1 = _forward_star(z)
    src = np.ascontiguousarray(z["sources"], np.int64)
    ns = len(src)
    dist = np.zeros(n1 * (ns + 1))
    pred = np.zeros(n1 * (ns + 1), np.int64)
    lib.pape_cuda.argtypes = [LP, LP, F64P, C.c_long, C.c_long, LP, C.c_long, C.c_long, F64P,
                              LP]
    lib.pape_cuda.restype = None
    lib.pape_cuda(va.ctypes.data_as(LP), ea.ctypes.data_as(LP), wa.ctypes.data_as(F64P), n1,
                  len(ea), src.ctypes.data_as(LP), ns, int(z["first_thru_node"]),
                  dist.ctypes.data_as(F64P), pred.ctypes.data_as(LP))
    for i, s in enumerate(src):
        d = dist[np.arange(n1) * ns + s]
        p = pred[np.arange(n1) * ns + s]
        np.testing.assert_array_equal(d[1:], z["dist"][i, 1:])
        _check_tight(z, d, p, range(1, n1), s)


@pytest.mark.parametrize("fn", ["sssp_pape", "sssp_pape_lll", "sssp_slf", "sssp_slf_lll"])
def test_single_source_entry_points(built_lib, fn):
    lib = built_lib
    z = np.load(os.path.join(GOLDEN_DIR, "sssp_martin.npz"))
    va, ea, wa, n1 = _forward_star(z)
    f = getattr(lib, fn)
    f.argtypes = [LP, LP, F64P, C.c_long, C.c_long, C.c_long, C.c_long, LP, F64P, LP]
    f.restype = None
    qn = np.zeros(n1, np.int64)
    for i, s in enumerate(z["sources"][:25]):
        d = np.zeros(n1)
        p = np.zeros(n1, np.int64)
        f(va.ctypes.data_as(LP), ea.ctypes.data_as(LP), wa.ctypes.data_as(F64P), n1, len(ea),
          int(s), int(z["first_thru_node"]), p.ctypes.data_as(LP), d.ctypes.data_as(F64P),
          qn.ctypes.data_as(LP))
        np.testing.assert_array_equal(d[1:], z["dist"][i, 1:])
        _check_tight(z, d, p, range(1, n1), s)


def test_fw_assign_loads(built_lib, tmp_path):
    lib = built_lib
    net, dem = synth.make_grid416()
    nd, dems = _parse_case(lib, net, dem, str(tmp_path))
    n1, m, zc = net.num_nodes + 1, net.num_links, net.num_zones
    va = np.zeros(n1 + 1, np.int64)
    ea = np.zeros(m, np.int64)
    wa = np.zeros(m)
    lib.adjlist_to_packed_arrays.argtypes = [C.POINTER(LinkData), C.c_long, C.c_long, LP, LP,
                                             F64P]
    lib.adjlist_to_packed_arrays(nd.links, n1, m, va.ctypes.data_as(LP), ea.ctypes.data_as(LP),
                                 wa.ctypes.data_as(F64P))
    lib.fw_assign.argtypes = [C.POINTER(NetData), C.POINTER(C.POINTER(DemandData)), LP, LP, F64P,
                              F64P, F64P, LP]
    lib.fw_assign.restype = None
    for t in (net.fft, _bpr(net, np.full(m, 900.0))):
        w = np.ascontiguousarray(t)
        vol = np.zeros(m)
        dist = np.zeros(n1 * (zc + 1))
        pred = np.zeros(n1 * (zc + 1), np.int64)
        lib.fw_assign(C.byref(nd), dems, va.ctypes.data_as(LP), ea.ctypes.data_as(LP),
                      w.ctypes.data_as(F64P), vol.ctypes.data_as(F64P),
                      dist.ctypes.data_as(F64P), pred.ctypes.data_as(LP))
        assert _rel(vol, oracle.aon(net, dem, w)) < 1e-12
        dref, _ = oracle.sssp_all(va, ea, w, n1, np.arange(1, zc + 1), net.first_thru_node)
        for s in range(1, zc + 1):
            np.testing.assert_array_equal(dist[np.arange(1, n1) * zc + s], dref[s - 1, 1:])


def test_link_array_operations(built_lib, tmp_path):
    lib = built_lib
    net, dem = synth.make_grid416()
    nd, _ = _parse_case(lib, net, dem, str(tmp_path))
    rng = np.random.default_rng(5)
    m = net.num_links
    x = rng.uniform(0, 2000, m)
    y = rng.uniform(0, 2000, m)
    d = y - x
    lib.update_link_costs.argtypes = [C.POINTER(NetData), F64P, F64P]
    lib.update_link_costs.restype = None
    t = np.zeros(m)
    lib.update_link_costs(C.byref(nd), x.ctypes.data_as(F64P), t.ctypes.data_as(F64P))
    assert _rel(t, _bpr(net, x)) < 1e-12
    lib.links_objective_function.argtypes = [C.POINTER(NetData), F64P]
    lib.links_objective_function.restype = C.c_double
    obj = lib.links_objective_function(C.byref(nd), x.ctypes.data_as(F64P))
    assert abs(obj - oracle.objective(net, x)) <= 1e-12 * abs(obj)
    lib.link_directional_derivative.argtypes = [C.POINTER(NetData), F64P, F64P, C.c_double]
    lib.link_directional_derivative.restype = C.c_double
    for lam in (0.0, 0.3, 1.0):
        g = lib.link_directional_derivative(C.byref(nd), x.ctypes.data_as(F64P),
                                            d.ctypes.data_as(F64P), lam)
        gr = oracle.directional_derivative(net, x, d, lam)
        assert abs(g - gr) <= 1e-12 * max(1.0, abs(gr))
    lib.total_link_cost.argtypes = [C.POINTER(NetData), F64P, F64P]
    lib.total_link_cost.restype = C.c_double
    tc = lib.total_link_cost(C.byref(nd), x.ctypes.data_as(F64P), t.ctypes.data_as(F64P))
    assert abs(tc - float(np.dot(x, t))) <= 1e-12 * tc
    lib.line_search.argtypes = [C.POINTER(NetData), F64P, F64P]
    lib.line_search.restype = C.c_double
    lam = lib.line_search(C.byref(nd), x.ctypes.data_as(F64P), d.ctypes.data_as(F64P))
    assert lam == oracle.line_search(net, x, d)


def test_cli_trip_mods_match_reference_golden(built_lib, tmp_path):
    """-t (trip modifications, tap/tap_main.c) against the reference's own run
    with the same file: flows, costs and log lines within 1e-6."""
    from test_oracle import load_tripmods_golden
    from traffic_assignment_gb300 import tripmods
    net, dem, mods, z = load_tripmods_golden()
    nf, tf = _write_case(net, dem, str(tmp_path))
    mf = os.path.join(str(tmp_path), "tripmods.txt")
    tripmods.write_trip_mods(mf, mods)
    _, _, vol, cost, hdr, log = _run_cli(["-n", "4", "-v", "-i", "60", "-t", mf, nf, tf])
    assert _rel(vol, z["volume"]) < 1e-6
    assert _rel(cost, z["cost"]) < 1e-6
    assert int(hdr["iterations"]) == 60
    assert abs(hdr["relgap"] - float(z["hdr_relgap"])) <= 1e-6 * abs(float(z["hdr_relgap"]))
    for col in (1, 2, 4):
        np.testing.assert_allclose(log[:, col], z["log"][:, col], rtol=1e-6)


def test_cli_checkpoint_on_sigusr2_and_clean_finish_on_sigterm(built_lib, tmp_path):
    """SIGUSR2 rewrites the flows file in place with the checkpoint header and
    the current flows while the solve goes on; SIGTERM then ends it cleanly
    with the final flows file (tap/tap_frankwolfe_pthread.c:215-254, 766-803).
    The signals are sent from the host between launches of iterations."""
    import signal
    import threading
    import time

    net, dem = synth.make_grid416()
    nf, tf = _write_case(net, dem, str(tmp_path))
    flows = str(tmp_path / "flows.txt")
    lines = []
    with open(flows, "w") as out:
        proc = subprocess.Popen([B.cli_path(), "-n", "1", "-i", "10000000", nf, tf], stdout=out,
                                stderr=subprocess.PIPE, text=True)
        reader = threading.Thread(target=lambda: lines.extend(proc.stderr), daemon=True)
        reader.start()
        try:
            time.sleep(3.0)  # past the set-up, inside the iteration loop
            assert proc.poll() is None, "".join(lines)
            proc.send_signal(signal.SIGUSR2)
            t0 = time.time()
            while not any("checkpointing to flows output file...done" in ln for ln in lines):
                assert time.time() - t0 < 60, "no checkpoint: " + "".join(lines)[-2000:]
                time.sleep(0.05)
            text = open(flows).read()
            assert text.startswith("~ checkpoint written at ")
            init, term, vol, cost, hdr = tntp.read_flows(text, is_text=True)
            assert len(vol) == net.num_links and hdr["iterations"] > 0
            np.testing.assert_array_equal(init, net.init)
            assert abs(hdr["totalcost"] - float(vol @ cost)) <= 1e-9 * hdr["totalcost"]
            # the status line of SIGUSR1 and the checkpoint's both carry the iteration
            assert any(ln.startswith("iter = ") for ln in lines)
            proc.send_signal(signal.SIGTERM)
            rc = proc.wait(timeout=120)
        finally:
            if proc.poll() is None:
                proc.kill()
                proc.wait()
    assert rc == 0, "".join(lines)[-2000:]
    # The final write rewinds the file without truncating it, as the reference
    # does (tap/tap_frankwolfe_pthread.c:795-803): it is shorter than the
    # checkpoint by the checkpoint's date line, so the checkpoint's last bytes
    # remain after the final flows.  Read the final header and M links.
    rows = open(flows).read().split("\n")
    keep, links = [], 0
    for ln in rows:  # the final header and metadata, then its first M link records
        if links == net.num_links:
            break
        if ln.startswith("\t") and ln.rstrip().endswith(";"):
            links += 1
        keep.append(ln)
    init, term, vol, cost, hdr = tntp.read_flows("\n".join(keep), is_text=True)
    assert not rows[0].startswith("~ checkpoint")
    assert len(vol) == net.num_links and hdr["iterations"] >= 1
    np.testing.assert_array_equal(init, net.init)
    assert np.all(vol >= 0) and abs(hdr["totalcost"] - float(vol @ cost)) <= 1e-9 * hdr["totalcost"]
