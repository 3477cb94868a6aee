"""CPU oracle for the Frank-Wolfe user-equilibrium loop (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this package, and only as the checker or the timed CPU
baseline.  The GPU library never imports, links or calls it.

Two oracles are exposed:

* the *port*: ``oracle_tap.c``, this project's C restatement of the reference
  CPU solver (built on any host by ``build_oracle.build_oracle``);
* the *reference*: the reference's own CPU solver compiled from its sources by
  ``build_oracle.build_reference`` into ``oracle/_ref`` (only where the
  reference tree exists).  Tests use it to pin the port.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile
from typing import Optional

import numpy as np

from . import build_oracle as _b

_LIB = None
_REFLIB = None

I64P = C.POINTER(C.c_int64)
F64P = C.POINTER(C.c_double)


class Problem(C.Structure):
    _fields_ = [
        ("num_nodes", C.c_int64),
        ("num_zones", C.c_int64),
        ("first_thru_node", C.c_int64),
        ("num_links", C.c_int64),
        ("init", I64P),
        ("term", I64P),
        ("capacity", F64P),
        ("fft", F64P),
        ("alpha", F64P),
        ("beta", F64P),
        ("od_ptr", I64P),
        ("od_dest", I64P),
        ("od_demand", F64P),
    ]


class IterRow(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("objective", "relgap", "avg_excess", "total_cost", "lambda_", "gap", "ms")]


def lib():
    global _LIB
    if _LIB is None:
        path = _b.build_oracle()
        L = C.CDLL(path)
        L.orc_frankwolfe.restype = C.c_int
        L.orc_frankwolfe.argtypes = [C.POINTER(Problem), C.c_int, F64P, C.c_int, C.c_double,
                                     F64P, F64P, C.POINTER(IterRow), C.c_int, F64P]
        L.orc_aon.restype = C.c_int
        L.orc_aon.argtypes = [C.POINTER(Problem), F64P, C.c_int, F64P]
        L.orc_sssp_many.restype = C.c_int
        L.orc_sssp_many.argtypes = [I64P, I64P, F64P, C.c_int64, C.c_int64, I64P, C.c_int64,
                                    C.c_int64, C.c_int, C.c_int, F64P, I64P]
        L.orc_line_search.restype = C.c_double
        L.orc_line_search.argtypes = [C.POINTER(Problem), F64P, F64P, F64P]
        L.orc_directional_derivative.restype = C.c_double
        L.orc_directional_derivative.argtypes = [C.POINTER(Problem), F64P, F64P, F64P,
                                                 C.c_double]
        L.orc_objective.restype = C.c_double
        L.orc_objective.argtypes = [C.POINTER(Problem), F64P, F64P]
        L.orc_bpr.restype = C.c_double
        L.orc_bpr.argtypes = [C.c_double] * 5
        L.orc_replay_vht.restype = C.c_double
        L.orc_replay_vht.argtypes = [C.POINTER(Problem), F64P, C.c_int, F64P, F64P, F64P]
        L.orc_adjoint_vht.restype = C.c_int
        L.orc_adjoint_vht.argtypes = [C.POINTER(Problem), F64P, C.c_int, F64P, F64P, F64P,
                                      F64P]
        _LIB = L
    return _LIB


def _p(a, t):
    return a.ctypes.data_as(t)


class _Bound:
    """Keeps the numpy arrays behind a Problem alive."""

    def __init__(self, net, dem, capacity=None):
        self.keep = dict(
            init=np.ascontiguousarray(net.init, np.int64),
            term=np.ascontiguousarray(net.term, np.int64),
            cap=np.ascontiguousarray(net.capacity if capacity is None else capacity,
                                     np.float64),
            fft=np.ascontiguousarray(net.fft, np.float64),
            alpha=np.ascontiguousarray(net.alpha, np.float64),
            beta=np.ascontiguousarray(net.beta, np.float64),
            od_ptr=np.ascontiguousarray(dem.od_ptr, np.int64),
            od_dest=np.ascontiguousarray(dem.od_dest, np.int64),
            od_demand=np.ascontiguousarray(dem.od_demand, np.float64),
        )
        k = self.keep
        self.prob = Problem(net.num_nodes, net.num_zones, net.first_thru_node, net.num_links,
                            _p(k["init"], I64P), _p(k["term"], I64P), _p(k["cap"], F64P),
                            _p(k["fft"], F64P), _p(k["alpha"], F64P), _p(k["beta"], F64P),
                            _p(k["od_ptr"], I64P), _p(k["od_dest"], I64P),
                            _p(k["od_demand"], F64P))


def frankwolfe(net, dem, threads: int = 1, max_iters: int = 0, target_relgap: float = 0.0,
               x0: Optional[np.ndarray] = None, capacity: Optional[np.ndarray] = None):
    """Run the oracle FW solve; returns dict(x, t, trace, iterations, objective,
    relgap, total_cost).  ``trace`` columns: objective, relgap, avg_excess,
    total_cost, lambda, gap, ms."""
    b = _Bound(net, dem, capacity)
    m = net.num_links
    x = np.zeros(m)
    t = np.zeros(m)
    cap = max(1, max_iters if max_iters > 0 else 100000)
    trace = (IterRow * cap)()
    summ = np.zeros(4)
    x0a = None if x0 is None else np.ascontiguousarray(x0, np.float64)
    rc = lib().orc_frankwolfe(C.byref(b.prob), threads,
                              None if x0a is None else _p(x0a, F64P), max_iters,
                              target_relgap, _p(x, F64P), _p(t, F64P), trace, cap,
                              _p(summ, F64P))
    if rc != 0:
        raise RuntimeError(f"oracle frankwolfe failed rc={rc}")
    n = int(summ[0])
    tr = np.array([[trace[i].objective, trace[i].relgap, trace[i].avg_excess,
                    trace[i].total_cost, trace[i].lambda_, trace[i].gap, trace[i].ms]
                   for i in range(min(n, cap))]).reshape(-1, 7)
    return dict(x=x, t=t, trace=tr, iterations=n, objective=summ[1], relgap=summ[2],
                total_cost=summ[3])


def aon(net, dem, t, threads: int = 1):
    b = _Bound(net, dem)
    y = np.zeros(net.num_links)
    ta = np.ascontiguousarray(t, np.float64)
    rc = lib().orc_aon(C.byref(b.prob), _p(ta, F64P), threads, _p(y, F64P))
    if rc != 0:
        raise RuntimeError(f"oracle aon failed rc={rc}")
    return y


def line_search(net, x, d, capacity=None):
    b = _Bound(net, _empty_demand(net), capacity)
    xa = np.ascontiguousarray(x, np.float64)
    da = np.ascontiguousarray(d, np.float64)
    return lib().orc_line_search(C.byref(b.prob), _p(b.keep["cap"], F64P), _p(xa, F64P),
                                 _p(da, F64P))


def directional_derivative(net, x, d, lam, capacity=None):
    b = _Bound(net, _empty_demand(net), capacity)
    xa = np.ascontiguousarray(x, np.float64)
    da = np.ascontiguousarray(d, np.float64)
    return lib().orc_directional_derivative(C.byref(b.prob), _p(b.keep["cap"], F64P),
                                            _p(xa, F64P), _p(da, F64P), lam)


def objective(net, x, capacity=None):
    b = _Bound(net, _empty_demand(net), capacity)
    xa = np.ascontiguousarray(x, np.float64)
    return lib().orc_objective(C.byref(b.prob), _p(b.keep["cap"], F64P), _p(xa, F64P))


def replay_vht(net, capacity, x0, loads):
    """VHT after the frozen-load FW map (loads [K][M], exact steps); also the steps."""
    b = _Bound(net, _empty_demand(net), capacity)
    Y = np.ascontiguousarray(loads, np.float64)
    k = Y.shape[0]
    xa = np.ascontiguousarray(x0, np.float64)
    lam = np.zeros(max(k, 1))
    v = lib().orc_replay_vht(C.byref(b.prob), _p(b.keep["cap"], F64P), k, _p(xa, F64P),
                             _p(Y, F64P), _p(lam, F64P))
    return v, lam[:k]


def adjoint_vht(net, capacity, x0, directions, lambdas):
    """FP64 reverse sweep of the frozen-load FW map on a tape -> dVHT/dcapacity."""
    b = _Bound(net, _empty_demand(net), capacity)
    D = np.ascontiguousarray(directions, np.float64)
    lam = np.ascontiguousarray(lambdas, np.float64)
    xa = np.ascontiguousarray(x0, np.float64)
    g = np.zeros(net.num_links)
    rc = lib().orc_adjoint_vht(C.byref(b.prob), _p(b.keep["cap"], F64P), D.shape[0],
                               _p(xa, F64P), _p(D, F64P), _p(lam, F64P), _p(g, F64P))
    if rc != 0:
        raise RuntimeError(f"oracle adjoint failed rc={rc}")
    return g


def _empty_demand(net):
    from traffic_assignment_gb300.synth import Demand
    z = net.num_zones
    return Demand(z, np.zeros(z + 2, np.int64), np.zeros(0, np.int64), np.zeros(0))


def sssp_all(va, ea, wa, num_nodes1, sources, first_thru, lll=True, threads=1):
    """dist/pred [S][num_nodes1] for each source (prevlink = link index, -1 none)."""
    va = np.ascontiguousarray(va, np.int64)
    ea = np.ascontiguousarray(ea, np.int64)
    wa = np.ascontiguousarray(wa, np.float64)
    src = np.ascontiguousarray(sources, np.int64)
    s = len(src)
    dist = np.zeros((s, num_nodes1))
    pred = np.zeros((s, num_nodes1), np.int64)
    rc = lib().orc_sssp_many(_p(va, I64P), _p(ea, I64P), _p(wa, F64P), num_nodes1, len(ea),
                             _p(src, I64P), s, first_thru, 1 if lll else 0, threads,
                             _p(dist, F64P), _p(pred, I64P))
    if rc != 0:
        raise RuntimeError("oracle sssp failed")
    return dist, pred


# ----------------------------------------------------------------------------
# the reference itself (only where its sources were compiled in this container)
# ----------------------------------------------------------------------------


def reference_path(name: str) -> Optional[str]:
    p = os.path.join(_b.REF_OUT, name)
    return p if os.path.exists(p) else None


def reference_available() -> bool:
    if _b.reference_available():
        try:
            _b.build_reference()
        except RuntimeError:
            return False
    return reference_path("tap_frankwolfe_pthread") is not None


def ref_sssp_lib():
    global _REFLIB
    if _REFLIB is None:
        p = reference_path("libref_sssp.so")
        if p is None:
            return None
        L = C.CDLL(p)
        for fn in ("sssp_pape", "sssp_pape_lll", "sssp_slf", "sssp_slf_lll"):
            f = getattr(L, fn)
            f.restype = None
            f.argtypes = [I64P, I64P, F64P, C.c_long, C.c_long, C.c_long, C.c_long, I64P,
                          F64P, I64P]
        _REFLIB = L
    return _REFLIB


def ref_sssp(va, ea, wa, num_nodes1, source, first_thru, fn="sssp_pape_lll"):
    L = ref_sssp_lib()
    va = np.ascontiguousarray(va, np.int64)
    ea = np.ascontiguousarray(ea, np.int64)
    wa = np.ascontiguousarray(wa, np.float64)
    prev = np.zeros(num_nodes1, np.int64)
    dist = np.zeros(num_nodes1)
    qn = np.zeros(num_nodes1, np.int64)
    getattr(L, fn)(_p(va, I64P), _p(ea, I64P), _p(wa, F64P), num_nodes1, len(ea), source,
                   first_thru, _p(prev, I64P), _p(dist, F64P), _p(qn, I64P))
    return dist, prev


def run_reference(net, dem, threads=1, iters=0, relgap=0.0, warm_flows=None,
                  binary="tap_frankwolfe_pthread", workdir=None, trip_mods=None):
    """Run the compiled reference CLI on TNTP files written from (net, dem)
    (``trip_mods``: a trip modifications file for its ``-t`` flag).

    Returns dict(volume, cost, header, log) where ``log`` rows are
    (iter, objective, relgap, avg_excess, total_cost) from the ``-v`` lines.
    """
    from traffic_assignment_gb300 import tntp
    exe = reference_path(binary)
    if exe is None:
        raise RuntimeError("reference binary not built")
    own = workdir is None
    wd = tempfile.mkdtemp(prefix="tapref_") if own else workdir
    netf = os.path.join(wd, "net.txt")
    tripf = os.path.join(wd, "trips.txt")
    tntp.write_net(netf, net)
    tntp.write_trips(tripf, dem)
    cmd = [exe]
    if binary == "tap_frankwolfe_pthread":
        cmd += ["-n", str(threads), "-v"]
        if iters:
            cmd += ["-i", str(iters)]
        if relgap:
            cmd += ["-r", repr(relgap)]
        if warm_flows is not None:
            cmd += ["-w", warm_flows]
        if trip_mods is not None:
            cmd += ["-t", trip_mods]
    else:
        cmd += ["-i", str(iters)] if iters else []
        cmd += ["-r", repr(relgap)] if relgap else []
    cmd += [netf, tripf]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"reference failed: {res.stderr[-2000:]}")
    init, term, vol, cost, hdr = tntp.read_flows(res.stdout, is_text=True)
    return dict(volume=vol, cost=cost, init=init, term=term, header=hdr,
                log=tntp.parse_iteration_log(res.stderr), stderr=res.stderr)
