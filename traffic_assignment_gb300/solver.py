"""Python front end of the GPU Frank-Wolfe solver (handle API of include/tap_gpu.h)."""

from __future__ import annotations

import ctypes as C
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _capi as K
from .synth import Demand, Network, Scenario

__all__ = ["Solver", "SolveResult"]


class SolveResult(dict):
    """iterations, error_bits, objective, relgap, total_cost, avg_excess, lambda_last."""

    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError as e:
            raise AttributeError(k) from e


def _net_struct(net: Network, keep: list):
    arrs = [np.ascontiguousarray(net.init, np.int64), np.ascontiguousarray(net.term, np.int64),
            np.ascontiguousarray(net.capacity, np.float64),
            np.ascontiguousarray(net.fft, np.float64),
            np.ascontiguousarray(net.alpha, np.float64),
            np.ascontiguousarray(net.beta, np.float64)]
    keep.extend(arrs)
    return K.Network(net.num_nodes, net.num_zones, net.first_thru_node, net.num_links,
                     K.ptr(arrs[0], K.I64P), K.ptr(arrs[1], K.I64P), K.ptr(arrs[2], K.F64P),
                     K.ptr(arrs[3], K.F64P), K.ptr(arrs[4], K.F64P), K.ptr(arrs[5], K.F64P))


def _dem_struct(dem: Demand, keep: list):
    arrs = [np.ascontiguousarray(dem.od_ptr, np.int64), np.ascontiguousarray(dem.od_dest, np.int64),
            np.ascontiguousarray(dem.od_demand, np.float64)]
    if arrs[1].size == 0:
        arrs[1] = np.zeros(1, np.int64)
        arrs[2] = np.zeros(1)
    keep.extend(arrs)
    return K.DemandS(dem.num_zones, K.ptr(arrs[0], K.I64P), K.ptr(arrs[1], K.I64P),
                     K.ptr(arrs[2], K.F64P))


class Solver:
    """One network + demand on one GPU.

    precision: "fp64" (all-FP64 shortest paths, parity with the reference) or
    "fp32" (FP32 path costs; gap, objective, line search and VHT stay FP64).
    """

    def __init__(self, net: Network, dem: Optional[Demand] = None, precision: str = "fp64",
                 device: int = 0, sssp_block: int = 0, aon_block: int = 0,
                 iters_per_launch: int = 0, use_graphs: bool = True, chunk_tasks: int = 0,
                 record_tape: bool = False, tape_capacity: int = 0,
                 global_scratch: int = 0, sssp_variant: str = "default",
                 nf_delta: float = 0.0, line_search: str = "reference",
                 tape_checkpoint: int = 0, sssp_ctas_per_sm: int = 0,
                 aon_ctas_per_sm: int = 0):
        self.L = K.load()
        self.net = net
        self.dem = dem
        opt = K.Options()
        self.L.tapgpu_default_options(C.byref(opt))
        opt.precision = K.TAPGPU_FP32_PATHS if precision in ("fp32", "fp32path") else K.TAPGPU_FP64
        opt.device = device
        opt.sssp_block = sssp_block
        opt.aon_block = aon_block
        opt.iters_per_launch = iters_per_launch
        opt.use_graphs = 1 if use_graphs else 0
        opt.chunk_tasks = chunk_tasks
        opt.record_tape = 1 if record_tape else 0
        opt.tape_capacity = tape_capacity
        # True / 1: labels in global memory; 2: the queue kernels' bitmaps and ring too
        opt.global_scratch = int(global_scratch)
        opt.sssp_variant = {"default": 0, "rounds": 1, "async": 2, "nearfar": 3,
                            "nearfar_queue": 4, "small": 6}[sssp_variant]
        opt.nf_delta = float(nf_delta)
        opt.line_search = {"reference": 0, "exact": 1}[line_search]
        opt.tape_checkpoint = int(tape_checkpoint)
        opt.sssp_ctas_per_sm = int(sssp_ctas_per_sm)
        opt.aon_ctas_per_sm = int(aon_ctas_per_sm)
        self.precision = "fp32" if opt.precision == K.TAPGPU_FP32_PATHS else "fp64"
        self.last_scenarios = 1
        keep: list = []
        ns = _net_struct(net, keep)
        ds = _dem_struct(dem, keep) if dem is not None else None
        h = C.c_void_p()
        K.check(self.L.tapgpu_create(C.byref(ns), C.byref(ds) if ds is not None else None,
                                     C.byref(opt), C.byref(h)))
        self.h = h
        self.m = net.num_links
        self.n1 = net.num_nodes + 1

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.tapgpu_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------------------
    def solve(self, max_iters: int = 0, target_relgap: float = 0.0,
              x0: Optional[np.ndarray] = None) -> SolveResult:
        r = K.Result()
        xa = None if x0 is None else np.ascontiguousarray(x0, np.float64)
        K.check(self.L.tapgpu_solve(self.h, int(max_iters), float(target_relgap),
                                    None if xa is None else K.ptr(xa, K.F64P), C.byref(r)))
        return SolveResult(r.as_dict())

    def begin(self, max_iters: int = 0, target_relgap: float = 0.0,
              x0: Optional[np.ndarray] = None):
        xa = None if x0 is None else np.ascontiguousarray(x0, np.float64)
        K.check(self.L.tapgpu_solve_begin(self.h, int(max_iters), float(target_relgap),
                                          None if xa is None else K.ptr(xa, K.F64P)))

    def advance(self, iters: int):
        r = K.Result()
        done = C.c_int(0)
        K.check(self.L.tapgpu_solve_advance(self.h, int(iters), C.byref(done), C.byref(r)))
        return bool(done.value), SolveResult(r.as_dict())

    def flows(self, scenario: int = 0):
        v = np.zeros(self.m)
        t = np.zeros(self.m)
        K.check(self.L.tapgpu_get_link_flows(self.h, scenario, K.ptr(v, K.F64P), K.ptr(t, K.F64P)))
        return v, t

    def flows_batch(self, first: int = 0, count: Optional[int] = None):
        """Volumes and costs [count][m] of scenarios first .. first+count-1 (of the
        last solve_scenarios call by default: all of them) in one call."""
        if count is None:
            count = self.last_scenarios - first
        v = np.zeros((count, self.m))
        t = np.zeros((count, self.m))
        K.check(self.L.tapgpu_get_link_flows_batch(self.h, first, count, K.ptr(v, K.F64P),
                                                   K.ptr(t, K.F64P)))
        return v, t

    def trace(self, scenario: int = 0, max_rows: int = 1000000) -> np.ndarray:
        """Rows: objective, relgap, avg_excess, vht, lambda, gap, iter, g0."""
        n = C.c_int(0)
        rows = np.zeros((max_rows, K.TRACE_COLS))
        K.check(self.L.tapgpu_get_trace(self.h, scenario, K.ptr(rows, K.F64P), max_rows,
                                        C.byref(n)))
        return rows[: n.value].copy()

    def set_capacity(self, cap: np.ndarray):
        ca = np.ascontiguousarray(cap, np.float64)
        K.check(self.L.tapgpu_set_capacity(self.h, K.ptr(ca, K.F64P)))

    def sssp(self, weights: np.ndarray, sources: Sequence[int], want_dist=True, want_pred=True):
        w = np.ascontiguousarray(weights, np.float64)
        src = np.ascontiguousarray(sources, np.int64)
        d = np.zeros((len(src), self.n1)) if want_dist else None
        p = np.zeros((len(src), self.n1), np.int64) if want_pred else None
        K.check(self.L.tapgpu_sssp(self.h, K.ptr(w, K.F64P), K.ptr(src, K.I64P), len(src),
                                   None if d is None else K.ptr(d, K.F64P),
                                   None if p is None else K.ptr(p, K.I64P)))
        return d, p

    def aon(self, weights: np.ndarray) -> np.ndarray:
        w = np.ascontiguousarray(weights, np.float64)
        y = np.zeros(self.m)
        K.check(self.L.tapgpu_aon(self.h, K.ptr(w, K.F64P), K.ptr(y, K.F64P)))
        return y

    def set_scenario_links(self, edits: Optional[Sequence] = None,
                           absent: Optional[Sequence] = None):
        """Per-scenario link records for the following solve_scenarios calls
        (the context's network is the union of every scenario's links).

        edits[s]: (links, fft, alpha, beta) arrays of scenario s's changed
        link parameters; absent[s]: the links scenario s's network does not
        have.  None returns to the one base network."""
        if edits is None and absent is None:
            K.check(self.L.tapgpu_set_scenario_links(self.h, 0, None, None, None, None, None,
                                                     None, None))
            return
        S = len(edits) if edits is not None else len(absent)
        edits = edits if edits is not None else [None] * S
        absent = absent if absent is not None else [None] * S
        if len(edits) != S or len(absent) != S:
            raise ValueError("edits and absent must list the same scenarios")
        cols = [[], [], [], []]
        eptr = np.zeros(S + 1, np.int64)
        aptr = np.zeros(S + 1, np.int64)
        alist = []
        for i in range(S):
            e = edits[i]
            n = 0
            if e is not None:
                arrs = [np.atleast_1d(np.asarray(a)) for a in e]
                n = len(arrs[0])
                if any(len(a) != n for a in arrs):
                    raise ValueError("edit arrays of one scenario differ in length")
                for c, a in zip(cols, arrs):
                    c.append(a)
            eptr[i + 1] = eptr[i] + n
            a = np.zeros(0, np.int64) if absent[i] is None else np.asarray(absent[i], np.int64)
            alist.append(a)
            aptr[i + 1] = aptr[i] + len(a)
        cat = [np.ascontiguousarray(np.concatenate(c) if c else np.zeros(0), t)
               for c, t in zip(cols, (np.int64, np.float64, np.float64, np.float64))]
        al = np.ascontiguousarray(np.concatenate(alist) if alist else np.zeros(0), np.int64)
        keep = [np.zeros(1, np.int64) if a.size == 0 else a for a in (cat[0], al)]
        fv = [np.zeros(1) if a.size == 0 else a for a in cat[1:]]
        K.check(self.L.tapgpu_set_scenario_links(
            self.h, S, K.ptr(eptr, K.I64P), K.ptr(keep[0], K.I64P), K.ptr(fv[0], K.F64P),
            K.ptr(fv[1], K.F64P), K.ptr(fv[2], K.F64P), K.ptr(aptr, K.I64P),
            K.ptr(keep[1], K.I64P)))

    def set_scenario_demand(self, demand: Optional[np.ndarray]):
        """Per-scenario OD demand [S][nnz] (entries in the order of the Demand
        given at construction) for the following solve_scenarios calls; None
        returns to the base demand."""
        if demand is None:
            K.check(self.L.tapgpu_set_scenario_demand(self.h, 0, None))
            return
        da = np.ascontiguousarray(demand, np.float64)
        if da.ndim != 2:
            raise ValueError("demand must be [scenarios][OD entries]")
        K.check(self.L.tapgpu_set_scenario_demand(self.h, da.shape[0], K.ptr(da, K.F64P)))

    def solve_scenarios(self, scenarios: List[Scenario], max_iters: int = 0,
                        target_relgap: float = 0.0, x0: Optional[np.ndarray] = None):
        ptr = [0]
        links, caps = [], []
        for sc in scenarios:
            links.extend(np.asarray(sc.links, np.int64).tolist())
            caps.extend(np.asarray(sc.new_capacity, np.float64).tolist())
            ptr.append(len(links))
        pa = np.asarray(ptr, np.int64)
        la = np.asarray(links if links else [0], np.int64)
        ca = np.asarray(caps if caps else [0.0], np.float64)
        res = (K.Result * len(scenarios))()
        xa = None if x0 is None else np.ascontiguousarray(x0, np.float64)
        K.check(self.L.tapgpu_solve_scenarios(self.h, len(scenarios), K.ptr(pa, K.I64P),
                                              K.ptr(la, K.I64P), K.ptr(ca, K.F64P),
                                              int(max_iters), float(target_relgap),
                                              None if xa is None else K.ptr(xa, K.F64P), res))
        self.last_scenarios = len(scenarios)
        return [SolveResult(r.as_dict()) for r in res]

    def adjoint_vht(self, scenario: int = 0):
        """(VHT, dVHT/dcapacity [M]) of the last solve (needs record_tape)."""
        g = np.zeros(self.m)
        v = np.zeros(1)
        K.check(self.L.tapgpu_adjoint_vht(self.h, scenario, K.ptr(g, K.F64P), K.ptr(v, K.F64P)))
        return float(v[0]), g

    def tape(self, iteration: int, scenario: int = 0, with_flows: bool = False):
        """(x_k or None, d_k, lambda_k) of the recorded solve."""
        d = np.zeros(self.m)
        lam = np.zeros(1)
        x = np.zeros(self.m) if with_flows else None
        K.check(self.L.tapgpu_get_tape(self.h, scenario, iteration,
                                       None if x is None else K.ptr(x, K.F64P),
                                       K.ptr(d, K.F64P), K.ptr(lam, K.F64P)))
        return x, d, float(lam[0])

    def stream_ptr(self) -> int:
        return int(self.L.tapgpu_stream(self.h) or 0)

    def run_iterations(self, iters: int):
        K.check(self.L.tapgpu_run_iterations(self.h, int(iters)))

    def set_timing(self, on: bool = True):
        K.check(self.L.tapgpu_set_timing(self.h, 1 if on else 0))

    def timing(self) -> Dict[str, float]:
        """Accumulated kernel times (ms) and launch counts since set_timing()."""
        ms = np.zeros(4)
        n = np.zeros(4, np.int64)
        kl = np.zeros(1, np.int64)
        K.check(self.L.tapgpu_get_timing(self.h, K.ptr(ms, K.F64P), K.ptr(n, K.I64P),
                                         K.ptr(kl, K.I64P)))
        names = ("sssp", "aon", "line_search", "step")
        out = {f"{k}_ms": float(ms[i]) for i, k in enumerate(names)}
        out.update({f"{k}_launches": int(n[i]) for i, k in enumerate(names)})
        out["kernel_launches"] = int(kl[0])
        st = np.zeros(6, np.int64)
        K.check(self.L.tapgpu_get_path_stats(self.h, K.ptr(st, K.I64P)))
        out["sssp_rounds"] = int(st[0])
        out["sssp_tasks"] = int(st[1])
        out["sssp_expansions"] = int(st[2])
        out["sssp_idle_polls"] = int(st[3])
        out["sssp_batches"] = int(st[4])
        out["sssp_scanned"] = int(st[5])
        return out

    def profile_iteration(self, reps: int = 5) -> Dict[str, float]:
        ms = (C.c_float * 5)()
        K.check(self.L.tapgpu_profile_iteration(self.h, int(reps), ms))
        return dict(sssp_ms=ms[0], aon_ms=ms[1], line_search_ms=ms[2], step_ms=ms[3],
                    iteration_ms=ms[4])
