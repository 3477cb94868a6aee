"""Benchmark: FW iterations/sec and scenarios/sec, batched FP32-path vs plain, 1 GB300.

Workload (both arms): the 10,000-node synthetic network (100 x 100 perturbed
grid + 200 two-way arterials, 40,000 links, 1,000 zones, gravity demand of
1.5M trips/h, BPR 0.15/4) with 256 upgrade scenarios (capacity +25-100% on
1-20 random links).  A *step* is one Frank-Wolfe iteration of all 256
scenarios in one batched launch sequence (FP32 path costs, FP64 gap /
objective / line search / VHT).  ``value`` is scenario-iterations per second
with everything resident in HBM; ``e2e`` is the same metric through the C ABI
from host buffers: tapgpu_solve_scenarios (the scenarios' capacity edits and
the warm-start flows in; the capacity rows are made on the device) and
tapgpu_get_link_flows_batch (every scenario's flows and costs out).

Also reported: scenarios/sec to relative gap 1e-4 for the batched solver and
for the plain single-scenario GPU path, the VHT change of each upgrade
(batched against individual plain solves), the same workload in FP64 mode
(``fp64_mode``), FW iterations/sec of the plain path on the 24-, 416- and
10,000-node networks in both precisions with the oracle on the host cores
beside them (``configs``), the FP32-path error against FP64 on each
(``precision_error``), the adjoint on the 10k- and 100k-node networks, the
roofline of the dominant kernel (all-origins shortest paths), per-kernel
times measured with CUDA events on the solver's stream, SM clocks sampled
during the timed region, and the CPU baseline (the oracle's pthread
Frank-Wolfe on the host cores).  ``--no-extras`` / ``--no-cpu`` skip the
extra measurements / the host-core legs.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FW iters/sec and scenarios/sec to rel-gap 1e-4, batched FP32 vs plain, 1 GB300"
UNIT = "scenario-FW-iterations/s"
WORKLOAD = ("grid10k x 256 upgrade scenarios: 10,000 nodes, 40,000 links, 1,000 zones, "
            "gravity OD 1.5M trips/h, BPR alpha 0.15 beta 4, batched FW iteration, FP32 paths")


def _env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class Dist:
    """Barrier and max-over-ranks for timing only (no data-path collective)."""

    def __init__(self, world):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, v):
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v):
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


# bytes of one scenario's device state record (sizeof the struct)
SCEN_STATE_BYTES = 144


def shard_scenarios(net, count, rank):
    """The upgrade scenarios of one rank: each rank draws its own set from a
    rank-specific seed (scenarios are independent; nothing is exchanged)."""
    from traffic_assignment_gb300 import synth
    return synth.make_scenarios(net, count, seed=1004 + 7919 * rank)


def whole_job_rate(dist, units, seconds):
    """Units processed by all ranks / the slowest rank's time."""
    return dist.sum(units) / dist.max(seconds)


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.idx = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, n in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0}, "fallback"


def profile_traffic():
    """DRAM bytes per shortest-path task (label write-out dominates), from the
    committed ncu summary of the near-far kernel on the batched 10k-node case."""
    p = os.path.join(ROOT, "profiles", "k_sssp_nfq_grid10k_batched.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_task:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def cpu_baseline(net, dem, scen, seconds=15.0):
    """The oracle's pthread FW (the reference's algorithm) on all host cores:
    FW iterations of one upgrade scenario, iterated until ~`seconds` elapse."""
    import oracle
    cores = os.cpu_count() or 1
    cap = net.capacity.copy()
    cap[scen.links] = scen.new_capacity
    t0 = time.perf_counter()
    it = 1
    while True:
        r = oracle.frankwolfe(net, dem, threads=cores, max_iters=it, capacity=cap)
        el = time.perf_counter() - t0
        if el >= seconds or it >= 64:
            break
        it *= 2
    # per-iteration time from the solver's own per-iteration wall clock
    ms = r["trace"][:, 6]
    per_iter = float(np.mean(ms)) / 1e3
    return {"value": 1.0 / per_iter, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"grid10k, 1 upgrade scenario, {len(ms)} FW iterations (oracle pthread "
                      f"FW on {cores} host threads, per-iteration wall clock)"}


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU algorithm (oracle port, all host
    threads) on the same workload; each step is one FW iteration of one
    upgrade scenario."""
    if rank != 0:
        return 0
    import oracle
    from traffic_assignment_gb300 import synth
    net, dem = synth.make_grid10k()
    scen = synth.make_scenarios(net, 256)[0]
    cap = net.capacity.copy()
    cap[scen.links] = scen.new_capacity
    cores = os.cpu_count() or 1
    total = args.warmup + args.steps
    r = oracle.frankwolfe(net, dem, threads=cores, max_iters=total, capacity=cap)
    ms = r["trace"][:, 6]
    timed = ms[args.warmup:]
    t = float(np.sum(timed)) / 1e3
    value = len(timed) / t
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / len(timed),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "step": "one FW iteration of one upgrade scenario "
                       "(the reference solves scenarios one at a time)", "threads": cores},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{len(timed)} FW iterations of scenario s0000 after "
                                       f"{args.warmup} warm-up iterations"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def cpu_config_rows(cores):
    """The oracle's pthread FW (the reference's algorithm, all host threads) on
    C1-C3: FW iterations per second on a bounded sample of each."""
    import oracle
    from traffic_assignment_gb300 import synth
    rows = {}
    for name, maker, iters in (("C1", synth.make_small24, 100), ("C2", synth.make_grid416, 2000),
                               ("C3", synth.make_grid10k, 20)):
        net, dem = maker()
        t0 = time.perf_counter()
        r = oracle.frankwolfe(net, dem, threads=cores, max_iters=iters)
        wall = time.perf_counter() - t0
        loop_s = float(np.sum(r["trace"][:, 6])) / 1e3
        rows[name] = {"fw_iterations_per_s": iters / loop_s, "iterations": iters,
                      "wall_s": wall, "threads": cores}
    return rows


def _plain_solve(net, dem, precision, iters=0, relgap=0.0):
    """One plain (single-scenario) GPU solve after an untimed warm-up solve:
    wall-clock iterations per second through Solver.solve, and the result."""
    import torch

    from traffic_assignment_gb300 import Solver
    with Solver(net, dem, precision=precision) as s:
        s.solve(max_iters=5)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = s.solve(max_iters=iters, target_relgap=relgap)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        x, _ = s.flows()
    return {"iterations": r["iterations"], "fw_iterations_per_s": r["iterations"] / wall,
            "ms_per_iteration": 1e3 * wall / max(1, r["iterations"]), "relgap": r["relgap"],
            "vht": r["total_cost"]}, r, x


def _errors(x32, r32, x64, r64):
    """FP32-path result against the FP64 one (the FP64 GPU path equals the
    all-FP64 oracle to ~1e-10 in the GPU tests): link flows relative to the
    largest flow, VHT, objective and relative gap relative to the FP64 value."""
    def rv(a, b):
        return abs(a - b) / abs(b) if b else abs(a - b)
    return {"flow_max": float(np.abs(x32 - x64).max() / max(1.0, np.abs(x64).max())),
            "flow_l1": float(np.abs(x32 - x64).sum() / max(1e-300, np.abs(x64).sum())),
            "vht": rv(r32["total_cost"], r64["total_cost"]),
            "objective": rv(r32["objective"], r64["objective"]),
            "relgap": rv(r32["relgap"], r64["relgap"])}


def gpu_config_rows():
    """C1-C3 on the plain single-scenario GPU path in both precisions, and the
    FP32-path error against FP64 on each."""
    from traffic_assignment_gb300 import synth
    rows, errs = {}, {}
    for name, maker, iters, relgap in (("C1", synth.make_small24, 100, 0.0),
                                       ("C2", synth.make_grid416, 0, 1e-5),
                                       ("C3", synth.make_grid10k, 500, 0.0)):
        net, dem = maker()
        row64, r64, x64 = _plain_solve(net, dem, "fp64", iters, relgap)
        row32, r32, x32 = _plain_solve(net, dem, "fp32", iters, relgap)
        rows[name] = {"network": f"{net.num_nodes} nodes, {net.num_links} links, "
                                 f"{net.num_zones} zones",
                      "stop": f"{iters} iterations" if iters else f"relative gap {relgap:g}",
                      "fp64": row64, "fp32_paths": row32}
        errs[name] = dict(_errors(x32, r32, x64, r64), compared=rows[name]["stop"])
    return rows, errs


def adjoint_check(net, dem, iters=50):
    """dVHT/dcapacity on the 10k-node network after `iters` FW iterations (FP32
    paths, exact line search): GPU forward and adjoint times.  Its accuracy is
    checked by the GPU tests against the FP64 CPU reverse sweep and central
    differences."""
    import torch

    from traffic_assignment_gb300 import Solver
    s = Solver(net, dem, precision="fp32", record_tape=True, tape_capacity=iters,
               line_search="exact")
    try:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.solve(max_iters=iters)
        t1 = time.perf_counter()
        vht, g = s.adjoint_vht()
        t2 = time.perf_counter()
    finally:
        s.close()
    return {"network": "grid10k", "iterations": iters, "precision": "fp32 paths, f64 adjoint",
            "forward_ms": 1e3 * (t1 - t0), "adjoint_ms": 1e3 * (t2 - t1), "vht": vht,
            "grad_nonzero_links": int(np.count_nonzero(g)),
            "accuracy": "tests/test_gpu_adjoint.py: 1e-9 of max |g| vs the FP64 CPU reverse "
                        "sweep; 1e-3 vs central differences (1% step) on 64 random links"}


def adjoint_large(iters=50):
    """C5 throughput: dVHT/dcapacity of the 100k-node network (99,856 nodes,
    ~400k links, 4,000 zones) through `iters` FW iterations, FP32 paths and an
    FP64 adjoint; forward (with the tape) and reverse sweep timed apart."""
    import torch

    from traffic_assignment_gb300 import Solver, synth
    net, dem = synth.make_grid100k()
    with Solver(net, dem, precision="fp32", record_tape=True, tape_capacity=iters,
                line_search="exact") as s:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.solve(max_iters=iters)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        vht, g = s.adjoint_vht()
        t2 = time.perf_counter()
    return {"network": "grid100k: 99,856 nodes, %d links, 4,000 zones" % net.num_links,
            "iterations": iters, "forward_ms": 1e3 * (t1 - t0), "adjoint_ms": 1e3 * (t2 - t1),
            "gradient_links_per_s": net.num_links / (t2 - t1), "vht": vht,
            "grad_nonzero_links": int(np.count_nonzero(g))}


def fp64_batched(net, dem, scen, xb, steps, warmup, x32_batch, res32):
    """The same C4 workload in FP64 mode (all-FP64 shortest paths, the
    reference's arithmetic): device-timed scenario-FW-iterations/s, and the
    FP32-path error over every scenario after the same warm-started
    iterations (x32_batch / res32: the FP32 run's flows and results)."""
    import torch

    from traffic_assignment_gb300 import Solver
    K = len(res32) and res32[0]["iterations"]
    with Solver(net, dem, precision="fp64") as s:
        res = s.solve_scenarios(scen, max_iters=K, x0=xb)
        x64, _ = s.flows_batch(0, len(scen))
        s.run_iterations(warmup)
        stream = torch.cuda.ExternalStream(s.stream_ptr())
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        s.run_iterations(steps)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / steps
    worst = {}
    for i in range(len(scen)):
        e = _errors(x32_batch[i], res32[i], x64[i], res[i])
        for k, v in e.items():
            worst[k] = max(worst.get(k, 0.0), v)
    worst["compared"] = f"all {len(scen)} scenarios after {K} warm-started iterations"
    return {"value": len(scen) / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "steps": steps,
            "dtype": "f64"}, worst


def large_network_rate(iters=6):
    """FW iterations per second of one scenario of the 100k-node network (C5:
    99,856 nodes, ~400k links, 4,000 zones, labels in global memory)."""
    import torch

    from traffic_assignment_gb300 import Solver, synth
    net, dem = synth.make_grid100k()
    with Solver(net, dem, precision="fp32") as s:
        s.solve(max_iters=2)
        s.set_timing(True)
        stream = torch.cuda.ExternalStream(s.stream_ptr())
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.run_iterations(iters)
        e1.record(stream)
        e1.synchronize()
        tm = s.timing()
    ms = e0.elapsed_time(e1) / iters
    return {"network": "grid100k: 99,856 nodes, %d links, 4,000 zones" % net.num_links,
            "fw_iterations_per_s": 1e3 / ms, "ms_per_iteration": ms,
            "kernels_ms_per_iteration": {k: tm[f"{k}_ms"] / iters
                                         for k in ("sssp", "aon", "line_search", "step")}}


def run_ours(args, rank, world, local_rank):
    import torch

    from traffic_assignment_gb300 import Solver, synth

    dist = Dist(world)
    torch.cuda.set_device(local_rank)
    net, dem = synth.make_grid10k()
    S = args.scenarios
    # each rank solves its own scenario set (weak scaling: no data exchange)
    scen = shard_scenarios(net, S, rank)
    solver = Solver(net, dem, precision="fp32", device=local_rank)

    # base equilibrium: the warm start of every scenario
    t0 = time.perf_counter()
    base = solver.solve(target_relgap=args.base_relgap, max_iters=args.base_max_iters)
    xb, _ = solver.flows()
    base_s = time.perf_counter() - t0

    # plain single-scenario path: a few scenarios one at a time to rel-gap 1e-4
    plain_n = min(args.plain_scenarios, S)
    t0 = time.perf_counter()
    plain_iters, plain_vht = [], []
    for sc in scen[:plain_n]:
        cap = net.capacity.copy()
        cap[sc.links] = sc.new_capacity
        solver.set_capacity(cap)
        q = solver.solve(target_relgap=1e-4, max_iters=args.max_iters, x0=xb)
        plain_iters.append(q["iterations"])
        plain_vht.append(q["total_cost"])
    plain_s = time.perf_counter() - t0
    solver.set_capacity(net.capacity)
    plain_sps = plain_n / plain_s

    # batched: all scenarios to rel-gap 1e-4 in one solve
    dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = solver.solve_scenarios(scen, target_relgap=1e-4, max_iters=args.max_iters, x0=xb)
    torch.cuda.synchronize()
    batched_s_local = time.perf_counter() - t0
    batched_iters = [q["iterations"] for q in res]
    batched_sps = whole_job_rate(dist, S, batched_s_local)

    # timed steps: batched FW iterations of all S scenarios (device timing)
    solver.run_iterations(args.warmup)
    solver.set_timing(True)
    stream = torch.cuda.ExternalStream(solver.stream_ptr())
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clk:
        torch.cuda.nvtx.range_push("timed_steps")
        ev0.record(stream)
        solver.run_iterations(args.steps)
        ev1.record(stream)
        ev1.synchronize()
        torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    dist.barrier()
    ms_local = ev0.elapsed_time(ev1)
    ms = dist.max(ms_local)
    tm = solver.timing()
    solver.set_timing(False)
    value = whole_job_rate(dist, S * args.steps, ms_local / 1e3)

    # end to end through the C ABI from host buffers
    torch.cuda.synchronize()
    e2e_iters = args.steps
    t0 = time.perf_counter()
    res2 = solver.solve_scenarios(scen, max_iters=e2e_iters, x0=xb)
    vols, costs = solver.flows_batch(0, S)
    e2e_value = whole_job_rate(dist, S * e2e_iters, time.perf_counter() - t0)
    m = net.num_links
    n_edits = sum(len(sc.links) for sc in scen)
    # host -> device per call: the scenario edits (link, capacity) with their
    # offsets and zero-capacity minima, the warm start once, the scenario list
    # and states; device -> host: every scenario's volumes and costs, results
    h2d = (S + 1) * 4 + n_edits * 12 + S * 8 + m * 8 + S * 4 + S * SCEN_STATE_BYTES
    d2h = S * m * 16 + S * 96
    assert vols.shape == (S, m) and costs.shape == (S, m)
    assert all(q["error_bits"] == 0 for q in res2)

    # roofline of the shortest-path kernel: 12 M + 8 N bytes per (scenario, origin)
    # task, averaged over the launches of the timed steps (the last label chunk
    # of a step is a partial one)
    Z, N, M = net.num_zones, net.num_nodes, m
    launches = max(1, tm["sssp_launches"])
    tasks_per_launch = S * Z * args.steps / launches
    bytes_per_launch = tasks_per_launch * (12 * M + 8 * N)
    sssp_avg_ms = tm["sssp_ms"] / launches
    achieved = bytes_per_launch / (sssp_avg_ms / 1e3) / 1e9
    peaks, peak_kind = measured_peaks()
    peak = float(peaks.get("hbm_gbs", 6800.0))
    per_task = profile_traffic()
    traffic = None if per_task is None else per_task * tasks_per_launch

    # VHT change of each upgrade (the reference farm's output): batched solves
    # against the plain path's individual solves of the same scenarios
    base_vht = base["total_cost"]
    dv_b = np.array([q["total_cost"] - base_vht for q in res])
    dv_p = np.array(plain_vht) - base_vht
    vht_change = {
        "base_vht": base_vht,
        "batched_delta_vht": {"mean": float(dv_b.mean()), "min": float(dv_b.min()),
                              "max": float(dv_b.max()), "scenarios": S},
        "plain_subset": [{"scenario": scen[i].change_id, "delta_vht_batched": float(dv_b[i]),
                          "delta_vht_plain": float(dv_p[i])} for i in range(plain_n)],
        "max_abs_diff_rel_base_vht": float(np.max(np.abs(dv_b[:plain_n] - dv_p)) / base_vht),
    }

    line = None
    if rank == 0:
        clocks = clk.summary()
        cpu = cpu_baseline(net, dem, scen[0], seconds=args.cpu_seconds) if not args.no_cpu else None
        cpu_rows = cpu_config_rows(os.cpu_count() or 1) if not args.no_cpu else None
        adj = None if args.no_extras else adjoint_check(net, dem)
        large = None if args.no_extras else large_network_rate()
        fp64 = rows = adj_large = None
        prec = {}
        if not args.no_extras:
            # FP32 paths and FP64 on the same warm-started C4 iterations
            res30 = solver.solve_scenarios(scen, max_iters=30, x0=xb)
            x30, _ = solver.flows_batch(0, S)
            fp64, prec["C4"] = fp64_batched(net, dem, scen, xb, args.steps, args.warmup, x30,
                                            res30)
            rows, errs = gpu_config_rows()
            prec.update(errs)
            adj_large = adjoint_large()
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "scenarios_per_gpu": S,
                       "parallelism": f"scenario shards x{world} (no collective)",
                       "l2": "working set per step ~%.1f GB (labels %d tasks x %d nodes x 4 B) "
                             "> 129 MB L2; no flush needed" % (
                                 S * Z * (N + 1) * 4 / 1e9, S * Z, N + 1),
                       "reductions": "f64", "path_costs": "f32"},
            "scenarios_per_sec": {
                "batched": batched_sps, "plain": plain_sps * world,
                "speedup": batched_sps / (plain_sps * world),
                "target_relgap": 1e-4, "warm_start": f"base equilibrium (relgap "
                f"{base['relgap']:.2e} after {base['iterations']} iterations, {base_s:.1f} s)",
                "batched_iters_mean": float(np.mean(batched_iters)),
                "batched_iters_max": int(np.max(batched_iters)),
                "plain_iters_mean": float(np.mean(plain_iters)), "plain_scenarios": plain_n,
                # the plain path's scenarios in the batch: same iteration counts, so the
                # per-iteration cost ratio isolates what batching itself buys
                "batched_iters_mean_plain_subset": float(np.mean(batched_iters[:plain_n])),
                "ms_per_scenario_iteration": {
                    "plain": 1e3 * plain_s / max(1, sum(plain_iters)),
                    "batched": 1e3 * batched_s_local / max(1, sum(batched_iters))}},
            "kernels_ms_per_step": {k: tm[f"{k}_ms"] / args.steps
                                    for k in ("sssp", "aon", "line_search", "step")},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "k_sssp_nfq", "peak_kind": f"{peak_kind} hbm_gbs",
                         "algorithmic_bytes_per_launch": bytes_per_launch,
                         "tasks_per_launch": tasks_per_launch,
                         "avg_launch_ms": sssp_avg_ms,
                         "traffic_source": "ncu dram__bytes_read+write per task of a "
                                           "16,000-task launch x tasks_per_launch",
                         "note": "the algorithmic bytes are edge records and labels served "
                                 "from L1/L2; the kernel is instruction-issue bound"},
            "cpu_baseline": cpu,
            "clocks": clocks,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d / e2e_iters,
                    "d2h_bytes_per_step": d2h / e2e_iters,
                    "call": "tapgpu_solve_scenarios(host scenario edits, warm flows) + "
                            "tapgpu_get_link_flows_batch (all scenarios' volumes and costs)",
                    "iterations": e2e_iters},
            "gpu_launches": tm["kernel_launches"],
            "fp64_mode": fp64,
            "vht_change": vht_change,
            "configs": {"gpu": rows, "cpu_port": cpu_rows},
            "precision_error": prec or None,
            "adjoint": adj,
            "adjoint_large": adj_large,
            "large_network": large,
        }
        print(json.dumps(line), flush=True)
    solver.close()
    dist.close()
    return 0


def profile_case(kind):
    """A few FW iterations on the 10k-node network: every kernel of the loop
    launches a handful of times (1,000 or 16,000 shortest-path tasks each);
    "small": the 416-node network (C2), one scenario, 20 iterations;
    "large": the 100k-node network (C5), one scenario, 3 iterations (4,000
    tasks per launch, labels in global memory)."""
    from traffic_assignment_gb300 import Solver, synth
    if kind == "large":
        net, dem = synth.make_grid100k()
        with Solver(net, dem, precision="fp32") as s:
            s.set_timing(True)
            r = s.solve(max_iters=3)
            tm = s.timing()
        print(json.dumps({"profile_case": kind, "iterations": r["iterations"], **tm}))
        return 0
    if kind == "small":
        net, dem = synth.make_grid416()
        with Solver(net, dem, precision="fp32") as s:
            r = s.solve(max_iters=20)
            s.set_timing(True)
            s.run_iterations(20)
            tm = s.timing()
        print(json.dumps({"profile_case": kind, "iterations": r["iterations"], **tm}))
        return 0
    net, dem = synth.make_grid10k()
    with Solver(net, dem, precision="fp32") as s:
        r = s.solve(max_iters=4)
        if kind == "batched":
            x0, _ = s.flows()
            s.solve_scenarios(synth.make_scenarios(net, 16), max_iters=3, x0=x0)
        s.set_timing(True)
        s.run_iterations(2)
        tm = s.timing()
    print(json.dumps({"profile_case": kind, "iterations": r["iterations"], **tm}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scenarios", type=int, default=256)
    ap.add_argument("--max-iters", type=int, default=400)
    ap.add_argument("--base-relgap", type=float, default=2e-5)
    ap.add_argument("--base-max-iters", type=int, default=4000)
    ap.add_argument("--plain-scenarios", type=int, default=8)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the adjoint check and the 100k-node rate")
    ap.add_argument("--profile-case", choices=["plain", "batched", "small", "large"],
                    default=None,
                    help="small case for ncu: a few FW iterations of the 10k-node network, "
                         "one scenario (plain) or 16 scenarios (batched), of the 416-node "
                         "network (small) or of the 100k-node network (large), then exit")
    args = ap.parse_args()
    rank, world, local_rank = _env_rank()
    if args.profile_case:
        return profile_case(args.profile_case)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    sys.exit(main())
