"""Batched upgrade scenarios (tapgpu_solve_scenarios) against individual
solves and against the oracle; the net-mods front end of the reference's
scenario farm (tap/tap_mpi_main.c)."""

import numpy as np
import pytest

import oracle
from mods_fixtures import mixed_mods
from traffic_assignment_gb300 import Solver, scenarios, synth, tntp

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(a - b).max() / max(1.0, np.abs(b).max())


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batched_equals_individual(built_lib, precision):
    net, dem = synth.make_grid416()
    scen = synth.make_scenarios(net, 12, seed=5, max_links=8)
    with Solver(net, dem, precision=precision) as s:
        res = s.solve_scenarios(scen, max_iters=25)
        batched = [s.flows(i)[0] for i in range(len(scen))]
    for i, sc in enumerate(scen):
        cap = net.capacity.copy()
        cap[sc.links] = sc.new_capacity
        with Solver(net, dem, precision=precision) as s1:
            s1.set_capacity(cap)
            r1 = s1.solve(max_iters=25)
            x1, _ = s1.flows()
        # the same kernels on the same inputs: identical bits
        np.testing.assert_array_equal(batched[i], x1)
        assert res[i]["total_cost"] == r1["total_cost"]
        assert res[i]["relgap"] == r1["relgap"]


def test_batched_matches_oracle_fp64(built_lib):
    net, dem = synth.make_grid416()
    scen = synth.make_scenarios(net, 6, seed=9)
    with Solver(net, dem, precision="fp64") as s:
        res = s.solve_scenarios(scen, max_iters=30)
        flows = [s.flows(i)[0] for i in range(len(scen))]
    for i, sc in enumerate(scen):
        cap = net.capacity.copy()
        cap[sc.links] = sc.new_capacity
        ref = oracle.frankwolfe(net, dem, threads=1, max_iters=30, capacity=cap)
        assert _rel(flows[i], ref["x"]) < 1e-6
        assert abs(res[i]["total_cost"] - ref["total_cost"]) <= 1e-6 * ref["total_cost"]


def test_batched_relgap_target_and_warm_start(built_lib):
    net, dem = synth.make_grid416()
    scen = synth.make_scenarios(net, 16, seed=11)
    with Solver(net, dem, precision="fp32") as s:
        base = s.solve(target_relgap=1e-4)
        x0, _ = s.flows()
        res = s.solve_scenarios(scen, target_relgap=1e-3, x0=x0, max_iters=2000)
    assert base["relgap"] <= 1e-4
    for r in res:
        assert r["relgap"] <= 1e-3 and r["error_bits"] == 0
        assert r["iterations"] >= 1


def test_farm_modes_from_net_mods_file(built_lib, tmp_path):
    net, dem = synth.make_grid416()
    scen = synth.make_scenarios(net, 4, seed=3, max_links=3)
    path = str(tmp_path / "mods.txt")
    tntp.write_net_mods(path, net, scen)
    single = scenarios.solve_farm(net, dem, path, "single", target_relgap=0, max_iters=10,
                                  warm_start=False, precision="fp64")
    assert [d["id"] for d in single] == [s.change_id for s in scen]
    assert all(d["batched"] for d in single)
    pairs = scenarios.solve_farm(net, dem, path, "pairs", target_relgap=0, max_iters=10,
                                 warm_start=False, precision="fp64")
    assert [d["id"] for d in pairs] == ["s0000_and_s0001", "s0000_and_s0002", "s0000_and_s0003",
                                        "s0001_and_s0002", "s0001_and_s0003", "s0002_and_s0003"]
    # a pair equals the single solve of the combined edit
    combo = synth.Scenario("x", np.concatenate([scen[0].links, scen[1].links]),
                           np.concatenate([scen[0].new_capacity, scen[1].new_capacity]))
    with Solver(net, dem, precision="fp64") as s:
        r = s.solve_scenarios([combo], max_iters=10)[0]
    assert pairs[0]["total_cost"] == r["total_cost"]
    subsets = scenarios.solve_farm(net, dem, path, "subsets", target_relgap=0, max_iters=5,
                                   warm_start=False, precision="fp32")
    assert len(subsets) == 5  # subsets of size >= 3 of 4 changes


def _trip_sets(dem):
    from traffic_assignment_gb300.tripmods import TripMod
    z = dem.num_zones
    return [[], [TripMod("p", "P2P", 2, 5, 3.0)], [TripMod("u", "UNIFORM", 4, 0, 0.5)],
            [TripMod("d", "UNIFORM", 0, z - 1, 1.7), TripMod("a", "ALL", 0, 0, 1.2)],
            [TripMod("z", "P2P", 1, 3, 0.0)]]


@pytest.mark.parametrize("with_caps", [False, True])
def test_trip_mod_demand_scenarios_match_oracle(built_lib, with_caps):
    """Trip modifications as batched demand scenarios (FP64 paths), optionally
    combined with capacity upgrades: each scenario against the oracle solving
    the modified demand (1e-6), average excess cost on its own demand total."""
    from traffic_assignment_gb300 import tripmods

    net, dem = synth.make_grid416()
    sets = _trip_sets(dem)
    D = tripmods.demand_scenarios(dem, sets)
    if with_caps:
        scen = synth.make_scenarios(net, len(sets), seed=21)
    else:
        scen = [synth.Scenario(f"t{i}", np.zeros(0, np.int64), np.zeros(0))
                for i in range(len(sets))]
    with Solver(net, dem, precision="fp64") as s:
        s.set_scenario_demand(D)
        res = s.solve_scenarios(scen, max_iters=30)
        flows = [s.flows(i)[0] for i in range(len(sets))]
        traces = [s.trace(i) for i in range(len(sets))]
        # back to the base demand: scenario 0 of a new batch is the base solve
        s.set_scenario_demand(None)
        s.solve_scenarios(scen[:1], max_iters=30)
        base_again = s.flows(0)[0]
    for i, ms in enumerate(sets):
        cap = net.capacity.copy()
        cap[scen[i].links] = scen[i].new_capacity
        ref = oracle.frankwolfe(net, tripmods.apply_trip_mods(dem, ms), threads=1, max_iters=30,
                                capacity=cap)
        assert res[i]["error_bits"] == 0
        assert _rel(flows[i], ref["x"]) < 1e-6, i
        assert abs(res[i]["total_cost"] - ref["total_cost"]) <= 1e-6 * ref["total_cost"]
        np.testing.assert_allclose(traces[i][:, 2], ref["trace"][:, 2], rtol=1e-6, atol=1e-9)
    if not with_caps:
        np.testing.assert_array_equal(flows[0], base_again)


def test_demand_scenarios_argument_checks(built_lib):
    net, dem = synth.make_small24()
    with Solver(net, dem) as s:
        D = np.tile(dem.od_demand[dem.od_ptr[1]:dem.od_ptr[dem.num_zones + 1]], (3, 1))
        s.set_scenario_demand(D)
        with pytest.raises(RuntimeError, match="demand scenarios were set for 3"):
            s.solve_scenarios(synth.make_scenarios(net, 2), max_iters=3)
        bad = D.copy()
        bad[1, 0] = np.nan
        with pytest.raises(RuntimeError, match="finite"):
            s.set_scenario_demand(bad)
        # single solves keep the base demand whatever is set
        s.set_scenario_demand(D * 2.0)
        r = s.solve(max_iters=5)
        ref = oracle.frankwolfe(net, dem, threads=1, max_iters=5)
        assert _rel(s.flows()[0], ref["x"]) < 1e-6 and r["iterations"] == 5


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_label_buffer_grows_with_the_batch(built_lib, precision):
    """The label buffer starts at 4,096 tasks per origin and grows when a batch
    holds more: 4,100 scenarios of the 24-node network (98,400 tasks).  The
    batched flows equal individual solves, and the one-shot shortest-path
    entry point, whose predecessor buffer is re-made with the label buffer,
    still matches the oracle afterwards."""
    net, dem = synth.make_small24()
    scen = synth.make_scenarios(net, 4100, seed=77)
    pick = [0, 2049, 4099]
    with Solver(net, dem, precision=precision) as s:
        d0, p0 = s.sssp(net.fft, [1, 5, 24])
        res = s.solve_scenarios(scen, max_iters=3)
        assert all(r["error_bits"] == 0 and r["iterations"] == 3 for r in res)
        batched = [s.flows(i)[0] for i in pick]
        d1, p1 = s.sssp(net.fft, [1, 5, 24])
    np.testing.assert_array_equal(d0, d1)
    np.testing.assert_array_equal(p0, p1)
    va, ea = net.csr()
    dref, _ = oracle.sssp_all(va, ea, net.fft, net.num_nodes + 1, np.array([1, 5, 24]),
                              net.first_thru_node)
    np.testing.assert_array_equal(d1, dref)
    for i, x in zip(pick, batched):
        cap = net.capacity.copy()
        cap[scen[i].links] = scen[i].new_capacity
        with Solver(net, dem, precision=precision) as s1:
            s1.set_capacity(cap)
            s1.solve(max_iters=3)
            np.testing.assert_array_equal(x, s1.flows()[0])


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_scenario_edits_zero_repeated_and_batch_readback(built_lib, precision):
    """Scenario capacity rows are made on the device from the base row and the
    edits: a zero capacity takes the row's smallest positive capacity (the
    zero-capacity fix-up), a link edited twice keeps its last value, and an
    edit can itself be the new smallest capacity.  Each batched scenario
    equals a solve with that capacity array; the batch read-back equals the
    per-scenario one."""
    net, dem = synth.make_grid416()
    a, b = 3, 10
    scen = [synth.Scenario("zero", np.array([a]), np.array([0.0])),
            synth.Scenario("twice", np.array([b, a, b]), np.array([5.0, 7.0, 9000.0])),
            synth.Scenario("smallest", np.array([a, b]), np.array([1e-3, 0.0]))]
    with Solver(net, dem, precision=precision) as s:
        res = s.solve_scenarios(scen, max_iters=5)
        assert all(r["error_bits"] == 0 for r in res)
        v, t = s.flows_batch()
        single = [s.flows(i) for i in range(len(scen))]
    for i in range(len(scen)):
        np.testing.assert_array_equal(v[i], single[i][0])
        np.testing.assert_array_equal(t[i], single[i][1])
    for i, sc in enumerate(scen):
        cap = net.capacity.copy()
        for k, c in zip(sc.links, sc.new_capacity):
            cap[k] = c
        with Solver(net, dem, precision=precision) as s1:
            s1.set_capacity(cap)
            s1.solve(max_iters=5)
            x1, t1 = s1.flows()
        np.testing.assert_array_equal(v[i], x1)
        np.testing.assert_array_equal(t[i], t1)


def test_demand_scenario_matches_reference_trip_mods_golden(built_lib):
    """The reference's -t run as a demand scenario of the batched solver (FP64):
    flows, costs and VHT within 1e-6 of the reference's own output."""
    from test_oracle import load_tripmods_golden
    from traffic_assignment_gb300 import tripmods
    net, dem, mods, z = load_tripmods_golden()
    with Solver(net, dem, precision="fp64") as s:
        s.set_scenario_demand(tripmods.demand_scenarios(dem, [mods]))
        res = s.solve_scenarios([synth.Scenario("base", np.zeros(0, np.int64), np.zeros(0))],
                                max_iters=60)
        x, t = s.flows(0)
    assert res[0]["error_bits"] == 0 and res[0]["iterations"] == 60
    assert _rel(x, z["volume"]) < 1e-6
    assert _rel(t, z["cost"]) < 1e-6
    assert abs(res[0]["total_cost"] - float(z["hdr_totalcost"])) <= 1e-6 * float(z["hdr_totalcost"])


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-6), ("fp32", 1e-4)])
def test_link_record_scenarios_match_oracle(built_lib, precision, tol):
    """Net-mods records of every kind (capacity and free-flow-time CHANGEs,
    ADDs, an ADD changed by a later record, a zero capacity) as one batch over
    the union network, warm-started from the base flows with zero flow on the
    added links (tap/tap_frankwolfe_pthread.c:564-597): each scenario against
    the oracle solving that scenario's own network (tap/tap_mpi_main.c:201-240
    applied, links sorted) from the same warm start.  FP64: flows, VHT and
    relative gap within 1e-6 and the same step every iteration; FP32 paths:
    flows within 1e-4."""
    net, dem = synth.make_grid416()
    groups = scenarios.group_mods(mixed_mods(net))
    scen = scenarios.enumerate_scenarios(list(groups), "pairs")
    recs = [(sid, [m for c in sel for m in groups[c]]) for sid, sel in scen]
    b = scenarios.build_link_batch(net, recs)
    base = oracle.frankwolfe(net, dem, threads=1, max_iters=40)
    x0 = b.warm_start(base["x"])
    K = 30
    with Solver(b.union, dem, precision=precision) as s:
        s.set_scenario_links(b.edits, b.absent)
        res = s.solve_scenarios(b.scenarios, max_iters=K, x0=x0)
        flows = [s.flows(i)[0] for i in range(len(recs))]
        traces = [s.trace(i, max_rows=100) for i in range(len(recs))]
    for i, (sid, _) in enumerate(recs):
        order = b.scenario_order(i)
        assert np.all(flows[i][b.absent[i]] == 0.0), sid
        ref = oracle.frankwolfe(b.scenario_network(i), dem, threads=1, max_iters=K,
                                x0=x0[order])
        assert res[i]["error_bits"] == 0 and res[i]["iterations"] == K
        assert _rel(flows[i][order], ref["x"]) < tol, sid
        if precision == "fp64":
            assert abs(res[i]["total_cost"] - ref["total_cost"]) <= tol * ref["total_cost"], sid
            assert abs(res[i]["relgap"] - ref["relgap"]) <= tol * abs(ref["relgap"]), sid
            np.testing.assert_array_equal(traces[i][:, 4], ref["trace"][:, 4], err_msg=sid)


def test_farm_batches_link_records(built_lib, tmp_path):
    """solve_farm solves ADD / CHANGE scenarios in one batch (no per-scenario
    contexts): the same VHT as the union-network batch solved directly."""
    net, dem = synth.make_grid416()
    mods = mixed_mods(net)
    path = str(tmp_path / "mods.txt")
    with open(path, "w") as f:
        for m in mods:
            f.write("\t".join([m.change_id, m.kind] + [repr(v) if isinstance(v, float) else str(v)
                                                        for v in m.link] + ["0"]) + "\n")
    out = scenarios.solve_farm(net, dem, path, "single", target_relgap=0, max_iters=12,
                               warm_start=False, precision="fp64")
    assert [d["id"] for d in out] == list(scenarios.group_mods(mods))
    assert all(d["batched"] for d in out)
    for d, sid in zip(out, scenarios.group_mods(mods)):
        recs = scenarios.group_mods(mods)[sid]
        ref = oracle.frankwolfe(scenarios.apply_mods(net, recs), dem, threads=1, max_iters=12)
        assert abs(d["total_cost"] - ref["total_cost"]) <= 1e-6 * ref["total_cost"], sid
