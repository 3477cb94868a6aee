"""Batched upgrade scenarios (tapgpu_solve_scenarios) against individual
solves and against the oracle; the net-mods front end of the reference's
scenario farm (tap/tap_mpi_main.c)."""

import numpy as np
import pytest

import oracle
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
