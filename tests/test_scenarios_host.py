"""Host-side scenario enumeration of the reference's farm (no GPU)."""

import numpy as np
import pytest

from mods_fixtures import mixed_mods
from traffic_assignment_gb300 import scenarios, synth


def test_subset_enumeration_order():
    ids = ["a", "b", "c", "d"]
    out = scenarios.enumerate_scenarios(ids, "subsets")
    # bit vectors 7, 11, 13, 14, 15 (tap/tap_mpi_main.c:553-560)
    assert [s for s, _ in out] == ["a+b+c", "a+b+d", "a+c+d", "b+c+d", "a+b+c+d"]
    assert len(scenarios.enumerate_scenarios(list("abcdefgh"), "subsets")) == 256 - 1 - 8 - 28


def test_pairs_and_list():
    assert scenarios.enumerate_scenarios(["x", "y", "z"], "pairs") == [
        ("x_and_y", ["x", "y"]), ("x_and_z", ["x", "z"]), ("y_and_z", ["y", "z"])]
    assert scenarios.enumerate_scenarios(["x", "y", "z"], "list", "z,x") == [("z+x", ["z", "x"])]
    with pytest.raises(KeyError):
        scenarios.enumerate_scenarios(["x"], "list", "q")
    with pytest.raises(ValueError):
        scenarios.enumerate_scenarios([str(i) for i in range(17)], "subsets")


def test_apply_mods_change_and_add():
    net, _ = synth.make_small24()
    k = 5
    ch = scenarios.NetMod("u1", "CHANGE", (int(net.init[k]), int(net.term[k]), 99999.0, 1.0,
                                           float(net.fft[k]), 0.15, 4.0, 0.0, 0.0, 1))
    add = scenarios.NetMod("u2", "ADD", (1, 24, 5000.0, 1.0, 3.0, 0.15, 4.0, 0.0, 0.0, 1))
    n2 = scenarios.apply_mods(net, [ch, add])
    assert n2.num_links == net.num_links + 1
    j = np.nonzero((n2.init == net.init[k]) & (n2.term == net.term[k]))[0][0]
    assert n2.capacity[j] == 99999.0
    assert np.all(np.diff(n2.init * 100 + n2.term) >= 0)
    grouped = scenarios.group_mods([add, ch])
    assert list(grouped) == ["u1", "u2"]


@pytest.mark.parametrize("mode", ["single", "pairs", "subsets"])
def test_link_batch_reproduces_each_scenario_network(mode):
    """The union network with each scenario's capacity and parameter edits,
    restricted to its own links, is the network the reference's farm builds
    for that scenario (tap/tap_mpi_main.c:201-240 records, then sorted)."""
    net, _ = synth.make_grid416()
    mods = mixed_mods(net)
    groups = scenarios.group_mods(mods)
    scen = scenarios.enumerate_scenarios(list(groups), mode)
    recs = [(sid, [m for c in sel for m in groups[c]]) for sid, sel in scen]
    b = scenarios.build_link_batch(net, recs)
    assert b.union.num_links == net.num_links + 3  # each ADD record once
    for s, (sid, r) in enumerate(recs):
        want = scenarios.apply_mods(net, r)
        got = b.scenario_network(s)
        for f in ("init", "term", "capacity", "fft", "alpha", "beta"):
            np.testing.assert_array_equal(getattr(got, f), getattr(want, f), err_msg=f"{sid} {f}")
        # links of the union that the scenario lacks are exactly the others' additions
        mine = set(b.members[s].tolist())
        assert set(b.absent[s].tolist()) == set(range(net.num_links, b.union.num_links)) - mine
    assert b.needs_links
    x = b.warm_start(np.arange(net.num_links, dtype=float))
    assert np.all(x[net.num_links:] == 0) and x[7] == 7
