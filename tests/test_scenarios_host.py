"""Host-side scenario enumeration of the reference's farm (no GPU)."""

import numpy as np
import pytest

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
