"""The autotuner on the GPU: every candidate runs, the winner is the fastest
row of its table, and a second call is served from the cache."""

import numpy as np
import pytest

from traffic_assignment_gb300 import autotune as A
from traffic_assignment_gb300 import Solver, synth

pytestmark = pytest.mark.gpu


def test_tune_and_cache(built_lib, tmp_path):
    net, dem = synth.make_grid416()
    cache = str(tmp_path / "tune.json")
    cands = [A.Candidate("rounds", 512), A.Candidate("async", 256),
             A.Candidate("nearfar", 256, 16.0), A.Candidate("nearfar_queue", 256, 16.0),
             A.Candidate("nearfar_queue", 128, 4.0, 256)]
    r = A.tune(net, dem, "fp32", scenarios=8, iters=2, warm_iters=10, cache=cache, cands=cands)
    assert not r.from_cache
    assert len(r.table) == len(cands)
    assert all(np.isfinite(row["ms_per_iteration"]) for row in r.table)
    assert r.ms_per_iteration == min(row["ms_per_iteration"] for row in r.table)
    r2 = A.tune(net, dem, "fp32", scenarios=8, cache=cache, cands=cands)
    assert r2.from_cache and r2.best == r.best
    # the tuned shape solves to the same equilibrium as the default one
    with Solver(net, dem, precision="fp64", **r.solver_kwargs(net)) as s:
        s.solve(max_iters=30)
        x1, _ = s.flows()
    with Solver(net, dem, precision="fp64") as s:
        s.solve(max_iters=30)
        x2, _ = s.flows()
    np.testing.assert_array_equal(x1, x2)
