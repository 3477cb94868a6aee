"""dVHT/dcapacity: the GPU adjoint against the FP64 CPU adjoint on the same tape,
against central finite differences of the frozen-load Frank-Wolfe map, and
through torch.autograd.

The map differentiated is the one the solve ran: x_0 = all-or-nothing at free
flow, loads y_k held fixed, d_k = y_k - x_k, lambda_k the exact root of the
directional derivative, x_{k+1} = x_k + lambda_k d_k, VHT = sum x_K t(x_K).
Finite differences replay that map on the CPU (oracle.replay_vht) with the
recorded loads.

Tolerances:
  GPU adjoint vs FP64 CPU adjoint on the GPU's tape: 1e-9 relative to max |g|
  central FD, step 1% of the link's capacity, 64 links:  |fd - g| <= 1e-3 |g|
    (the step's own truncation error is about 5 (h/c)^2 = 5e-4 for BPR power 4)
  Richardson-extrapolated FD (steps 1% and 0.5%):        |fd - g| <= 1e-6 |g|
"""

import numpy as np
import pytest

import oracle
from traffic_assignment_gb300 import synth
from traffic_assignment_gb300.solver import Solver

pytestmark = pytest.mark.gpu

K_ITERS = 30


def _tape(s: Solver, iters: int):
    m = s.m
    x0, _, _ = s.tape(0, with_flows=True)
    D = np.zeros((iters, m))
    lam = np.zeros(iters)
    for k in range(iters):
        _, D[k], lam[k] = s.tape(k)
    X = [x0]
    for k in range(iters):
        X.append(X[-1] + lam[k] * D[k])
    Y = np.array([D[k] + X[k] for k in range(iters)])
    return x0, D, lam, Y


def _solve(net, dem, precision, iters=K_ITERS, **kw):
    s = Solver(net, dem, precision=precision, record_tape=True, tape_capacity=iters,
               line_search="exact", **kw)
    r = s.solve(max_iters=iters)
    assert r.iterations == iters
    return s


@pytest.fixture(scope="module")
def grid416():
    return synth.make_grid416()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_adjoint_matches_cpu_reverse_sweep(built_lib, grid416, precision):
    net, dem = grid416
    with _solve(net, dem, precision) as s:
        v, g = s.adjoint_vht()
        x0, D, lam, Y = _tape(s, K_ITERS)
    g_cpu = oracle.adjoint_vht(net, net.capacity, x0, D, lam)
    scale = np.abs(g_cpu).max()
    assert scale > 0
    np.testing.assert_allclose(g, g_cpu, rtol=0, atol=1e-9 * scale)
    v_cpu, lam_cpu = oracle.replay_vht(net, net.capacity, x0, Y)
    assert abs(v - v_cpu) <= 1e-9 * abs(v_cpu)
    # the GPU's exact steps are the CPU's roots of the same directional derivative
    np.testing.assert_allclose(lam, lam_cpu, rtol=1e-9, atol=1e-12)
    assert np.all((lam > 0) & (lam < 1))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_adjoint_vs_central_differences(built_lib, grid416, precision):
    net, dem = grid416
    with _solve(net, dem, precision) as s:
        _, g = s.adjoint_vht()
        x0, _, _, Y = _tape(s, K_ITERS)
    cap = net.capacity
    links = np.argsort(-np.abs(g), kind="stable")[:64]

    def f(a, h):
        c = cap.copy()
        c[a] += h
        return oracle.replay_vht(net, c, x0, Y)[0]

    for a in links:
        h = 0.01 * cap[a]
        fd = (f(a, h) - f(a, -h)) / (2 * h)
        fd2 = (f(a, h / 2) - f(a, -h / 2)) / h
        rich = (4 * fd2 - fd) / 3
        assert abs(fd - g[a]) <= 1e-3 * abs(g[a]), (a, fd, g[a])
        assert abs(rich - g[a]) <= 1e-6 * abs(g[a]), (a, rich, g[a])


def test_checkpoint_interval_does_not_change_gradient(built_lib):
    net, dem = synth.make_small24()
    grads = []
    for ck in (1, 4, 7, K_ITERS, 0):
        with _solve(net, dem, "fp64", tape_checkpoint=ck) as s:
            v, g = s.adjoint_vht()
            grads.append((v, g))
    for v, g in grads[1:]:
        assert v == grads[0][0]
        np.testing.assert_array_equal(g, grads[0][1])


def test_adjoint_on_upgrade_scenarios(built_lib, grid416):
    """Each scenario of a batched solve has its own tape and gradient."""
    net, dem = grid416
    scen = synth.make_scenarios(net, 3, seed=11)
    with Solver(net, dem, precision="fp32", record_tape=True, tape_capacity=20,
                line_search="exact") as s:
        s.solve_scenarios(scen, max_iters=20)
        for i, sc in enumerate(scen):
            v, g = s.adjoint_vht(i)
            x0, D, lam, _ = _tape_s(s, 20, i)
            cap = net.capacity.copy()
            cap[np.asarray(sc.links)] = sc.new_capacity
            g_cpu = oracle.adjoint_vht(net, cap, x0, D, lam)
            np.testing.assert_allclose(g, g_cpu, rtol=0, atol=1e-9 * np.abs(g_cpu).max())


def _tape_s(s, iters, scen):
    x0, _, _ = s.tape(0, scenario=scen, with_flows=True)
    D = np.zeros((iters, s.m))
    lam = np.zeros(iters)
    for k in range(iters):
        _, D[k], lam[k] = s.tape(k, scenario=scen)
    return x0, D, lam, None


def test_tape_too_short_is_an_error(built_lib):
    net, dem = synth.make_small24()
    with Solver(net, dem, record_tape=True, tape_capacity=5, line_search="exact") as s:
        s.solve(max_iters=8)
        with pytest.raises(RuntimeError, match="tape"):
            s.adjoint_vht()
    with Solver(net, dem) as s:
        s.solve(max_iters=3)
        with pytest.raises(RuntimeError, match="record_tape"):
            s.adjoint_vht()


def test_torch_autograd(built_lib):
    torch = pytest.importorskip("torch")
    from traffic_assignment_gb300 import adjoint

    net, dem = synth.make_small24()
    cap = torch.tensor(net.capacity, dtype=torch.float64, requires_grad=True)
    v = adjoint.vht(cap, net, dem, iters=K_ITERS, precision="fp64")
    (2.0 * v).backward()
    v_ref, g_ref = adjoint.vht_and_grad(net, dem, None, K_ITERS, "fp64")
    assert v.item() == v_ref
    np.testing.assert_array_equal(cap.grad.numpy(), 2.0 * g_ref)


def test_screen_upgrades_first_order(built_lib, grid416):
    """The first-order estimate tracks the frozen-load VHT change of a small upgrade."""
    from traffic_assignment_gb300 import adjoint

    net, dem = grid416
    with _solve(net, dem, "fp64") as s:
        v0, g = s.adjoint_vht()
        x0, _, _, Y = _tape(s, K_ITERS)
    top = np.argsort(g)[:4]  # most negative: upgrades that cut VHT most
    est, v_base, g2 = adjoint.screen_upgrades(net, dem, [top[:1], top[1:4]],
                                              [[0.002], [0.002] * 3], iters=K_ITERS,
                                              precision="fp64")
    assert v_base == v0
    np.testing.assert_array_equal(g2, g)
    for links, e in zip([top[:1], top[1:4]], est):
        cap = net.capacity.copy()
        cap[links] *= 1.002
        dv = oracle.replay_vht(net, cap, x0, Y)[0] - v0
        assert e < 0 and dv < 0
        assert abs(dv - e) <= 0.02 * abs(e)


def test_adjoint_grid10k_random_links(built_lib):
    """The 10,000-node network, 50 FW iterations with FP32 paths, 64 random
    loaded links: central differences with a 1%-of-capacity step within 1e-3
    relative (links whose gradient is below 1e-3 of the largest are held to
    1e-6 of the largest instead: there the VHT's own rounding dominates)."""
    from concurrent.futures import ThreadPoolExecutor

    net, dem = synth.make_grid10k()
    iters = 50
    with _solve(net, dem, "fp32", iters=iters) as s:
        v, g = s.adjoint_vht()
        x0, D, lam, Y = _tape(s, iters)
        x_end, _ = s.flows()
    g_cpu = oracle.adjoint_vht(net, net.capacity, x0, D, lam)
    gmax = np.abs(g_cpu).max()
    np.testing.assert_allclose(g, g_cpu, rtol=0, atol=1e-9 * gmax)
    rng = np.random.default_rng(2024)
    links = rng.choice(np.flatnonzero(x_end > 0), 64, replace=False)
    cap = net.capacity

    def f(args):
        a, h = args
        c = cap.copy()
        c[a] += h
        return oracle.replay_vht(net, c, x0, Y)[0]

    jobs = [(a, sgn * 0.01 * cap[a]) for a in links for sgn in (1.0, -1.0)]
    with ThreadPoolExecutor(max_workers=16) as ex:  # ctypes calls release the GIL
        vals = list(ex.map(f, jobs))
    for i, a in enumerate(links):
        fd = (vals[2 * i] - vals[2 * i + 1]) / (0.02 * cap[a])
        if abs(g[a]) >= 1e-3 * gmax:
            assert abs(fd - g[a]) <= 1e-3 * abs(g[a]), (a, fd, g[a])
        else:
            assert abs(fd - g[a]) <= 1e-6 * gmax, (a, fd, g[a])


def test_screening_ranks_c3_upgrades_like_full_resolves(built_lib):
    """The use the gradient serves: screening candidate upgrades before any
    full re-solve.  On the 10k-node network, 12 single-link upgrades (+25 %
    capacity; the 6 links of most negative dVHT/dcapacity after 50
    iterations and 6 random loaded links) are ranked by the first-order
    estimate and by re-solving each to relative gap 2e-5 from the base
    equilibrium (one batch).  The rank correlation is high and the estimate
    picks the best upgrade; magnitudes are first-order (measured in FP64 on
    16 candidates: Spearman 0.92, estimates 1.5-4x the re-solved change)."""
    from scipy.stats import spearmanr

    from traffic_assignment_gb300 import adjoint

    net, dem = synth.make_grid10k()
    _, _, g = adjoint.screen_upgrades(net, dem, [[0]], [[0.0]], iters=50)
    with Solver(net, dem, precision="fp32") as s:
        base = s.solve(target_relgap=2e-5, max_iters=20000)
        xb, _ = s.flows()
    rng = np.random.default_rng(11)
    top = np.argsort(g)[:6]
    loaded = np.setdiff1d(np.nonzero(xb > 100)[0], top)
    cands = [[int(k)] for k in np.concatenate([top, rng.choice(loaded, 6, replace=False)])]
    est, _, _ = adjoint.screen_upgrades(net, dem, cands, [[0.25]] * len(cands), iters=50)
    scen = [synth.Scenario(f"c{i}", np.array(c), net.capacity[c] * 1.25)
            for i, c in enumerate(cands)]
    with Solver(net, dem, precision="fp32") as s:
        res = s.solve_scenarios(scen, target_relgap=2e-5, max_iters=20000, x0=xb)
    dv = np.array([r["total_cost"] for r in res]) - base["total_cost"]
    assert all(r["error_bits"] == 0 and r["relgap"] <= 2e-5 for r in res)
    rho = spearmanr(est, dv).correlation
    assert rho >= 0.75, (rho, est, dv)
    assert int(np.argmin(dv)) in np.argsort(est)[:3]
    big = np.abs(est) >= 1000
    assert np.all(dv[big] < 0)
