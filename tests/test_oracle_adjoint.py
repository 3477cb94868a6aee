"""The FP64 CPU adjoint (oracle/oracle_adjoint.c) against finite differences.

A tape is produced on the CPU: all-or-nothing loads from the oracle, exact
steps from oracle.replay_vht.  The reverse sweep must then match central
differences of the frozen-load map: plain 1%-of-capacity steps within 1e-3
relative (their truncation error is about 5e-4 for BPR power 4) and the
Richardson combination of 1% and 0.5% steps within 1e-6.
"""

import numpy as np

import oracle
from traffic_assignment_gb300 import synth


def _bpr(net, cap, x):
    return net.fft * (1.0 + net.alpha * (x / cap) ** net.beta)


def _cpu_tape(net, dem, cap, iters):
    x = oracle.aon(net, dem, net.fft.copy())
    x0 = x.copy()
    Y = []
    for _ in range(iters):
        y = oracle.aon(net, dem, _bpr(net, cap, x))
        Y.append(y)
        _, lam = oracle.replay_vht(net, cap, x, np.array([y]))
        x = x + lam[0] * (y - x)
    return x0, np.array(Y)


def test_cpu_adjoint_vs_finite_differences():
    net, dem = synth.make_small24()
    cap = net.capacity.copy()
    x0, Y = _cpu_tape(net, dem, cap, 25)
    v, lam = oracle.replay_vht(net, cap, x0, Y)
    X, D = [x0], []
    for k in range(len(Y)):
        D.append(Y[k] - X[-1])
        X.append(X[-1] + lam[k] * D[-1])
    g = oracle.adjoint_vht(net, cap, x0, np.array(D), lam)
    assert np.all(np.abs(g) > 0)

    def f(a, h):
        c = cap.copy()
        c[a] += h
        return oracle.replay_vht(net, c, x0, Y)[0]

    for a in range(net.num_links):
        h = 0.01 * cap[a]
        fd = (f(a, h) - f(a, -h)) / (2 * h)
        fd2 = (f(a, h / 2) - f(a, -h / 2)) / h
        assert abs(fd - g[a]) <= 1e-3 * abs(g[a])
        assert abs((4 * fd2 - fd) / 3 - g[a]) <= 1e-6 * abs(g[a])


def test_cpu_adjoint_zero_iterations():
    """With no iterations VHT = sum x t(x) at x_0 and only the direct term remains."""
    net, dem = synth.make_small24()
    x0 = oracle.aon(net, dem, net.fft.copy())
    g = oracle.adjoint_vht(net, net.capacity, x0, np.zeros((0, net.num_links)), np.zeros(0))
    direct = -x0 * net.fft * net.alpha * net.beta * (x0 / net.capacity) ** net.beta / net.capacity
    np.testing.assert_allclose(g, direct, rtol=1e-13, atol=0)
