"""Net-mods records shared by the host and GPU scenario tests."""

import numpy as np

from traffic_assignment_gb300 import scenarios


def mixed_mods(net):
    """Records of every kind on the 416-node network: capacity-only CHANGEs, a
    CHANGE of free-flow time and BPR parameters, ADDs of new links (one
    change id adds a link and then changes it), so the farm's scenarios differ
    in topology as well as in costs."""
    NM = scenarios.NetMod
    rng = np.random.default_rng(5)
    ks = rng.choice(net.num_links, 4, replace=False)

    def rec(cid, kind, k=None, cap=None, fft=None, alpha=None, beta=None, ends=None):
        i, j = ends if ends is not None else (int(net.init[k]), int(net.term[k]))
        base = (lambda a, d: float(getattr(net, a)[k]) if k is not None else d)
        return NM(cid, kind, (i, j, cap if cap is not None else base("capacity", 3000.0), 1.0,
                              fft if fft is not None else base("fft", 1.0),
                              alpha if alpha is not None else base("alpha", 0.15),
                              beta if beta is not None else base("beta", 4.0), 0.0, 0.0, 1))
    present = set(zip(net.init.tolist(), net.term.tolist()))
    free = [(a, b) for a in range(1, 40) for b in range(200, 260) if (a, b) not in present]
    return [
        rec("c_cap", "CHANGE", ks[0], cap=float(net.capacity[ks[0]]) * 1.8),
        rec("c_cap", "CHANGE", ks[1], cap=float(net.capacity[ks[1]]) * 1.3),
        rec("c_fft", "CHANGE", ks[2], cap=float(net.capacity[ks[2]]), fft=float(net.fft[ks[2]]) * 0.6,
            alpha=0.3, beta=3.0),
        rec("d_add", "ADD", ends=free[0], cap=4000.0, fft=0.4),
        rec("d_add", "ADD", ends=(free[0][1], free[0][0]), cap=4000.0, fft=0.4),
        rec("e_addchg", "ADD", ends=free[7], cap=2500.0, fft=0.7),
        rec("e_addchg", "CHANGE", ends=free[7], cap=5000.0, fft=0.5, alpha=0.2, beta=4.0),
        rec("f_zero", "CHANGE", ks[3], cap=0.0),
    ]
