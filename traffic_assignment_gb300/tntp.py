"""TNTP text formats: ``_net``, ``_trips``, flows output and net-mods files.

Layouts follow the reference parsers and printers:
  net file      tap/parsetapfiles.c:62-146   (10 whitespace fields per link)
  trips file    tap/parsetapfiles.c:181-311  (``Origin o`` then ``d : v;``)
  flows file    tap/tap_functions.c:431-445 and tap/parsetapfiles.c:344-423
  net mods      tap/parsetapfiles.c:457-516  (tab separated, ADD / CHANGE)
  trip mods     tap/parsetapfiles.c:573-638  (tab separated, P2P/UNIFORM/ALL)

Numbers are written with ``repr`` so the C ``atof`` of the reference reads
back the same doubles.
"""

from __future__ import annotations

import io
import re
from typing import Dict, List, Tuple

import numpy as np

from .synth import Demand, Network, Scenario

__all__ = [
    "write_net",
    "write_trips",
    "read_net",
    "read_trips",
    "read_flows",
    "write_flows",
    "write_net_mods",
    "read_net_mods",
    "parse_iteration_log",
]


def _r(x: float) -> str:
    return repr(float(x))


def write_net(path: str, net: Network) -> None:
    with open(path, "w") as f:
        f.write(f"<NUMBER OF ZONES> {net.num_zones}\n")
        f.write(f"<NUMBER OF NODES> {net.num_nodes}\n")
        f.write(f"<FIRST THRU NODE> {net.first_thru_node}\n")
        f.write(f"<NUMBER OF LINKS> {net.num_links}\n")
        f.write("<END OF METADATA>\n\n\n")
        f.write("~ \tInit node \tTerm node \tCapacity \tLength \tFree Flow Time \tB"
                "\tPower\tSpeed limit \tToll \tType\t;\n")
        lines = []
        for k in range(net.num_links):
            lines.append(
                f"\t{int(net.init[k])}\t{int(net.term[k])}\t{_r(net.capacity[k])}\t"
                f"{_r(net.length[k])}\t{_r(net.fft[k])}\t{_r(net.alpha[k])}\t"
                f"{_r(net.beta[k])}\t{_r(net.speed[k])}\t{_r(net.toll[k])}\t"
                f"{int(net.link_type[k])}\t;\n")
        f.write("".join(lines))


def write_trips(path: str, dem: Demand) -> None:
    with open(path, "w") as f:
        f.write(f"<NUMBER OF ZONES> {dem.num_zones}\n")
        f.write(f"<TOTAL OD FLOW> {_r(dem.total)}\n")
        f.write("<END OF METADATA>\n\n\n")
        parts = []
        for o in range(1, dem.num_zones + 1):
            s, e = int(dem.od_ptr[o]), int(dem.od_ptr[o + 1])
            parts.append(f"Origin {o}\n")
            row = []
            for i in range(s, e):
                row.append(f"{int(dem.od_dest[i])} : {_r(dem.od_demand[i])};")
                if len(row) == 5:
                    parts.append("    " + "\t".join(row) + "\n")
                    row = []
            if row:
                parts.append("    " + "\t".join(row) + "\n")
            parts.append("\n")
        f.write("".join(parts))


def _meta(line: str) -> Tuple[str, str]:
    close = line.index(">")
    return line[: close + 1], line[close + 1 :].strip()


def read_net(path: str) -> Network:
    """Parse a TNTP ``_net`` file; links are returned sorted by (init, term)."""
    meta: Dict[str, str] = {}
    rows: List[List[str]] = []
    with open(path) as f:
        for line in f:
            if not line.strip() or line.startswith("~"):
                continue
            if line.startswith("<"):
                k, v = _meta(line)
                meta[k] = v
                continue
            toks = line.split()
            rows.append(toks[:10])
    m = int(meta["<NUMBER OF LINKS>"])
    if len(rows) != m:
        raise ValueError(f"num_links {m} but {len(rows)} links")
    a = rows
    net = Network(
        num_nodes=int(meta["<NUMBER OF NODES>"]),
        num_zones=int(meta["<NUMBER OF ZONES>"]),
        first_thru_node=int(meta.get("<FIRST THRU NODE>", "1")),
        init=np.array([int(r[0]) for r in a], dtype=np.int64),
        term=np.array([int(r[1]) for r in a], dtype=np.int64),
        capacity=np.array([float(r[2]) for r in a]),
        length=np.array([float(r[3]) for r in a]),
        fft=np.array([float(r[4]) for r in a]),
        alpha=np.array([float(r[5]) for r in a]),
        beta=np.array([float(r[6]) for r in a]),
        speed=np.array([float(r[7]) for r in a]),
        toll=np.array([float(r[8]) for r in a]),
        link_type=np.array([int(float(r[9].rstrip(";"))) if len(r) > 9 and r[9] != ";"
                            else 0 for r in a], dtype=np.int16),
    )
    return net.sort_links()


_PAIR = re.compile(r"(\d+)\s*:\s*([-+0-9.eE]+)\s*;")


def read_trips(path: str) -> Demand:
    """Parse a TNTP ``_trips`` file, keeping each origin's entries in file order."""
    z = None
    per: Dict[int, List[Tuple[int, float]]] = {}
    cur = None
    with open(path) as f:
        for line in f:
            if not line.strip() or line.startswith("~"):
                continue
            if line.startswith("<"):
                k, v = _meta(line)
                if k == "<NUMBER OF ZONES>":
                    z = int(v)
                continue
            if line.startswith("Origin"):
                cur = int(line.split()[1])
                per[cur] = []
                continue
            for d, v in _PAIR.findall(line):
                per[cur].append((int(d), float(v)))
    ptr = [0, 0]
    dests, vals = [], []
    for o in range(1, z + 1):
        lst = per.get(o, [])
        dests.extend(d for d, _ in lst)
        vals.extend(v for _, v in lst)
        ptr.append(ptr[-1] + len(lst))
    return Demand(num_zones=z, od_ptr=np.asarray(ptr, np.int64),
                  od_dest=np.asarray(dests, np.int64), od_demand=np.asarray(vals))


def read_flows(path_or_text: str, is_text: bool = False):
    """Parse a flows file: returns (init, term, volume, cost, header dict).

    The header dict holds ``iterations``, ``objvalue``, ``relgap`` and
    ``totalcost`` when the ``~`` summary lines written by
    tap/tap_frankwolfe_pthread.c:798-801 are present.
    """
    text = path_or_text if is_text else open(path_or_text).read()
    init, term, vol, cost = [], [], [], []
    hdr: Dict[str, float] = {}
    for line in io.StringIO(text):
        if line.startswith("~"):
            for key in ("iterations", "objvalue", "relgap", "totalcost"):
                mm = re.search(key + r"\s*=\s*([-+0-9.eEinfa]+)", line)
                if mm:
                    hdr[key] = float(mm.group(1))
            continue
        if not line.strip() or line.startswith("<"):
            continue
        toks = line.replace(";", " ").split()
        # \tTail\tHead\t:\tVolume\tCost;
        init.append(int(toks[0]))
        term.append(int(toks[1]))
        vol.append(float(toks[3]))
        cost.append(float(toks[4]))
    return (np.asarray(init, np.int64), np.asarray(term, np.int64), np.asarray(vol),
            np.asarray(cost), hdr)


def write_flows(path: str, net: Network, volume, cost, iterations=None, objvalue=None,
                relgap=None, totalcost=None) -> None:
    """Write the flows output format of tap/tap_functions.c:431-445."""
    with open(path, "w") as f:
        if iterations is not None:
            f.write("~ iterations = %d objvalue = %.15f relgap = %.15f\n"
                    % (iterations, objvalue, relgap))
            f.write("~ totalcost = %.15f\n" % totalcost)
        f.write("<NUMBER OF NODES>\t%d\n" % net.num_nodes)
        f.write("<NUMBER OF LINKS>\t%d\n" % net.num_links)
        f.write("<END OF METADATA>\n\n")
        f.write("~\tTail\tHead\t:\tVolume\tCost\t;\n")
        for k in range(net.num_links):
            f.write("\t%d\t%d\t:\t%.15f\t%.15f;\n"
                    % (net.init[k], net.term[k], volume[k], cost[k]))


def write_net_mods(path: str, net: Network, scenarios: List[Scenario]) -> None:
    """Scenarios as CHANGE records of the net-mods format (one change id each)."""
    with open(path, "w") as f:
        for sc in scenarios:
            for k, c in zip(sc.links.tolist(), sc.new_capacity.tolist()):
                f.write("\t".join([
                    sc.change_id, "CHANGE", str(int(net.init[k])), str(int(net.term[k])),
                    _r(c), _r(net.length[k]), _r(net.fft[k]), _r(net.alpha[k]),
                    _r(net.beta[k]), _r(net.speed[k]), _r(net.toll[k]),
                    str(int(net.link_type[k])), "0"]) + "\n")


def read_net_mods(path: str):
    """Return a list of (change_id, kind, link tuple of 10 fields, project_cost)."""
    out = []
    with open(path) as f:
        for line in f:
            if not line.strip() or line.startswith("~"):
                continue
            t = line.rstrip("\n").split("\t")
            out.append((t[0], t[1], (int(t[2]), int(t[3]), float(t[4]), float(t[5]),
                                     float(t[6]), float(t[7]), float(t[8]), float(t[9]),
                                     float(t[10]), int(t[11])),
                        float(t[12]) if len(t) > 12 and t[12] else 0.0))
    return out


_ITER = re.compile(
    r"iter = (\d+) objective value = ([-+0-9.einfa]+) relative gap = ([-+0-9.einfa]+) "
    r"average exccess cost = ([-+0-9.einfa]+) total cost = ([-+0-9.einfa]+)")


def parse_iteration_log(text: str) -> np.ndarray:
    """Per-iteration (iter, objective, relgap, avg_excess, total_cost) rows from the
    ``-v`` lines printed at tap/tap_frankwolfe_pthread.c:751-753."""
    rows = [[float(g) for g in m.groups()] for m in _ITER.finditer(text)]
    return np.asarray(rows).reshape(-1, 5)
