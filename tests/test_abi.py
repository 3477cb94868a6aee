"""The C ABI: libtapgpu.so loads without a GPU and exports every declaration
of include/tap_gpu.h; the host-side TNTP parsers and printers of the library
read and write the reference's formats (no GPU compute is called here)."""

import ctypes as C
import os
import re
import tempfile

import numpy as np
import pytest

import oracle
from traffic_assignment_gb300 import _capi, synth, tntp

HEADER = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include", "tap_gpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", src)
    skip = {"if", "while", "for", "return", "sizeof"}
    return sorted(set(n for n in names if n not in skip))


def declared_data():
    src = open(HEADER).read()
    return re.findall(r"^extern\s+(?:unsigned\s+)?int\s+(\w+);", src, flags=re.M)


@pytest.fixture(scope="module")
def lib(built_lib):
    return built_lib


def test_header_lists_match_binding():
    assert set(declared_functions()) == set(_capi.EXPORTED)
    assert set(declared_data()) == set(_capi.EXPORTED_DATA)


def test_every_declared_symbol_exported(lib):
    missing = [n for n in declared_functions() + declared_data() if not hasattr(lib, n)]
    assert not missing, missing


class LinkData(C.Structure):
    _fields_ = [("init_node", C.c_long), ("term_node", C.c_long), ("capacity", C.c_double),
                ("length", C.c_double), ("free_flow_time", C.c_double), ("B", C.c_double),
                ("power", C.c_double), ("speed_limit", C.c_double), ("toll", C.c_double),
                ("link_type", C.c_short)]


class NetData(C.Structure):
    _fields_ = [("num_zones", C.c_long), ("num_nodes", C.c_long),
                ("first_thru_node", C.c_long), ("num_links", C.c_long),
                ("links", C.POINTER(LinkData))]


class DemandData(C.Structure):
    _fields_ = [("dest", C.c_long), ("demand", C.c_double)]


def _libc():
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    return libc


def test_link_struct_layout_matches_reference():
    # tap/tap_types.h:20-32 on LP64: 2 longs, 7 doubles, 1 short, padded to 80 bytes
    assert C.sizeof(LinkData) == 80
    assert C.sizeof(NetData) == 40


def test_parse_net_and_trips(lib):
    net, dem = synth.make_grid416()
    d = tempfile.mkdtemp()
    nf, tf = os.path.join(d, "net.txt"), os.path.join(d, "trips.txt")
    tntp.write_net(nf, net)
    tntp.write_trips(tf, dem)
    libc = _libc()
    lib.parse_net_file.argtypes = [C.c_void_p, C.POINTER(NetData)]
    fp = libc.fopen(nf.encode(), b"r")
    nd = NetData()
    assert lib.parse_net_file(fp, C.byref(nd)) == 0
    libc.fclose(fp)
    assert (nd.num_nodes, nd.num_zones, nd.num_links, nd.first_thru_node) == (
        net.num_nodes, net.num_zones, net.num_links, net.first_thru_node)
    got = np.array([(nd.links[k].init_node, nd.links[k].term_node) for k in range(nd.num_links)])
    np.testing.assert_array_equal(got[:, 0], net.init)
    np.testing.assert_array_equal(got[:, 1], net.term)
    caps = np.array([nd.links[k].capacity for k in range(nd.num_links)])
    np.testing.assert_array_equal(caps, net.capacity)

    lib.parse_trips_file.argtypes = [C.c_void_p, C.POINTER(C.POINTER(C.POINTER(DemandData))),
                                     C.POINTER(C.c_long)]
    fp = libc.fopen(tf.encode(), b"r")
    arr = C.POINTER(C.POINTER(DemandData))()
    nz = C.c_long()
    assert lib.parse_trips_file(fp, C.byref(arr), C.byref(nz)) == 0
    libc.fclose(fp)
    assert nz.value == dem.num_zones
    for o in range(1, nz.value + 1):
        s, e = dem.od_ptr[o], dem.od_ptr[o + 1]
        lst = []
        i = 0
        while arr[o][i].dest != 0:
            lst.append((arr[o][i].dest, arr[o][i].demand))
            i += 1
        assert [a for a, _ in lst] == dem.od_dest[s:e].tolist()
        np.testing.assert_array_equal([b for _, b in lst], dem.od_demand[s:e])
    lib.demand_sum.restype = C.c_double
    lib.demand_sum.argtypes = [C.POINTER(C.POINTER(DemandData)), C.c_long]
    assert lib.demand_sum(arr, nz.value + 1) == pytest.approx(dem.total, rel=1e-12)


def test_print_flow_format(lib, tmp_path):
    net, _ = synth.make_small24()
    m = net.num_links
    links = (LinkData * m)()
    for k in range(m):
        links[k].init_node = int(net.init[k])
        links[k].term_node = int(net.term[k])
    nd = NetData(net.num_zones, net.num_nodes, 1, m, links)
    vol = np.linspace(0, 1000, m)
    cost = np.linspace(1, 9, m)
    libc = _libc()
    path = str(tmp_path / "flows.txt")
    fp = libc.fopen(path.encode(), b"w")
    lib.print_flow.argtypes = [C.c_void_p, C.POINTER(NetData), C.POINTER(C.c_double),
                               C.POINTER(C.c_double)]
    lib.print_flow(fp, C.byref(nd), vol.ctypes.data_as(C.POINTER(C.c_double)),
                   cost.ctypes.data_as(C.POINTER(C.c_double)))
    libc.fclose(fp)
    text = open(path).read()
    lines = text.splitlines()
    assert lines[0] == f"<NUMBER OF NODES>\t{net.num_nodes}"
    assert lines[4] == "~\tTail\tHead\t:\tVolume\tCost\t;"
    assert lines[5] == "\t%d\t%d\t:\t%.15f\t%.15f;" % (net.init[0], net.term[0], vol[0], cost[0])
    i, t, v, c, _ = tntp.read_flows(text, is_text=True)
    np.testing.assert_array_equal(i, net.init)


def test_python_tntp_roundtrip(tmp_path):
    net, dem = synth.make_grid416()
    tntp.write_net(str(tmp_path / "n.txt"), net)
    tntp.write_trips(str(tmp_path / "t.txt"), dem)
    n2 = tntp.read_net(str(tmp_path / "n.txt"))
    d2 = tntp.read_trips(str(tmp_path / "t.txt"))
    np.testing.assert_array_equal(n2.init, net.init)
    np.testing.assert_array_equal(n2.capacity, net.capacity)
    np.testing.assert_array_equal(n2.fft, net.fft)
    np.testing.assert_array_equal(d2.od_ptr, dem.od_ptr)
    np.testing.assert_array_equal(d2.od_demand, dem.od_demand)


def test_synthetic_shapes():
    net, dem = synth.make_small24()
    assert (net.num_nodes, net.num_links, net.num_zones) == (24, 76, 24)
    net, dem = synth.make_grid416()
    assert (net.num_nodes, net.num_links, net.num_zones) == (416, 914, 38)
    frac = len(dem.od_demand) / (38 * 37)  # nonzero off-diagonal OD pairs
    assert 0.25 < frac < 0.35 and (dem.od_demand > 0).all()
    net, dem = synth.make_grid10k()
    assert (net.num_nodes, net.num_links, net.num_zones) == (10000, 40000, 1000)
    assert abs(dem.total - 1.5e6) < 1.0
    # links sorted by (init, term) and every node reachable on the grid backbone
    assert np.all(np.diff(net.init * (net.num_nodes + 1) + net.term) > 0)


def test_oracle_no_path_reported():
    net, dem = synth.make_grid416(first_thru_node=39)
    with pytest.raises(RuntimeError, match="rc=2"):
        oracle.frankwolfe(net, dem, threads=1, max_iters=2)


def test_bench_counts_the_scenario_state_size(tmp_path):
    """bench.py counts host-to-device bytes with the size of the device's
    per-scenario state record: compile a host program against the header."""
    import importlib.util
    import shutil
    import subprocess

    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc absent")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "sz.cu"
    src.write_text('#include <cstdio>\n#include "fw_kernels.cuh"\n'
                   'int main() { std::printf("%zu", sizeof(tapgpu::ScenState)); return 0; }\n')
    exe = tmp_path / "sz"
    subprocess.run([nvcc, "-std=c++17", "-I", os.path.join(root, "include"), "-I",
                    os.path.join(root, "traffic_assignment_gb300", "csrc"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    size = int(subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout)
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    assert bench.SCEN_STATE_BYTES == size


def test_options_struct_matches_header(tmp_path):
    """The Python front end's tapgpu_options mirror has the header's size and
    field offsets (compiled with the C compiler against include/tap_gpu.h)."""
    import shutil
    import subprocess

    from traffic_assignment_gb300 import _capi

    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    names = [f[0] for f in _capi.Options._fields_]
    body = "".join(f'  printf("%zu ", offsetof(tapgpu_options, {n}));\n' for n in names)
    src = tmp_path / "opt.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "tap_gpu.h"\n'
                   'int main(void) {\n' + body +
                   '  printf("%zu", sizeof(tapgpu_options));\n  return 0;\n}\n')
    exe = tmp_path / "opt"
    subprocess.run([cc, "-I", os.path.join(root, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True,
                                          text=True).stdout.split()]
    want = [getattr(_capi.Options, n).offset for n in names] + [C.sizeof(_capi.Options)]
    assert got == want


# num_nodes1 (node 0 counted) whose FP64 labels and bitmaps still fit one
# per-CTA slice of the allocation-free entry point's fixed 32 MiB array
NOALLOC_MAX_NODES1 = 4_067_172


def test_noalloc_size_limit_is_exact(lib):
    """The allocation-free entry point applies its size limit before any CUDA
    call: one node over the limit is refused, the limit itself passes the size
    check (with no sources the call then returns without touching the GPU)."""
    dummy = C.c_void_p(16)  # never dereferenced: the calls return before any device work
    args = (0, 1, dummy, dummy, dummy, dummy, 0, None, None)
    rc = lib.tapgpu_sssp_labels_noalloc(NOALLOC_MAX_NODES1 + 1, *args)
    assert rc == _capi.TAPGPU_ERR_UNSUPPORTED
    assert lib.tapgpu_sssp_labels_noalloc(NOALLOC_MAX_NODES1, *args) == _capi.TAPGPU_OK
