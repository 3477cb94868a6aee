"""ctypes binding of libtapgpu.so (the C ABI declared in include/tap_gpu.h).

The library is the only compute path: if it has not been built this module
raises instead of falling back to anything else.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

I64P = C.POINTER(C.c_int64)
F64P = C.POINTER(C.c_double)

TAPGPU_OK = 0
TAPGPU_ERR_ARG = 1
TAPGPU_ERR_CUDA = 2
TAPGPU_ERR_NO_PATH = 3
TAPGPU_ERR_NO_CONVERGENCE = 4
TAPGPU_ERR_ALLOC = 5
TAPGPU_ERR_UNSUPPORTED = 6
TAPGPU_ERR_NO_DEVICE = 7
TAPGPU_FP64 = 0
TAPGPU_FP32_PATHS = 1
TRACE_COLS = 8


class Network(C.Structure):
    _fields_ = [("num_nodes", C.c_int64), ("num_zones", C.c_int64),
                ("first_thru_node", C.c_int64), ("num_links", C.c_int64),
                ("init", I64P), ("term", I64P), ("capacity", F64P), ("fft", F64P),
                ("alpha", F64P), ("beta", F64P)]


class DemandS(C.Structure):
    _fields_ = [("num_origins", C.c_int64), ("od_ptr", I64P), ("od_dest", I64P),
                ("od_demand", F64P)]


class Options(C.Structure):
    _fields_ = [("precision", C.c_int), ("device", C.c_int), ("sssp_block", C.c_int),
                ("aon_block", C.c_int), ("iters_per_launch", C.c_int), ("use_graphs", C.c_int),
                ("chunk_tasks", C.c_int64), ("record_tape", C.c_int),
                ("tape_capacity", C.c_int), ("global_scratch", C.c_int),
                ("sssp_variant", C.c_int), ("nf_delta", C.c_double),
                ("line_search", C.c_int), ("tape_checkpoint", C.c_int),
                ("sssp_ctas_per_sm", C.c_int), ("aon_ctas_per_sm", C.c_int)]


class Result(C.Structure):
    _fields_ = [("iterations", C.c_int), ("error_bits", C.c_int), ("objective", C.c_double),
                ("relgap", C.c_double), ("total_cost", C.c_double),
                ("avg_excess", C.c_double), ("lambda_last", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class TapGpuError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{message} (status {status})")
        self.status = status


_LIB = None

# every function exported by include/tap_gpu.h
EXPORTED = [
    "tap_frankwolfe", "fw_assign", "pape_cuda", "sssp_pape", "sssp_slf", "sssp_slf_lll",
    "sssp_pape_lll", "get_shortest_path", "bpr_cost_function", "linkcost_integral",
    "links_objective_function", "link_directional_derivative", "adjlist_to_packed_arrays",
    "adjlist_entry_compar", "update_link_costs", "demand_sum", "total_link_cost", "print_flow",
    "line_search", "apply_trip_modification", "parse_net_file", "parse_trips_file",
    "parse_flows_file", "parse_net_mod_file", "link_data_compar", "parse_trip_mod_file",
    "tapgpu_default_options", "tapgpu_status_string", "tapgpu_last_message", "tapgpu_create",
    "tapgpu_destroy", "tapgpu_solve", "tapgpu_solve_begin", "tapgpu_solve_advance",
    "tapgpu_get_link_flows", "tapgpu_get_link_flows_batch", "tapgpu_get_trace",
    "tapgpu_set_capacity", "tapgpu_solve_scenarios", "tapgpu_sssp", "tapgpu_aon", "tapgpu_stream",
    "tapgpu_profile_iteration", "tapgpu_run_iterations", "tapgpu_set_timing",
    "tapgpu_get_timing", "tapgpu_get_path_stats", "tapgpu_sssp_labels_noalloc",
    "tapgpu_adjoint_vht", "tapgpu_get_tape", "tapgpu_set_scenario_demand",
    "tapgpu_set_scenario_links",
]
EXPORTED_DATA = ["num_cores", "num_threads", "using_fermi_architecture"]


def library_path() -> str:
    return _build.lib_path()


def load(path: str | None = None):
    """Load libtapgpu.so; raises if it was not built (no fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = path or library_path()
    if not os.path.exists(p):
        raise RuntimeError(
            f"libtapgpu.so not found at {p}: build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(p)
    vp = C.c_void_p
    L.tapgpu_default_options.argtypes = [C.POINTER(Options)]
    L.tapgpu_default_options.restype = None
    L.tapgpu_status_string.argtypes = [C.c_int]
    L.tapgpu_status_string.restype = C.c_char_p
    L.tapgpu_last_message.argtypes = []
    L.tapgpu_last_message.restype = C.c_char_p
    L.tapgpu_create.argtypes = [C.POINTER(Network), C.POINTER(DemandS), C.POINTER(Options),
                                C.POINTER(vp)]
    L.tapgpu_destroy.argtypes = [vp]
    L.tapgpu_destroy.restype = None
    L.tapgpu_solve.argtypes = [vp, C.c_int, C.c_double, F64P, C.POINTER(Result)]
    L.tapgpu_solve_begin.argtypes = [vp, C.c_int, C.c_double, F64P]
    L.tapgpu_solve_advance.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(Result)]
    L.tapgpu_get_link_flows.argtypes = [vp, C.c_int, F64P, F64P]
    L.tapgpu_get_link_flows_batch.argtypes = [vp, C.c_int, C.c_int, F64P, F64P]
    L.tapgpu_get_trace.argtypes = [vp, C.c_int, F64P, C.c_int, C.POINTER(C.c_int)]
    L.tapgpu_set_capacity.argtypes = [vp, F64P]
    L.tapgpu_solve_scenarios.argtypes = [vp, C.c_int, I64P, I64P, F64P, C.c_int, C.c_double,
                                         F64P, C.POINTER(Result)]
    L.tapgpu_sssp.argtypes = [vp, F64P, I64P, C.c_int64, F64P, I64P]
    L.tapgpu_aon.argtypes = [vp, F64P, F64P]
    L.tapgpu_stream.argtypes = [vp]
    L.tapgpu_stream.restype = vp
    L.tapgpu_profile_iteration.argtypes = [vp, C.c_int, C.POINTER(C.c_float)]
    L.tapgpu_run_iterations.argtypes = [vp, C.c_int]
    L.tapgpu_set_timing.argtypes = [vp, C.c_int]
    L.tapgpu_get_timing.argtypes = [vp, F64P, I64P, I64P]
    L.tapgpu_get_path_stats.argtypes = [vp, I64P]
    L.tapgpu_get_path_stats.restype = C.c_int
    L.tapgpu_sssp_labels_noalloc.argtypes = [C.c_int32, C.c_int32, C.c_int32, vp, vp, vp, vp,
                                             C.c_int32, vp, vp]
    L.tapgpu_sssp_labels_noalloc.restype = C.c_int
    L.tapgpu_adjoint_vht.argtypes = [vp, C.c_int, F64P, F64P]
    L.tapgpu_adjoint_vht.restype = C.c_int
    L.tapgpu_get_tape.argtypes = [vp, C.c_int, C.c_int, F64P, F64P, F64P]
    L.tapgpu_get_tape.restype = C.c_int
    L.tapgpu_set_scenario_demand.argtypes = [vp, C.c_int, F64P]
    L.tapgpu_set_scenario_demand.restype = C.c_int
    L.tapgpu_set_scenario_links.argtypes = [vp, C.c_int, I64P, I64P, F64P, F64P, F64P, I64P,
                                            I64P]
    L.tapgpu_set_scenario_links.restype = C.c_int
    for fn in ("tapgpu_create", "tapgpu_solve", "tapgpu_solve_begin", "tapgpu_solve_advance",
               "tapgpu_get_link_flows", "tapgpu_get_link_flows_batch", "tapgpu_get_trace",
               "tapgpu_set_capacity", "tapgpu_solve_scenarios", "tapgpu_sssp", "tapgpu_aon",
               "tapgpu_profile_iteration", "tapgpu_run_iterations", "tapgpu_set_timing",
               "tapgpu_get_timing"):
        getattr(L, fn).restype = C.c_int
    _LIB = L
    return L


def check(status: int):
    if status != TAPGPU_OK:
        L = load()
        raise TapGpuError(status, "%s: %s" % (L.tapgpu_status_string(status).decode(),
                                              L.tapgpu_last_message().decode()))


def ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)
