"""Trip modifications on the host: the Python restatement against the
library's C drop-ins (parse_trip_mod_file, apply_trip_modification, which
follow tap/parsetapfiles.c:573-638 and tap/tap_functions.c:521-598)."""

import ctypes as C

import numpy as np
import pytest

from test_abi import DemandData, _libc
from traffic_assignment_gb300 import synth, tntp
from traffic_assignment_gb300 import tripmods as T


class TripModS(C.Structure):
    _fields_ = [("trip_change_id", C.c_char * 128), ("trip_modtype", C.c_int),
                ("origin", C.c_long), ("dest", C.c_long), ("multiplier", C.c_double)]


MODS = [T.TripMod("p1", "P2P", 3, 7, 1.5), T.TripMod("u1", "UNIFORM", 5, 0, 0.25),
        T.TripMod("u2", "UNIFORM", 0, 11, 2.0), T.TripMod("a1", "ALL", 0, 0, 1.1),
        T.TripMod("p0", "P2P", 2, 9, 0.0)]


@pytest.fixture(scope="module")
def lib():
    from traffic_assignment_gb300 import _capi
    return _capi.load()


def _c_demands(lib, dem, tmp_path):
    tf = str(tmp_path / "trips.txt")
    tntp.write_trips(tf, dem)
    libc = _libc()
    lib.parse_trips_file.argtypes = [C.c_void_p, C.POINTER(C.POINTER(C.POINTER(DemandData))),
                                     C.POINTER(C.c_long)]
    fp = libc.fopen(tf.encode(), b"r")
    arr = C.POINTER(C.POINTER(DemandData))()
    nz = C.c_long()
    assert lib.parse_trips_file(fp, C.byref(arr), C.byref(nz)) == 0
    libc.fclose(fp)
    return arr, nz.value


def _c_to_entries(arr, dem):
    out = []
    for o in range(1, dem.num_zones + 1):
        j = 0
        while arr[o][j].dest != 0:
            out.append((o, arr[o][j].dest, arr[o][j].demand))
            j += 1
    return out


def test_trip_mod_file_roundtrip_and_c_parser(lib, tmp_path):
    p = str(tmp_path / "tripmods.txt")
    T.write_trip_mods(p, MODS)
    assert T.read_trip_mods(p) == MODS
    libc = _libc()
    lib.parse_trip_mod_file.argtypes = [C.c_void_p, C.POINTER(C.POINTER(TripModS)),
                                        C.POINTER(C.c_int)]
    fp = libc.fopen(p.encode(), b"r")
    mods = C.POINTER(TripModS)()
    n = C.c_int()
    assert lib.parse_trip_mod_file(fp, C.byref(mods), C.byref(n)) == 0
    libc.fclose(fp)
    assert n.value == len(MODS)
    kinds = {1: "P2P", 2: "UNIFORM", 3: "ALL"}
    for i, m in enumerate(MODS):
        c = mods[i]
        assert (c.trip_change_id.decode(), kinds[c.trip_modtype], c.origin, c.dest,
                c.multiplier) == (m.change_id, m.kind, m.origin, m.dest, m.multiplier)


@pytest.mark.parametrize("bad", [T.TripMod("x", "P2P", 0, 3, 2.0),
                                 T.TripMod("x", "UNIFORM", 0, 0, 2.0),
                                 T.TripMod("x", "HALF", 1, 1, 2.0)])
def test_invalid_mods_rejected(bad, tmp_path):
    p = str(tmp_path / "bad.txt")
    with open(p, "w") as f:
        f.write(f"{bad.change_id}\t{bad.kind}\t{bad.origin}\t{bad.dest}\t{bad.multiplier}\n")
    with pytest.raises(ValueError):
        T.read_trip_mods(p)


def test_apply_matches_c_drop_in(lib, tmp_path):
    net, dem = synth.make_small24()
    arr, nz = _c_demands(lib, dem, tmp_path)
    lib.apply_trip_modification.argtypes = [C.POINTER(C.POINTER(DemandData)),
                                            C.POINTER(TripModS), C.c_long]
    lib.apply_trip_modification.restype = C.c_int
    kinds = {"P2P": 1, "UNIFORM": 2, "ALL": 3}
    cur = dem
    for m in MODS:
        cm = TripModS(m.change_id.encode(), kinds[m.kind], m.origin, m.dest, m.multiplier)
        assert lib.apply_trip_modification(arr, C.byref(cm), nz) == 0
        cur = T.apply_trip_mod(cur, m)
        ents = _c_to_entries(arr, dem)
        np.testing.assert_array_equal(np.array([e[2] for e in ents]), T.demand_entries(cur))
        np.testing.assert_array_equal(np.array([e[1] for e in ents]),
                                      dem.od_dest[dem.od_ptr[1]:dem.od_ptr[dem.num_zones + 1]])
    bad = TripModS(b"b", 1, nz + 1, 1, 2.0)
    assert lib.apply_trip_modification(arr, C.byref(bad), nz) == -1
    with pytest.raises(ValueError):
        T.apply_trip_mod(dem, T.TripMod("b", "P2P", nz + 1, 1, 2.0))


def test_demand_scenario_matrix():
    net, dem = synth.make_small24()
    sets = [[], [MODS[0]], [MODS[3], MODS[1]]]
    D = T.demand_scenarios(dem, sets)
    assert D.shape == (3, dem.od_ptr[dem.num_zones + 1] - dem.od_ptr[1])
    np.testing.assert_array_equal(D[0], T.demand_entries(dem))
    assert D[2].sum() != D[0].sum()
