"""The reference's own CLI driver (tap/tap_main.c with tap/utils.c),
compiled unmodified from the reference checkout with the reference's own
headers, links against libtapgpu.so with no symbol left unresolved, and the
resulting binary calls into the library: on a host without a GPU the solve
stops at context creation with the library's no-device message.  Skipped
where the reference checkout is absent (the GPU host has none)."""

import os
import shutil
import subprocess

import pytest

from oracle import build_oracle as ob
from traffic_assignment_gb300 import build as B
from traffic_assignment_gb300 import synth, tntp

pytestmark = pytest.mark.skipif(not os.path.isdir(ob.REF_TAP) or shutil.which("gcc") is None,
                                reason="reference checkout or gcc absent")


@pytest.fixture(scope="module")
def ref_driver(built_lib, tmp_path_factory):
    out = str(tmp_path_factory.mktemp("refdrv") / "tap_main_on_tapgpu")
    lib = os.path.dirname(B.lib_path())
    srcs = [os.path.join(ob.REF_TAP, f) for f in ("tap_main.c", "utils.c")]
    cmd = ["gcc", "-O2", "-pthread", "-DUNIX", "-w", "-I", ob.REF_TAP, "-o", out, *srcs,
           "-L", lib, "-ltapgpu", "-Wl,--no-undefined", "-Wl,-rpath," + lib, "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]
    return out


def test_reference_driver_links_unchanged(ref_driver):
    assert os.access(ref_driver, os.X_OK)
    res = subprocess.run(["nm", "-D", "--undefined-only", ref_driver], capture_output=True,
                         text=True)
    undefined = {ln.split()[-1].split("@")[0] for ln in res.stdout.splitlines() if ln.strip()}
    # the FW entry points resolve to the library
    for sym in ("tap_frankwolfe", "parse_net_file", "parse_trips_file", "link_data_compar",
                "apply_trip_modification", "parse_trip_mod_file"):
        if sym in undefined:
            res2 = subprocess.run(["nm", "-D", "--defined-only", B.lib_path()],
                                  capture_output=True, text=True)
            assert sym in res2.stdout, sym


def test_reference_driver_reaches_the_library(ref_driver, tmp_path):
    net, dem = synth.make_small24()
    nf, tf = str(tmp_path / "net.txt"), str(tmp_path / "trips.txt")
    tntp.write_net(nf, net)
    tntp.write_trips(tf, dem)
    env = dict(os.environ, TAPGPU_NO_SIGNALS="1", CUDA_VISIBLE_DEVICES="")
    res = subprocess.run([ref_driver, "-i", "5", nf, tf], capture_output=True, text=True,
                         timeout=120, env=env)
    # parsed by the library's TNTP readers, then the GPU solver reports no device
    assert res.returncode != 0
    assert "CUDA" in res.stderr or "device" in res.stderr, res.stderr[-2000:]
