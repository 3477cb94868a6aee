"""Build recipe for the CPU oracle (test infrastructure only).

* ``build_oracle()`` compiles this directory's own C restatement
  (``oracle_tap.c``) into ``oracle/_build/liboracle_tap.so``.  It runs on any
  machine with gcc, including the GPU host, where it is rebuilt from source.
* ``build_reference()`` compiles the reference's own CPU solver from the
  sources where they lie under ``$TAP_REFERENCE_ROOT/trunk/tap`` (the
  reference checkout; default ``/root/reference``) into
  ``oracle/_ref/`` (never copying a source file), with the reference's flags
  (tap/common.mk:50 ``-O3 -fno-associative-math`` plus ``-pthread``):

    oracle/_ref/tap_frankwolfe_pthread   parsetapfiles.c tap_functions.c utils.c
                                          sssp_pape.c tap_frankwolfe_pthread.c tap_main.c
    oracle/_ref/tap_frankwolfe           ... tap_frankwolfe.c (serial driver)
    oracle/_ref/libref_sssp.so           sssp_pape.c alone (shortest-path entry points)

  It is skipped when the reference tree is absent.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# the reference checkout: one setting for every recipe and test that reads it
REFERENCE_ROOT = os.environ.get("TAP_REFERENCE_ROOT", "/root/reference")
REF_TRUNK = os.path.join(REFERENCE_ROOT, "trunk")
REF_TAP = os.path.join(REF_TRUNK, "tap")
CFLAGS = ["-O3", "-fno-associative-math", "-pthread", "-DUNIX"]


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), res.stdout, res.stderr))


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, "liboracle_tap.so")
    srcs = [os.path.join(HERE, "oracle_tap.c"), os.path.join(HERE, "oracle_adjoint.c"),
            os.path.join(HERE, "oracle_tap.h")]
    if force or _stale(out, srcs):
        tmp = out + ".tmp"
        # no fused multiply-add: the Arm host would otherwise round differently
        _run(["gcc", *CFLAGS, "-ffp-contract=off", "-std=c11", "-fPIC", "-shared", "-o", tmp,
              srcs[0], srcs[1], "-lm"])
        os.replace(tmp, out)
    return out


def reference_available() -> bool:
    return os.path.isdir(REF_TAP)


def build_reference(force: bool = False) -> bool:
    if not reference_available() or shutil.which("gcc") is None:
        return False
    os.makedirs(REF_OUT, exist_ok=True)
    common = ["parsetapfiles.c", "tap_functions.c", "utils.c", "sssp_pape.c"]
    targets = {
        "tap_frankwolfe_pthread": common + ["tap_frankwolfe_pthread.c", "tap_main.c"],
        "tap_frankwolfe": common + ["tap_frankwolfe.c"],
    }
    for name, files in targets.items():
        out = os.path.join(REF_OUT, name)
        srcs = [os.path.join(REF_TAP, f) for f in files]
        if force or _stale(out, srcs):
            _run(["gcc", *CFLAGS, "-w", "-I", REF_TAP, "-o", out, *srcs, "-lm"])
    out = os.path.join(REF_OUT, "libref_sssp.so")
    src = os.path.join(REF_TAP, "sssp_pape.c")
    if force or _stale(out, [src]):
        _run(["gcc", *CFLAGS, "-w", "-fPIC", "-shared", "-I", REF_TAP, "-o", out, src, "-lm"])
    return True


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print("reference built" if build_reference(force="--force" in sys.argv)
          else "reference sources absent: skipped")
