"""Build libtapgpu.so (CUDA sm_103a) and the tap_frankwolfe_gpu CLI in-tree.

Everything is compiled with nvcc / gcc directly (no cmake), translation units in
parallel, into ``traffic_assignment_gb300/_lib/``:

  libtapgpu.so          kernels + host solver + C ABI of include/tap_gpu.h
  tap_frankwolfe_gpu    drop-in CLI with the flags of the reference's tap_main.c
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "_lib")
OBJ = os.path.join(OUT, "obj")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INC, "-I", CSRC,
              "--expt-relaxed-constexpr"]
CU_SOURCES = ["fw_kernels.cu", "solver.cu", "linkops.cu", "adjoint.cu", "noalloc.cu"]
CXX_SOURCES = ["capi.cpp"]
C_SOURCES = ["tntp_io.c"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def cuda_home() -> str:
    return os.path.dirname(os.path.dirname(nvcc()))


def lib_path() -> str:
    return os.path.join(OUT, "libtapgpu.so")


def cli_path() -> str:
    return os.path.join(OUT, "tap_frankwolfe_gpu")


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), res.stdout, res.stderr))
    return res.stdout + res.stderr


def _headers():
    hs = [os.path.join(INC, f) for f in os.listdir(INC)]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, extra=()):
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ, src + ".o")
    if not _stale(obj, [path, *_headers(), __file__]):
        return obj, ""
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", path, "-o", obj]
    elif src.endswith(".cpp"):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-I", INC, "-I", CSRC,
               "-I", os.path.join(cuda_home(), "include"), "-c", path, "-o", obj]
    else:
        cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-Wall", "-I", INC, "-c", path, "-o", obj]
    log = _run(cmd)
    return obj, log


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    srcs = [s for s in CU_SOURCES + CXX_SOURCES + C_SOURCES
            if os.path.exists(os.path.join(CSRC, s))]
    extra = ("-Xptxas", "-v") if ptxas_info else ()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda s: _compile(s, extra if s.endswith(".cu") else ()), srcs))
    objs = [r[0] for r in results]
    if verbose or ptxas_info:
        for r in results:
            if r[1]:
                print(r[1], file=sys.stderr)
    lib = lib_path()
    if _stale(lib, objs):
        tmp = lib + ".tmp"
        _run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lpthread"])
        os.replace(tmp, lib)
    cli_src = os.path.join(CSRC, "tap_main_gpu.c")
    if os.path.exists(cli_src) and _stale(cli_path(), [cli_src, lib]):
        _run(["gcc", "-O2", "-std=gnu11", "-Wall", "-I", INC, "-o", cli_path(), cli_src,
              "-L", OUT, "-ltapgpu", "-Wl,-rpath,$ORIGIN", "-lm"])
    return lib


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv))
