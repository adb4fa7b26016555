"""Builds the CUDA C-ABI library libstormbird_gb300.so in-tree (sm_103a only).

Each .cu translation unit is compiled in parallel with nvcc
(-gencode arch=compute_103a,code=sm_103a -lineinfo -O3), then linked into
stormbird_gb300/_build/libstormbird_gb300.so. No cmake, no relocatable device code.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libstormbird_gb300.so")
UNITS = ["k_biot_savart.cu", "k_wake.cu", "k_solve.cu", "k_probe.cu", "sim_host.cu", "batch_host.cu", "noalloc_sweep.cu", "k_mlp.cu",
         "mlp_host.cu", "k_wind.cu", "csm_host.cu",
         "result_io.cu"]
HEADERS = ["sb_device.cuh", "sb_kernels.h", "sb_setup.hpp", "json_min.hpp", "sim_core.hpp", "sb_ptx.cuh", "sb_mlp.h", "sb_wind_setup.hpp",
           "sb_controller_setup.hpp", "batch_access.hpp", "result_io.hpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA library cannot be built")


def _deps():
    inc = os.path.join(HERE, "..", "include", "stormbird_gb300.h")
    return [os.path.join(CSRC, f) for f in UNITS + HEADERS] + [inc, os.path.abspath(__file__)]


def stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(d) > t for d in _deps())


def build(force: bool = False, verbose: bool = False, ptxas_verbose: bool = False) -> str:
    if not force and not stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    common = [cc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I", CSRC, "-I", os.path.join(HERE, "..", "include")]
    if ptxas_verbose:
        common += ["-Xptxas", "-v"]
    tag = f"{os.getpid()}"

    def compile_unit(u: str) -> str:
        obj = os.path.join(OUT_DIR, u.replace(".cu", f".{tag}.o"))
        cmd = common + ["-c", os.path.join(CSRC, u), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {u}:\n{r.stdout}\n{r.stderr}")
        if ptxas_verbose or verbose:
            sys.stdout.write(r.stdout + r.stderr)
        return obj

    objs = []
    try:
        with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
            objs = list(ex.map(compile_unit, UNITS))
    finally:
        if len(objs) != len(UNITS):
            for u in UNITS:
                o = os.path.join(OUT_DIR, u.replace(".cu", f".{tag}.o"))
                if os.path.exists(o):
                    os.remove(o)
    tmp = LIB + f".tmp{tag}"
    cmd = [cc, "-shared", *ARCH, "-cudart", "static", "-o", tmp] + objs + ["-lrt", "-ldl", "-lpthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    for o in objs:
        os.remove(o)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, ptxas_verbose="--ptxas" in sys.argv))
