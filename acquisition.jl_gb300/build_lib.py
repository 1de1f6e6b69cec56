"""Build libacqgb300.so in-tree (sm_103a only).

    python acquisition.jl_gb300/build_lib.py [--debug] [--bounds-check]

Compiles the host C++ (g++) and the CUDA runtime/kernels (nvcc) in parallel and links
``acquisition.jl_gb300/acqgb300/libacqgb300.so``. No cmake. Host code is compiled with
-ffp-contract=off so double-precision geometry rounds identically on x86-64 and aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "acqgb300")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libacqgb300.so")
CHECKED_LIB = os.path.join(OUT_DIR, "libacqgb300_checked.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def build(verbose: bool = False, debug: bool = False, ptxas_verbose: bool = False, bounds_check: bool = False) -> str:
    """Build the library; bounds_check=True builds the checked variant (device index checks that
    record the first out-of-buffer access instead of faulting) as libacqgb300_checked.so, in its
    own object directory. Returns the compiler output."""
    build_dir = BUILD_DIR + ("_checked" if bounds_check else "")
    lib = CHECKED_LIB if bounds_check else LIB
    os.makedirs(build_dir, exist_ok=True)
    nvcc = _nvcc()
    opt = ["-O0", "-g"] if debug else ["-O3"]
    if bounds_check:
        opt = opt + ["-DACQ_BOUNDS_CHECK"]
    host_obj = os.path.join(build_dir, "acq_host.o")
    dev_obj = os.path.join(build_dir, "acq_runtime.o")
    na_obj = os.path.join(build_dir, "acq_noalloc.o")
    corr_obj = os.path.join(build_dir, "acq_corr.o")
    synth_obj = os.path.join(build_dir, "acq_synth.o")
    inst = ["acq_inst_tile", "acq_inst_col", "acq_inst_sign", "acq_inst_mma"]
    inst_objs = [os.path.join(build_dir, f"{n}.o") for n in inst]
    host_cmd = ["g++", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function", *opt,
                f"-I{INCLUDE}", "-c", os.path.join(CSRC, "acq_host.cpp"), "-o", host_obj]
    dev_cmd = [nvcc, "-std=c++17", *ARCH, "-lineinfo", *opt, "-Xcompiler", "-fPIC,-ffp-contract=off",
               f"-I{INCLUDE}", f"-I{CSRC}", "-c", os.path.join(CSRC, "acq_runtime.cu"), "-o", dev_obj]
    na_cmd = [nvcc, "-std=c++17", *ARCH, "-lineinfo", *opt, "-Xcompiler", "-fPIC,-ffp-contract=off",
              f"-I{INCLUDE}", f"-I{CSRC}", "-c", os.path.join(CSRC, "acq_noalloc.cu"), "-o", na_obj]
    corr_cmd = [nvcc, "-std=c++17", *ARCH, "-lineinfo", *opt, "-Xcompiler", "-fPIC,-ffp-contract=off",
                f"-I{INCLUDE}", f"-I{CSRC}", "-c", os.path.join(CSRC, "acq_corr.cu"), "-o", corr_obj]
    synth_cmd = [nvcc, "-std=c++17", *ARCH, "-lineinfo", *opt, "-Xcompiler", "-fPIC,-ffp-contract=off",
                 f"-I{INCLUDE}", f"-I{CSRC}", "-c", os.path.join(CSRC, "acq_synth.cu"), "-o", synth_obj]
    if ptxas_verbose:
        dev_cmd.insert(1, "-Xptxas=-v")
        corr_cmd.insert(1, "-Xptxas=-v")
    inst_cmds = [[nvcc, "-std=c++17", *ARCH, "-lineinfo", *opt, "-Xcompiler", "-fPIC,-ffp-contract=off",
                  f"-I{INCLUDE}", f"-I{CSRC}", "-c", os.path.join(CSRC, f"{n}.cu"), "-o", o]
                 for n, o in zip(inst, inst_objs)]
    if ptxas_verbose:
        for c in inst_cmds:
            c.insert(1, "-Xptxas=-v")
    cmds = [host_cmd, dev_cmd, na_cmd, corr_cmd, synth_cmd, *inst_cmds]
    with ThreadPoolExecutor(len(cmds)) as ex:
        outs = list(ex.map(_run, cmds))
    link_cmd = [nvcc, "-shared", *ARCH, host_obj, dev_obj, na_obj, corr_obj, synth_obj, *inst_objs, "-o", lib + ".tmp", "-lcudart_static", "-lrt", "-ldl",
                "-lpthread"]
    outs.append(_run(link_cmd))
    os.replace(lib + ".tmp", lib)
    log = "".join(outs)
    if verbose:
        print(log)
    return log


if __name__ == "__main__":
    checked = "--bounds-check" in sys.argv
    print(build(verbose=False, debug="--debug" in sys.argv, ptxas_verbose="-v" in sys.argv, bounds_check=checked))
    print("built", CHECKED_LIB if checked else LIB)
