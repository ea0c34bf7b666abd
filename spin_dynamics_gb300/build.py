"""Builds libspinchem_gpu.so in-tree (spin_dynamics_gb300/_build/) with nvcc
for sm_103a. Translation units compile in parallel; the shared library links
against the CUDA runtime only.

    python -m spin_dynamics_gb300.build
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libspinchem_gpu.so")
SOURCES = ["spc_propagate.cu", "spc_hamiltonian.cu", "spc_diag.cu", "spc_host.cpp", "spc_api.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code keeps the reference's rounding points (no FMA contraction), so the
# host-side sample generator and Hamiltonian coefficients are bit-identical on
# x86-64 and aarch64.
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libspinchem_gpu")


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "spinchem_gpu.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc(), *ARCH, *COMMON, "-c", path, "-o", obj]
    if src.endswith(".cu") and verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False) -> str:
    """Compile every translation unit and link the shared library; returns its path."""
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if not (os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs)):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    build_cli()
    return LIB


CLI = os.path.join(OUT, "spinchem")
CLI_SRC = os.path.join(CSRC, "spinchem_main.cpp")


def build_cli() -> str:
    """The `spinchem input.ini` drop-in executable, linked against the library."""
    if os.path.exists(CLI) and os.path.getmtime(CLI) >= max(os.path.getmtime(CLI_SRC),
                                                           os.path.getmtime(LIB)):
        return CLI
    cxx = shutil.which(os.environ.get("CXX", "g++")) or "g++"
    # no FMA contraction: the weighted block sums round as the Python driver's
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", CLI_SRC, "-o", CLI, "-L", OUT, "-lspinchem_gpu",
           "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CLI build failed:\n{r.stdout}\n{r.stderr}")
    return CLI


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
