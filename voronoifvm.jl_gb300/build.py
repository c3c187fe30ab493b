"""Build the CUDA library ``_build/libvfvm_gb300.so`` in-tree with nvcc for sm_103a.

Every ``csrc/*.cu`` file is compiled to an object in parallel, then linked into
one shared library exporting the C ABI declared in ``include/vfvm_gb300.h``.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libvfvm_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall", "-Xcompiler", "-Wno-unknown-pragmas",
              "-Xcompiler", "-Wno-unused-function", "--expt-relaxed-constexpr"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvfvm_gb300.so")


# The persistent engine's kernels are instantiated once per registered physics
# and precision from one source (vfvm_persist_inst.cu), each pair into its own
# object, so these heavy instantiations compile in parallel.
INST_SOURCE = "vfvm_persist_inst.cu"
INST_PHYSICS = ["PhysEx105", "PhysEx106", "PhysEx110", "PhysEx160", "PhysEx207", "PhysEx301", "PhysEx440",
                "PhysLaplaceDir", "PhysNLPoisson", "PhysPorous", "PhysBipolar", "PhysRD2", "PhysKappaExp",
                "PhysSurfaceHeat", "PhysBoundarySpecies", "PhysEdgeReaction", "PhysJouleHeat",
                "PhysEx161", "PhysTestFunction", "PhysEx430", "PhysOutflow",
                "PhysEx210", "PhysEx102", "PhysEx107", "PhysEx115", "PhysEx215", "PhysEx220",
                "PhysEx203"]


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu") and f != INST_SOURCE)


def _units():
    """(source, object, extra flags) for every object of the library."""
    units = [(s, os.path.join(BUILD, os.path.basename(s)[:-3] + ".o"), []) for s in sources()]
    inst = os.path.join(CSRC, INST_SOURCE)
    for ph in INST_PHYSICS:
        for kt in ("double", "float"):
            units.append((inst, os.path.join(BUILD, f"vfvm_persist_inst_{ph}_{kt}.o"),
                          [f"-DVFVM_INST_PHYS=vfvm::{ph}", f"-DVFVM_INST_KT={kt}"]))
    return units


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(os.path.dirname(HERE), "include", "vfvm_gb300.h"))
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_library(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    """Compile (if needed) and return the path of the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    units = _units()
    objs = [o for _, o, _ in units]
    jobs = []
    for s, o, flags in units:
        if force or _stale(o, [s] + hdrs):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, *flags, *extra_flags, "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return cmd[-1]

    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose=True))
