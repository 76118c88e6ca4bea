"""Build libsbpgpu.so (CUDA kernels + C ABI) for sm_103a, in tree.

    python hpc-reading-course_gb300/build.py [--force] [--verbose]

Translation units compile in parallel: one per SBP order for the fused wave
stage kernels, one for the remaining kernels, one for the host runtime.
Outputs: hpc-reading-course_gb300/_build/*.o and hpc-reading-course_gb300/lib/libsbpgpu.so.
"""
from __future__ import annotations

import argparse
import os
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIB_DIR, "libsbpgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -Xptxas -v: ptxas reports each kernel's registers, stack and spills; build() keeps
# the report of every unit beside its object (resource_report() reads them)
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2", "-I", os.path.join(ROOT, "include"),
              "--expt-relaxed-constexpr", "-Xptxas", "-v"] + ARCH


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsbpgpu.so")
    return path


def units():
    """(object file, source, extra flags) for every translation unit."""
    out = []
    for order in (2, 4, 6):
        out.append((f"wave2d_o{order}.o", "wave2d_inst.cu", [f"-DSBP_ORDER={order}"]))
    for order in (2, 4, 6):
        out.append((f"wave_batch_o{order}.o", "wave_batch_inst.cu", [f"-DSBP_ORDER={order}"]))
    out.append(("kernels.o", "kernels.cu", []))
    out.append(("sbp_runtime.o", "sbp_runtime.cpp", ["-x", "cu"]))
    out.append(("noalloc.o", "noalloc.cu", []))
    out.append(("petsc_io.o", "petsc_io.cpp", []))
    out.append(("batch_runtime.o", "batch_runtime.cpp", ["-x", "cu"]))
    out.append(("cnn.o", "cnn.cu", []))
    out.append(("rk45.o", "rk45.cu", []))
    out.append(("wave3d.o", "wave3d.cu", []))
    out.append(("decomp.o", "decomp.cu", []))
    return out


def _sources_mtime() -> float:
    m = 0.0
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            m = max(m, os.path.getmtime(os.path.join(d, f)))
    return max(m, os.path.getmtime(__file__))


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    """Compile and link; returns the path of the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime():
        return LIB
    cc = nvcc()
    flags = NVCC_FLAGS + (extra_flags or [])

    def compile_one(u):
        obj, src, extra = u
        cmd = [cc] + flags + extra + ["-c", os.path.join(CSRC, src), "-o", os.path.join(BUILD, obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode == 0:
            with open(os.path.join(BUILD, obj + ".ptxas.txt"), "w") as f:
                f.write(r.stderr)
        return obj, r

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        results = list(ex.map(compile_one, units()))
    failed = [(o, r) for o, r in results if r.returncode != 0]
    for o, r in results:
        if verbose or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
    if failed:
        raise RuntimeError("nvcc failed for: " + ", ".join(o for o, _ in failed))
    objs = [os.path.join(BUILD, o) for o, _, _ in units()]
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("link of libsbpgpu.so failed")
    os.replace(tmp, LIB)
    return LIB


def resource_report() -> dict[str, dict[str, int]]:
    """Per kernel (mangled name) its registers, stack frame and spill bytes, from the ptxas
    reports the last build kept for every translation unit."""
    out: dict[str, dict[str, int]] = {}
    for obj, _, _ in units():
        path = os.path.join(BUILD, obj + ".ptxas.txt")
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path}: no ptxas report (rebuild with build(force=True))")
        cur = None
        with open(path) as f:
            for line in f:
                m = re.search(r"Compiling entry function '(\S+)'", line)
                if m:
                    cur = out.setdefault(m.group(1), {"registers": 0, "stack": 0, "spill_stores": 0, "spill_loads": 0})
                    continue
                if cur is None:
                    continue
                m = re.search(r"(\d+) bytes stack frame, (\d+) bytes spill stores, (\d+) bytes spill loads", line)
                if m:
                    cur["stack"], cur["spill_stores"], cur["spill_loads"] = map(int, m.groups())
                m = re.search(r"Used (\d+) registers", line)
                if m:
                    cur["registers"] = int(m.group(1))
                    cur = None
    return out


DRIVER = os.path.join(LIB_DIR, "sbp_demo")


def build_driver(force: bool = False) -> str:
    """The demo driver (drivers/sbp_demo.cpp): plain C++ against include/sbpgpu.h, linked to the
    library beside it (rpath $ORIGIN). Returns its path."""
    lib = build()
    src = os.path.join(PKG, "drivers", "sbp_demo.cpp")
    if not force and os.path.exists(DRIVER) and os.path.getmtime(DRIVER) >= max(os.path.getmtime(src),
                                                                                  os.path.getmtime(lib)):
        return DRIVER
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), src, "-o", DRIVER + ".tmp",
           "-L", LIB_DIR, "-lsbpgpu", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("build of sbp_demo failed")
    os.replace(DRIVER + ".tmp", DRIVER)
    return DRIVER


PETSC_LIB = os.path.join(LIB_DIR, "libsbpgpu_petsc.so")


def petsc_include_dirs() -> list[str] | None:
    """PETSc's include directories from $PETSC_DIR (and $PETSC_ARCH), or None when its headers
    are not there."""
    base = os.environ.get("PETSC_DIR")
    if not base:
        return None
    dirs = [os.path.join(base, "include")]
    arch = os.environ.get("PETSC_ARCH")
    if arch:
        dirs.append(os.path.join(base, arch, "include"))
    return dirs if os.path.exists(os.path.join(dirs[0], "petscts.h")) else None


def build_petsc_adapter(force: bool = False) -> str | None:
    """libsbpgpu_petsc.so (petsc/sbp_petsc.cpp, include/sbp_petsc.h): the TSSetRHSFunction
    callback and ts_rk4 / ts_rk45 drop-ins over libsbpgpu, built where PETSc's headers are
    found ($PETSC_DIR[/$PETSC_ARCH]). Returns its path, or None without PETSc."""
    inc = petsc_include_dirs()
    if inc is None:
        return None
    lib = build()
    src = os.path.join(PKG, "petsc", "sbp_petsc.cpp")
    if not force and os.path.exists(PETSC_LIB) and os.path.getmtime(PETSC_LIB) >= max(os.path.getmtime(src),
                                                                                       os.path.getmtime(lib)):
        return PETSC_LIB
    base, arch = os.environ["PETSC_DIR"], os.environ.get("PETSC_ARCH", "")
    cmd = (["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include")] +
           [a for d in inc for a in ("-I", d)] +
           [src, "-o", PETSC_LIB + ".tmp", "-L", LIB_DIR, "-lsbpgpu", "-Wl,-rpath,$ORIGIN",
            "-L", os.path.join(base, arch, "lib"), "-lpetsc"])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("build of libsbpgpu_petsc failed")
    os.replace(PETSC_LIB + ".tmp", PETSC_LIB)
    return PETSC_LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose))
