"""Builds liblmm_gb300.so in-tree for sm_103a (GB300).

Each CUDA/C++ translation unit under csrc/ is compiled by its own nvcc
process (in parallel), then linked into one shared library with the CUDA
runtime linked statically, so the library loads with nothing but the driver.
Objects are rebuilt only when a source or header is newer.

  python financial-services-workload-samples_gb300/build_lib.py [--force] [-j N]
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "liblmm_gb300.so")
CLI_SRC = os.path.join(PKG, "cli", "lmm_bench.cpp")
CLI = os.path.join(PKG, "lmm_bench")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblmm_gb300.so")


def common_flags():
    return ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O3", "-I" + INCLUDE, "-I" + CSRC,
            "-Xptxas", "-warn-spills"]


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _compile(src: str, force: bool, extra) -> tuple[str, str]:
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    newest_dep = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in headers()])
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep:
        return obj, ""
    cmd = [nvcc()] + ARCH + common_flags() + list(extra) + ["-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj, (r.stdout + r.stderr).strip()


def build(force: bool = False, jobs: int | None = None, extra=(), verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    srcs = sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, force, extra), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for o, log in results:
            if log:
                print(f"[{os.path.basename(o)}]\n{log}")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    build_cli(force)
    return LIB


SHIM = os.path.join(PKG, "shim", "liborSwaptionGreeks_gb300.cpp")
MKL_STANDIN = os.path.join(PKG, "shim", "include")


def build_dropin(reference_root: str, out_dir: str, double: bool = True) -> str:
    """Links the reference's own driver (LiborMarketModel/main.cpp, unmodified,
    from `reference_root`) with the drop-in shim and this library: the check
    that a user of the reference can switch by replacing two source files.
    Returns the executable's path."""
    lmm_dir = os.path.join(reference_root, "LiborMarketModel")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "liborSwaptionGreeks_gb300" + ("" if double else "_f32"))
    cmd = [shutil.which("g++") or "g++", "-O2", "-std=c++11", "-fopenmp", "-w", "-I" + lmm_dir,
           "-I" + INCLUDE, "-I" + MKL_STANDIN, os.path.join(lmm_dir, "main.cpp"), SHIM,
           "-L" + PKG, "-llmm_gb300", "-Wl,-rpath," + PKG, "-o", exe]
    if double:
        cmd.insert(1, "-DUSE_DOUBLE")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"drop-in build failed:\n{r.stdout}\n{r.stderr}")
    return exe


def build_cli(force: bool = False) -> str:
    """The benchmark driver (cli/lmm_bench.cpp), linked against the library
    beside it (rpath $ORIGIN)."""
    deps = [CLI_SRC, LIB, os.path.join(INCLUDE, "lmm_gb300.h")]
    if force or not os.path.exists(CLI) or os.path.getmtime(CLI) < max(os.path.getmtime(d) for d in deps):
        tmp = CLI + f".tmp{os.getpid()}"
        cmd = [shutil.which("g++") or "g++", "-O2", "-std=c++17", "-Wall", "-Wextra", "-I" + INCLUDE, CLI_SRC,
               "-L" + PKG, "-llmm_gb300", "-Wl,-rpath,$ORIGIN", "-o", tmp]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"lmm_bench build failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, CLI)
    return CLI


if __name__ == "__main__":
    j = None
    if "-j" in sys.argv:
        j = int(sys.argv[sys.argv.index("-j") + 1])
    print(build(force="--force" in sys.argv, jobs=j, verbose="-v" in sys.argv))
