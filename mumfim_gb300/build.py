"""Builds libmumfim_gpu.so in-tree (mumfim_gb300/_lib/) for sm_103a, and
libmumfim_netgen.so, the seeded synthetic-network generator of the tests and
benchmarks (host code only, kept out of the solver library).

Every translation unit is compiled in parallel; the CUDA ones with
``-gencode arch=compute_103a,code=sm_103a``. Host code and the bit-exact FP64
kernels are compiled without floating-point contraction (``-ffp-contract=off``
for g++, ``--fmad=false`` for nvcc) so their results do not depend on the
compiler's choice of fused multiply-adds; the mixed-precision kernel keeps
FMA on. cudart is linked statically, so the library loads on machines
without a GPU driver (the C ABI then reports MFG_E_NO_DEVICE).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(REPO, "include")
OUT_DIR = os.path.join(PKG, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB_NAME = "libmumfim_gpu.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)
NETGEN_PATH = os.path.join(OUT_DIR, "libmumfim_netgen.so")
NETGEN_SRC = os.path.join(CSRC, "netgen.cpp")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, kind, extra flags)
SOURCES = [
    ("mfg_host.cpp", "cxx", []),
    ("mfg_metrics.cpp", "cxx", []),
    ("mfg_coupling.cpp", "cxx", []),
    ("mfg_mixed_order.cpp", "cxx", []),
    ("mfg_relax_f64.cu", "cuda", ["--fmad=false"]),
    ("mfg_aux.cu", "cuda", ["--fmad=false"]),
    ("mfg_relax_mixed.cu", "cuda", []),
]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _headers() -> list[str]:
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def _compile(src: str, kind: str, extra: list[str], cuda: str, newest_header: float) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ_DIR, src + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(path), newest_header,
                                                             os.path.getmtime(__file__)):
        return obj
    inc = ["-I" + INCLUDE, "-I" + CSRC, "-I" + os.path.join(cuda, "include")]
    if kind == "cxx":
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
               "-Wno-unused-function", *inc, *extra, "-c", path, "-o", obj]
    else:
        cmd = [os.path.join(cuda, "bin", "nvcc"), *ARCH, "-O3", "-lineinfo", "-std=c++17",
               "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-v",
               *inc, *extra, "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {src} failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if kind == "cuda":
        with open(obj + ".ptxas.txt", "w") as fh:
            fh.write(r.stderr)
    return obj


def build_netgen(out_path: str = NETGEN_PATH, force: bool = False) -> str:
    """Compiles the network generator (netgen.cpp, IEEE +-*/ only, no
    contraction: the same networks on every platform) into its own shared
    library at out_path; returns the path."""
    deps = [NETGEN_SRC, os.path.join(INCLUDE, "mumfim_netgen.h"), __file__]
    if (not force and os.path.exists(out_path)
            and os.path.getmtime(out_path) >= max(os.path.getmtime(d) for d in deps)):
        return out_path
    os.makedirs(os.path.dirname(out_path), exist_ok=True)
    tmp = out_path + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-Wall",
           "-I" + INCLUDE, NETGEN_SRC, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling netgen.cpp failed:\n{' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, out_path)
    return out_path


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles (incrementally) and links the library and the network
    generator; returns the library's path."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    cuda = _cuda_home()
    newest = max(os.path.getmtime(h) for h in _headers())
    if force:
        for f in os.listdir(OBJ_DIR):
            os.remove(os.path.join(OBJ_DIR, f))
    with ThreadPoolExecutor(max_workers=len(SOURCES) + 1) as ex:
        ng = ex.submit(build_netgen, NETGEN_PATH, force)
        objs = list(ex.map(lambda s: _compile(s[0], s[1], s[2], cuda, newest), SOURCES))
        ng.result()
    if (not os.path.exists(LIB_PATH)
            or os.path.getmtime(LIB_PATH) < max(os.path.getmtime(o) for o in objs)):
        tmp = LIB_PATH + ".tmp"
        cmd = [os.path.join(cuda, "bin", "nvcc"), *ARCH, "-shared", "-cudart", "static",
               "-Xlinker", "--no-undefined", *objs, "-o", tmp, "-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"linking failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB_PATH)
    if verbose:
        print(LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
