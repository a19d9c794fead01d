"""Builds the CUDA extension libbirp_gb300.so in-tree (sm_103a only).

Every translation unit is compiled in parallel with nvcc (host code with
-ffp-contract=off so the FP64 camera frame gives the same bits as the
oracle's on every host), then linked into birp_cpp_gb300/lib/.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libbirp_gb300.so")
CLASSES_LIB = os.path.join(LIBDIR, "libbirp_classes.so")
CPP = os.path.join(HERE, "cpp")
ABI_INCLUDE = os.path.normpath(os.path.join(HERE, "..", "include"))  # include/birp_gb300.h, the C ABI

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["render.cu", "capi.cu", "cube.cu", "batch.cu", "server.cu", "noalloc.cu", "cmem_host.cpp", "tune.cpp"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
                   "-I", os.path.join(HERE, "..", "include")]


def _compile(src: str) -> str:
    out = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".inc"))]
    deps.append(os.path.join(HERE, "..", "include", "birp_gb300.h"))
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    lang = [] if src.endswith(".cu") else ["-x", "cu"]
    cmd = [nvcc()] + _flags() + lang + ["-c", path, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return out


def build(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    build_classes()
    build_cli()
    if verbose:
        print("built", LIB, CLASSES_LIB, "and", CLI)
    return LIB


CLI = os.path.join(LIBDIR, "birp")
DEBUG_LIB = os.path.join(LIBDIR, "libbirp_gb300_debug.so")


def build_debug_bounds() -> str:
    """The bounds-checking library lib/libbirp_gb300_debug.so: render.cu with
    BIRP_DEBUG_BOUNDS (every table access of the kernels checked, the first
    violation recorded for birp_debug_bounds), the other units as built."""
    build()
    out = os.path.join(OBJ, "render_debug_bounds.o")
    src = os.path.join(CSRC, "render.cu")
    cmd = [nvcc()] + _flags() + ["-DBIRP_DEBUG_BOUNDS", "-c", src, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    objs = [out] + [os.path.join(OBJ, os.path.splitext(s)[0] + ".o") for s in SOURCES if s != "render.cu"]
    cmd = [nvcc()] + ARCH + ["-shared", "-o", DEBUG_LIB] + objs + ["-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return DEBUG_LIB


def build_variant(defines: dict, tag: str) -> str:
    """lib/libbirp_gb300_<tag>.so: render.cu compiled with the given macro
    definitions (the autotuner's candidates), the other units as built."""
    build()
    out = os.path.join(OBJ, f"render_{tag}.o")
    src = os.path.join(CSRC, "render.cu")
    cmd = [nvcc()] + _flags() + [f"-D{k}={v}" for k, v in defines.items()] + ["-c", src, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    lib = os.path.join(LIBDIR, f"libbirp_gb300_{tag}.so")
    objs = [out] + [os.path.join(OBJ, os.path.splitext(s)[0] + ".o") for s in SOURCES if s != "render.cu"]
    r = subprocess.run([nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lpthread"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    return lib


def build_cli() -> str:
    """The command-line front-end (cli/birp.cpp) over the classes: lib/birp."""
    src = os.path.join(HERE, "cli", "birp.cpp")
    deps = [src, CLASSES_LIB] + [os.path.join(CPP, "include", "birp", h)
                                 for h in os.listdir(os.path.join(CPP, "include", "birp"))]
    if os.path.exists(CLI) and all(os.path.getmtime(CLI) >= os.path.getmtime(d) for d in deps):
        return CLI
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", src, "-I", os.path.join(CPP, "include"), "-I", ABI_INCLUDE, "-L", LIBDIR,
           "-lbirp_classes", "-lbirp_gb300", "-lpthread", "-Wl,-rpath,$ORIGIN", "-o", CLI]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CLI build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return CLI


def build_classes() -> str:
    """The reference-API C++ classes (cpp/) over the C ABI: libbirp_classes.so."""
    srcs = [os.path.join(CPP, "src", f) for f in ("classes.cpp", "helper.cpp")]
    deps = srcs + [LIB, os.path.join(ABI_INCLUDE, "birp_gb300.h")] + [os.path.join(CPP, "include", "birp", h)
                           for h in os.listdir(os.path.join(CPP, "include", "birp"))]
    if os.path.exists(CLASSES_LIB) and all(os.path.getmtime(CLASSES_LIB) >= os.path.getmtime(d) for d in deps):
        return CLASSES_LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall", *srcs, "-I", os.path.join(CPP, "include"),
           "-I", ABI_INCLUDE,
           "-L", LIBDIR, "-lbirp_gb300", "-Wl,-rpath,$ORIGIN", "-o", CLASSES_LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"classes build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return CLASSES_LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
