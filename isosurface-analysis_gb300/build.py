"""Builds libisosim.so (the engine's CUDA kernels and C ABI) for sm_103a.

Usage: python build.py [--force]

Each translation unit is compiled by its own nvcc process in parallel, then
linked into lib/libisosim.so.  Objects are rebuilt when the source, a header or
this file is newer than the object.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_obj")
LIB = os.path.join(HERE, "lib")
TARGET = os.path.join(LIB, "libisosim.so")
HOST = os.path.join(HERE, "host")
CLI = os.path.join(HERE, "bin", "isosim")
HOST_SOURCES = ["main.cpp", "modules.cpp"]

SOURCES = [
    "iso_context.cu",
    "iso_surface.cu",
    "iso_distance.cu",
    "iso_distance_tc.cu",
    "iso_histogram.cu",
    "iso_mi_ref32.cu",
    "iso_pipeline.cu",
    "iso_server.cu",
    "iso_multi.cu",
    "iso_reps.cpp",
    "iso_tune.cpp",
]
HEADERS = [os.path.join(CSRC, "iso_internal.cuh"), os.path.join(CSRC, "iso_tc.cuh"),
           os.path.join(ROOT, "include", "isosim.h")]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = [
    "-std=c++17", "-O3", "-lineinfo",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden", "-Xcompiler", "-ffp-contract=off",
    # exact IEEE arithmetic everywhere: no implicit FMA contraction, IEEE
    # division and square root, denormals preserved
    "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-I", os.path.join(ROOT, "include"), "-I", CSRC,
]


# Files compiled with nvcc's default multiply-add contraction instead of
# -fmad=false: the reference-order FP32 MI must fuse exactly where the
# reference's kernel does (its build passes no -fmad flag).
DEFAULT_CONTRACTION = {"iso_mi_ref32.cu"}


def flags_for(src):
    if src in DEFAULT_CONTRACTION:
        return [f for f in COMMON if f not in ("-fmad=false",)]
    return COMMON


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(src, obj):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src, os.path.abspath(__file__)] + HEADERS
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src, force):
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ, src + ".o")
    if not force and not _stale(path, obj):
        return obj, None
    cmd = [nvcc()] + flags_for(src) + ARCH + ["-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "cu"] + flags_for(src) + ARCH + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, "compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr)
    return obj, None


def build(force=False, verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, force), SOURCES))
    errors = [e for _, e in results if e]
    if errors:
        raise RuntimeError("\n".join(errors))
    objs = [o for o, _ in results]
    if force or not os.path.exists(TARGET) or any(os.path.getmtime(o) > os.path.getmtime(TARGET) for o in objs):
        cmd = [nvcc(), "-shared"] + ARCH + ["-Xcompiler", "-fPIC", "-o", TARGET] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    build_cli(force)
    if verbose:
        print("built", TARGET, "and", CLI)
    return TARGET


def build_cli(force=False):
    """The module CLI (host C++ only, linked against libisosim.so)."""
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    srcs = [os.path.join(HOST, s) for s in HOST_SOURCES]
    deps = srcs + [os.path.join(HOST, h) for h in ("json.hpp", "dao.hpp", "modules.hpp")] + [TARGET]
    if not force and os.path.exists(CLI) and all(os.path.getmtime(d) <= os.path.getmtime(CLI) for d in deps):
        return CLI
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-Wall", "-ffp-contract=off",
           "-I", os.path.join(ROOT, "include"), "-o", CLI] + srcs + \
          ["-L", LIB, "-lisosim", "-Wl,-rpath,$ORIGIN/../lib", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("CLI build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return CLI


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
