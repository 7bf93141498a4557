"""Build recipe of the CUDA library (sm_103a only).

``build_library()`` compiles ``csrc/*.cu`` and ``csrc/*.cpp`` with nvcc into
``_lib/libswgpu.so`` (in-tree), one translation unit per process, in
parallel.  ``build_cpp_programs()`` builds the C++ drop-in programs under
``tests/cpp`` against the C++ class layer in ``cxx/``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libswgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def nvcc() -> str:
    p = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required")
    return p


def _flags(extra=()):
    return (ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                    "-Xcompiler", "-O3", "--expt-relaxed-constexpr"]
            + list(extra))


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp")))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> str:
    srcs = _sources()
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(
        (".h", ".cuh"))] + [os.path.join(ROOT, "include", "swgpu.h")]
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    if not force and not _stale(LIB, srcs + hdrs):
        return LIB

    def compile_one(src):
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        if force or _stale(obj, [src] + hdrs):
            cmd = [nvcc()] + _flags() + ["-c", src, "-o", obj]
            if src.endswith(".cpp"):
                cmd[1:1] = ["-x", "cu"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
            if verbose and r.stderr:
                print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    cmd = ([nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB]
           + objs + ["-Xlinker", f"-rpath,{CUDA_HOME}/lib64"])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB


def build_cpp_programs(force: bool = False) -> list:
    """Build tests/cpp/*.cu (C++ drop-in programs) linked to libswgpu.so."""
    lib = build_library()
    src_dir = os.path.join(ROOT, "tests", "cpp")
    if not os.path.isdir(src_dir):
        return []
    out_dir = os.path.join(LIBDIR, "bin")
    os.makedirs(out_dir, exist_ok=True)
    hdrs = [os.path.join(PKG, "cxx", f) for f in os.listdir(
        os.path.join(PKG, "cxx"))] + [os.path.join(ROOT, "include", "swgpu.h")]
    srcs = sorted(f for f in os.listdir(src_dir) if f.endswith(".cu"))

    def one(f):
        exe = os.path.join(out_dir, f[:-3])
        src = os.path.join(src_dir, f)
        if force or _stale(exe, [src, lib] + hdrs):
            cmd = ([nvcc()] + _flags() + ["-I", os.path.join(ROOT, "include"),
                                          "-I", os.path.join(PKG, "cxx"),
                                          "-o", exe, src, "-L", LIBDIR,
                                          "-lswgpu", "-cudart", "shared",
                                          "-Xlinker", f"-rpath,{LIBDIR}",
                                          "-Xlinker",
                                          f"-rpath,{CUDA_HOME}/lib64"])
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        return exe

    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(srcs)))) as ex:
        return list(ex.map(one, srcs))


if __name__ == "__main__":
    print(build_library(force=True, verbose=True))
