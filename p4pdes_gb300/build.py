"""Build libfishgpu.so (sm_103a), the C `fish` driver and the CPU oracle, in-tree.

    python -m p4pdes_gb300.build        # or: import p4pdes_gb300.build as b; b.build()

Outputs (all git-ignored): p4pdes_gb300/lib/libfishgpu.so,
p4pdes_gb300/bin/fish, p4pdes_gb300/_build/*.o, oracle/_build/*.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
BINDIR = os.path.join(PKG, "bin")
LIB = os.path.join(LIBDIR, "libfishgpu.so")

SOURCES = ["common.cu", "callbacks.cu", "solver.cu", "noalloc.cu", "server.cu", "msurf.cu", "petscbin.cu"]
HEADERS = ["fishgpu_internal.cuh", "kernels.cuh", "common.cuh", "vkernels.cuh", "mg_hooks.cuh", "graph_loop.cuh",
           "tma.cuh", "vblock.cuh", "bitconv.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), p.stdout))
    if verbose and p.stdout.strip():
        print(p.stdout)
    return p.stdout


def build_library(verbose=False, extra_flags=()):
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "fishgpu.h")]
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE,
                    "--expt-relaxed-constexpr"] + list(extra_flags)
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + hdrs + [__file__]):
            jobs.append([nvcc] + flags + ["-c", s, "-o", o])
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for f in [ex.submit(_run, j, verbose) for j in jobs]:
                f.result()
    if _stale(LIB, objs):
        cudalib = os.path.join(_cuda_home(nvcc), "lib64")
        _run([nvcc] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB] + objs +
             ["-Xlinker", "-rpath", "-Xlinker", cudalib], verbose)
    return LIB


def build_driver(verbose=False):
    """The C drivers: fish, minimal and bratu2D, with the reference programs' flags."""
    os.makedirs(BINDIR, exist_ok=True)
    exes = []
    for name in ("fish", "minimal", "bratu2D", "obstacle"):
        src = os.path.join(PKG, "host", name + ".c")
        exe = os.path.join(BINDIR, name)
        if _stale(exe, [src, LIB, os.path.join(INCLUDE, "fishgpu.h")]):
            cc = os.environ.get("CC", "gcc")
            _run([cc, "-O2", "-std=c99", "-Wall", "-I", INCLUDE, src, "-o", exe, "-L", LIBDIR,
                  "-lfishgpu", "-Wl,-rpath," + LIBDIR, "-lm"], verbose)
        exes.append(exe)
    return exes[0]


def build_oracle(verbose=False):
    """The CPU oracle (test infrastructure) is built by its own Makefile."""
    _run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], verbose)
    return os.path.join(ROOT, "oracle", "_build", "liboracle.so")


def build(verbose=False):
    build_library(verbose)
    build_driver(verbose)
    build_oracle(verbose)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
