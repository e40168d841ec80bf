"""In-tree build of the native library ``_build/libfluidsim.so`` (sm_103a) and
the ``_build/fluidsim`` command-line driver.

The CUDA translation unit is compiled with nvcc for ``compute_103a/sm_103a``
only; host C++ translation units with g++ (``-ffp-contract=off`` so that the
FP32 parameter derivation rounds like the reference host code on both x86 and
Arm).  Units compile in parallel; nothing is rebuilt when up to date.
"""
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(BUILD, "libfluidsim.so")
CLI = os.path.join(BUILD, "fluidsim")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_UNITS = ["fsim_kernels.cu", "fsim_sim.cu", "fsim_noalloc.cu", "fsim_probe.cu"]
HOST_UNITS = ["fsim_host.cpp"]
HEADERS = ["fsim_internal.h", "fsim_types.h"]
# FSIM_DEVICE_CHECKS=1 in the environment compiles the kernels' index checks
# in (a debugging build; see FSIM_DCHECK in fsim_kernels.cu)
DEBUG_FLAGS = ["-DFSIM_DEVICE_CHECKS"] if os.environ.get("FSIM_DEVICE_CHECKS") == "1" else []


def _deps():
    deps = [os.path.join(CSRC, f) for f in HEADERS]
    deps.append(os.path.join(INCLUDE, "fluidsim.h"))
    deps.append(os.path.abspath(__file__))
    return deps


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _run_parallel(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in cmds]
    errors = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append("$ %s\n%s" % (" ".join(c), out.decode(errors="replace")))
    if errors:
        raise RuntimeError("native build failed:\n" + "\n".join(errors))


def build(force=False, verbose=False):
    """Compile libfluidsim.so and the CLI; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    deps = _deps()
    objs, cmds = [], []
    for u in CUDA_UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + deps):
            cmds.append([NVCC] + ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                                         "-Xptxas", "-v" if verbose else "-O3"] + DEBUG_FLAGS +
                        ["-I", INCLUDE, "-c", src, "-o", obj])
    for u in HOST_UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + deps):
            cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                         "-I", INCLUDE, "-c", src, "-o", obj])
    if cmds:
        _run_parallel(cmds)
    if force or _stale(LIB, objs):
        _run_parallel([[NVCC] + ARCH + ["-shared", "-o", LIB] + objs])
    cli_src = os.path.join(CSRC, "fsim_cli.cpp")
    if os.path.exists(cli_src) and (force or _stale(CLI, [cli_src, LIB] + deps)):
        _run_parallel([["g++", "-O2", "-std=c++17", "-I", INCLUDE, cli_src, "-o", CLI, "-L", BUILD,
                        "-lfluidsim", "-Wl,-rpath,$ORIGIN"]])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
