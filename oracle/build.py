"""Build recipe for the oracle (test infrastructure only).

* ``build_oracle()`` compiles oracle.c twice with gcc + OpenMP:
  ``_build/liboracle_f64.so`` (FP64) and ``_build/liboracle_f32.so`` (FP32).
* ``build_ref()`` compiles the reference's own host sources that derive the
  simulation parameters (src/config.cpp, src/kernel.cpp, src/properties.cpp,
  src/domain.cpp, src/physics.cpp, src/sim_time.cpp) unmodified, straight from
  the read-only reference checkout, together with ref_params_main.cpp, into
  ``_ref/ref_params``.  ``-include math.h`` supplies the <cmath> overloads that
  MSVC's headers pull in implicitly (unqualified ``pow(float, float)`` is the
  float overload there), and ``compat/windows.h`` is an empty stand-in for the
  one Windows header src/properties.cpp includes but does not use.
* ``build_refcuda()`` compiles the reference's CUDA kernels (its unmodified
  src/{memory_copy,pair,fluid,virt,solid}.cu, through refcuda/ref_device.cu)
  into loadable sm_103a device images: ``_ref/refcuda_release.fatbin`` with the
  reference's Release flags (CMakeLists.txt:18-22: -O3, -Xptxas -dlcm=cg,
  -use_fast_math) and ``_ref/refcuda_precise.fatbin`` without fast math.  The
  reference does not vendor glm; refcuda/glm/ is a subset written here from
  the mathematical definitions.  ``_ref/ref_layout`` prints the reference's
  struct offsets for the layout test.  Device images carry no host code, so
  the ones built here serve the Arm GPU host too.
* ``build_harness()`` compiles refcuda/ref_harness.cpp (the host program
  around those images) into ``_build/librefharness.so``; it needs no
  reference source and is built on every machine.

The reference checkout is found at ``$FSIM_REFERENCE_ROOT``, else at
``../reference`` beside this repository.  Run ``python oracle/build.py`` or
call the functions.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
REFERENCE_ROOT = os.environ.get("FSIM_REFERENCE_ROOT", os.path.join(os.path.dirname(REPO), "reference"))
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
REFCUDA = os.path.join(HERE, "refcuda")
REF_DEVICE_UNITS = ["memory_copy", "pair", "fluid", "virt", "solid"]
REF_SOURCES = ["config", "kernel", "properties", "domain", "physics", "sim_time"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def oracle_lib_path(precision="f64"):
    return os.path.join(HERE, "_build", "liboracle_%s.so" % precision)


def build_oracle(force=False):
    os.makedirs(os.path.join(HERE, "_build"), exist_ok=True)
    src = os.path.join(HERE, "oracle.c")
    hdr = os.path.join(HERE, "oracle.h")
    procs = []
    for prec, extra in (("f64", []), ("f32", ["-DORACLE_F32"])):
        out = oracle_lib_path(prec)
        if not force and not _stale(out, [src, hdr]):
            continue
        cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
               "-fno-fast-math"] + extra + [src, "-o", out, "-lm"]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("oracle build failed: %s\n%s" % (" ".join(cmd), out.decode()))


def ref_params_path():
    return os.path.join(HERE, "_ref", "ref_params")


def build_ref(force=False):
    """Compile the reference host sources; returns False when the reference
    checkout is absent (as on the GPU machine)."""
    src_dir = os.path.join(REFERENCE_ROOT, "src")
    if not os.path.isdir(src_dir):
        return False
    os.makedirs(os.path.join(HERE, "_ref"), exist_ok=True)
    sources = [os.path.join(src_dir, s + ".cpp") for s in REF_SOURCES]
    sources.append(os.path.join(HERE, "ref_params_main.cpp"))
    out = ref_params_path()
    if not force and not _stale(out, sources):
        return True
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-include", "math.h",
           "-I", os.path.join(HERE, "compat"), "-I", os.path.join(REFERENCE_ROOT, "include")]
    cmd += sources + ["-o", out]
    _run(cmd)
    return True


def refcuda_image_path(variant="release"):
    return os.path.join(HERE, "_ref", "refcuda_%s.fatbin" % variant)


def ref_layout_path():
    return os.path.join(HERE, "_ref", "ref_layout")


def harness_lib_path():
    return os.path.join(HERE, "_build", "librefharness.so")


def _glm_headers():
    out = []
    for base, _, files in os.walk(os.path.join(REFCUDA, "glm")):
        out += [os.path.join(base, f) for f in files]
    return out


def build_refcuda(force=False):
    """Compile the reference's CUDA kernels into device images; returns False
    when the reference checkout is absent (as on the GPU machine, which uses the
    images built here)."""
    src_dir = os.path.join(REFERENCE_ROOT, "src")
    inc_dir = os.path.join(REFERENCE_ROOT, "include")
    if not os.path.isdir(src_dir):
        return False
    os.makedirs(os.path.join(HERE, "_ref"), exist_ok=True)
    unity = os.path.join(REFCUDA, "ref_device.cu")
    deps = [unity] + _glm_headers() + [os.path.join(src_dir, u + ".cu") for u in REF_DEVICE_UNITS]
    deps += [os.path.join(inc_dir, f) for f in os.listdir(inc_dir)]
    common = ["-std=c++17", "-diag-suppress", "427", "-Xcudafe", "--diag_suppress=esa_on_defaulted_function_ignored",
              "-I", REFCUDA, "-I", src_dir, "-I", inc_dir]
    cmds = []
    for variant, flags in (("release", ["-O3", "-Xptxas", "-O3,-dlcm=cg", "-use_fast_math"]),
                           ("precise", ["-O3", "-Xptxas", "-O3,-dlcm=cg"])):
        out = refcuda_image_path(variant)
        if force or _stale(out, deps):
            cmds.append([NVCC] + ARCH + flags + common + ["-fatbin", unity, "-o", out])
    probe = os.path.join(REFCUDA, "layout_probe.cu")
    if force or _stale(ref_layout_path(), deps + [probe]):
        cmds.append([NVCC] + common + [probe, "-o", ref_layout_path()])
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in cmds]
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("reference CUDA build failed: %s\n%s" % (" ".join(c), out.decode()))
    return True


def build_harness(force=False):
    os.makedirs(os.path.join(HERE, "_build"), exist_ok=True)
    src = os.path.join(REFCUDA, "ref_harness.cpp")
    hdr = os.path.join(REPO, "include", "fluidsim.h")
    out = harness_lib_path()
    if force or _stale(out, [src, hdr]):
        _run([NVCC, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-I", os.path.join(REPO, "include"),
              src, "-o", out])
    return out


if __name__ == "__main__":
    f = "--force" in sys.argv
    build_oracle(force=f)
    print("oracle built:", oracle_lib_path("f64"), oracle_lib_path("f32"))
    print("reference host sources built:", build_ref(force=f))
    print("reference CUDA kernels built:", build_refcuda(force=f))
    print("reference build harness:", build_harness(force=f))
