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
  one Windows header src/properties.cpp includes but does not use.  The
  reference's CUDA sources need the unvendored glm library and are not built.

Run ``python oracle/build.py`` or call the functions.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE_ROOT = os.environ.get("FSIM_REFERENCE_ROOT", "/root/reference")
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


if __name__ == "__main__":
    build_oracle(force="--force" in sys.argv)
    print("oracle built:", oracle_lib_path("f64"), oracle_lib_path("f32"))
    print("reference host sources built:", build_ref(force="--force" in sys.argv))
