"""Regenerate the golden fixtures of tests/golden/ from the reference itself.

Runs oracle/_ref/ref_params — the reference's own host sources
(src/config.cpp, src/kernel.cpp, src/properties.cpp, src/domain.cpp,
src/physics.cpp, src/sim_time.cpp) compiled unmodified by oracle/build.py — on
every INI file in tests/golden/ini/ and records what the reference reads and
derives (raw values, FP32 kernel/EOS/material constants, the cell grid and the
reader's error flag) in params_<name>.json.  It also runs the reference's
particle-count readers ({Fluid,Solid,Virtual}Properties::readNumber) on small
.dat sets and records the counts and the mismatch flag in counts_<name>.json.

Needs the reference checkout (this container only):  python tests/golden/make_golden.py
"""
import glob
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build as oracle_build  # noqa: E402


def run_ref(ini, prefix=None):
    cmd = [oracle_build.ref_params_path(), ini] + ([prefix] if prefix else [])
    text = subprocess.check_output(cmd, text=True)
    # the reference readers print their own diagnostics before the JSON
    brace = text.index("{")
    out = json.loads(text[brace:])
    out["messages"] = [m for m in text[:brace].splitlines() if m.strip()]
    return out


# .dat sets for the count reader: (name, {file: text})
DAT_SETS = {
    "ok": {
        "fluid_particle.dat": "2\n0.1 0.2 0.3 0 0 0 1000 0\n0.4 0.5 0.6 0 0 0 1000 0\n",
        "solid_particle.dat": "1\n0.5 0.5 0.5 0 0 0 0.5 0.5 0.5 0\n",
        "virt_particle.dat": "3\n-0.01 0 0 0\n-0.02 0 0 0\n-0.03 0 0 0\n",
    },
    "mismatch": {
        "fluid_particle.dat": "3\n0.1 0.2 0.3 0 0 0 1000 0\n0.4 0.5 0.6 0 0 0 1000 0\n",
        "solid_particle.dat": "0\n",
        "virt_particle.dat": "1\n-0.01 0 0 0\n",
    },
    "empty_solid": {
        "fluid_particle.dat": "1\n0.1 0.2 0.3 0 0 0 1000 0\n",
        "solid_particle.dat": "0\n",
        "virt_particle.dat": "0\n",
    },
}


def main():
    if not oracle_build.build_ref():
        sys.exit("reference checkout not found; cannot regenerate golden fixtures")
    for ini in sorted(glob.glob(os.path.join(HERE, "ini", "*.ini"))):
        name = os.path.splitext(os.path.basename(ini))[0]
        out = run_ref(ini)
        with open(os.path.join(HERE, "params_%s.json" % name), "w") as f:
            json.dump(out, f, indent=1, sort_keys=True)
        print("params", name, "read_error=%d" % out.get("read_error", -1))
    ini = os.path.join(HERE, "ini", "small_dam_break.ini")
    for name, files in DAT_SETS.items():
        with tempfile.TemporaryDirectory() as tmp:
            # the reference opens <prefix>\<file> (a backslash path); on Linux that
            # backslash is part of the file name
            prefix = os.path.join(tmp, "data")
            for fn, text in files.items():
                with open(prefix + "\\" + fn, "w") as f:
                    f.write(text)
            out = run_ref(ini, prefix)
        rec = {"files": files, "count_error": out["count_error"], "n_fluid": out["n_fluid"],
               "n_solid": out["n_solid"], "n_virt": out["n_virt"]}
        with open(os.path.join(HERE, "counts_%s.json" % name), "w") as f:
            json.dump(rec, f, indent=1, sort_keys=True)
        print("counts", name, rec["count_error"], rec["n_fluid"], rec["n_solid"], rec["n_virt"])


if __name__ == "__main__":
    main()
