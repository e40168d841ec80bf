"""Per-field error of the plain FP32 and the mixed form against the FP64
oracle, at chosen step counts, from the same initial state, beside the error
of the FP32 oracle (the same formulas restated in single precision on the
CPU) and of the reference build (the reference's own CUDA kernels, Release
build with fast math and a build without) on the same input.

    python tests/accuracy_report.py --case fsi_4m_jitter --steps 1,200,1000 \
        --json out/accuracy.json

Errors per field (fluid and solid), with d = gpu - fp64:
  max_rel = |d|_inf / |fp64|_inf            (the normalised max error of the tests)
  rms_rel = rms(d) / rms(fp64)
and for positions also max|d| and rms|d| in particle diameters.
Runs on one GPU; the oracle uses every host core.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from fluidsim_gb300 import api, cases  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from oracle import refbuild  # noqa: E402

FIELDS = ("fluid_pos", "fluid_vel", "fluid_rho", "fluid_p", "solid_pos", "solid_vel", "solid_PK1")


def field_errors(got, want, dx):
    g = np.asarray(got, np.float64)
    w = np.asarray(want, np.float64)
    d = g - w
    out = {"max_rel": float(np.abs(d).max() / max(np.abs(w).max(), 1e-30)),
           "rms_rel": float(np.sqrt((d * d).mean()) / max(np.sqrt((w * w).mean()), 1e-30))}
    if dx:
        n = np.sqrt((d.reshape(len(d), -1) ** 2).sum(1))
        out["max_dx"] = float(n.max() / dx)
        out["rms_dx"] = float(np.sqrt((n * n).mean()) / dx)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="fsi_4m_jitter")
    ap.add_argument("--steps", default="1,200,1000")
    ap.add_argument("--json", default=None)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--no-fp32-oracle", action="store_true")
    ap.add_argument("--no-reference-build", action="store_true")
    args = ap.parse_args()
    checkpoints = [int(x) for x in args.steps.split(",")]
    make = getattr(cases, args.case)
    cfg_p, pa = cases.make(make(precision=api.PRECISION_FP32))
    cfg_m = api.Config.from_buffer_copy(cfg_p)
    cfg_m.precision = api.PRECISION_MIXED
    dx = float(cfg_p.particle_diameter)
    plain = api.Simulation(cfg_p, pa, device=0)
    mixed = api.Simulation(cfg_m, pa, device=0)
    threads = args.threads or (os.cpu_count() or 1)
    ref = orc.OracleSim(cfg_p, pa, "f64", threads=threads)
    others = {}  # further columns: name -> object with step(n) / get(field)
    if not args.no_fp32_oracle:
        others["fp32_oracle"] = orc.OracleSim(cfg_p, pa, "f32", threads=threads)
    if not args.no_reference_build:
        for variant in ("release", "precise"):
            if refbuild.available(variant):
                others["ref_" + variant] = refbuild.RefBuildSim(cfg_p, pa, variant)
    report = {"case": args.case, "n_fluid": pa.n_fluid, "n_solid": pa.n_solid, "n_virt": pa.n_virt,
              "host_cores": os.cpu_count(), "checkpoints": {}}
    done = 0
    for c in checkpoints:
        n = c - done
        t0 = time.perf_counter()
        plain.step(n)
        mixed.step(n)
        ref.step(n)
        for o in others.values():
            o.step(n)
        plain.sync()
        mixed.sync()
        done = c
        row = {}
        for f in FIELDS:
            if f.startswith("solid") and pa.n_solid == 0:
                continue
            want = ref.get(f)
            pos = f.endswith("_pos")
            row[f] = {"plain": field_errors(plain.get(f), want, dx if pos else 0.0),
                      "mixed": field_errors(mixed.get(f), want, dx if pos else 0.0)}
            for name, o in others.items():
                row[f][name] = field_errors(o.get(f), want, dx if pos else 0.0)
        # where the largest fluid errors sit: distance of the worst particles to the nearest domain wall
        lo = np.array([cfg_p.xmin, cfg_p.ymin, cfg_p.zmin])
        hi = np.array([cfg_p.xmax, cfg_p.ymax, cfg_p.zmax])
        pos = ref.get("fluid_pos")
        wall = np.minimum(pos - lo, hi - pos).min(1) / dx
        for f in ("fluid_vel", "fluid_p"):
            want = ref.get(f)
            for form, sim in (("plain", plain), ("mixed", mixed)):
                d = np.abs(np.asarray(sim.get(f), np.float64) - want)
                d = d.reshape(len(d), -1).max(1)
                top = np.argsort(d)[-5:][::-1]
                row[f][form]["worst_wall_dist_dx"] = [float(wall[k]) for k in top]
                row[f][form]["share_of_max_err_within_3dx_of_wall"] = float(
                    (d[wall < 3.0] > 0.5 * d.max()).sum() / max(1, (d > 0.5 * d.max()).sum()))
        report["checkpoints"][str(c)] = row
        print("step %d (%.0f s)" % (c, time.perf_counter() - t0), flush=True)
        for f, e in row.items():
            extra = "".join(" | %s max %.3g rms %.3g" % (k, e[k]["max_rel"], e[k]["rms_rel"]) for k in others)
            print("  %-10s plain max %.3g rms %.3g | mixed max %.3g rms %.3g%s %s" % (
                f, e["plain"]["max_rel"], e["plain"]["rms_rel"], e["mixed"]["max_rel"], e["mixed"]["rms_rel"],
                extra, e["mixed"].get("worst_wall_dist_dx", "")), flush=True)
        if args.json:
            with open(args.json, "w") as fh:
                json.dump(report, fh, indent=1)
    plain.close()
    mixed.close()
    for o in others.values():
        o.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
