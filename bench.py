"""Benchmark: particle-updates/s of the FluidSim hot path on the 4M-particle FSI case.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One step = one fluid step of the full hot path (cell sort, fluid-solid coupling,
virtual walls, fused fluid sweep + update, 4 solid sub-steps) over the
``fsi_4m`` workload: 4,194,304 fluid + 27,000 solid + 912,600 wall particles
(dx = 0.005 m, dt = 5e-5 s).  particle-updates/s = (N_fluid + N_solid) * steps
/ time; wall particles are not counted (their cost is included).

* ``value``: device time of K steps (CUDA-graph replays; state resident in
  HBM; the 300+ MB particle state is larger than the 129 MB L2), CUDA events
  on the handle's stream, max over ranks.  The step graphs replayed carry
  event nodes around the fluid sweep, so the same replays time that kernel.
* ``e2e``: the same metric through the C ABI with host buffers, over the 20
  steps right after the timed region: every step copies the fluid and solid
  state in from pinned host memory (fsim_set_fields), advances one step
  (fsim_step) and reads the state back (fsim_get_fields).  ``serial_bound``
  is the rate if the step took its device time (measured just before, from
  the same state) plus the upload and download at the link's measured copy
  rates (``link_*_gbps``, one pinned buffer of the step's bytes each way).
* ``phases_ms_per_step``: per-phase device time, launch by launch with events
  around every launch, over K steps after the e2e run (the dam break has
  developed further by then, so the sum can exceed ``ms_per_step``).
* ``roofline``: the fluid sweep (the dominant kernel) in the timed region
  against the measured HBM bandwidth, with the algorithmic 64 B per fluid
  particle-step; ``roofline_fp32`` against the measured FP32 FMA peak.
* ``cpu_baseline``: the FP64 CPU oracle on this host's cores, 2 steps of the
  same workload; ``single_thread``: one step of it on one thread.
* ``reference_build``: the reference's own CUDA kernels (its unmodified
  src/pair.cu, fluid.cu, virt.cu, solid.cu, compiled for sm_103a with its
  Release flags; oracle/refcuda) on the same workload and GPU, with the
  reference's launch shapes and a synchronisation after every launch.
* ``forms``: the small dam break for its 2000 steps beside the reference build
  (``config0``), the mixed-precision form, the batched 64-instance ensemble and
  the served request stream.

``--impl reference`` times the reference build on the GPU (the reference is a
CUDA program with no CPU path); where its device image is absent it falls back
to the CPU restatement of its algorithm (FP32 oracle, all host threads), which
it also samples for ``cpu_baseline``.  ``--cpu-full`` times the FP64 oracle on
the small dam break for all 2000 steps and on 200 steps of the 4M case, on all
host cores and on one thread (minutes; not part of the default run).
Multi-GPU: replicas only (independent instances, no collective).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ALG_BYTES_FLUID = 64   # per fluid particle-step (pos, vel, rho read+write; cell key write+read)
ALG_BYTES_SOLID = 132  # per solid particle-sub-step
ALG_BYTES_SOLID_STEP = 16
ALG_BYTES_VIRT = 32    # per wall particle-step


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier and max-reduction across replicas (gloo on host tensors)."""

    def __init__(self):
        self.ws, self.rank, self.local = _dist()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as td

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group("gloo", rank=self.rank, world_size=self.ws)
            self.pg = td

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v):
        if not self.pg:
            return v
        import torch

        t = torch.tensor([float(v)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        return summarize_clocks(self.lines)


def summarize_clocks(lines):
    sm, smax, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for ln in lines:
        f = [x.strip() for x in ln.split(",")]
        if len(f) < 9:
            continue
        try:
            sm.append(float(f[1]))
            smax.append(float(f[2]))
        except ValueError:
            continue
        for name, v in zip(names, f[5:9]):
            if v.lower() == "active":
                reasons.add(name)
    if not sm:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
    sm.sort()
    return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(smax), "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def workload(args):
    from fluidsim_gb300 import cases

    cfg, pa = cases.make(cases.fsi_4m())
    return cfg, pa


def workload_desc(cfg, pa):
    return {
        "workload": "fsi_4m: dam break, %d fluid + %d solid (free 30^3 cube) + %d wall particles, dx=0.005 m, "
                    "dt=5e-5 s, %d solid sub-steps, Gaussian kernel h=1.3dx, FP32" %
                    (pa.n_fluid, pa.n_solid, pa.n_virt, cfg.solid_sub_step),
        "n_fluid": pa.n_fluid, "n_solid": pa.n_solid, "n_virt": pa.n_virt,
        "l2": "inputs larger than L2 (particle state > 300 MB vs 129 MB L2); no flush",
    }


def cpu_oracle_rate(cfg, pa, precision, steps, threads=0):
    from oracle import oracle as orc

    o = orc.OracleSim(cfg, pa, precision, threads=threads)
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    o.close()
    return (pa.n_fluid + pa.n_solid) * steps / dt, dt


def reference_build_rate(cfg, pa, steps, warmup, dev=0):
    """The reference's own CUDA kernels (unmodified src/*.cu, Release flags,
    sm_103a; oracle/refcuda) on this GPU through the harness that restates its
    host loop: particle-updates/s over `steps` steps after `warmup`, CUDA
    events on the default stream, a device synchronisation after every launch
    as in the reference.  None when the device image is absent."""
    from oracle import refbuild

    if not refbuild.available("release"):
        return None
    with refbuild.RefBuildSim(cfg, pa, "release", device=dev) as ref:
        ref.step(warmup)
        ms = ref.time_steps(steps)
    return {"value": (pa.n_fluid + pa.n_solid) * steps / (ms * 1e-3), "unit": "particle-updates/s",
            "ms_per_step": ms / steps, "steps": steps, "warmup": warmup, "thread_num": cfg.thread_num,
            "build": "reference CUDA kernels (src/pair.cu, fluid.cu, virt.cu, solid.cu, unmodified) for sm_103a "
                     "with -O3 -Xptxas -dlcm=cg -use_fast_math, glm subset written here; host loop of "
                     "src/calculation.cu:20-35 restated (oracle/refcuda/ref_harness.cpp)"}


def run_reference(args, dist):
    """The reference arm: the reference's own CUDA build on this GPU (its
    kernels are the whole of its hot path; it has no CPU path).  Where the
    device image is absent, the CPU restatement of its algorithm instead."""
    if dist.rank != 0:
        return 0
    cfg, pa = workload(args)
    cores = os.cpu_count() or 1
    desc = workload_desc(cfg, pa)
    # CPU restatement (FP32 oracle, all host threads): a short bounded sample
    warm = 1
    _, tw = cpu_oracle_rate(cfg, pa, "f32", warm, cores)
    cpu_steps = max(1, min(args.steps, int(20.0 / max(tw / warm, 1e-3))))
    cpu_rate, cpu_dt = cpu_oracle_rate(cfg, pa, "f32", cpu_steps, cores)
    cpu = {"value": cpu_rate, "unit": "particle-updates/s", "cores": cores, "kind": "port",
           "sample": "%d fluid steps of the full workload in the FP32 CPU restatement of the reference path "
                     "(OpenMP, all host threads) in %.1f s, after 1 untimed step; at most --steps, about 20 s"
                     % (cpu_steps, cpu_dt)}
    ref = None
    try:
        ref = reference_build_rate(cfg, pa, args.steps, max(args.warmup, 3), dist.local)
    except Exception as e:  # the reference build failing is reported, not hidden
        ref = None
        cpu["reference_build_error"] = str(e)
    if ref is not None:
        line = {
            "impl": "reference", "metric": "particle-updates/s", "value": ref["value"], "unit": "particle-updates/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": ref["warmup"], "ms_per_step": ref["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": desc, "reference_build": ref, "cpu_baseline": cpu,
            "e2e": {"value": ref["value"], "unit": "particle-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "the reference is a CUDA program; its own kernels run here on the GPU, state resident for "
                    "the whole run as in the reference (its loop copies nothing per step); cpu_baseline is the "
                    "CPU restatement of the same path, a separate sample",
        }
    else:
        line = {
            "impl": "reference", "metric": "particle-updates/s", "value": cpu_rate, "unit": "particle-updates/s",
            "n_gpus": args.gpus, "steps": cpu_steps, "warmup": warm, "ms_per_step": cpu_dt * 1e3 / cpu_steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": desc, "cpu_baseline": cpu,
            "e2e": {"value": cpu_rate, "unit": "particle-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "the reference build's device image is absent, so the reference arm is the CPU restatement "
                    "of its algorithm",
        }
    print(json.dumps(line), flush=True)
    return 0


def run_config0(dev, steps=2000):
    """The small dam break (32,000 fluid, 3,680 solid, 144,216 wall particles,
    dt 1e-4, 4 sub-steps) for its full 2000 steps: this build and the
    reference build on the same GPU."""
    from fluidsim_gb300 import api, cases

    cfg, pa = cases.make(cases.small_dam_break())
    nupd = pa.n_fluid + pa.n_solid
    with api.Simulation(cfg, pa, device=dev) as sim:
        sim.step(10)
        sim.sync()
        ms = sim.time_steps(steps)
    out = {"workload": "small dam break: %d fluid + %d solid + %d wall particles, dx=0.01, dt=1e-4, %d steps "
                       "after 10 warm-up steps" % (pa.n_fluid, pa.n_solid, pa.n_virt, steps),
           "value": nupd * steps / (ms * 1e-3), "ms_per_step": ms / steps, "unit": "particle-updates/s"}
    try:
        ref = reference_build_rate(cfg, pa, steps, 10, dev)
    except Exception as e:
        ref = {"error": str(e)}
    out["reference_build"] = ref
    if ref and "value" in ref:
        out["ratio_vs_reference_build"] = out["value"] / ref["value"]
    return out


def run_gb300(args, dist):
    from fluidsim_gb300 import api

    dev = dist.local
    cfg, pa = workload(args)
    nupd = pa.n_fluid + pa.n_solid
    sim = api.Simulation(cfg, pa, device=dev)
    launches = sim.launches_per_step()
    sim.step(max(args.warmup, 3))
    sim.sync()

    # ---- device-resident timed region
    clocks = ClockSampler(dev)
    dist.barrier()
    sim.sync()
    lists0 = sim.list_stats()
    clocks.start()
    t_wall = time.perf_counter()
    # the timed region: K replays of the step graph, whose event nodes around
    # the fluid sweep time that kernel inside the same replays
    ms, sweep_ms = sim.time_sweep(args.steps)
    t_wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    lists1 = sim.list_stats()
    neighbor_lists = {"enabled": bool(lists1["enabled"]), "skin": cfg.neighbor_skin,
                      "capacity": lists1["capacity"], "builds_in_timed_steps": lists1["builds"] - lists0["builds"],
                      "cell_check": bool(lists1["check"])}
    dist.barrier()
    ms = dist.max(ms)
    sweep_ms = dist.max(sweep_ms)
    value = nupd * args.steps * dist.ws / (ms * 1e-3)

    # ---- end to end through the C ABI with pinned host buffers, right after
    #      the timed region (the dam break keeps developing as steps accumulate)
    bufs = {k: api.PinnedBuffer(shape) for k, shape in (
        ("fluid_pos", (pa.n_fluid, 3)), ("fluid_vel", (pa.n_fluid, 3)), ("fluid_rho", (pa.n_fluid,)),
        ("fluid_p", (pa.n_fluid,)), ("solid_pos", (pa.n_solid, 3)), ("solid_vel", (pa.n_solid, 3)))}
    for k, b in bufs.items():
        sim.get(k, out=b.array)
    h2d = sum(b.nbytes for b in bufs.values())
    d2h = h2d
    e2e_steps = max(1, min(args.steps, 20))
    # device time of the same number of steps from the same state, for the serial bound
    dev_ms_e2e = dist.max(sim.time_steps(e2e_steps))
    dist.barrier()
    sim.sync()
    t0 = time.perf_counter()
    names = list(bufs)
    ptrs = [bufs[k].ptr for k in names]
    sizes = [bufs[k].nbytes for k in names]
    for _ in range(e2e_steps):
        sim.set_many_ptr(names, ptrs, sizes)   # fsim_set_fields: the step's whole input state
        sim.step(1)
        sim.get_many_ptr(names, ptrs, sizes)   # fsim_get_fields: the step's whole result
    sim.sync()
    e2e_s = dist.max(time.perf_counter() - t0)
    e2e = nupd * e2e_steps * dist.ws / e2e_s
    # the serial bound: device step + upload + download at the link's measured rates
    link = link_bandwidth(dev, h2d)
    bound_s = dev_ms_e2e * 1e-3 / e2e_steps + h2d / (link["h2d_gbps"] * 1e9) + d2h / (link["d2h_gbps"] * 1e9)
    e2e_bound = nupd * dist.ws / bound_s
    for b in bufs.values():
        b.free()

    chosen, tune_ms = sim.sweep_tuning()
    tuning = {"chosen_shape": chosen, "shape": api.SWEEP_SHAPES[chosen] if chosen >= 0 else None,
              "shapes": "(warps per block, list capacity)", "sweep_ms_per_shape": tune_ms}

    # ---- the dominant kernel (fluid sweep): its launches in the timed region
    t_launch = sweep_ms * 1e-3 / args.steps
    alg_bytes = ALG_BYTES_FLUID * pa.n_fluid
    peaks, peak_src = measured_peaks()
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    achieved = alg_bytes / t_launch / 1e9
    step_bytes = (ALG_BYTES_FLUID * pa.n_fluid + pa.n_solid * (ALG_BYTES_SOLID * cfg.solid_sub_step +
                                                               ALG_BYTES_SOLID_STEP) + ALG_BYTES_VIRT * pa.n_virt)
    fp32 = sweep_flop_roofline(api, sim, dev, t_launch)
    phases = {k: v / args.steps for k, v in sim.time_phases(args.steps).items()}
    traffic = None
    prof = os.path.join(ROOT, "profiles", "fluid_sweep_traffic.json")
    if os.path.exists(prof):
        try:
            with open(prof) as f:
                traffic = json.load(f).get("bytes_per_launch_full_size")
        except (OSError, ValueError):
            traffic = None

    sim.close()

    # ---- the reference build on the same workload and GPU (its own kernels)
    ref_build = None
    if not args.no_forms:
        try:
            ref_build = reference_build_rate(cfg, pa, max(10, min(args.steps, 50)), 3, dev)
        except Exception as e:
            ref_build = {"error": str(e)}
        if ref_build and "value" in ref_build:
            ref_build["ratio_device"] = value / ref_build["value"]
            ref_build["ratio_e2e"] = e2e / ref_build["value"]

    # ---- the other forms and the small dam break
    forms = None
    if not args.no_forms:
        forms = {"config0": run_config0(dev),
                 "mixed": run_mixed(dev, max(10, min(args.steps, 100))),
                 "ensemble64": run_ensemble(dev, max(10, min(args.steps, 50))), "served": run_served(dev)}

    # ---- CPU baseline (rank 0, N=1 only)
    cpu = None
    if dist.ws == 1 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        rate, dt = cpu_oracle_rate(cfg, pa, "f64", args.cpu_steps, cores)
        cpu = {"value": rate, "unit": "particle-updates/s", "cores": cores, "kind": "port",
               "sample": "%d fluid steps of the full workload in the FP64 oracle (%.1f s)" % (args.cpu_steps, dt)}
        if cores > 1:
            rate1, dt1 = cpu_oracle_rate(cfg, pa, "f64", 1, 1)
            cpu["single_thread"] = {"value": rate1, "unit": "particle-updates/s", "cores": 1,
                                    "sample": "1 fluid step of the full workload in the FP64 oracle on one "
                                              "thread (%.1f s)" % dt1}

    if dist.rank == 0:
        line = {
            "metric": "particle-updates/s", "value": value, "unit": "particle-updates/s", "n_gpus": dist.ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(workload_desc(cfg, pa), parallelism="replicas%d" % dist.ws),
            "e2e": {"value": e2e, "unit": "particle-updates/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": e2e_steps, "link_h2d_gbps": link["h2d_gbps"],
                    "link_d2h_gbps": link["d2h_gbps"], "serial_bound": e2e_bound, "frac_of_bound": e2e / e2e_bound},
            "roofline": {"bound": "hbm", "kernel": "k_fluid_sweep", "achieved": achieved, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": traffic,
                         "peak_source": peak_src,
                         "alg_bytes_per_launch": alg_bytes, "launch_ms": t_launch * 1e3,
                         "step_alg_bytes": step_bytes,
                         "step_frac": step_bytes / (ms * 1e-3 / args.steps) / 1e9 / hbm_peak},
            "roofline_fp32": fp32,
            "autotuner": tuning,
            "phases_ms_per_step": phases,
            "cpu_baseline": cpu,
            "reference_build": ref_build,
            "clocks": clk,
            "forms": forms,
            "neighbor_lists": neighbor_lists,
            "gpu_launches": launches * args.steps,
            "wall_s_timed": t_wall,
        }
        print(json.dumps(line), flush=True)
    return 0


def sweep_flop_roofline(api, sim, dev, t_launch):
    """The sweep against the FP32 roofline (it is a gather bound by FP32/ALU
    issue, not by HBM): algorithmic FLOPs of one launch = 10 per candidate
    distance test over the reference's 27-cell candidates + 80 per in-range
    pair (FMA = 2, exp/rsqrt/div = 1), counted on the current state; the peak
    is the device's FP32 FMA throughput measured here by fsim_measure_fp32_peak."""
    import numpy as np

    d = sim.derived()
    nx, ny, nz = d.cell_number[0], d.cell_number[1], d.cell_number[2]
    occ = np.zeros((nx, ny, nz), np.int64)
    for sp in (0, 1, 2):
        start, _ = sim.cells(sp)
        occ += np.diff(start.astype(np.int64)).reshape(nx, ny, nz)
    pad = np.pad(occ, 1)
    box = sum(pad[1 + a:1 + a + nx, 1 + b:1 + b + ny, 1 + c:1 + c + nz]
              for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1))
    fstart, _ = sim.cells(0)
    nfc = np.diff(fstart.astype(np.int64)).reshape(nx, ny, nz)
    cand = float((nfc * box).sum())
    pairs = float(sim.neighbor_counts().astype(np.int64).sum())
    flop = 10.0 * cand + 80.0 * pairs
    peak = api.measure_fp32_peak(dev)
    achieved = flop / t_launch / 1e12
    nf = max(1, int(nfc.sum()))
    return {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "peak_source": "measured (fsim_measure_fp32_peak, FMA chains at full residency)",
            "flop_per_launch": flop, "candidates_per_particle": cand / nf, "pairs_per_particle": pairs / nf,
            "flop_model": "10 FLOP per 27-cell candidate test + 80 FLOP per in-range pair"}


def link_bandwidth(dev, nbytes, reps=5):
    """Host<->device copy rate of one pinned buffer of nbytes each way (GB/s),
    timed with CUDA events: the bound the end-to-end figure is held to."""
    import torch

    with torch.cuda.device(dev):
        h = torch.empty(max(1, nbytes // 4), dtype=torch.float32, pin_memory=True)
        d = torch.empty_like(h, device="cuda")
        out = {}
        for name, fn in (("h2d_gbps", lambda: d.copy_(h, non_blocking=True)),
                         ("d2h_gbps", lambda: h.copy_(d, non_blocking=True))):
            fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                fn()
            e1.record()
            torch.cuda.synchronize()
            out[name] = h.numel() * 4 * reps / (e0.elapsed_time(e1) * 1e-3) / 1e9
        del h, d
        torch.cuda.empty_cache()
    return out


def run_mixed(dev, steps):
    """The mixed-precision workload: the 4M FSI case with +-0.01 dx position
    jitter (seed 12345) in the plain FP32 form and in the mixed form, same input.  Device
    time of `steps` graph steps each; the per-field error of both forms against
    the FP64 oracle is measured separately (tests/accuracy_report.py)."""
    from fluidsim_gb300 import api, cases

    out = {}
    for name, prec in (("plain", api.PRECISION_FP32), ("mixed", api.PRECISION_MIXED)):
        cfg, pa = cases.make(cases.fsi_4m_jitter(precision=prec))
        with api.Simulation(cfg, pa, device=dev) as sim:
            sim.step(5)
            sim.sync()
            ms = sim.time_steps(steps)
            tot, sweep = sim.time_sweep(steps)
        out[name] = (pa.n_fluid + pa.n_solid) * steps / (ms * 1e-3)
        out[name + "_ms_per_step"] = ms / steps
        out[name + "_sweep_ms"] = sweep / steps
    out.update({"workload": "fsi_4m with uniform +-0.01 dx jitter (seed 12345)", "steps": steps,
                "unit": "particle-updates/s", "ratio_mixed_over_plain": out["mixed"] / out["plain"]})
    return out


def run_ensemble(dev, steps):
    """The ensemble workload: 64 seeded dam-break instances (8k-250k fluid
    particles, plate E log-uniform 1e5-1e7 Pa, nu 0.3-0.45, gate 0.6-1.0 m),
    advanced (a) one instance after another in the plain form and (b) all at
    once by batched launches.  Returns aggregate particle-updates/s of both."""
    from fluidsim_gb300 import api, cases

    members = [cases.make(s) for s in cases.ensemble(64, 2024)]
    total = sum(pa.n_fluid + pa.n_solid for _, pa in members)
    sims = [api.Simulation(cfg, pa, device=dev) for cfg, pa in members]
    for sm in sims:
        sm.step(3)
        sm.sync()
    one_by_one_ms = sum(sm.time_steps(steps) for sm in sims)
    with api.Batch(sims) as b:
        b.step(3)
        b.sync()
        batched_ms = b.time_steps(steps)
        launches = b.launches_per_step()
        chosen, tune_ms = b.sweep_tuning()
    for sm in sims:
        sm.close()
    # the same ensemble with the solid sub-steps as one persistent cooperative launch
    for cfg, _ in members:
        cfg.solid_fused = 1
    sims = [api.Simulation(cfg, pa, device=dev) for cfg, pa in members]
    with api.Batch(sims) as b:
        b.step(3)
        b.sync()
        fused_ms = b.time_steps(steps)
        fused_launches = b.launches_per_step()
    for sm in sims:
        sm.close()
    # the reference build, one instance after another (how the reference runs an ensemble)
    ref_ms, ref_err = 0.0, None
    try:
        from oracle import refbuild

        if refbuild.available("release"):
            for cfg, pa in members:
                cfg.solid_fused = 0
                with refbuild.RefBuildSim(cfg, pa, "release", device=dev) as r:
                    r.step(3)
                    ref_ms += r.time_steps(steps)
        else:
            ref_err = "reference device image absent"
    except Exception as e:
        ref_err = str(e)
    ref_rate = total * steps / (ref_ms * 1e-3) if ref_ms > 0 and not ref_err else None
    return {
        "reference_build_one_by_one": ref_rate,
        "ratio_batched_vs_reference_build": (total * steps / (batched_ms * 1e-3)) / ref_rate if ref_rate else None,
        "reference_build_error": ref_err,
        "workload": "ensemble of 64 dam-break instances (seed 2024), %d fluid+solid particles in total, "
                    "dx=0.01, dt=1e-4, 4-5 solid sub-steps" % total,
        "steps": steps,
        "batched": total * steps / (batched_ms * 1e-3),
        "one_by_one": total * steps / (one_by_one_ms * 1e-3),
        "ratio": one_by_one_ms / batched_ms,
        "unit": "particle-updates/s",
        "batched_launches_per_step": launches,
        "autotuner": {"chosen_shape": chosen, "sweep_ms_per_shape": tune_ms},
        "batched_fused_solid": total * steps / (fused_ms * 1e-3),
        "batched_fused_solid_launches_per_step": fused_launches,
    }


def run_served(dev, n=24):
    """The served workload, shortened in request count only: a seeded Poisson
    stream (20 requests/s) of ensemble-style dam-break scenarios (fluid 10k-1M
    log-uniform, solid 1k-27k, 200-2000 steps), served with continuous
    batching under a 150 GB budget, and the same stream
    served one request at a time.  Request data is generated before the clock
    starts.  The default 24 requests keep the run to tens of seconds; at 20
    requests/s the stream saturates the GPU, as the 2000-request stream does.
    `--served-requests N` runs the first N requests of the same stream alone."""
    from fluidsim_gb300 import serve

    spec = dict(n=n, rate=20.0, seed=7, fluid_range=(10_000, 1_000_000), solid_range=(1_000, 27_000),
                steps_range=(200, 2000))
    reqs = serve.pregenerate(serve.poisson_stream(**spec))
    batched = serve.Server(budget_bytes=150 * 10 ** 9, backend=serve.GpuBackend(dev), quantum=20,
                           max_particles=6_000_000).run(reqs)
    again = serve.poisson_stream(**spec)  # same stream, same data
    for r, q in zip(reqs, again):
        q.data, q.particles = r.data, r.particles
    plain = serve.serve_one_by_one(again, device=dev)
    return {"workload": "Poisson stream, %d requests at %g/s (seed 7), fluid %d-%d log-uniform, solid %d-%d, "
                        "steps %d-%d uniform, dx=0.01, 150 GB HBM budget and a 6M-particle work budget; a "
                        "2000-request stream shortened to %d"
                        % (spec["n"], spec["rate"], spec["fluid_range"][0], spec["fluid_range"][1],
                           spec["solid_range"][0], spec["solid_range"][1], spec["steps_range"][0],
                           spec["steps_range"][1], spec["n"]),
            "served": batched, "one_by_one": plain,
            "throughput_ratio": batched["throughput"] / plain["throughput"]}


def run_cpu_full(args):
    """The FP64 CPU oracle on the two plain workloads as the measurement plan
    asks: the small dam break for all 2000 steps and the 4M case for 200 steps,
    on every host core; one thread on 20 and 2 steps of them (per-step rates
    extrapolate, the oracle's cost per step varies little)."""
    from fluidsim_gb300 import cases

    cores = os.cpu_count() or 1
    out = {"cores": cores, "unit": "particle-updates/s", "kind": "port (FP64 oracle, OpenMP)"}
    for name, make, steps, steps1 in (("small_dam_break", cases.small_dam_break, 2000, 20),
                                      ("fsi_4m", cases.fsi_4m, 200, 2)):
        cfg, pa = cases.make(make())
        rate, dt = cpu_oracle_rate(cfg, pa, "f64", steps, cores)
        rate1, dt1 = cpu_oracle_rate(cfg, pa, "f64", steps1, 1)
        out[name] = {"all_cores": rate, "all_cores_steps": steps, "all_cores_s": dt,
                     "one_thread": rate1, "one_thread_steps": steps1, "one_thread_s": dt1,
                     "particles": pa.n_fluid + pa.n_solid, "wall_particles": pa.n_virt}
        print(json.dumps({name: out[name]}), flush=True)
    print(json.dumps(out), flush=True)
    return 0


def run_profile(args):
    """Fewest launches for an ncu capture: creation, the autotuner's step
    (the sweep once per launch shape and round), then N steps of the timed
    region's graph.  --profile-form picks the plain
    4M case, the mixed form of the jittered 4M case, or the batched ensemble."""
    from fluidsim_gb300 import api, cases

    if args.profile_form == "ensemble":
        members = [cases.make(s) for s in cases.ensemble(64, 2024)]
        sims = [api.Simulation(cfg, pa, device=0) for cfg, pa in members]
        with api.Batch(sims) as b:
            ms = b.time_steps(args.profile_steps)
        for sm in sims:
            sm.close()
        print(json.dumps({"profile_steps": args.profile_steps, "form": "ensemble",
                          "ms_per_step": ms / args.profile_steps}))
        return 0
    if args.profile_form == "mixed":
        cfg, pa = cases.make(cases.fsi_4m_jitter(precision=api.PRECISION_MIXED))
    else:
        cfg, pa = workload(args)
    sim = api.Simulation(cfg, pa, device=0)
    sim.step(1)  # the autotuner's step: every sweep shape, then the fastest is kept
    tot, sweep = sim.time_sweep(args.profile_steps)
    sim.close()
    print(json.dumps({"profile_steps": args.profile_steps, "form": args.profile_form,
                      "ms_per_step": tot / args.profile_steps, "sweep_ms": sweep / args.profile_steps}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the batched-ensemble measurement")
    ap.add_argument("--profile-form", choices=("plain", "mixed", "ensemble"), default="plain")
    ap.add_argument("--cpu-full", action="store_true",
                    help="time the FP64 oracle on the small dam break (2000 steps) and the 4M case (200 steps)")
    ap.add_argument("--served-requests", type=int, default=0,
                    help="run only the served stream, with this many requests, and print its JSON")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="profiling run for ncu: create the workload, run this many steps, print nothing else")
    args = ap.parse_args()
    if args.profile_steps:
        return run_profile(args)
    if args.served_requests:
        print(json.dumps({"served": run_served(0, args.served_requests)}), flush=True)
        return 0
    if args.cpu_full:
        return run_cpu_full(args)
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    dist = Dist()
    try:
        if args.impl == "reference":
            return run_reference(args, dist)
        return run_gb300(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    sys.exit(main())
