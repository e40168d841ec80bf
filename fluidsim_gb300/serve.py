"""Served stream of FSI requests with continuous batching.

A request is one dam-break scenario (a config + case) and a number of steps.
Requests arrive on a schedule; the server keeps the admitted ones resident on
the GPU and advances all of them together with batched launches
(fsim_batch_*).  At every step-quantum boundary it retires finished requests
(their results are read back) and admits waiting ones first-come first-served
while their estimated device memory (fsim_estimate_bytes) fits the budget, so
requests that arrive while others run join the running batch.  The reference
runs one scenario per process; this loop has no reference counterpart.

`serve_one_by_one` processes the same stream with one standalone instance at a
time (the plain form), for comparison.
"""
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import api, cases


@dataclass
class Request:
    rid: int
    arrival: float           # seconds after the start of the stream
    cfg: object
    case: object
    steps: int
    particles: int = 0       # fluid + solid, set when generated
    done_at: float = float("nan")
    result: dict = field(default_factory=dict)
    data: object = None      # (config, particles) when generated ahead of the stream
    error: str = ""          # set when the request failed or was cancelled


def poisson_stream(n, rate, seed=7, fluid_range=(10_000, 1_000_000), solid_range=(1_000, 27_000),
                   steps_range=(200, 2000), dx=0.01):
    """Seeded request stream: Poisson arrivals at `rate` per second; fluid count
    log-uniform in fluid_range; a solid plate (or block) of solid_range
    particles; steps uniform in steps_range."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for rid in range(n):
        t += rng.exponential(1.0 / rate)
        cfg, case = cases.ensemble_member(rng, dx=dx, n_range=fluid_range)
        # solid block: 4 cells thick, height and width sized to the drawn count
        ns = int(math.exp(rng.uniform(math.log(solid_range[0]), math.log(solid_range[1]))))
        sz = max(4, min(case.tank_n[2], int(round(math.sqrt(ns / 4.0)))))
        sy = max(2, min(case.tank_n[1] - 1, ns // (4 * sz)))
        case.solid_n[0], case.solid_n[1], case.solid_n[2] = 4, sy, sz
        steps = int(rng.integers(steps_range[0], steps_range[1] + 1))
        cfg.iend = steps
        out.append(Request(rid, t, cfg, case, steps))
    return out


def pregenerate(requests):
    """Generate every request's particles ahead of the stream (a served request
    arrives with its data; generation is not part of serving)."""
    for r in requests:
        r.data = cases.make((r.cfg, r.case))
        r.particles = r.data[1].n_fluid + r.data[1].n_solid
    return requests


def _result_fields(sim):
    out = {"fluid_pos": sim.get("fluid_pos"), "fluid_vel": sim.get("fluid_vel"), "fluid_rho": sim.get("fluid_rho")}
    if sim.n["solid"]:
        out["solid_pos"] = sim.get("solid_pos")
    return out


def _percentile(xs, q):
    return float(np.percentile(np.asarray(xs, dtype=np.float64), q)) if xs else float("nan")


class GpuBackend:
    """Instances are fsim handles; a batch is an fsim_batch over them."""

    def __init__(self, device=0):
        self.device = device

    def prepare(self, r):
        """Generate the request's particles; returns (particles, device bytes)."""
        cfg, pa = r.data if r.data is not None else cases.make((r.cfg, r.case))
        return (cfg, pa), api.estimate_bytes(cfg, pa.n_fluid, pa.n_solid, pa.n_virt), pa.n_fluid + pa.n_solid

    def create(self, prepared):
        cfg, pa = prepared
        return api.Simulation(cfg, pa, device=self.device)

    def batch(self, instances):
        return api.Batch(instances)

    def add(self, batch, inst):
        batch.add(inst)

    def remove(self, batch, inst):
        batch.remove(inst)

    def result(self, inst):
        return _result_fields(inst)

    def member_status(self, batch):
        """Per-member status codes after the batch's last step (waits for it)."""
        return batch.sync_members()

    def destroy(self, inst):
        inst.close()


class Server:
    """Continuous-batching server over one GPU.

    Every loop turn: release requests whose arrival time has passed into the
    waiting queue; admit from its head while the estimated device memory of
    the admitted requests stays within the HBM budget and their particles
    within the work budget `max_particles` (a request larger than a budget is
    admitted alone when nothing else runs); rebuild the batch when its
    membership changed; advance the batch by `quantum` steps (fewer if a member
    needs fewer); retire members whose steps are done.

    The work budget bounds the batch at about what saturates the GPU: beyond
    that, admitting more only slows every running request down (they share the
    GPU), raising latency without raising throughput.

    Failures stay per request: a request whose instance cannot be created
    (e.g. out of device memory) fails at admission; a member whose own error
    flag is set (its particles left the cell grid) is evicted at the next
    quantum boundary while the others continue; cancel(rid) drops a waiting
    request or evicts a running one.  Failed and cancelled requests carry
    `error` and count in the summary's "failed"."""

    def __init__(self, budget_bytes, backend=None, quantum=10, keep_results=False, max_particles=None):
        self.budget = budget_bytes
        self.max_particles = max_particles
        self.backend = backend or GpuBackend()
        self.quantum = quantum
        self.keep_results = keep_results
        self.log = []  # (event, request id, time)
        self._cancel = set()

    def cancel(self, rid):
        """Cancel request `rid` (takes effect at the next loop turn)."""
        self._cancel.add(rid)

    def run(self, requests, clock=time.perf_counter, sleep=time.sleep):
        be = self.backend
        reqs = sorted(requests, key=lambda r: r.arrival)
        waiting, active = [], []  # active entries: [request, instance, steps left, bytes]
        pending = []  # admitted while the batch stepped: they join it at the next quantum
        prepared = {}
        st = {"nxt": 0, "used": 0, "load": 0, "completed": 0, "failed": 0, "work": 0, "rebuilds": 0, "joins": 0,
              "leaves": 0}
        # host time per activity: stepping (enqueue + the wait for the quantum),
        # admission (instance creation), retirement (read-back + free),
        # batch membership changes, idle (nothing to run)
        tm = {"step": 0.0, "admit": 0.0, "retire": 0.0, "membership": 0.0, "idle": 0.0}
        batch, batch_members = None, []
        t0 = clock()

        def close_request(r, now, event, error=""):
            r.done_at, r.error = now, error
            st["completed"] += 1
            st["failed"] += bool(error)
            self.log.append((event, r.rid, now))

        def retire(a, now, error=""):
            t_r = clock()
            if self.keep_results and not error:
                a[0].result = be.result(a[1])
            be.destroy(a[1])
            st["used"] -= a[3]
            st["load"] -= a[0].particles
            close_request(a[0], now, "failed" if error else "done", error)
            tm["retire"] += clock() - t_r

        def arrivals():
            now = clock() - t0
            while st["nxt"] < len(reqs) and reqs[st["nxt"]].arrival <= now:
                waiting.append(reqs[st["nxt"]])
                st["nxt"] += 1

        def admit(running):
            """Admit waiting requests first-come first-served while the budgets
            allow; `running`: instances already on the GPU (active or pending)."""
            out = []
            while waiting:
                r = waiting[0]
                if r.rid not in prepared:
                    prepared[r.rid] = be.prepare(r)
                data, need, npart = prepared[r.rid]
                if running and st["used"] + need > self.budget:
                    break
                if running and self.max_particles is not None and st["load"] + npart > self.max_particles:
                    break
                waiting.pop(0)
                del prepared[r.rid]
                r.particles = npart
                t_a = clock()
                try:
                    inst = be.create(data)
                except Exception as exc:  # this request fails; the others go on
                    close_request(r, clock() - t0, "failed", "admission failed: %s" % exc)
                    continue
                finally:
                    tm["admit"] += clock() - t_a
                out.append([r, inst, r.steps, need])
                running = True
                st["used"] += need
                st["load"] += npart
                self.log.append(("admit", r.rid, clock() - t0))
            return out

        while st["completed"] < len(reqs):
            arrivals()
            now = clock() - t0
            changed = bool(pending)
            active.extend(pending)
            pending = []
            if self._cancel:
                for r in [r for r in waiting if r.rid in self._cancel]:
                    waiting.remove(r)
                    prepared.pop(r.rid, None)
                    close_request(r, now, "cancelled", "cancelled")
                for a in [a for a in active if a[0].rid in self._cancel]:
                    active.remove(a)
                    if batch is not None:
                        batch.close()
                        batch = None
                    retire(a, now, "cancelled")
                    changed = True
            if not active:
                # nothing runs: admit now, there is nothing to overlap with
                new = admit(False)
                active.extend(new)
                changed = changed or bool(new)
            if not active:
                if batch is not None:
                    batch.close()
                    batch = None
                if st["nxt"] < len(reqs):
                    t_i = clock()
                    sleep(max(0.0, min(0.05, reqs[st["nxt"]].arrival - (clock() - t0))))
                    tm["idle"] += clock() - t_i
                continue
            t_m = clock()
            if batch is not None and changed and hasattr(be, "add"):
                # keep the live batch: admit the new members into it
                current = list(batch_members)
                for a in active:
                    if not any(a[1] is c for c in current):
                        be.add(batch, a[1])
                        batch_members.append(a[1])
                        st["joins"] += 1
                changed = False
            if changed or batch is None:
                if batch is not None:
                    batch.close()
                batch = be.batch([a[1] for a in active])
                batch_members = [a[1] for a in active]
                st["rebuilds"] += 1
            tm["membership"] += clock() - t_m
            k = min(self.quantum, min(a[2] for a in active))
            t_s = clock()
            batch.step(k)
            # while the quantum runs on the GPU: admit what has arrived (the new
            # instances join at the next quantum)
            arrivals()
            t_p = clock()
            pending = admit(True)
            t_s += clock() - t_p  # admission time is counted as admission, not stepping
            status = be.member_status(batch)
            tm["step"] += clock() - t_s
            now = clock() - t0
            finished, broken = [], []
            for a, code in zip(active, status):
                if code:
                    broken.append((a, code))
                    continue
                a[2] -= k
                st["work"] += a[0].particles * k
                if a[2] == 0:
                    finished.append(a)
            if finished or broken:
                leaving = finished + [a for a, _ in broken]
                t_m = clock()
                if hasattr(be, "remove") and len(leaving) < len(active):
                    for a in leaving:
                        be.remove(batch, a[1])
                        batch_members = [c for c in batch_members if c is not a[1]]
                        st["leaves"] += 1
                else:
                    batch.close()
                    batch = None
                tm["membership"] += clock() - t_m
                for a in finished:
                    retire(a, now)
                for a, code in broken:
                    retire(a, now, "instance error %d" % code)
                gone = {id(a) for a in finished} | {id(a) for a, _ in broken}
                active = [a for a in active if id(a) not in gone]
        if batch is not None:
            batch.close()
        makespan = clock() - t0
        lat = [r.done_at - r.arrival for r in reqs if not r.error]
        return {"requests": len(reqs), "makespan_s": makespan, "particle_updates": st["work"],
                "throughput": st["work"] / makespan, "p50_latency_s": _percentile(lat, 50),
                "p99_latency_s": _percentile(lat, 99), "batch_rebuilds": st["rebuilds"],
                "batch_joins": st["joins"], "batch_leaves": st["leaves"], "failed": st["failed"],
                "host_time_s": {k: round(v, 3) for k, v in tm.items()}}


def serve_one_by_one(requests, device=0, clock=time.perf_counter, keep_results=False):
    """The plain form: one standalone instance at a time, first-come first-served."""
    reqs = sorted(requests, key=lambda r: r.arrival)
    t0 = clock()
    work = 0
    for r in reqs:
        wait = r.arrival - (clock() - t0)
        if wait > 0:
            time.sleep(wait)
        cfg, pa = r.data if r.data is not None else cases.make((r.cfg, r.case))
        r.particles = pa.n_fluid + pa.n_solid
        with api.Simulation(cfg, pa, device=device) as sim:
            sim.step(r.steps)
            sim.sync()
            r.done_at = clock() - t0
            if keep_results:
                r.result = _result_fields(sim)
        work += r.particles * r.steps
    makespan = clock() - t0
    lat = [r.done_at - r.arrival for r in reqs]
    return {"requests": len(reqs), "makespan_s": makespan, "particle_updates": work, "throughput": work / makespan,
            "p50_latency_s": _percentile(lat, 50), "p99_latency_s": _percentile(lat, 99)}
