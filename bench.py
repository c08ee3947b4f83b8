"""Benchmark of the GB300 transport engine.

Workload (the metric's configuration): forward straggled energy loss and
mixed Coulomb scattering of muons through a 1 km StandardRock slab
(z in [0, 1000] m, vacuum outside), stop on exit or at 1 GeV; 1e7 events
per step, 50/50 mu+/mu-, kinetic energy log-uniform in [10 GeV, 100 TeV],
direction +z, FP64 state, Philox streams keyed by (seed, event id).

One step transports the whole batch. Timed legs:

* value: events/s with the initial states resident in HBM (device structure
  of arrays, restored from a pristine copy at the start of each step), CUDA
  events on the launching stream, max over ranks;
* e2e: the same through the C ABI call a user makes
  (gpumas_context_transport) with pinned host pumas_state arrays: host to
  device copy of the states, transport, device to host copy of states and
  per event results, all inside the timed region;
* roofline: FP64 operations per reference step (F_step, measured once with
  ncu on this kernel) x steps / kernel time, against the FP64 throughput of
  a DFMA microbenchmark run in the same process;
* cpu_baseline: the C restatement of the reference transport (oracle/port.c)
  with OpenMP over all host cores on a bounded sample of the same workload.

`--impl reference` runs only the CPU reference arm.
"""
import argparse
import json
import os
import platform
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic FP64 work of one reference step (one step_transport call,
# pumas.c:6296-6925, with its share of DEL / EHS work) for the rock slab
# workload: FP64 flops (DADD, DMUL: 1, DFMA: 2, per thread) counted by ncu
# on the one thread per event restatement of the algorithm (gp_kernel_plain)
# over 20 000 rock slab events (5 482 614 steps), frozen here. The pool
# engine's own executed count over the same events (its kernels) is
# reported beside it.
F_STEP = 680.4
F_STEP_EXECUTED = 681.7
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum over every pool
# kernel launch) per reference step, from one ncu launch list of two
# 2e6-event rock slab batches (820.2 GB over 1.0957e9 steps); the traffic
# of a batch is this times its steps.
TRAFFIC_STEP = 749.0
# The plain CSDA workload (closed form transport_with_csda, one thread per
# event): FP64 flops per event (DADD and DMUL 1, DFMA 2) and DRAM bytes per
# event, from one ncu capture of 2e7 events.
F_CSDA = 101.0
TRAFFIC_CSDA = 197.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--events", type=int, default=10_000_000)
    p.add_argument("--impl", default="gb300")
    p.add_argument("--seed", type=int, default=7)
    p.add_argument("--no-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--cpu-events", type=int, default=0)
    p.add_argument("--engine", type=int, default=2,
                   help="1: one thread per event, 2: slot pool")
    p.add_argument("--pool-slots", type=int, default=0)
    p.add_argument("--max-inner", type=int, default=0)
    p.add_argument("--batch", type=int, default=0)
    p.add_argument("--tail", type=int, default=0,
                   help="drain threshold in slots (0: off, <0: automatic)")
    p.add_argument("--workload", default="rock_slab",
                   choices=["rock_slab", "slab_jobs", "terrain",
                            "plain_csda", "serve", "atmosphere",
                            "tabulate"])
    p.add_argument("--jobs", type=int, default=8192)
    p.add_argument("--job-scale", type=float, default=0.01,
                   help="slab_jobs: factor on the events per job")
    p.add_argument("--plain-stride", type=int, default=8,
                   help="slab_jobs: plain comparison on every n-th job")
    p.add_argument("--per-direction", type=int, default=10_000,
                   help="terrain: events per direction")
    p.add_argument("--atm-events", type=int, default=1_000_000,
                   help="atmosphere: events per step")
    p.add_argument("--rates",
                   default="100,200,300,500,700,1000,1500,2000,3000,5000,"
                           "10000",
                   help="serve: Poisson arrival rates (requests/s)")
    p.add_argument("--serve-seconds", type=float, default=3.0)
    p.add_argument("--serve-scale", type=float, default=1E-03)
    p.add_argument("--serve-plain", type=int, default=300,
                   help="serve: requests of each rate also served by the "
                        "plain one-request-at-a-time server (0: none)")
    p.add_argument("--autotune", action="store_true",
                   help="slab_jobs: tune the pool on every 8th job first")
    p.add_argument("--no-c3", action="store_true",
                   help="rock_slab: skip the batched jobs sub-object")
    p.add_argument("--no-c4", action="store_true",
                   help="rock_slab: skip the serving sub-object")
    p.add_argument("--c3-scale", type=float, default=0.1,
                   help="rock_slab: event scale of the batched jobs")
    p.add_argument("--e2e-steps", type=int, default=5,
                   help="timed end to end calls (at most --steps)")
    return p.parse_args()


def rank_first_event(rank):
    """First event id of a rank: replicas transport disjoint event ranges
    (events are independent; there is no exchange on the data path)."""
    return rank * 10 ** 12


def max_over_ranks(value, device, world):
    """The maximum of a per rank value (the step time of the slowest
    replica), through the default process group when world > 1."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,"
             "clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        import statistics
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[0]))
                mx.append(float(s[1]))
            except (ValueError, IndexError):
                continue
            for k, v in zip(names, s[3:7]):
                if v.lower() == "active":
                    reasons.add(k)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def fp64_peak_tflops(torch):
    """Measured FP64 throughput of a DFMA microbenchmark, in TFLOP/s."""
    import pumas_gb300 as pg
    lib = pg.library()
    import ctypes
    lib.gpumas_bench_dfma.restype = ctypes.c_int
    lib.gpumas_bench_dfma.argtypes = [ctypes.POINTER(ctypes.c_double)]
    best = 0.
    for _ in range(3):
        v = ctypes.c_double(0.)
        rc = lib.gpumas_bench_dfma(ctypes.byref(v))
        if rc == 0:
            best = max(best, v.value)
    return best


def cpu_baseline(n_events, seed, first_event=0, single=True):
    """All-core OpenMP run of the C restatement on a bounded sample, with
    the host's core count and, on a smaller sample, the one thread rate
    (so that the per core speed and the thread scaling can be read from
    the line)."""
    import numpy as np
    import oracle
    import pumas_gb300 as pg
    from pumas_gb300 import workloads as W
    oracle.build_port()
    port = oracle.Port(pg.default_dump())
    rock = port.material_index("StandardRock")
    geo = oracle.make_geometry(1, [(rock, 0.)], slab_z=[0., 1000.],
                               slab_medium=[0])
    cfg = oracle.Config(seed=seed, **W.config_dict("rock_slab"))
    threads = port.max_threads()
    s0 = W.rock_slab(n_events, seed=seed, first_event=first_event)
    t0 = time.perf_counter()
    _, r = port.transport(cfg, geo, s0, first_event, threads)
    dt = time.perf_counter() - t0
    out = {"value": n_events / dt, "unit": "events/s", "cores": threads,
           "kind": "port",
           "steps_per_s": float(r["steps"].sum()) / dt,
           "nproc": os.cpu_count(), "omp_max_threads": threads,
           "sample": "%d events of the rock slab workload (first event "
                     "id %d), %.1f s wall on %d OpenMP threads"
                     % (n_events, first_event, dt, threads)}
    if single:
        m = max(1, n_events // (4 * threads))
        t0 = time.perf_counter()
        port.transport(cfg, geo, s0[:m], first_event, 1)
        d1 = time.perf_counter() - t0
        out["one_thread"] = {"value": m / d1, "unit": "events/s",
                             "sample": "the first %d events of the same "
                                       "sample on 1 thread, %.1f s" % (m, d1)}
        out["thread_scaling"] = out["value"] / out["one_thread"]["value"]
        # The reference computes the Coulomb functions of hard scatters in
        # long double, which aarch64 implements in software (IEEE quad):
        # the same sample through the port built with double there.
        try:
            dbl = oracle.PortDouble(pg.default_dump(), private=True)
            t0 = time.perf_counter()
            _, r2 = dbl.transport(cfg, geo, s0[:m], first_event, 1)
            d2 = time.perf_counter() - t0
            out["one_thread_coulomb_double"] = {
                "value": m / d2, "unit": "events/s",
                "same_steps": bool(np.array_equal(
                    r2["steps"], r[:m]["steps"])),
                "note": "the port with its Coulomb functions in double "
                        "instead of the reference's long double (%s); "
                        "not a baseline" % platform.machine()}
        except (OSError, RuntimeError):
            pass
    return out


def run_reference_arm(args, rank, world):
    if rank != 0:
        return
    n = args.cpu_events or 200_000
    vals, steps = [], []
    base = None
    for k in range(args.warmup + args.steps):
        r = cpu_baseline(n, args.seed, first_event=k * n,
                         single=(k == args.warmup + args.steps - 1))
        if k >= args.warmup:
            vals.append(r["value"])
            steps.append(r["steps_per_s"])
            base = r
    value = sum(vals) / len(vals)
    line = {
        "impl": "reference", "metric": "events/s", "value": value,
        "unit": "events/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1E+03 * n / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": "rock_slab: forward straggled + mixed "
                               "scattering, 1 km StandardRock slab, "
                               "10 GeV-100 TeV, stop at 1 GeV or exit",
                   "events_per_step": n},
        "steps_per_s": sum(steps) / len(steps),
        "cpu_baseline": {"value": value, "unit": "events/s",
                         "cores": base["cores"], "kind": "port",
                         "sample": base["sample"], "nproc": base["nproc"],
                         "omp_max_threads": base["omp_max_threads"],
                         "one_thread": base.get("one_thread"),
                         "thread_scaling": base.get("thread_scaling")},
        "e2e": {"value": value, "unit": "events/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


class DeviceEvents:
    """Events of several jobs in one device structure of arrays (torch
    tensors), with a pristine copy to restore them between steps."""

    FIELDS = ("charge", "energy", "distance", "grammage", "time", "weight")

    def __init__(self, states, dev):
        import numpy as np
        import torch
        self.n = len(states)
        self.cols = {}
        for f in self.FIELDS:
            self.cols[f] = torch.from_numpy(
                np.ascontiguousarray(states[f])).to(dev)
        for k in range(3):
            self.cols["position%d" % k] = torch.from_numpy(
                np.ascontiguousarray(states["position"][:, k])).to(dev)
            self.cols["direction%d" % k] = torch.from_numpy(
                np.ascontiguousarray(states["direction"][:, k])).to(dev)
        self.cols["decayed"] = torch.from_numpy(
            np.ascontiguousarray(states["decayed"])).to(dev)
        self.work = {k: v.clone() for k, v in self.cols.items()}
        import pumas_gb300 as pg
        self.rsize = pg.RESULT_DTYPE.itemsize
        self.results = torch.zeros((self.n, self.rsize), dtype=torch.uint8,
                                   device=dev)

    def restore(self, stream=None):
        import torch
        with torch.cuda.stream(stream) if stream is not None else \
                _nullcontext():
            for k in self.work:
                self.work[k].copy_(self.cols[k], non_blocking=True)

    def soa(self, offset=0):
        w = self.work
        d = {f: w[f].data_ptr() + 8 * offset for f in self.FIELDS}
        d["decayed"] = w["decayed"].data_ptr() + 4 * offset
        d["position"] = [w["position%d" % k].data_ptr() + 8 * offset
                         for k in range(3)]
        d["direction"] = [w["direction%d" % k].data_ptr() + 8 * offset
                          for k in range(3)]
        d["result"] = self.results.data_ptr() + self.rsize * offset
        return d

    def result_records(self):
        import numpy as np
        import pumas_gb300 as pg
        return np.frombuffer(self.results.cpu().numpy().tobytes(),
                             dtype=pg.RESULT_DTYPE)

    def final_states(self):
        import numpy as np
        import pumas_gb300 as pg
        s = np.zeros(self.n, dtype=pg.STATE_DTYPE)
        for f in self.FIELDS + ("decayed",):
            s[f] = self.work[f].cpu().numpy()
        for k in range(3):
            s["position"][:, k] = self.work["position%d" % k].cpu().numpy()
            s["direction"][:, k] = self.work["direction%d" % k].cpu().numpy()
        return s


class _nullcontext:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def base_line(args, world, metric, value, unit, ms_per_step, config,
              higher=True):
    return {"metric": metric, "value": value, "unit": unit,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_per_step, "higher_is_better": higher,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config}


def measure_slab_jobs(args, physics, dev, scale, steps, warmup,
                      plain_stride=8, cpu_stride=100, baseline=True,
                      autotune=False):
    """Batched uneven jobs (the slab-stack workload at `scale` times its
    events per job): every job in one engine run (one pool, CUDA graph
    batches) per step, against one plain one-thread-per-event launch per
    job on every plain_stride-th job, and the C restatement over all host
    cores on every cpu_stride-th job, whose events are also compared with
    the GPU's. Returns a dict of the measurements."""
    import numpy as np
    import torch
    import pumas_gb300 as pg
    from pumas_gb300 import serving
    from pumas_gb300 import workloads as W
    jobs = W.slab_jobs(args.jobs, seed=args.seed, event_scale=scale)
    t0 = time.perf_counter()
    ctxs, states, offsets = [], [], []
    off = 0
    for k, job in enumerate(jobs):
        c = pg.Context(physics)
        W.apply_config(c, W.slab_job_config(job))
        c.seed = args.seed * 100003 + k
        c.set_geometry(W.slab_job_geometry(physics, job))
        ctxs.append(c)
        states.append(W.slab_job_states(job, seed=args.seed))
        offsets.append(off)
        off += job["n"]
    s0 = np.concatenate(states)
    ev = DeviceEvents(s0, dev)
    setup_s = time.perf_counter() - t0
    spec = [(c, job["n"], None, job["first_event"])
            for c, job in zip(ctxs, jobs)]
    tuned = None
    # The uneven jobs keep more slots busy than the rock slab: 4 M slots
    # (1.5 GB) run them 8 % faster than the 1 M default (measured on the
    # GB300: 0.99e6, 1.10e6, 1.16e6 and 1.19e6 events/s at 0.5, 1, 2 and
    # 4 M slots, events per job x 0.1).
    pool = dict(pool_slots=args.pool_slots or (1 << 22),
                max_inner=args.max_inner, batch=args.batch, tail=args.tail)
    if autotune:
        from pumas_gb300 import autotune as at

        def sample_run(eng):
            ev.restore()
            eng.run([(c, n, ev.soa(o), fe) for k, ((c, n, _, fe), o) in
                     enumerate(zip(spec, offsets)) if k % 8 == 0])
            torch.cuda.synchronize()

        tuned = at.tune(physics, sample_run)
        at.save(tuned)
        pool = {k: tuned[k] for k in pool}
    eng = pg.Engine(physics, max_jobs=len(jobs) + 1, **pool)

    def batched(sub=None):
        ev.restore()
        torch.cuda.synchronize()
        t = time.perf_counter()
        ks = range(len(jobs)) if sub is None else sub
        eng.run([(spec[k][0], spec[k][1], ev.soa(offsets[k]), spec[k][3])
                 for k in ks])
        torch.cuda.synchronize()
        return time.perf_counter() - t

    stream = torch.cuda.Stream(device=dev)
    # The one-launch-per-job comparison runs on every plain_stride-th job
    # (the plain form takes minutes on the whole set), both ways.
    sub = list(range(0, len(jobs), plain_stride))

    def plain():
        ev.restore()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in sub:
            c, n, _, fe = spec[k]
            rc = c.transport_device(n, ev.soa(offsets[k]), fe,
                                    stream.cuda_stream)
            if rc != 0:
                raise RuntimeError("plain transport: %d" % rc)
        e1.record(stream)
        stream.synchronize()
        return e0.elapsed_time(e1) * 1E-03

    for c in ctxs:
        c.tuning(engine=pg.ENGINE_PLAIN)
    for _ in range(warmup):
        batched(sub)
    st0 = eng.stats()
    tb = [batched() for _ in range(steps)]
    st1 = eng.stats()
    res = ev.result_records()
    fin = ev.final_states()
    steps_total = float(res["steps"].sum())
    n = len(s0)
    n_sub = sum(jobs[k]["n"] for k in sub)
    idx_sub = np.concatenate([np.arange(offsets[k], offsets[k] + jobs[k]["n"])
                              for k in sub])
    tbs = batched(sub)
    tp = plain()
    res_p = ev.result_records()
    same = bool(np.array_equal(res_p[idx_sub], res[idx_sub]))
    tb_m = sum(tb) / len(tb)
    kernel_ms = (st1["kernel_ms"] - st0["kernel_ms"]) / steps
    out = {"jobs": len(jobs), "events": n, "event_scale": scale,
           "events_per_job": [int(min(j["n"] for j in jobs)),
                              int(max(j["n"] for j in jobs))],
           "setup_s": setup_s, "batched_s": tb_m,
           "value": n / tb_m, "unit": "events/s",
           "steps_per_s": steps_total / tb_m,
           "steps_per_event": steps_total / n,
           "event_errors": int(np.count_nonzero(res["status"])),
           "kernel_ms": kernel_ms,
           "gpu_launches": (st1["launches"] - st0["launches"]) // steps,
           "plain": {"value": n_sub / tp, "unit": "events/s",
                     "ms": tp * 1E+03, "jobs": len(sub), "events": n_sub,
                     "batched_same_jobs": n_sub / tbs,
                     "detail": "every %d-th job: one gp_kernel_plain "
                               "launch per job on one stream, against one "
                               "engine run of the same jobs" % plain_stride,
                     "identical_results": same},
           "batched_over_plain": tp / tbs,
           "engine": dict(pool, autotuned=None if tuned is None else {
               "sample": "every 8th job", "trials": tuned["trials"]})}
    if baseline:
        cpu, parity = slab_jobs_cpu(jobs, ctxs, states, fin, res, offsets,
                                    cpu_stride)
        out["cpu_baseline"] = cpu
        out["batched_over_cpu"] = out["value"] / cpu["value"]
        out["parity_cpu_sample"] = parity
    return out


def run_slab_jobs(args, rank, world, local):
    """Batched uneven jobs (C3), as its own bench line."""
    import torch
    import pumas_gb300 as pg
    dev = torch.device("cuda", local)
    physics = pg.Physics()
    with ClockSampler(local) as clocks:
        m = measure_slab_jobs(args, physics, dev, args.job_scale, args.steps,
                              max(1, args.warmup // 3), args.plain_stride,
                              baseline=not args.no_baseline,
                              autotune=args.autotune)
    peak = fp64_peak_tflops(torch)
    achieved = F_STEP * m["steps_per_s"] * m["batched_s"] / (
        m["kernel_ms"] * 1E-03) * 1E-12
    if rank != 0:
        return
    line = base_line(args, world, "events/s", world * m["value"],
                     "events/s", m["batched_s"] * 1E+03, {
                         "workload": "slab_jobs: %d uneven jobs, 1-8 slabs "
                                     "of rock / water / iron, 50/50 "
                                     "forward / backward, straggled + "
                                     "mixed" % m["jobs"],
                         "events_per_step": m["events"],
                         "event_scale": m["event_scale"],
                         "events_per_job": m["events_per_job"],
                         "setup_s": m["setup_s"]})
    line.update({k: v for k, v in m.items() if k not in (
        "jobs", "events", "event_scale", "events_per_job", "setup_s",
        "value", "unit")})
    line["impl_detail"] = ("one engine run per step (all jobs in one slot "
                           "pool, CUDA graph batches)")
    line["roofline"] = {"bound": "fp64", "achieved": achieved, "peak": peak,
                        "unit": "TFLOP/s", "frac": achieved / peak,
                        "traffic": None, "f_step": F_STEP}
    line["clocks"] = clocks.summary()
    print(json.dumps(line), flush=True)


def slab_jobs_cpu(jobs, ctxs, states, fin, res, offsets, stride=100):
    """The C restatement with OpenMP over all host cores on every
    `stride`-th job of the slab-stack workload (a seeded 1 % job subset),
    scaled to events/s; its events are compared with the GPU's final
    states `fin` and results `res` (fraction within 1e-9)."""
    import numpy as np
    import oracle
    import pumas_gb300 as pg
    from pumas_gb300 import serving
    from pumas_gb300 import workloads as W
    oracle.build_port()
    port = oracle.Port(pg.default_dump())
    threads = port.max_threads()
    n = 0
    dt = 0.
    n_close = n_same = 0
    for k in range(0, len(jobs), stride):
        job = jobs[k]
        mats = [port.material_index(m) for m in job["materials"]]
        geo = oracle.make_geometry(
            1, [(m, 0.) for m in mats], slab_z=job["slab_z"],
            slab_medium=list(range(len(mats))))
        cfg = oracle.Config(seed=ctxs[k].seed, **W.slab_job_config(job))
        t = time.perf_counter()
        b, rb = port.transport(cfg, geo, states[k], job["first_event"],
                               threads)
        dt += time.perf_counter() - t
        sl = slice(offsets[k], offsets[k] + job["n"])
        same, close = serving.agreement(fin[sl], res[sl], b, rb)
        n_same += int(same.sum())
        n_close += int(close.sum())
        n += job["n"]
    cpu = {"value": n / dt, "unit": "events/s", "cores": threads,
           "kind": "port", "nproc": os.cpu_count(),
           "sample": "every %d-th job (%d jobs, %d events), %.1f s on %d "
                     "OpenMP threads, one job after the other"
                     % (stride, (len(jobs) + stride - 1) // stride, n, dt,
                        threads)}
    parity = {"events": n, "within_1e-9": n_close, "bit_identical": n_same,
              "fraction_within_1e-9": n_close / max(n, 1)}
    return cpu, parity


def port_transport(states, cfg_dict, geometry_spec, seed, first_event):
    """The C restatement with OpenMP over all host cores: final states and
    results of `states` with event ids from first_event."""
    import oracle
    import pumas_gb300 as pg
    oracle.build_port()
    port = oracle.Port(pg.default_dump())
    media = [(port.material_index(m), d) for m, d in geometry_spec["media"]]
    kw = {k: v for k, v in geometry_spec.items()
          if k not in ("kind", "media")}
    geo = oracle.make_geometry(geometry_spec["kind"], media, **kw)
    cfg = oracle.Config(seed=seed, **cfg_dict)
    return port.transport(cfg, geo, states, first_event, port.max_threads())


def port_baseline(name, states, cfg_dict, geometry_spec, seed, first_event,
                  sample):
    """The C restatement with OpenMP over all host cores on `states` (a
    bounded sample of a workload), in events/s."""
    import oracle
    import pumas_gb300 as pg
    oracle.build_port()
    port = oracle.Port(pg.default_dump())
    media = [(port.material_index(m), d) for m, d in geometry_spec["media"]]
    kw = {k: v for k, v in geometry_spec.items()
          if k not in ("kind", "media")}
    geo = oracle.make_geometry(geometry_spec["kind"], media, **kw)
    cfg = oracle.Config(seed=seed, **cfg_dict)
    threads = port.max_threads()
    t0 = time.perf_counter()
    _, r = port.transport(cfg, geo, states, first_event, threads)
    dt = time.perf_counter() - t0
    return {"value": len(states) / dt, "unit": "events/s",
            "cores": threads, "kind": "port",
            "steps_per_s": float(r["steps"].sum()) / dt,
            "sample": "%s: %s, %.1f s wall on %d OpenMP threads"
                      % (name, sample, dt, threads)}


def run_terrain(args, rank, world, local):
    """Backward muography over the synthetic terrain: 32 x 64 directions x
    per-direction events through the context's device entry point."""
    import numpy as np
    import torch
    import pumas_gb300 as pg
    from pumas_gb300 import workloads as W
    dev = torch.device("cuda", local)
    physics = pg.Physics()
    ctx = pg.Context(physics)
    W.apply_config(ctx, W.config_dict("terrain"))
    ctx.seed = args.seed
    t0 = time.perf_counter()
    heights = W.terrain_heights()
    ctx.set_geometry(W.terrain_geometry(physics))
    dirs = W.terrain_directions()
    s0, d = W.terrain(args.per_direction, seed=args.seed, heights=heights,
                      directions=dirs)
    setup_s = time.perf_counter() - t0
    ctx.tuning(engine=args.engine, pool_slots=args.pool_slots,
               max_inner=args.max_inner, batch=args.batch, tail=args.tail)
    ev = DeviceEvents(s0, dev)
    stream = torch.cuda.Stream(device=dev)
    n = len(s0)

    def step(k):
        ev.restore(stream)
        rc = ctx.transport_device(n, ev.soa(), 0, stream.cuda_stream)
        if rc != 0:
            raise RuntimeError("transport_device: %d" % rc)

    for k in range(args.warmup):
        step(k)
    stream.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        e0.record(stream)
        for k in range(args.steps):
            step(k)
        e1.record(stream)
        stream.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    res = ev.result_records()
    fin = ev.final_states()
    flux = W.terrain_flux(fin, res, d, len(dirs[0]))
    steps_total = float(res["steps"].sum())
    st = ctx.stats()
    peak = fp64_peak_tflops(torch)
    achieved = F_STEP * steps_total / (st["kernel_ms"] * 1E-03) * 1E-12
    if rank != 0:
        return
    line = base_line(args, world, "events/s", world * n / (ms * 1E-03),
                     "events/s", ms, {
                         "workload": "terrain: backward muography, 512 x "
                                     "512 heightmap (10 m), 32 x 64 "
                                     "directions x %d events, 1 GeV - "
                                     "100 TeV, straggled + mixed, "
                                     "weighted decay, stop at 3 km or "
                                     "1e8 GeV"
                                     % args.per_direction,
                         "events_per_step": n, "setup_s": setup_s})
    cpu = parity = None
    if not args.no_baseline:
        from pumas_gb300 import serving
        # Every 100th initial state, over all directions, transported with
        # event ids 0 .. n/100 - 1 (a sample of the same distribution).
        sub = np.arange(0, n, 100)
        cpu = port_baseline("terrain", s0[sub], W.config_dict("terrain"),
                            W.terrain_spec(), args.seed, 0,
                            "every 100th initial state (%d events)"
                            % len(sub))
        # Parity: the first events of the workload with their own event
        # ids, against the GPU's final states.
        m = min(n, 20000)
        b, rb = port_transport(s0[:m], W.config_dict("terrain"),
                               W.terrain_spec(), args.seed, 0)
        same, close = serving.agreement(fin[:m], res[:m], b, rb)
        parity = {"events": m, "within_1e-9": int(close.sum()),
                  "bit_identical": int(same.sum()),
                  "fraction_within_1e-9": float(close.mean()),
                  "sample": "the first %d events (event ids 0 .. %d)"
                            % (m, m - 1)}
    line.update({
        "cpu_baseline": cpu,
        "parity_cpu_sample": parity,
        "steps_per_s": steps_total / (ms * 1E-03),
        "steps_per_event": steps_total / n,
        "event_errors": int(np.count_nonzero(res["status"])),
        "flux_total": float(flux.sum()),
        "flux_zenith_profile": [float(x) for x in
                                flux.reshape(32, 64).mean(axis=1)[::4]],
        "gpu_launches": st["launches"],
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak,
                     "traffic": None, "f_step": F_STEP},
        "clocks": clocks.summary()})
    print(json.dumps(line), flush=True)


def run_atmosphere(args, rank, world, local):
    """Muons from 15 km through the exponential atmosphere with the
    geomagnetic field into 200 m of rock: media with local properties,
    transported by the one thread per event kernel that carries them."""
    import numpy as np
    import torch
    import pumas_gb300 as pg
    from pumas_gb300 import workloads as W
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    physics = pg.Physics()
    ctx = pg.Context(physics)
    W.apply_config(ctx, W.config_dict("atmosphere"))
    ctx.seed = args.seed
    ctx.set_geometry(W.atmosphere_geometry(physics))
    n = args.atm_events
    first = rank_first_event(rank)
    s0 = W.atmosphere(n, seed=args.seed, first_event=first)
    ev = DeviceEvents(s0, dev)
    stream = torch.cuda.Stream(device=dev)

    def step(k):
        ev.restore(stream)
        rc = ctx.transport_device(n, ev.soa(), first, stream.cuda_stream)
        if rc != 0:
            raise RuntimeError("transport_device: %d" % rc)

    for k in range(args.warmup):
        step(k)
    stream.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        e0.record(stream)
        for k in range(args.steps):
            step(k)
        e1.record(stream)
        stream.synchronize()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, dev, world)
    res = ev.result_records()
    steps_total = float(res["steps"].sum())
    st = ctx.stats()
    if rank != 0:
        return
    line = base_line(args, world, "events/s", world * n / (ms * 1E-03),
                     "events/s", ms, {
                         "workload": "atmosphere: forward straggled + mixed "
                                     "scattering from 15 km through an "
                                     "exponential atmosphere (12 km scale "
                                     "height, geomagnetic field) into 200 m "
                                     "of StandardRock, 1 GeV - 1 TeV, stop "
                                     "at 1 GeV or exit",
                         "events_per_step": n})
    cpu = None
    if not args.no_baseline:
        sub = max(1, n // 100)
        cpu = port_baseline("atmosphere", s0[:sub],
                            W.config_dict("atmosphere"), W.atmosphere_spec(),
                            args.seed, first, "the first %d events" % sub)
    line.update({
        "cpu_baseline": cpu,
        "steps_per_s": steps_total / (ms * 1E-03),
        "steps_per_event": steps_total / n,
        "event_errors": int(np.count_nonzero(res["status"])),
        "gpu_launches": st["launches"],
        "roofline": None,
        "clocks": clocks.summary()})
    print(json.dumps(line), flush=True)


def run_plain_csda(args, rank, world, local):
    """Deterministic CSDA in infinite rock: one thread per event, streaming
    8 B in and 32 B out per event (HBM roofline)."""
    import numpy as np
    import torch
    import pumas_gb300 as pg
    from pumas_gb300 import workloads as W
    dev = torch.device("cuda", local)
    physics = pg.Physics()
    ctx = pg.Context(physics)
    W.plain_csda_config(ctx)
    ctx.seed = args.seed
    ctx.set_geometry(pg.Geometry.uniform(
        physics.material_index("StandardRock")))
    n = args.events
    s0 = W.plain_csda(n, seed=args.seed)
    ev = DeviceEvents(s0, dev)
    stream = torch.cuda.Stream(device=dev)
    soa = ev.soa()
    soa["result"] = None

    def step():
        with torch.cuda.stream(stream):
            ev.work["energy"].copy_(ev.cols["energy"], non_blocking=True)
        rc = ctx.transport_device(n, soa, 0, stream.cuda_stream)
        if rc != 0:
            raise RuntimeError("transport_device: %d" % rc)

    for _ in range(args.warmup):
        step()
    stream.synchronize()
    kms = []
    with ClockSampler(local) as clocks:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
            kms.append(None)
        e1.record(stream)
        stream.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    kernel_ms = ctx.stats()["kernel_ms"]
    hbm = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))[
        "hbm_gbs"] if os.path.exists(os.path.join(
            ROOT, "MEASURED_PEAKS.json")) else 6800.
    peak = fp64_peak_tflops(torch)
    # 8 B in (kinetic energy) + 32 B out (energy, distance, grammage,
    # time) per event; position z is also written (8 B).
    algo = 48. * n
    if rank != 0:
        return
    line = base_line(args, world, "events/s", world * n / (ms * 1E-03),
                     "events/s", ms, {
                         "workload": "plain_csda: forward CSDA, infinite "
                                     "StandardRock, mu-, 10 GeV - 10 TeV, "
                                     "stop at 1 GeV",
                         "events_per_step": n,
                         "l2": "state %.1f GB larger than L2"
                               % (n * 104 / 1E+09)})
    cpu = None
    if not args.no_baseline:
        m = min(n, 20_000_000)
        cpu = port_baseline("plain_csda", s0[:m],
                            W.config_dict("plain_csda"),
                            dict(kind=0, media=[("StandardRock", 0.)]),
                            args.seed, 0, "first %d events" % m)
    line.update({
        "cpu_baseline": cpu,
        "kernel_ms": kernel_ms,
        "roofline": {"bound": "fp64",
                     "achieved": F_CSDA * n / (kernel_ms * 1E-03) * 1E-12,
                     "peak": peak, "unit": "TFLOP/s",
                     "frac": F_CSDA * n / (kernel_ms * 1E-03) * 1E-12 / peak,
                     "traffic": TRAFFIC_CSDA * n, "flops_per_event": F_CSDA,
                     "hbm": {"achieved": algo / (kernel_ms * 1E-03) * 1E-09,
                             "peak": hbm, "unit": "GB/s",
                             "frac": algo / (kernel_ms * 1E-03) * 1E-09 / hbm,
                             "algorithmic_bytes_per_event": 48}},
        "gpu_launches": 1, "clocks": clocks.summary()})
    print(json.dumps(line), flush=True)


def run_tabulate(args, rank, world, local):
    """Device table builder: the per element DEL tables of the shipped
    physics (4 materials, 7 elements, 194 energies) recomputed from its
    elements and energy grid -- 5 432 restricted cross sections of 180 DCS
    evaluations each and 3 x 7 x 194 DCS table rows of 36 points -- per
    step, against the C restatement over all host cores. The e2e time is
    the whole gpumas_physics_tabulate call, host arrays included."""
    import numpy as np
    import torch
    import oracle
    import pumas_gb300 as pg
    dump = pg.default_dump()
    physics = pg.Physics(dump)
    for _ in range(args.warmup):
        physics.tabulate()
    ms, wall = [], []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            r = physics.tabulate()
            wall.append(time.perf_counter() - t0)
            ms.append(r["ms"])
    evals = 3 * physics.n_elements * physics.n_energies * (
        180 + physics.n_table_dcs)
    ms_m = sum(ms) / len(ms)
    cpu = None
    if not args.no_baseline and rank == 0:
        oracle.build_port()
        port = oracle.Port(dump)
        threads = port.max_threads()
        t0 = time.perf_counter()
        port.dcs_tabulate(threads)
        dt = time.perf_counter() - t0
        cpu = {"value": 1. / dt, "unit": "tabulations/s", "cores": threads,
               "kind": "port", "nproc": os.cpu_count(),
               "sample": "one tabulation of the shipped physics, %.2f s on "
                         "%d OpenMP threads" % (dt, threads)}
    if rank != 0:
        return
    line = base_line(args, world, "tabulations/s", 1E+03 / ms_m,
                     "tabulations/s", ms_m, {
                         "workload": "tabulate: per element DEL tables of "
                                     "the shipped physics (CSn, CSn_dK, DCS "
                                     "tables, envelope exponents)",
                         "dcs_evaluations": evals})
    line.update({
        "dcs_evaluations_per_s": evals / (ms_m * 1E-03),
        "e2e": {"value": 1. / (sum(wall) / len(wall)),
                "unit": "tabulations/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(r["csn"].nbytes +
                                          r["csn_dk"].nbytes +
                                          r["dcs"].nbytes +
                                          r["alpha"].nbytes)},
        "cpu_baseline": cpu, "gpu_launches": 6, "roofline": None,
        "clocks": clocks.summary()})
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_info()
    if args.impl == "reference":
        return run_reference_arm(args, rank, world)
    if args.workload != "rock_slab":
        import torch
        import pumas_gb300 as pg
        torch.cuda.set_device(local)
        pg.library(build=True)
        fn = {"slab_jobs": run_slab_jobs, "terrain": run_terrain,
              "plain_csda": run_plain_csda, "atmosphere": run_atmosphere,
              "tabulate": run_tabulate}.get(args.workload)
        if fn is None:
            from pumas_gb300 import serving
            return serving.bench(args, rank, world, local)
        return fn(args, rank, world, local)

    import numpy as np
    import torch
    import pumas_gb300 as pg
    from pumas_gb300 import workloads as W

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    pg.library(build=True)
    physics = pg.Physics()
    ctx = pg.Context(physics)
    W.rock_slab_config(ctx)
    ctx.seed = args.seed
    ctx.set_geometry(W.rock_slab_geometry(physics))
    tuning = ctx.tuning(engine=args.engine, pool_slots=args.pool_slots,
                        max_inner=args.max_inner, batch=args.batch,
                        tail=args.tail)

    n = args.events
    first = rank_first_event(rank)
    s0 = W.rock_slab(n, seed=args.seed, first_event=first)
    dev = torch.device("cuda", local)
    cols = {}
    for f in ("charge", "energy", "distance", "grammage", "time", "weight"):
        cols[f] = torch.from_numpy(np.ascontiguousarray(s0[f])).to(dev)
    for k in range(3):
        cols["position%d" % k] = torch.from_numpy(
            np.ascontiguousarray(s0["position"][:, k])).to(dev)
        cols["direction%d" % k] = torch.from_numpy(
            np.ascontiguousarray(s0["direction"][:, k])).to(dev)
    cols["decayed"] = torch.from_numpy(
        np.ascontiguousarray(s0["decayed"])).to(dev)
    work = {k: v.clone() for k, v in cols.items()}
    results = torch.zeros((n, pg.RESULT_DTYPE.itemsize), dtype=torch.uint8,
                          device=dev)
    soa = {f: work[f].data_ptr() for f in
           ("charge", "energy", "distance", "grammage", "time", "weight",
            "decayed")}
    soa["position"] = [work["position%d" % k].data_ptr() for k in range(3)]
    soa["direction"] = [work["direction%d" % k].data_ptr() for k in range(3)]
    soa["result"] = results.data_ptr()
    stream = torch.cuda.Stream(device=dev)

    def device_step(k):
        with torch.cuda.stream(stream):
            for key in work:
                work[key].copy_(cols[key], non_blocking=True)
        rc = ctx.transport_device(n, soa, first + k * n,
                                  stream.cuda_stream)
        if rc != 0:
            raise RuntimeError("transport_device: %d" % rc)

    for k in range(args.warmup):
        device_step(k)
    stream.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    kernel_ms = []
    with ClockSampler(local) as clocks:
        ev0.record(stream)
        for k in range(args.steps):
            device_step(args.warmup + k)
            kernel_ms.append(None)
        ev1.record(stream)
        stream.synchronize()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    total_ms = ev0.elapsed_time(ev1)
    # Device time of the last step's transport (CUDA events on the same
    # stream around the engine's launches, recorded by the library).
    st = ctx.stats()
    last_kernel_ms = st["kernel_ms"]
    res = np.frombuffer(results.cpu().numpy().tobytes(),
                        dtype=pg.RESULT_DTYPE)
    steps_per_event = float(res["steps"].mean())
    bad = int(np.count_nonzero(res["status"]))
    ms_per_step = max_over_ranks(total_ms / args.steps, dev, world)
    value = world * n / (ms_per_step * 1E-03)

    # End to end through the C ABI with pinned host buffers.
    e2e = None
    if not args.no_e2e:
        host = torch.empty(n * pg.STATE_DTYPE.itemsize, dtype=torch.uint8,
                           pin_memory=True)
        hres = torch.empty(n * pg.RESULT_DTYPE.itemsize, dtype=torch.uint8,
                           pin_memory=True)
        hview = np.frombuffer(host.numpy(), dtype=pg.STATE_DTYPE)
        e2e_ms = []
        for k in range(1 + min(args.steps, args.e2e_steps)):
            hview[:] = s0
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rc = ctx.transport_raw(n, host.data_ptr(), hres.data_ptr(),
                                   first + (k + 1000) * n)
            t1 = time.perf_counter()
            if rc != 0:
                raise RuntimeError("transport: %d" % rc)
            if k > 0:
                e2e_ms.append(1E+03 * (t1 - t0))
        e2e_step = sum(e2e_ms) / len(e2e_ms)
        e2e = {"value": world * n / (e2e_step * 1E-03), "unit": "events/s",
               "h2d_bytes_per_step": n * pg.STATE_DTYPE.itemsize,
               "d2h_bytes_per_step": n * (pg.STATE_DTYPE.itemsize +
                                          pg.RESULT_DTYPE.itemsize),
               "ms_per_step": e2e_step}

    peak = fp64_peak_tflops(torch)
    steps_total = steps_per_event * n
    kernel_s = last_kernel_ms * 1E-03
    roofline = None
    if F_STEP is not None and peak > 0:
        achieved = F_STEP * steps_total / kernel_s * 1E-12
        roofline = {"bound": "fp64", "achieved": achieved, "peak": peak,
                    "unit": "TFLOP/s", "frac": achieved / peak,
                    "traffic": (None if TRAFFIC_STEP is None else
                                TRAFFIC_STEP * steps_total),
                    "kernel": "transport of one batch: gp_pool_drain, "
                              "gp_pool_step, gp_pool_del, gp_pool_polar, "
                              "gp_pool_ehs",
                    "f_step": F_STEP,
                    "f_step_executed": F_STEP_EXECUTED,
                    "peak_source": "measured: DFMA microbenchmark in this "
                                   "process (MEASURED_PEAKS.json has no "
                                   "FP64 figure)"}
    base = None
    if rank == 0 and not args.no_baseline:
        base = cpu_baseline(args.cpu_events or 200_000, args.seed,
                            first_event=first)
    # The batched-jobs and serving targets, measured once after the timed
    # region on this rank's GPU.
    # A failure of one of them is recorded in its object; the line of the
    # timed region above is printed all the same.
    c3 = c4 = None
    if rank == 0 and not args.no_c3:
        try:
            c3 = measure_slab_jobs(args, physics, dev, args.c3_scale, 1, 1,
                                   baseline=not args.no_baseline)
            c3["workload"] = ("slab_jobs: %d uneven jobs, 1-8 slabs of "
                              "rock / water / iron, 50/50 forward / "
                              "backward, straggled + mixed, events per job "
                              "x %g" % (c3["jobs"], c3["event_scale"]))
        except (RuntimeError, MemoryError, pg.PumasError) as err:
            c3 = {"error": "%s: %s" % (type(err).__name__, err)}
        torch.cuda.empty_cache()
    if rank == 0 and not args.no_c4:
        from pumas_gb300 import serving
        try:
            c4 = serving.sweep(physics, [float(x) for x in
                                         args.rates.split(",")],
                               args.serve_seconds, args.serve_scale,
                               args.seed)
        except (RuntimeError, MemoryError, pg.PumasError) as err:
            c4 = {"error": "%s: %s" % (type(err).__name__, err)}
    if rank != 0:
        return
    line = {
        "metric": "events/s", "value": value, "unit": "events/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": "rock_slab: forward straggled + mixed "
                               "scattering, 1 km StandardRock slab, "
                               "10 GeV-100 TeV, stop at 1 GeV or exit",
                   "events_per_step": n, "parallelism": "replicas",
                   "l2": "inputs (%.2f GB) larger than L2" % (
                       n * 104 / 1E+09)},
        "steps_per_s": world * steps_total / (ms_per_step * 1E-03),
        "steps_per_event": steps_per_event,
        "kernel_ms": last_kernel_ms,
        "event_errors": bad,
        "gpu_launches": args.steps * st["launches"],
        "engine": tuning,
        "e2e": e2e, "roofline": roofline, "cpu_baseline": base,
        "clocks": clocks.summary(),
        "c3": c3, "c4": c4,
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
