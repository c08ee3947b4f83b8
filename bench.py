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
# engine's own executed count over the same events (its four kernels) is
# reported beside it.
F_STEP = 680.4
F_STEP_EXECUTED = 681.7
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum over the four
# pool kernels) per reference step, from ncu on 200 000 rock slab events;
# None until captured.
TRAFFIC_STEP = None


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
    return p.parse_args()


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


def cpu_baseline(n_events, seed, first_event=0):
    """All-core OpenMP run of the C restatement on a bounded sample."""
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
    return {"value": n_events / dt, "unit": "events/s", "cores": threads,
            "kind": "port",
            "steps_per_s": float(r["steps"].sum()) / dt,
            "sample": "%d events of the rock slab workload (first event "
                      "id %d), %.1f s wall on %d OpenMP threads"
                      % (n_events, first_event, dt, threads)}


def run_reference_arm(args, rank, world):
    if rank != 0:
        return
    n = args.cpu_events or 200_000
    vals, steps = [], []
    base = None
    for k in range(args.warmup + args.steps):
        r = cpu_baseline(n, args.seed, first_event=k * n)
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
                         "sample": base["sample"]},
        "e2e": {"value": value, "unit": "events/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_info()
    if args.impl == "reference":
        return run_reference_arm(args, rank, world)

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
                        max_inner=args.max_inner, batch=args.batch)

    n = args.events
    first = rank * 10 ** 12
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
    results = torch.zeros((n, 32), dtype=torch.uint8, device=dev)
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
    ms_per_step = total_ms / args.steps
    if world > 1:
        t = torch.tensor([ms_per_step], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_per_step = float(t.item())
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
        for k in range(1 + args.steps):
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
                    "kernel": "transport of one batch: gp_pool_step, "
                              "gp_pool_del, gp_pool_polar, gp_pool_ehs",
                    "f_step": F_STEP,
                    "f_step_executed": F_STEP_EXECUTED,
                    "peak_source": "measured: DFMA microbenchmark in this "
                                   "process (MEASURED_PEAKS.json has no "
                                   "FP64 figure)"}
    base = None
    if rank == 0 and not args.no_baseline:
        base = cpu_baseline(args.cpu_events or 200_000, args.seed,
                            first_event=first)
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
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
