"""Benchmark of the Flockers continuous-space step (boid-updates/s).

Workload (default): 1,048,576 boids, f32, density 0.025 boids per unit^2
(torus side 6476.34), radius 10, discretization 10/1.5, all weights 1.0,
jump 0.7, uniform positions and unit headings, seed 7.  A "step" is one
Schedule::step of the whole flock: the agent pass (every Bird::step) and the
field's lazy_update, on inputs resident in HBM.  L2 is flushed (a 512 MiB
write) before every timed step; the JSON line says so.

  python bench.py [--steps K] [--warmup W] [--workload flock1m|flock1k|clustered4m] [--impl ours|reference]

--impl reference times the reference-equivalent CPU path (the oracle's
priority-queue schedule, one host core: the reference's sequential path is
single-threaded) on the same workload, a bounded number of steps.
Under torchrun each rank runs an independent replica on its own GPU (the
step does not shard: replicas only) and rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

D_C = float(np.float32(10.0) / np.float32(1.5))
WORKLOADS = {
    # name: (n, side, seed, generator, sim steps of the workload)
    "flock1k": dict(n=1000, side=200.0, seed=42, gen="uniform", steps=200,
               desc="Flockers 1,000 boids, torus 200x200"),
    "flock1m": dict(n=1 << 20, side=float(np.float32(np.sqrt((1 << 20) / 0.025))), seed=7,
               gen="uniform", steps=1000,
               desc="Flockers 1,048,576 boids, density 0.025 (torus side 6476.34)"),
    "clustered4m": dict(n=1 << 22, side=12952.0, seed=11, gen="clustered", steps=500,
               desc="Flockers 4,194,304 boids in 256 Gaussian clusters (sigma 40), torus 12952"),
}
METRIC = "boid-updates/s (1M boids, 1 GB300)"
UNIT = "boid-updates/s"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def bag_count(side, d=D_C):
    """Bags of a square field: (ceil(side/d) + 1)^2 in f32, the bag matrix of
    Field2D::new (field_2d.rs:304-322)."""
    return (int(np.ceil(np.float32(side) / np.float32(d))) + 1) ** 2


def algorithmic_bytes(n, ncells):
    """Algorithmic bytes of one step: the metric's unit figure, 32 B per boid
    (its float4 state read, its next state written) and 8 B per bag (one bag
    offset written and read).  The dominant kernel's roofline divides this
    step figure by its own launch time (one launch processes one step's
    boids and bags).  The per-kernel "impl_bytes" count what each kernel of
    this implementation touches once (ids, keys, counts included)."""
    return {
        "step": n * 32 + ncells * 8,
        "force": n * 44 + ncells * 8,  # record in 20, record + key out 24; offsets in, counts out
        "scan": ncells * 8,            # counts in, offsets out
        "rebin": n * 44 + ncells * 8,  # key + record in 24, record out 20; two offset arrays
    }


def ncu_traffic(kernel):
    """DRAM bytes (read + write) per launch of `kernel` from the committed ncu
    summary of the same workload (profiles/<kernel>_flock1m.md, a line
    `dram_bytes_per_launch: <int>`), or None when there is none."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_flock1m.md")
    if not os.path.exists(p):
        return None
    with open(p) as fh:
        for ln in fh:
            if ln.startswith("dram_bytes_per_launch:"):
                return int(ln.split(":", 1)[1].strip())
    return None


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def gen(wl, src):
    """The workload's seeded flock from `src`: the library (krabmaga_gb300) for
    the GPU arm, the oracle for the CPU arms, so that those never load the GPU
    library.  Both give the same bits (tests/test_workload_gen.py)."""
    if wl["gen"] == "uniform":
        return src.gen_uniform(wl["n"], wl["side"], wl["side"], wl["seed"], 1.0)
    return src.gen_clustered(wl["n"], wl["side"], wl["side"], 256, 40.0, 0.3, wl["seed"])


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def allmax(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_reference(wl, steps, warmup=0):
    """The oracle's reference-equivalent run, `steps` timed steps after
    `warmup` untimed ones: returns (boid-updates/s, sample text)."""
    import oracle

    ids, xy, dxy = gen(wl, oracle)
    p = oracle.params(seed=wl["seed"], query_mode=0)
    secs, _ = oracle.simulate_timed(wl["side"], wl["side"], D_C, p, ids, xy, dxy, steps,
                                    warmup=warmup)
    return wl["n"] * steps / secs, (f"{wl['desc']}, {steps} steps after {warmup} warm-up steps "
                                    f"through the priority-queue schedule (oracle restatement "
                                    f"of the reference, 1 core)")


def cpu_reference_threads(wl, steps, warmup=0):
    """The oracle's run with the agent pass on every host core (not what the
    reference can do: its schedule runs agents one at a time): returns
    (boid-updates/s, threads, sample text)."""
    import oracle

    threads = max(1, os.cpu_count() or 1)
    ids, xy, dxy = gen(wl, oracle)
    p = oracle.params(seed=wl["seed"], query_mode=0)
    secs, _ = oracle.simulate_timed_threads(wl["side"], wl["side"], D_C, p, ids, xy, dxy, steps,
                                            threads, warmup=warmup)
    return wl["n"] * steps / secs, threads, (f"{wl['desc']}, {steps} steps after {warmup} "
                                             f"warm-up steps, agent pass on {threads} host "
                                             f"threads (oracle, not the reference's sequential "
                                             f"schedule)")


def run_sweep(args, dev):
    """Batched exploration sweep: `sweep_reps` replicas (N log-uniform over
    [1024, 65536] at density 0.025, per-replica weights/jump/radius, seed =
    replica index), `sweep_steps` steps of all replicas together, in the
    tiled mode (tile shape from the autotuner) and the separate-kernel mode;
    against running the plain field replica by replica on the same GPU."""
    import torch

    import krabmaga_gb300 as kg
    from krabmaga_gb300 import _lib as L

    reps = kg.sweep_replicas(args.sweep_reps)
    total = sum(r.n for r in reps)
    steps = args.sweep_steps

    def batched(mode):
        b = kg.Batch(reps, device=dev)
        b.set_step_options(mode)
        # the autotuner's trials are real steps of the sweep: the tile shape of
        # the tiled modes, the force block size of the separate kernels
        tx, ty, used, tune_ms = b.autotune(0, 4)
        step = used
        b.step(step, 10, 1, 0)
        step += 10
        b.synchronize()
        stream = torch.cuda.ExternalStream(b.cuda_stream(), device=dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.step(step, steps, 1, 100)  # one launch group per step, 100-step graphs
        e1.record(stream)
        b.synchronize()
        bs = e0.elapsed_time(e1) / 1e3
        step += steps
        one = None
        if mode == 1:
            e0.record(stream)
            b.step(step, steps, steps, 0)  # all steps in one persistent launch
            e1.record(stream)
            b.synchronize()
            one = total * steps / (e0.elapsed_time(e1) / 1e3)
        stats = b.step_stats()
        b.close()
        return {"mode": mode, "value": total * steps / bs, "ms_per_step": 1e3 * bs / steps,
                "autotuned": ({"tile": [tx, ty]} if mode in (1, 2)
                              else {"force_block_threads": tx, "replicas_per_block": ty}),
                "autotune_ms_per_step": tune_ms, "fused": stats,
                "one_launch_value": one}

    runs = [batched(m) for m in (2, 0)]
    best = max(runs, key=lambda r: r["value"])
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    plain_s = 0.0
    for r in reps:  # the plain field's default (fastest) step path
        f = kg.Field2D(r.width, r.height, r.discretization, True, device=dev, capacity_hint=r.n)
        f.set_locations(*r.state)
        f.lazy_update()
        pc = r.params.to_c()
        L.call("kb_flock_step", f.handle, C.byref(pc), C.c_uint64(0), C.c_uint32(2))
        f.synchronize()
        fs = torch.cuda.ExternalStream(f.cuda_stream(), device=dev)
        e0.record(fs)
        L.call("kb_flock_step", f.handle, C.byref(pc), C.c_uint64(2), C.c_uint32(steps))
        e1.record(fs)
        f.synchronize()
        plain_s += e0.elapsed_time(e1) / 1e3
        f.close()
    bv = best["value"]
    pv = total * steps / plain_s
    return {
        "workload": f"{args.sweep_reps} Flockers replicas, N log-uniform [1024, 65536] "
                    f"(total {total}), density 0.025, per-replica weights/jump/radius, "
                    f"{steps} steps",
        "batched_value": bv, "plain_replica_by_replica_value": pv, "speedup": bv / pv,
        "unit": UNIT, "batched_ms_per_step": best["ms_per_step"], "best_mode": best["mode"],
        "modes": runs,
        "launch": "mode 2: tile step + scan per step, CUDA graphs of 100 steps; mode 0: force + "
                  "offsets scan (three launches at this bag count) + rebin (64-bag segments) per "
                  "step over all replicas, CUDA graphs of 100 steps, programmatic dependent "
                  "launch between the kernels",
        "data": "synthetic (seeded)", "l2": "working set larger than L2 (no flush)",
    }


def run_configs(args, dev):
    """The other configurations of the workload table at their own sizes,
    fast arithmetic: C1 (1,000 boids, torus 200, seed 42, 200 steps: one call,
    whole steps on the thread-block cluster path; and end to end from host
    arrays) and C3 (4,194,304 boids in 256 Gaussian clusters, torus 12952,
    seed 11: graph-replayed steps on inputs larger than L2)."""
    import torch

    import krabmaga_gb300 as kg
    from krabmaga_gb300 import _lib as L

    out = {}
    for name, steps in (("flock1k", 200), ("clustered4m", args.c3_steps)):
        wl = WORKLOADS[name]
        ids, xy, dxy = gen(wl, kg)
        p = kg.FlockParams(seed=wl["seed"], arith=kg.KB_ARITH_FAST).to_c()
        f = kg.Field2D(wl["side"], wl["side"], D_C, True, device=dev, capacity_hint=wl["n"])
        f.set_locations(ids, xy, dxy)
        f.lazy_update()
        L.call("kb_flock_step", f.handle, C.byref(p), C.c_uint64(0), C.c_uint32(steps))  # warm-up
        f.synchronize()
        stream = torch.cuda.ExternalStream(f.cuda_stream(), device=dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        L.call("kb_flock_step", f.handle, C.byref(p), C.c_uint64(steps), C.c_uint32(steps))
        e1.record(stream)
        f.synchronize()
        sec = e0.elapsed_time(e1) / 1e3
        entry = {"workload": wl["desc"], "steps": steps, "value": wl["n"] * steps / sec,
                 "unit": UNIT, "ms_per_step": 1e3 * sec / steps, "path": f.step_path(),
                 "candidate_walk": "per-run (dense)" if f.dense_active() else "flat"}
        f.close()
        if name == "flock1k":
            t0 = time.perf_counter()
            g = kg.Field2D(wl["side"], wl["side"], D_C, True, device=dev, capacity_hint=wl["n"])
            g.set_locations(ids, xy, dxy)
            g.lazy_update()
            L.call("kb_flock_step", g.handle, C.byref(p), C.c_uint64(0), C.c_uint32(steps))
            g.get_state()
            t1 = time.perf_counter()
            g.close()
            entry["e2e"] = {"value": wl["n"] * steps / (t1 - t0), "unit": UNIT,
                            "call": f"create + set_locations + lazy_update + {steps} steps + "
                                    f"get_state, host arrays in and out"}
        out[name] = entry
    return out


def run_serving(args, dev):
    """Served request stream: Poisson arrivals (`serve_rate` per second for
    `serve_seconds`), each a Flockers simulation with N log-uniform over
    [1024, 262144], steps uniform in [100, 1000], per-request weights/jump/
    radius and seeds; admitted under a 120 GB HBM budget and `serve_slots`
    slots, merged into batched persistent launches (continuous batching)."""
    import krabmaga_gb300 as kg

    stream = kg.request_stream(args.serve_rate, args.serve_seconds)
    srv = kg.Server(max_slots=args.serve_slots, hbm_budget_bytes=120 << 30,
                    quantum_steps=args.serve_quantum, max_request_boids=262144,
                    max_request_cells=1 << 20, device=dev)
    t0 = time.perf_counter()
    tickets = []
    for ta, req in stream:
        now = time.perf_counter() - t0
        if ta > now:
            time.sleep(ta - now)
        tickets.append(srv.submit(req))
    srv.wait_idle(max(600.0, 10 * args.serve_seconds))
    st = srv.stats()
    srv.close()
    offered = sum(r.nboids * r.steps for _, r in stream) / args.serve_seconds
    return {
        "workload": f"Poisson {args.serve_rate:g} req/s for {args.serve_seconds:g} s "
                    f"({len(stream)} requests), N log-uniform [1024, 262144], steps U[100, 1000]",
        "requests": len(stream), "completed": st["completed"], "failed": st["failed"],
        "p50_latency_s": st["p50_s"], "p99_latency_s": st["p99_s"], "max_latency_s": st["max_s"],
        "aggregate_value": st["boid_updates"] / st["wall_s"] if st["wall_s"] else None,
        "offered_boid_updates_per_s": offered, "unit": UNIT,
        "busy_fraction": st["busy_s"] / st["wall_s"] if st["wall_s"] else None,
        "launches": st["launches"], "repacks": st["repacks"], "max_active": st["max_active"],
        "slots": args.serve_slots, "quantum_steps": args.serve_quantum,
        "latency": "arrival -> final state on the host",
    }


def run_reference(args, wl):
    ws, rank, _ = dist_setup()
    if rank != 0:
        return
    # a bounded sample of the workload: at most ref_steps timed steps after
    # at most ref_warmup warm-up steps, so that the run stays within minutes
    steps = max(1, min(args.steps, args.ref_steps))
    warm = max(0, min(args.warmup, args.ref_warmup))
    value, sample = cpu_reference(wl, steps, warm)
    pv, threads, psample = cpu_reference_threads(wl, steps, warm)
    # rank 0 alone runs the CPU arm (one core), whatever the number of ranks
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1,
        "ranks": ws,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * wl["n"] / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Philox uniform flock)",
        "config": {"workload": wl["desc"], "global_batch": wl["n"], "parallelism": "cpu",
                   "host": platform.machine()},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        # informational: the same restatement with its agent pass on every host core
        "cpu_all_cores": {"value": pv, "unit": UNIT, "cores": threads, "kind": "port",
                          "sample": psample},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, wl):
    import torch

    import krabmaga_gb300 as kg
    from krabmaga_gb300 import _lib as L

    ws, rank, local = dist_setup()
    dev = local
    torch.cuda.set_device(dev)
    n, side = wl["n"], wl["side"]
    ids, xy, dxy = gen(wl, kg)
    params = kg.FlockParams(seed=wl["seed"], query_mode=kg.KB_QUERY_RELAX,
                            arith=kg.KB_ARITH_FAST if args.arith == "fast" else kg.KB_ARITH_STRICT)
    pc = params.to_c()

    f = kg.Field2D(side, side, D_C, True, device=dev, capacity_hint=n)
    tx, ty = (int(v) for v in args.tile.split("x"))
    f.set_step_options(args.mode, tx, ty)
    f.set_locations(ids, xy, dxy)
    f.lazy_update()
    stream = torch.cuda.ExternalStream(f.cuda_stream(), device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{dev}")

    def one_step(t):
        L.call("kb_flock_step", f.handle, C.byref(pc), C.c_uint64(t), C.c_uint32(1))

    step_no = 0
    tuned = None
    if args.mode in (1, 2) and args.tile == "0x0" and not args.profile:
        # the autotuner's trials are real steps of this simulation (warm-up)
        tuned = f.autotune(params, step_no, 4)
        step_no += tuned[2]
    for _ in range(args.warmup):
        one_step(step_no)
        step_no += 1
    f.synchronize()
    if args.profile:  # a short plain run for a profiler: warm-up, then `steps` calls
        if args.phase_clocks:
            L.call("kb_field_phase_clocks", f.handle, C.c_int32(1), None)
        k = max(1, args.profile_call_steps)  # steps per kb_flock_step call
        for _ in range(args.steps):
            L.call("kb_flock_step", f.handle, C.byref(pc), C.c_uint64(step_no), C.c_uint32(k))
            step_no += k
        f.synchronize()
        out = {"profile_run": True, "steps": args.steps, "stats": f.step_stats()}
        if args.phase_clocks:
            clk = (C.c_uint64 * 16)()
            L.call("kb_field_phase_clocks", f.handle, C.c_int32(0), clk)
            names = ["tile_setup", "segments_offsets", "serial_prefix", "stage_wait", "keys",
                     "gather", "force", "hist_flush", "tile_fetch", "barrier1", "scan", "barrier2"]
            ctas = out["stats"]["ctas"] if args.mode == 1 else 1
            # mode 1: per CTA (persistent); mode 2: summed over all tile CTAs
            out["phase_us_per_step"] = {nm: clk[i] / ctas / args.steps / 2070.0
                                        for i, nm in enumerate(names)}
        print(json.dumps(out))
        return

    K = args.steps
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(K)]
    barrier(ws)
    torch.cuda.synchronize(dev)
    with ClockSampler(dev) as clk:
        with torch.cuda.stream(stream):
            for k in range(K):
                flush.fill_(k & 0xFF)  # evict L2 between timed steps
                ev[k][0].record(stream)
                one_step(step_no)  # the whole step (its launches, chained)
                ev[k][1].record(stream)
                step_no += 1
        torch.cuda.synchronize(dev)
    f.synchronize()  # raises if a kernel set the device error word
    barrier(ws)
    step_ms = [ev[k][0].elapsed_time(ev[k][1]) for k in range(K)]
    kernel_ms, kernel_steps = (None, 0)
    if args.mode == 0:
        # Per-kernel durations: the same K steps again (L2 flushed before each)
        # with CUDA events around each launch.  A separate pass, because an
        # event between two launches stops the next one from being scheduled
        # before the previous ends, which the timed steps above do not have.
        f.kernel_times()
        f.set_kernel_timing(True)
        with torch.cuda.stream(stream):
            for k in range(K):
                flush.fill_(k & 0xFF)
                one_step(step_no)
                step_no += 1
        f.synchronize()
        kernel_ms, kernel_steps = f.kernel_times()
        f.set_kernel_timing(False)
    dense = f.dense_active()  # the walk the timed steps used (chosen from the occupancies)
    total_s = allmax(ws, sum(step_ms) / 1e3)
    value = ws * n * K / total_s
    stats = f.step_stats()

    # warm-L2 throughput (no flush, graph-replayed steps), informational
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    warm_steps = min(200, max(10, K))
    with torch.cuda.stream(stream):
        L.call("kb_flock_step", f.handle, C.byref(pc), C.c_uint64(step_no), C.c_uint32(warm_steps))
        step_no += warm_steps
        e0.record(stream)
        L.call("kb_flock_step", f.handle, C.byref(pc), C.c_uint64(step_no), C.c_uint32(warm_steps))
        step_no += warm_steps
        e1.record(stream)
    torch.cuda.synchronize(dev)
    warm_value = n * warm_steps / (e0.elapsed_time(e1) / 1e3)

    # e2e: the public API from host arrays to host arrays, one whole simulation
    e2e_steps = wl["steps"] if not args.e2e_steps else args.e2e_steps
    pinned = [torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).pin_memory()
              for a in (ids, xy, dxy)]
    out_ids = torch.empty(n, dtype=torch.int32).pin_memory()
    out_st = torch.empty((n, 4), dtype=torch.float32).pin_memory()
    e2e_times = []
    for _ in range(args.e2e_reps):
        barrier(ws)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        g = kg.Field2D(side, side, D_C, True, device=dev, capacity_hint=n)
        L.call("kb_field_set_locations", g.handle, C.c_size_t(n),
               C.cast(pinned[0].data_ptr(), L._U32), C.cast(pinned[1].data_ptr(), L._F),
               C.cast(pinned[2].data_ptr(), L._F))
        L.call("kb_field_lazy_update", g.handle)
        L.call("kb_flock_step", g.handle, C.byref(pc), C.c_uint64(0), C.c_uint32(e2e_steps))
        cnt = C.c_size_t()
        L.call("kb_field_get_state", g.handle, C.cast(out_ids.data_ptr(), L._U32),
               C.cast(out_st.data_ptr(), L._F), C.c_size_t(n), C.byref(cnt))
        t1 = time.perf_counter()
        g.close()
        e2e_times.append(allmax(ws, t1 - t0))
    e2e_t = min(e2e_times)
    e2e_value = ws * n * e2e_steps / e2e_t
    h2d = n * (4 + 8 + 8)
    d2h = n * (4 + 16)

    if rank != 0:
        return
    hbm, peak_kind = peaks()
    ab = algorithmic_bytes(n, bag_count(side))
    step_bytes, force_bytes, scan_bytes, rebin_bytes = ab["step"], ab["force"], ab["scan"], ab["rebin"]
    kernels = None
    if kernel_ms is not None and kernel_steps == K:
        fm, sm, rm = (v / K for v in kernel_ms)
        kernels = {"k_flock_force": {"ms_mean": fm, "impl_bytes": force_bytes,
                                     "impl_gbs": force_bytes / fm / 1e6}}
        if sm < 1e-3:  # the offsets scan runs inside the rebin launch
            ob = scan_bytes + rebin_bytes
            kernels["k_offsets_rebin"] = {"ms_mean": sm + rm, "impl_bytes": ob,
                                          "impl_gbs": ob / (sm + rm) / 1e6}
        else:
            kernels["k_scan"] = {"ms_mean": sm, "impl_bytes": scan_bytes,
                                 "impl_gbs": scan_bytes / sm / 1e6}
            kernels["k_rebin"] = {"ms_mean": rm, "impl_bytes": rebin_bytes,
                                  "impl_gbs": rebin_bytes / rm / 1e6}
        kname, kbytes, kms = "k_flock_force", step_bytes, fm
    else:  # tiled modes: the whole step is the measured unit
        kname = {2: "k_tile_step + k_scan (two launches per step)",
                 1: "k_fused (whole step, one launch)", 0: "whole step"}[args.mode]
        kbytes, kms = step_bytes, statistics.mean(step_ms)
    achieved = kbytes / kms / 1e6
    traffic = ncu_traffic(kname) if kernels else None
    clocks = clk.summary()

    configs = run_configs(args, dev) if (args.c3_steps > 0 and ws == 1) else None
    sweep = run_sweep(args, dev) if (args.sweep_reps > 0 and ws == 1) else None
    serving = run_serving(args, dev) if (args.serve_seconds > 0 and ws == 1) else None

    cpu = None
    if not args.no_cpu_baseline and ws == 1:
        cwarm = max(0, min(args.warmup, args.ref_warmup))
        cval, sample = cpu_reference(wl, args.cpu_steps, cwarm)
        pv, threads, psample = cpu_reference_threads(wl, args.cpu_steps, cwarm)
        cpu = {"value": cval, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample,
               "all_cores": {"value": pv, "cores": threads, "sample": psample}}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K,
        "warmup": args.warmup, "ms_per_step": total_s * 1e3 / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Philox uniform flock)",
        "config": {"workload": wl["desc"], "global_batch": n * ws, "seq_len": None,
                   "parallelism": f"replicas{ws}", "arith": args.arith, "query": "relax",
                   "l2": "flushed (512 MiB write) before every timed step",
                   "kernel_timing": "per-launch CUDA events over a second pass of the same "
                                    "K steps (L2 flushed before each)",
                   "candidate_walk": "per-run (dense)" if dense else "flat",
                   "warm_l2_value": warm_value},
        "roofline": {"bound": "hbm", "kernel": kname,
                     "achieved": achieved, "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic,
                     "algorithmic_bytes_per_launch": kbytes, "launch_ms_mean": kms,
                     "kernels": kernels,
                     "step_bytes": step_bytes, "step_ms_mean": statistics.mean(step_ms),
                     "step_ms_median": statistics.median(step_ms),
                     "step_frac": step_bytes / (statistics.mean(step_ms) / 1e3) / 1e9 / hbm,
                     "fused": stats, "autotuned": tuned},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d / e2e_steps,
                "d2h_bytes_per_step": d2h / e2e_steps, "h2d_bytes_per_call": h2d,
                "d2h_bytes_per_call": d2h,
                "call": f"Field2D create + set_locations + lazy_update + {e2e_steps} steps + "
                        f"get_state, host arrays in and out"},
        # per step: force + tile sums + offsets + rebin (mode 0); plus, in mode 0, the
        # bag-occupancy measurement that the field launches every 64 steps
        "gpu_launches": K * ({2: 3, 1: 1}.get(args.mode) or (1 + len(kernels) if kernels else 3))
                        + (((args.warmup + K) // 64 - args.warmup // 64) if args.mode == 0 else 0),
        "configs": configs,
        "sweep": sweep,
        "serving": serving,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--workload", default="flock1m", choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--arith", default="fast", choices=["fast", "strict"])
    ap.add_argument("--cpu-steps", type=int, default=10)
    ap.add_argument("--ref-steps", type=int, default=20)
    ap.add_argument("--ref-warmup", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=0)
    ap.add_argument("--e2e-reps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--tile", default="0x0", help="fused tile shape TXxTY in bags (0x0: automatic)")
    ap.add_argument("--mode", type=int, default=0,
                    help="step path: 0 the default choice (separate kernels on this workload), "
                         "1 persistent tiled, 2 split tiled, 3 separate kernels whatever the size")
    ap.add_argument("--profile", action="store_true", help="short plain run for ncu, no timing")
    ap.add_argument("--profile-call-steps", type=int, default=1,
                    help="with --profile: steps per kb_flock_step call (runs of 2 or more take "
                         "the cluster path on fields of at most 4096 boids)")
    ap.add_argument("--c3-steps", type=int, default=20,
                    help="steps of the C1/C3 configuration runs (0: skip them)")
    ap.add_argument("--sweep-reps", type=int, default=512)
    ap.add_argument("--sweep-steps", type=int, default=500)
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-slots", type=int, default=64)
    ap.add_argument("--serve-quantum", type=int, default=50)
    ap.add_argument("--phase-clocks", action="store_true", help="with --profile: per-phase cycles")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, wl)
    else:
        run_ours(args, wl)


if __name__ == "__main__":
    main()
