#!/usr/bin/env python
"""Benchmark of the OpenABL near() hot path on GB300.

Workload: examples/boids2d.abl with 1,048,576 agents in FP64
(-P num_agents=1048576 -P agent_density=3200.0: about 8 agents per
interaction-radius cell), synthetic seeded state (positions uniform in
[0, L)^2, velocity directions uniform on the circle, speed in [0.5, 1]).
A step is one timestep of the simulate loop: uniform-grid binning of all
agents followed by the update_boid step kernel.

Metric: agent-steps/s.  `value` is device time of K timesteps with the state
resident in HBM and L2 flushed between timesteps; `e2e` runs the same steps
through the C ABI with the state copied from pinned host memory before and
back after every timestep.  `--impl reference` times the reference
algorithm (the `c` backend's brute-force near loop, CPrinter.cpp:148-173,
restated in oracle/) on the host cores instead.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

CONFIG = "boids2d_1m"
METRIC = "agent-steps/s (1M boids2d fp64)"
BYTES_PER_AGENT_STEP = 80        # SoA pos+vel read + written, binning key/id written + read
FP64_FLOP_PER_AGENT_STEP = 560   # ~72 candidates x 5 + ~25 in-radius x 8 FP64 ops


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_reference_sample(state, consts, target_seconds, n_total):
    """Brute-force reference step (every agent scans all agents) on a bounded
    sample of agents, all host threads.  Returns (agent-steps/s, sample, cores)."""
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    count = 512
    t0 = time.perf_counter()
    O.boids2d_step(state, consts, mode=0, nthreads=cores, first=0, count=count)
    dt = time.perf_counter() - t0
    count = int(max(count, min(n_total, count * target_seconds / max(dt, 1e-6))))
    t0 = time.perf_counter()
    O.boids2d_step(state, consts, mode=0, nthreads=cores, first=0, count=count)
    dt = time.perf_counter() - t0
    return count / dt, count, cores, dt


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.file,
                stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.file.flush()
        self.file.seek(0)
        rows = [r.split(",") for r in self.file.read().strip().splitlines() if r.strip()]
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            if len(r) < 9:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(rows)}


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    import openabl_gb300.workloads as W
    cfg = json.load(open(os.path.join(REPO, "openabl_gb300", "generated", "configs.json")))[CONFIG]
    g = cfg["globals"]
    n = int(g["num_agents"])
    state = W.boids2d(n, float(g["max_pos"]), seed=0)
    from oracle import oracle as O
    consts = {k: float(g[k]) for k in O.BOIDS2D_KEYS}
    per_step = max(1.0, 60.0 / max(1, args.steps + args.warmup))
    for _ in range(args.warmup):
        cpu_reference_sample(state, consts, min(per_step, 2.0), n)
    rates = []
    sample = 0
    cores = os.cpu_count()
    for _ in range(args.steps):
        r, sample, cores, _ = cpu_reference_sample(state, consts, per_step, n)
        rates.append(r)
    value = statistics.mean(rates)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "agent-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * n / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, uniform positions)",
        "config": {"workload": "boids2d 1,048,576 agents FP64, agent_density 3200.0",
                   "agents": n, "l2": "n/a (host)"},
        "cpu_baseline": {"value": value, "unit": "agent-steps/s", "cores": cores, "kind": "port",
                         "sample": f"brute-force near loop (reference c backend algorithm, "
                                   f"oracle/abl_oracle.c) for {sample} of {n} agents per step"},
        "e2e": {"value": value, "unit": "agent-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_ours(args):
    import numpy as np
    import torch
    import openabl_gb300 as o
    import openabl_gb300.workloads as W

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    model, g = o.globals_for_config(CONFIG)
    n = g.get("num_agents")
    state = W.boids2d(n, g.get("max_pos"), seed=rank)
    sim = o.Simulation(model, g)
    sim.upload("Boid", state)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # warm-up (graph capture included)
    sim.run(max(3, args.warmup))
    for _ in range(args.warmup):
        flush.zero_()
        torch.cuda.synchronize()
        sim.step()

    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    times, launches = [], 0
    for _ in range(args.steps):
        flush.zero_()                 # evict the state from L2 between timesteps
        torch.cuda.synchronize()
        sim.step()
        times.append(sim.last_exec_time())
        launches += sim.last_launch_count()
    barrier()
    clock_info = clocks.stop()
    total = sum(times)
    if world > 1:
        t = torch.tensor([total], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total = float(t.item())
    value = world * n * args.steps / total

    # graph replay of the same timesteps, back to back (no flush)
    sim.run(args.steps)
    graph_rate = n * args.steps / sim.last_exec_time()

    # dominant kernel: update_boid, timed with events on the runtime's stream
    sim.set_profiling(True)
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        sim.step()
    ksec, klaunch = sim.step_kernel_time(0)
    sim.set_profiling(False)
    kernel_s = ksec / max(1, klaunch)
    peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(REPO, "MEASURED_PEAKS.json")) else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    achieved_gbs = BYTES_PER_AGENT_STEP * n / kernel_s / 1e9
    dfma, dadd, dmul = o.runtime.fp64_rates()
    fp64_peak_tflops = 2 * dfma / 1e12
    achieved_fp64 = FP64_FLOP_PER_AGENT_STEP * n / kernel_s / 1e12

    # end to end through the C ABI: pinned host state in, step, state out
    pin = {k: torch.from_numpy(v).pin_memory().numpy() for k, v in state.items()}
    out = {k: torch.empty(v.shape, dtype=torch.float64).pin_memory().numpy()
           for k, v in state.items()}
    e2e_steps = max(3, args.steps // 2)
    sim.upload("Boid", pin)
    sim.step()
    sim.download("Boid", out)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sim.upload("Boid", pin)
        sim.step()
        sim.download("Boid", out)
    e2e_wall = time.perf_counter() - t0
    e2e_value = world * n * e2e_steps / e2e_wall
    h2d = sum(v.nbytes for v in pin.values())

    cpu = None
    if rank == 0:
        from oracle import oracle as O
        consts = {k: g.get(k) for k in O.BOIDS2D_KEYS}
        rate, sample, cores, dt = cpu_reference_sample(state, consts, args.cpu_seconds, n)
        cpu = {"value": rate, "unit": "agent-steps/s", "cores": cores, "kind": "port",
               "sample": f"brute-force near loop (reference c backend algorithm restated in "
                         f"oracle/abl_oracle.c) for {sample} of {n} agents, {dt:.1f} s"}
    sim.close()
    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "value": value, "unit": "agent-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded: uniform positions, unit-circle headings, speed U[0.5,1])",
        "config": {"workload": "boids2d 1,048,576 agents FP64, agent_density 3200.0, "
                               "per-step bit-exact", "agents": n, "cell": "0.05 (+2^-10)",
                   "l2": "flushed (256 MB write) before every timed timestep",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "graph_replay_value": graph_rate,
        "e2e": {"value": e2e_value, "unit": "agent-steps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": h2d},
        "roofline": {"bound": "hbm", "kernel": "update_boid", "achieved": achieved_gbs,
                     "peak": hbm_peak, "unit": "GB/s", "frac": achieved_gbs / hbm_peak,
                     "traffic": None, "bytes_per_agent": BYTES_PER_AGENT_STEP,
                     "kernel_ms": kernel_s * 1e3, "peak_source": "measured (MEASURED_PEAKS.json)"},
        "fp64": {"achieved_tflops": achieved_fp64, "peak_tflops": fp64_peak_tflops,
                 "frac": achieved_fp64 / fp64_peak_tflops,
                 "flop_per_agent": FP64_FLOP_PER_AGENT_STEP,
                 "peak_source": "measured DFMA rate (abl_diag_fp64_rates)",
                 "dadd_per_s": dadd, "dmul_per_s": dmul},
        "gpu_launches": launches,
        "clocks": clock_info,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
