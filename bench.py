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
# FP64 instructions per agent executed by update_boid on this workload (ncu
# smsp__sass_thread_inst_executed_op_d{add,mul,fma}_pred_on, one launch, per
# agent).  The FP32 band decides most radius tests without FP64; FP64 sums
# issue as fused multiply-adds with a multiplier of one.
UPDATE_BOID_FP64_INSTR = {"dadd": 1, "dmul": 18, "dfma": 129}
# DRAM bytes of one update_boid launch on this workload (ncu capture, L2 cold
# as in the timed steps, which flush L2 first).
UPDATE_BOID_DRAM_BYTES = 240.00e6
# game_of_life 4096^2 step kernel with kept neighbour lists: algorithmic bytes
# per cell and timestep, and ncu's DRAM bytes for one launch
GOL_BYTES_PER_CELL = 41
GOL_DRAM_BYTES_4096 = 671.98e6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the ensemble and precision measurements")
    ap.add_argument("--ensemble-replicas", type=int, default=256)
    ap.add_argument("--ensemble-steps", type=int, default=200)
    ap.add_argument("--ensemble-only", action="store_true",
                    help="print only the ensemble measurement, graph replay and persistent, "
                         "without the replica-by-replica baseline (for profiling)")
    ap.add_argument("--ensemble-no-autotune", action="store_true",
                    help="run the ensemble with its default launch configuration")
    ap.add_argument("--serve-jobs", type=int, default=48)
    ap.add_argument("--serve-slots", type=int, default=8)
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def slowest_rank_seconds(total, world, device="cuda"):
    """Time of the whole job: every rank times the same K timesteps of its
    own replica; the job takes as long as its slowest rank."""
    if world <= 1:
        return total
    import torch
    import torch.distributed as dist
    t = torch.tensor([total], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, agents, steps, seconds):
    """Agent-steps per second of the whole job: each of `world` ranks
    advances its own replica of `agents` agents by `steps` timesteps."""
    return world * agents * steps / seconds


def cpu_reference_sample(state, consts, target_seconds, n_total):
    """Brute-force reference step (every agent scans all agents: the `c`
    backend's near loop, CPrinter.cpp:148-173) on a bounded sample of agents,
    all host threads.  Returns (agent-steps/s, sample, cores, seconds)."""
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


def cpu_whole_steps(step, state, agents, target_seconds, max_steps=1000):
    """Whole timesteps of a CPU oracle step function `step(state) -> state`
    (all host threads), repeated until `target_seconds` have passed.
    Returns (agent-steps/s, timesteps, seconds)."""
    t0 = time.perf_counter()
    k = 0
    while k < max_steps:
        state = step(state)
        k += 1
        if time.perf_counter() - t0 >= target_seconds:
            break
    dt = time.perf_counter() - t0
    return agents * k / dt, k, dt


def binned_cpu_baseline(kind_label, step, state, agents, target_seconds):
    """`cpu_baseline` object for a CPU oracle timed on whole timesteps."""
    rate, k, dt = cpu_whole_steps(step, state, agents, target_seconds)
    return {"value": rate, "unit": "agent-steps/s", "cores": os.cpu_count() or 1,
            "kind": "port",
            "sample": f"{kind_label}: {k} whole timesteps of all {agents} agents from the "
                      f"initial state, {dt:.1f} s, all host threads"}


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
                 "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.file,
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


def measure_ensemble(args, o, W, np):
    """Form (2): boids2d replicas in FP32 with log-uniform agent counts in
    [1e3, 2e5] and steer/match/collision weights within +-20% of the file's,
    one seed each, run as one ensemble (segmented grid, graph replay,
    autotuned launch configuration) against the same replicas run one after
    another through the plain single-model path; and the same ensemble run
    as one persistent cooperative launch for all its timesteps."""
    model, base = o.globals_for_config("boids2d_float_4096")
    gl, states, seeds = W.boids2d_ensemble(model, base, replicas=args.ensemble_replicas,
                                           n_min=1000, n_max=200000, seed=0)
    states = [{k: v.astype(np.float32) for k, v in s.items()} for s in states]
    total = sum(len(s["pos"]) for s in states)
    T = args.ensemble_steps
    tune = (lambda e: e.tuning()) if args.ensemble_no_autotune else (lambda e: e.autotune(3))
    ens = o.Ensemble(model, gl, seeds=seeds)
    ens.upload("Boid", states)
    tuning = tune(ens)
    ens.run(3)
    ens.upload("Boid", states)
    ens.run(T)
    ens_s = ens.last_exec_time()
    launches = ens.last_launch_count()
    final = ens.download("Boid")
    ens.close()
    # The same run as one persistent cooperative launch (its own autotune).
    pe = o.Ensemble(model, gl, seeds=seeds)
    pe.set_persistent(True)
    pe.upload("Boid", states)
    p_tuning = tune(pe)
    pe.run(3)
    pe.upload("Boid", states)
    pe.run(T)
    pers_s = pe.last_exec_time()
    pers = {"value": total * T / pers_s, "seconds": pers_s,
            "gpu_launches": pe.last_launch_count(), "blocks": pe.persistent_blocks(),
            "tuning": p_tuning,
            # per phase of the first timesteps: assign, cell scan (2), scatter,
            # sort, gather, list merge, step; block 0's clock at each barrier
            "phase_ms_first": [round(x * 1e3, 4) for x in pe.phase_times(24)],
            "equal_to_per_phase_run": all(np.array_equal(a[k], b[k])
                                          for a, b in zip(pe.download("Boid"), final)
                                          for k in a)}
    pe.close()
    base_s = 0.0
    base_launches = 0
    if getattr(args, "ensemble_only", False):
        # profiling runs: the ensemble's two ways only, not the replicas one
        # by one (which would add T x 15 launches per replica)
        return {"value": total * T / ens_s, "seconds": ens_s, "gpu_launches": launches,
                "tuning": tuning, "persistent": pers}
    for g, st in zip(gl, states):
        sim = o.Simulation(model, g)
        sim.upload("Boid", st)
        sim.run(2)
        sim.upload("Boid", st)
        sim.run(T)
        base_s += sim.last_exec_time()
        base_launches += sim.last_launch_count()
        sim.close()
    return {"workload": f"{args.ensemble_replicas} boids2d replicas FP32, agents log-uniform "
                        f"1e3-2e5 (total {total}), weights +-20%, {T} timesteps",
            "value": total * T / ens_s, "unit": "agent-steps/s", "seconds": ens_s,
            "gpu_launches": launches, "tuning": tuning,
            "persistent": pers,
            "baseline_value": total * T / base_s, "baseline_seconds": base_s,
            "baseline_gpu_launches": base_launches,
            "baseline": "same replicas one after another, each in its own context",
            "speedup": base_s / ens_s}


def measure_precision(args, o, W, np, steps=100):
    """Form (1): the use_float model (all agent arithmetic in FP32, as
    LIBABL_USE_FLOAT) against FP64 on the 1M boids2d workload."""
    m64, g64 = o.globals_for_config(CONFIG)
    m32, g32 = o.globals_for_config("boids2d_float_1m")
    n = g64.get("num_agents")
    st = W.boids2d(n, g64.get("max_pos"), seed=0)
    a = o.Simulation(m64, g64)
    a.upload("Boid", st)
    a.run(steps)
    t64 = a.last_exec_time()
    r64 = a.download("Boid")
    a.close()
    b = o.Simulation(m32, g32)
    b.upload("Boid", {k: v.astype(np.float32) for k, v in st.items()})
    b.run(steps)
    t32 = b.last_exec_time()
    r32 = b.download("Boid")
    b.close()
    L = g64.get("max_pos")
    dp = np.abs(r32["pos"].astype(np.float64) - r64["pos"]).max(axis=1) / L
    # boundPosition moves an agent leaving the domain to the opposite side, so
    # also measure the error up to that jump (minimum image).
    d = np.abs(r32["pos"].astype(np.float64) - r64["pos"])
    dpi = np.minimum(d, np.abs(L - d)).max(axis=1) / L
    dv = np.abs(r32["velocity"].astype(np.float64) - r64["velocity"]).max(axis=1)
    # The mixed form (-C cuda.precision=mixed): FP64 state and arithmetic,
    # near-loop sums of neighbour members in FP32.
    mm, gm = o.globals_for_config("boids2d_mixed_1m")
    c = o.Simulation(mm, gm)
    c.upload("Boid", st)
    c.run(steps)
    tmx = c.last_exec_time()
    rmx = c.download("Boid")
    c.close()
    dm = np.abs(rmx["pos"] - r64["pos"])
    dmi = np.minimum(dm, np.abs(L - dm)).max(axis=1) / L
    dmv = np.abs(rmx["velocity"] - r64["velocity"]).max(axis=1)
    mixed = {"value": n * steps / tmx, "unit": "agent-steps/s",
             "speedup_vs_fp64": t64 / tmx,
             "pos_rel_err_min_image_max": float(dmi.max()),
             "pos_rel_err_min_image_median": float(np.median(dmi)),
             "pos_rel_err_min_image_p99": float(np.quantile(dmi, 0.99)),
             "frac_agents_min_image_err_le_1e-5": float((dmi <= 1e-5).mean()),
             "vel_abs_err_max": float(dmv.max()), "vel_abs_err_median": float(np.median(dmv)),
             "form": "FP64 state, integration and radius tests; near-loop sums of neighbour "
                     "positions (as offsets from the agent) and velocities in FP32"}
    return {"workload": f"boids2d {n} agents, {steps} timesteps, FP32 (use_float) vs FP64",
            "mixed": mixed,
            "fp32_value": n * steps / t32, "fp64_value": n * steps / t64, "unit": "agent-steps/s",
            "pos_rel_err_max": float(dp.max()), "pos_rel_err_median": float(np.median(dp)),
            "pos_rel_err_p99": float(np.quantile(dp, 0.99)),
            "vel_abs_err_median": float(np.median(dv)),
            "frac_agents_rel_err_le_1e-5": float((dp <= 1e-5).mean()),
            "pos_rel_err_min_image_max": float(dpi.max()),
            "frac_agents_min_image_err_le_1e-5": float((dpi <= 1e-5).mean()),
            "error_metric": "per agent max |pos32 - pos64| / max_pos"}


def measure_serving(args, o, W, np):
    """Form (5): a Poisson stream (200 jobs/s) of circle, circle3d, boids2d and
    predator_prey simulations, agents log-uniform in [1e3, 1e6], timesteps
    uniform in [50, 1000], FP32/FP64 50/50, admitted by an 80 GB device-memory
    budget into `slots` concurrent workers.  Latency = completion - arrival."""
    stream = W.serving_stream(jobs=args.serve_jobs, rate=200.0, seed=0)
    prepared = [(t, W.served_job(m, n, prec, seed=k), steps, n, m, prec)
                for k, (t, m, n, steps, prec, seed) in enumerate(stream)]
    srv = o.Server(slots=args.serve_slots, hbm_budget=80 * 10**9)
    ids = []
    t0 = time.perf_counter()
    for t_arr, (model, g, state), steps, n, m, prec in prepared:
        delay = t0 + t_arr - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        ids.append((srv.submit(model, g, state, steps, seed=len(ids)), n, steps, m, prec))
    for jid, *_ in ids:
        srv.wait(jid, timeout=1800.0)
    infos = [srv.info(jid) for jid, *_ in ids]
    srv.close()
    lat = np.array([i["done"] - i["submit"] for i in infos])
    wait = np.array([i["admit"] - i["submit"] for i in infos])
    # Where the time goes, per model: the jobs' device time in timesteps and
    # their time in a slot (admission to completion), summed.
    per_model = {}
    for (jid, n, steps, m, prec), i in zip(ids, infos):
        d = per_model.setdefault(m, {"jobs": 0, "agent_steps": 0, "device_s": 0.0, "slot_s": 0.0})
        d["jobs"] += 1
        d["agent_steps"] += n * steps
        d["device_s"] += i["exec_s"]
        d["slot_s"] += i["done"] - i["admit"]
    first = min(i["submit"] for i in infos)
    last = max(i["done"] for i in infos)
    work = sum(n * steps for _, n, steps, _, _ in ids)
    failed = sum(1 for i in infos if i["status"] != 2)
    arrivals = max(t for t, *_ in prepared) - min(t for t, *_ in prepared)
    # The plain path on the same jobs: one after another, each in its own
    # context (upload, run, download), wall clock.
    tp = time.perf_counter()
    for _, (model, g, state), steps, n, m, prec in prepared:
        sim = o.Simulation(model, g)
        for tname, cols in state.items():
            sim.upload(tname, cols)
        sim.run(steps)
        for tname in state:
            sim.download(tname)
        sim.close()
    plain_s = time.perf_counter() - tp
    return {"workload": f"{len(ids)} jobs, Poisson 200/s, circle/circle3d/boids2d/predator_prey, "
                        "agents log-uniform 1e3-1e6, timesteps U[50,1000], FP32/FP64 50/50, "
                        f"80 GB budget, {args.serve_slots} slots",
            "value": work / (last - first), "unit": "agent-steps/s",
            "offered_agent_steps_per_s": work / max(arrivals, 1e-9),
            "arrival_span_s": arrivals,
            "plain_serial_value": work / plain_s, "plain_serial_seconds": plain_s,
            "speedup_vs_plain_serial": plain_s / (last - first),
            "latency_p50_s": float(np.percentile(lat, 50)),
            "latency_p99_s": float(np.percentile(lat, 99)),
            "queue_wait_p50_s": float(np.percentile(wait, 50)),
            "makespan_s": last - first, "jobs": len(ids), "failed": failed,
            "per_model": per_model}


def measure_other_workloads(args, o, W, np):
    """The other hot-path configurations: circle 4,000 agents (the reference's
    CPU-sized case), game_of_life 4096 x 4096 with 50% alive, boids (3D) with
    1,048,576 agents, sugarscape on a 1024 x 1024 grid, and predator_prey
    with 800,000 prey + 200,000 predators (+ 1,000,000 grass) for 500
    timesteps in FP64 and FP32."""
    import sys as _sys
    _sys.path.insert(0, os.path.join(REPO, "tests"))
    out = {}
    # circle, 4000 agents, 100 timesteps (reference init from the golden case)
    from golden_io import load_case
    meta, st = load_case("circle_4000")
    model, g = o.globals_for_config("circle_4000")
    sim = o.Simulation(model, g)
    sim.upload("Point", st)
    sim.run(3)
    sim.upload("Point", st)
    sim.run(100)
    out["circle_4000"] = {"value": 4000 * 100 / sim.last_exec_time(), "unit": "agent-steps/s",
                          "ms_per_step": sim.last_exec_time() * 10.0}
    sim.close()
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    cc = {"r": g.get("r"), "k_rep": g.get("k_rep"), "k_att": g.get("k_att"), "W": g.get("W")}
    out["circle_4000"]["cpu_baseline"] = binned_cpu_baseline(
        "brute-force near loop (the reference c backend's algorithm, oracle/abl_oracle.c "
        "mode 0)", lambda s_: O.circle_step(s_, cc, mode=0, nthreads=cores), st, 4000, 3.0)
    # game of life 4096^2, 50% live, 100 timesteps
    model, g = o.globals_for_config("game_of_life_4096")
    st = W.game_of_life(g.get("size"), 0.5, seed=0)
    sim = o.Simulation(model, g)
    sim.upload("Cell", st)
    sim.run(3)
    sim.upload("Cell", st)
    sim.run(100)
    n = len(st["alive"])
    out["game_of_life_4096"] = {"value": n * 100 / sim.last_exec_time(), "unit": "agent-steps/s",
                                "ms_per_step": sim.last_exec_time() * 10.0}
    # its step kernel against HBM: per cell 40 B read (position 16, alive and
    # the double buffer's alive 2, list offset 4, nine int16 list entries 18)
    # and 1 B written; neighbours' alive bytes come from L1/L2
    sim.set_profiling(True)
    sim.run(20)
    ksec, klaunch = sim.step_kernel_time(0)
    sim.set_profiling(False)
    kernel_s = ksec / max(1, klaunch)
    peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(REPO, "MEASURED_PEAKS.json")) else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    gbs = GOL_BYTES_PER_CELL * n / kernel_s / 1e9
    out["game_of_life_4096"]["roofline"] = {
        "bound": "hbm", "kernel": "step_move", "achieved": gbs, "peak": hbm_peak, "unit": "GB/s",
        "frac": gbs / hbm_peak, "kernel_ms": kernel_s * 1e3, "bytes_per_agent": GOL_BYTES_PER_CELL,
        "traffic": GOL_DRAM_BYTES_4096,
        "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch"}
    sim.close()
    gc = {"radius": g.get("radius"), "size": g.get("size")}
    out["game_of_life_4096"]["cpu_baseline"] = binned_cpu_baseline(
        "binned CPU oracle (oracle/abl_oracle.c mode 1)",
        lambda s_: O.game_of_life_step(s_, gc, mode=1, nthreads=cores), st, n, 5.0)
    # boids (3D), 1,048,576 agents (~9 per interaction cell), and sugarscape
    # on a 1024 x 1024 grid, 100 timesteps each
    for name, cfg, agent, make in (
            ("boids3d_1m", "boids3d_1m", "Boid",
             lambda g: W.boids3d(g.get("num_agents"), g.get("max_pos"), seed=0)),
            ("sugarscape_1m", "sugarscape_1m", "Agent",
             lambda g: W.sugarscape(g.get("grid_width"), g.get("occupiedFrac"), seed=0))):
        model, g = o.globals_for_config(cfg)
        st = make(g)
        sim = o.Simulation(model, g)
        sim.upload(agent, st)
        sim.run(3)
        sim.upload(agent, st)
        sim.run(100)
        n = len(st["pos"])
        out[name] = {"value": n * 100 / sim.last_exec_time(), "unit": "agent-steps/s",
                     "ms_per_step": sim.last_exec_time() * 10.0, "agents": n}
        sim.close()
        if name == "boids3d_1m":
            bc = {k: g.get(k) for k in O.BOIDS2D_KEYS}
            stepf = (lambda bc_: lambda s_: O.boids3d_step(s_, bc_, mode=1, nthreads=cores))(bc)
        else:
            sg = O.Sugarscape(st, radius=g.get("radius"), grid_width=float(g.get("grid_width")),
                              nthreads=cores)
            stepf = (lambda sg_: lambda s_: sg_.step())(sg)
        out[name]["cpu_baseline"] = binned_cpu_baseline(
            "binned CPU oracle (oracle/abl_oracle.c mode 1)", stepf, st, n, 5.0)
    # predator_prey, 500 timesteps, FP64 and FP32
    from pp_setup import case
    cfg, st, consts = case("predator_prey_1m")
    res = {}
    for name in ("predator_prey", "predator_prey_float"):
        model = o.Model(name)
        g = model.default_globals().update(cfg["globals"])
        sim = o.Simulation(model, g)
        sim.set_seed(1)
        fd = np.float32 if model.float_bytes == 4 else np.float64
        for t, cols in st.items():
            sim.upload(t, {k: (v.astype(fd) if v.dtype.kind == "f" else v)
                           for k, v in cols.items()})
        sim.run(500)
        rows = [list(map(float, r.split(","))) for r in sim.log_text().strip().splitlines()]
        agents = sum(r[0] + r[1] for r in rows) + 1e6 * len(rows)  # prey + predators + grass
        res[name] = {"seconds": sim.last_exec_time(), "rows": rows}
        out[name + "_1m"] = {"value": agents / sim.last_exec_time(), "unit": "agent-steps/s",
                             "ms_per_step": sim.last_exec_time() * 2.0,
                             "final_prey": rows[-1][0], "final_predators": rows[-1][1],
                             "final_grass_available": rows[-1][2]}
        sim.close()
    a = np.array(res["predator_prey"]["rows"])[:, :3]
    b = np.array(res["predator_prey_float"]["rows"])[:, :3]
    rel = np.abs(a - b) / np.maximum(a, 1)
    out["predator_prey_fp32_vs_fp64"] = {
        "metric": "relative difference of the per-timestep counts (prey, predators, available "
                  "grass) between the FP32 and FP64 runs",
        "max_at_step_100": float(rel[:100].max()), "max_over_500": float(rel.max())}
    out["predator_prey_fp32_vs_fp64"].update(pp_agent_error(o, np, cfg, st))
    # CPU baselines: the oracle's restatement (the reference `c` backend
    # refuses this model), binned, all host threads, whole timesteps
    for name, cls in (("predator_prey_1m", O.PredatorPrey),
                      ("predator_prey_float_1m", O.PredatorPreyF32)):
        st_ = st
        if cls is O.PredatorPreyF32:
            st_ = {t: {k: (v.astype(np.float32) if v.dtype.kind == "f" else v)
                       for k, v in d.items()} for t, d in st.items()}
        ref = cls(st_, consts, seed=1)
        t0 = time.perf_counter()
        k, agent_steps = 0, 0
        while True:
            agent_steps += sum(ref._fn("oracle_pp_count")(ref.h, i) for i in range(3))
            ref.run(1, mode=1, nthreads=cores)
            k += 1
            if time.perf_counter() - t0 >= 5.0:
                break
        dt = time.perf_counter() - t0
        ref.close()
        out[name]["cpu_baseline"] = {
            "value": agent_steps / dt, "unit": "agent-steps/s", "cores": cores, "kind": "port",
            "sample": f"binned CPU restatement (oracle/abl_oracle.c predator_prey): {k} whole "
                      f"timesteps from the initial state, {dt:.1f} s, all host threads"}
    return out


def pp_agent_error(o, np, cfg, st, steps=100):
    """Per-animal error of the FP32 predator_prey run against the FP64 run.

    Births and deaths are decided by comparisons, so after the first flipped
    comparison the two populations differ and agents can no longer be
    matched by index.  Each FP32 animal is therefore matched to the nearest
    FP64 animal of its type (scipy cKDTree; animals are ~1/40 of the domain
    apart, far more than the FP32 error); the error is that distance over
    env_size.  Animals born or killed in one run only find a farther partner,
    so the distribution's tail includes them: the median and p99 describe
    the arithmetic, the maximum the population differences."""
    from scipy.spatial import cKDTree
    sims = []
    for name in ("predator_prey", "predator_prey_float"):
        model = o.Model(name)
        g = model.default_globals().update(cfg["globals"])
        sim = o.Simulation(model, g)
        sim.set_seed(1)
        fd = np.float32 if model.float_bytes == 4 else np.float64
        for t, cols in st.items():
            sim.upload(t, {k: (v.astype(fd) if v.dtype.kind == "f" else v)
                           for k, v in cols.items()})
        sims.append(sim)
    L = float(cfg["globals"]["env_size"])
    errs = {}
    for t in range(1, steps + 1):
        for sim in sims:
            sim.step()
        if t not in (1, 10, 100) and t != steps:
            continue
        d, counts = [], {}
        for ty in ("Predator", "Prey"):
            a = sims[0].download(ty)["pos"]
            b = sims[1].download(ty)["pos"].astype(np.float64)
            counts[ty] = [len(a), len(b)]
            if len(a) and len(b):
                d.append(cKDTree(a).query(b, k=1)[0] / L)
        d = np.concatenate(d) if d else np.zeros(1)
        errs[f"step_{t}"] = {"pos_rel_err_median": float(np.median(d)),
                             "pos_rel_err_p99": float(np.quantile(d, 0.99)),
                             "pos_rel_err_max": float(d.max()),
                             "frac_le_1e-5": float((d <= 1e-5).mean()),
                             "animals_fp64_fp32": counts}
    for sim in sims:
        sim.close()
    return {"agent_error_metric": "per FP32 animal: distance to the nearest FP64 animal of "
                                  "its type / env_size", "agent_error": errs}


def headline_config(n, world):
    """`config` of the headline line, the same for both arms."""
    return {"workload": "boids2d 1,048,576 agents FP64, agent_density 3200.0, "
                        "per-step bit-exact", "agents": n, "cell": "0.05 (+2^-10)",
            "l2": "flushed (256 MB write) before every timed timestep (GPU arm)",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def run_reference(args):
    """The reference's own algorithm for the path -- the `c` backend's
    brute-force near loop (src/backend/CPrinter.cpp:148-173), restated in
    oracle/abl_oracle.c and pinned bit for bit to the reference programs --
    on all host cores.  One whole timestep of 1,048,576 agents is ~10^12
    distance tests, so each step here is a bounded sample: a block of agents
    each scanning all N agents; `ms_per_step` is that sample's wall time and
    `value` the agent-steps per second it achieved."""
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
    per_step = min(10.0, max(1.0, 120.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        cpu_reference_sample(state, consts, min(per_step, 1.0), n)
    secs, samples = [], []
    cores = os.cpu_count()
    for _ in range(args.steps):
        r, sample, cores, dt = cpu_reference_sample(state, consts, per_step, n)
        secs.append(dt)
        samples.append(sample)
    value = sum(samples) / sum(secs)
    mean_sample = int(statistics.mean(samples))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "agent-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * sum(secs) / len(secs), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded: uniform positions, unit-circle headings, speed U[0.5,1])",
        "config": headline_config(n, 1),
        "step_definition": f"one bounded sample: ~{mean_sample} of {n} agents, each scanning "
                           f"all agents (a whole timestep would take {n / value:.0f} s)",
        "cpu_baseline": {"value": value, "unit": "agent-steps/s", "cores": cores, "kind": "port",
                         "sample": f"brute-force near loop (reference c backend algorithm, "
                                   f"oracle/abl_oracle.c), ~{mean_sample} of {n} agents per "
                                   f"step, extrapolated to agent-steps/s"},
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

    if args.ensemble_only:
        print(json.dumps({"ensemble": measure_ensemble(args, o, W, np)}))
        return 0

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

    # Every measured section starts from the initial state, so `value` covers
    # timesteps 1..K of the workload (boids flock over time and later
    # timesteps have more neighbours).
    sim.upload("Boid", state)
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
    total = slowest_rank_seconds(sum(times), world)
    value = job_rate(world, n, args.steps, total)

    # Boids flock over time, so later timesteps have more neighbours: the
    # average over the configuration's whole run (timesteps 1..100) too.
    ts = times
    if args.steps < 100:
        sim.upload("Boid", state)
        ts = []
        for _ in range(100):
            flush.zero_()
            torch.cuda.synchronize()
            sim.step()
            ts.append(sim.last_exec_time())
    run100 = {"value": n * len(ts[:100]) / sum(ts[:100]), "unit": "agent-steps/s",
              "ms_per_step": 1000.0 * sum(ts[:100]) / len(ts[:100]),
              "timesteps": f"1..{len(ts[:100])}, L2 flushed before each"}

    # graph replay of the same timesteps, back to back (no flush)
    sim.upload("Boid", state)
    sim.run(args.steps)
    graph_rate = n * args.steps / sim.last_exec_time()

    # dominant kernel: update_boid, timed with events on the runtime's stream
    sim.upload("Boid", state)
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
    # FP64 floor of the kernel: its executed FP64 instructions, each class at
    # its own measured issue rate (DADD, DMUL, DFMA share the FP64 pipe).
    rate = {"dadd": dadd, "dmul": dmul, "dfma": dfma}
    fp64_floor_s = n * sum(c / rate[k] for k, c in UPDATE_BOID_FP64_INSTR.items())

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
    e2e_serial_value = world * n * e2e_steps / e2e_wall
    h2d = sum(v.nbytes for v in pin.values())

    # The same steps with two requests in flight: two contexts (each its own
    # stream), driven by two host threads through the same C ABI calls, so
    # one context's copies overlap the other's kernels.  Every step still
    # uploads its input from pinned host memory and downloads its result.
    import threading
    lanes = [sim, o.Simulation(model, g)]
    outs = [out] + [{k: torch.empty(v.shape, dtype=torch.float64).pin_memory().numpy()
                     for k, v in state.items()} for _ in lanes[1:]]
    for s_, q_ in zip(lanes, outs):
        s_.upload("Boid", pin)
        s_.step()
        s_.download("Boid", q_)
    same = all(np.array_equal(outs[0][k], q_[k]) for q_ in outs[1:] for k in q_)
    e2e_steps2 = 2 * e2e_steps

    def lane(j):
        for _ in range(j, e2e_steps2, len(lanes)):
            lanes[j].upload("Boid", pin)
            lanes[j].step()
            lanes[j].download("Boid", outs[j])
    barrier()
    t0 = time.perf_counter()
    threads = [threading.Thread(target=lane, args=(j,)) for j in range(len(lanes))]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    e2e_wall2 = time.perf_counter() - t0
    e2e_value = world * n * e2e_steps2 / e2e_wall2
    same = same and all(np.array_equal(outs[0][k], q_[k]) for q_ in outs[1:] for k in q_)
    lanes[1].close()

    forms = {}
    if not args.no_forms:
        forms["ensemble"] = measure_ensemble(args, o, W, np)
        forms["precision"] = measure_precision(args, o, W, np)
        forms["serving"] = measure_serving(args, o, W, np)
        forms["other_workloads"] = measure_other_workloads(args, o, W, np)

    cpu = cpu_bf = None
    if rank == 0:
        from oracle import oracle as O
        consts = {k: g.get(k) for k in O.BOIDS2D_KEYS}
        cores = os.cpu_count() or 1
        cpu = binned_cpu_baseline(
            "binned CPU oracle (oracle/abl_oracle.c mode 1: the reference c backend's "
            "arithmetic and neighbour order, uniform-grid candidates)",
            lambda st: O.boids2d_step(st, consts, mode=1, nthreads=cores), state, n,
            args.cpu_seconds)
        rate_bf, sample, cores, dt = cpu_reference_sample(state, consts, args.cpu_seconds, n)
        cpu_bf = {"value": rate_bf, "unit": "agent-steps/s", "cores": cores, "kind": "port",
                  "sample": f"brute-force near loop (the reference c backend's algorithm, "
                            f"CPrinter.cpp:148-173, restated in oracle/abl_oracle.c): "
                            f"extrapolated from {sample} of {n} agents, {dt:.1f} s"}
    sim.close()
    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "value": value, "unit": "agent-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded: uniform positions, unit-circle headings, speed U[0.5,1])",
        "config": headline_config(n, world),
        "graph_replay_value": graph_rate,
        "timesteps_1_100": run100,
        "e2e": {"value": e2e_value, "unit": "agent-steps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": h2d, "requests_in_flight": len(lanes),
                "one_in_flight_value": e2e_serial_value, "lanes_agree": same},
        "roofline": {"bound": "hbm", "kernel": "update_boid", "achieved": achieved_gbs,
                     "peak": hbm_peak, "unit": "GB/s", "frac": achieved_gbs / hbm_peak,
                     "traffic": UPDATE_BOID_DRAM_BYTES,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one "
                                       "launch, L2 cold",
                     "bytes_per_agent": BYTES_PER_AGENT_STEP,
                     "kernel_ms": kernel_s * 1e3, "peak_source": "measured (MEASURED_PEAKS.json)"},
        "fp64": {"instr_per_agent": UPDATE_BOID_FP64_INSTR,
                 "instr_source": "ncu executed DADD/DMUL/DFMA of one launch / agents",
                 "rates_per_s": rate, "rates_source": "measured (abl_diag_fp64_rates)",
                 "floor_ms": fp64_floor_s * 1e3, "kernel_ms": kernel_s * 1e3,
                 "frac": fp64_floor_s / kernel_s},
        "gpu_launches": launches,
        "clocks": clock_info,
        "cpu_baseline": cpu,
        "cpu_baseline_brute_force": cpu_bf,
        "speedup_vs_cpu_baseline": value / cpu["value"] if cpu else None,
        "e2e_speedup_vs_cpu_baseline": e2e_value / cpu["value"] if cpu else None,
    }
    line.update(forms)
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
