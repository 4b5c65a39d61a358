"""Serving: jobs that run together in the server (overlapping on the device,
admitted as slots and memory free up) give exactly the results they give
alone."""
import numpy as np
import pytest

import openabl_gb300 as o
from openabl_gb300 import workloads

pytestmark = pytest.mark.gpu

JOBS = [("circle", 3000, "fp64", 40), ("boids2d", 8000, "fp32", 60), ("predator_prey", 6000,
        "fp64", 25), ("circle3d", 2000, "fp32", 30), ("boids2d", 20000, "fp64", 35),
        ("predator_prey", 4000, "fp32", 20)]


def run_alone(model, g, state, steps, seed):
    sim = o.Simulation(model, g)
    sim.set_seed(seed)
    for t, cols in state.items():
        sim.upload(t, cols)
    sim.run(steps)
    out = {t: sim.download(t) for t, _ in model.agent_types}
    sim.close()
    return out


def test_results_in_the_mix_equal_results_alone():
    srv = o.Server(slots=4)
    submitted = []
    for k, (m, n, prec, steps) in enumerate(JOBS):
        model, g, state = workloads.served_job(m, n, prec, seed=k)
        jid = srv.submit(model, g, state, steps, seed=100 + k)
        submitted.append((jid, model, g, state, steps, 100 + k))
    for jid, model, g, state, steps, seed in submitted:
        srv.wait(jid)
        got = srv.result(jid)
        want = run_alone(model, g, state, steps, seed)
        for t in want:
            for k in want[t]:
                assert np.array_equal(got[t][k], want[t][k]), (jid, t, k)
        srv.release(jid)
    srv.close()


def test_small_budget_serialises_admission():
    model, g, state = workloads.served_job("boids2d", 50000, "fp64", seed=1)
    srv = o.Server(slots=4, hbm_budget=100 << 20)  # room for one such job (~76 MB) at a time
    ids = [srv.submit(model, g, state, 10) for _ in range(3)]
    for j in ids:
        srv.wait(j)
    info = [srv.info(j) for j in ids]
    assert all(i["status"] == 2 for i in info)
    assert info[1]["admit"] >= info[0]["done"] - 1e-3
    assert info[2]["admit"] >= info[1]["done"] - 1e-3
    srv.close()


def test_batched_small_jobs_equal_results_alone():
    """Small jobs of one model queued behind a busy slot are admitted
    together and run as one ensemble; each completes at its own timestep
    count with the bits it computes alone.  A job above the batching size
    runs in a context of its own."""
    srv = o.Server(slots=1)
    srv.set_batching(64, 10000)
    # the first (large) job holds the one slot while the others queue
    specs = [("boids2d", 300000, "fp64", 60), ("boids2d", 3000, "fp64", 30),
             ("boids2d", 5000, "fp64", 12), ("boids2d", 1200, "fp64", 30),
             ("boids2d", 20000, "fp64", 8), ("boids2d", 800, "fp64", 45),
             ("circle", 2000, "fp64", 20)]
    submitted = []
    for k, (m, n, prec, steps) in enumerate(specs):
        model, g, state = workloads.served_job(m, n, prec, seed=20 + k)
        jid = srv.submit(model, g, state, steps, seed=200 + k)
        submitted.append((jid, model, g, state, steps, 200 + k, n))
    infos = {}
    for jid, model, g, state, steps, seed, n in submitted:
        srv.wait(jid)
        infos[jid] = srv.info(jid)
        got = srv.result(jid)
        want = run_alone(model, g, state, steps, seed)
        for t in want:
            for k in want[t]:
                assert np.array_equal(got[t][k], want[t][k]), (jid, t, k)
        srv.release(jid)
    srv.close()
    small = [infos[s[0]]["admit"] for s in submitted if s[1].name == "boids2d" and s[6] <= 10000]
    assert len(small) == 4 and max(small) - min(small) < 1e-6  # admitted as one batch
