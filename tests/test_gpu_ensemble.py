"""Ensembles: each replica of a batched run equals the same replica run in its
own context, bit for bit, with uneven agent counts and parameter points,
through graph replay and after autotuning."""
import numpy as np
import pytest

import openabl_gb300 as o
from openabl_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("model_name,config", [("boids2d", "boids2d_4096"),
                                                ("boids2d_float", "boids2d_float_4096")])
def test_replicas_equal_separate_contexts(model_name, config):
    model, base = o.globals_for_config(config)
    gl, states, seeds = workloads.boids2d_ensemble(model, base, replicas=12, n_min=300,
                                                   n_max=5000, seed=3)
    fd = np.float32 if model.float_bytes == 4 else np.float64
    states = [{k: v.astype(fd) for k, v in s.items()} for s in states]
    ens = o.Ensemble(model, gl, seeds=seeds)
    ens.upload("Boid", states)
    ens.run(9)
    got = ens.download("Boid")
    for r in range(len(gl)):
        sim = o.Simulation(model, gl[r])
        sim.upload("Boid", states[r])
        sim.run(9)
        want = sim.download("Boid")
        sim.close()
        for k in want:
            assert np.array_equal(got[r][k], want[k]), (r, k)
    ens.close()


def test_autotune_keeps_results():
    model, base = o.globals_for_config("boids2d_4096")
    gl, states, seeds = workloads.boids2d_ensemble(model, base, replicas=8, n_min=500,
                                                   n_max=4000, seed=5)
    a = o.Ensemble(model, gl, seeds=seeds)
    a.upload("Boid", states)
    choice = a.autotune(2)
    assert choice["block"] in (64, 128)
    a.run(5)
    b = o.Ensemble(model, gl, seeds=seeds)
    b.upload("Boid", states)
    b.run(5)
    for ra, rb in zip(a.download("Boid"), b.download("Boid")):
        for k in ra:
            assert np.array_equal(ra[k], rb[k])
    a.close()
    b.close()


@pytest.mark.parametrize("tiling", [0, 256, 1024, 4096])
def test_block_tiling_keeps_results(tiling):
    """The cells-per-block tiling knob (abl_ensemble_set_tiling) changes how
    ordered near loops gather neighbours, never what they compute: every
    setting gives the replicas the bits of separate contexts.  256 entries
    are too few for most blocks, which then fall back to per-agent merging."""
    model, base = o.globals_for_config("boids2d_4096")
    gl, states, seeds = workloads.boids2d_ensemble(model, base, replicas=6, n_min=500,
                                                   n_max=6000, seed=8)
    ens = o.Ensemble(model, gl, seeds=seeds)
    ens.set_tiling(tiling)
    assert ens.tuning()["tiling_entries"] == tiling
    ens.upload("Boid", states)
    ens.run(6)
    got = ens.download("Boid")
    for r in range(len(gl)):
        sim = o.Simulation(model, gl[r])
        sim.upload("Boid", states[r])
        sim.run(6)
        want = sim.download("Boid")
        sim.close()
        for k in want:
            assert np.array_equal(got[r][k], want[k]), (tiling, r, k)
    with pytest.raises(o.AblError):
        ens.set_tiling(100)
    ens.close()
