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


def _prefix_replicas(config, sizes):
    """Replicas cut from a golden case's initial state: the first n agents,
    for each n in sizes, all with the case's globals."""
    import sys, os
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from golden_io import load_case
    meta, st = load_case(config)
    model, g = o.globals_for_config(config)
    tname = model.agent_types[0][0]
    states = [{k: np.ascontiguousarray(v[:n]) for k, v in st.items()} for n in sizes]
    return model, [g] * len(sizes), tname, states


@pytest.mark.parametrize("config,sizes", [
    ("circle_4000", [4000, 1500, 700, 2500]),          # 2D ordered: row lists
    ("circle3d_4000", [4000, 900, 2600]),              # 3D ordered: three list levels
    ("game_of_life_64", [4096, 2048, 1000]),           # order-free loop: no lists
    ("boids3d_5000", [5000, 1200, 3100]),
    ("sugarscape_10000", [10000, 4000]),               # members kept from two swaps before
])
def test_persistent_run_equals_separate_contexts(config, sizes):
    """One cooperative launch for all timesteps of every replica gives each
    replica the bits of its own context, over an odd number of timesteps (the
    program alternates two buffer sets) and in two runs in a row."""
    model, gl, tname, states = _prefix_replicas(config, sizes)
    ens = o.Ensemble(model, gl, seeds=list(range(len(gl))))
    ens.set_persistent(True)
    ens.upload(tname, states)
    ens.run(5)
    assert ens.last_launch_count() == 1
    assert ens.persistent_blocks() >= 152
    ens.run(2)
    got = ens.download(tname)
    for r in range(len(gl)):
        sim = o.Simulation(model, gl[r])
        sim.set_seed(r)
        sim.upload(tname, states[r])
        sim.run(7)
        want = sim.download(tname)
        sim.close()
        for k in want:
            assert np.array_equal(got[r][k], want[k]), (config, r, k)
    ens.close()


@pytest.mark.parametrize("model_name,config", [("boids2d", "boids2d_4096"),
                                                ("boids2d_float", "boids2d_float_4096")])
def test_persistent_boids_equal_per_phase_launches(model_name, config):
    """The boids ensemble of uneven replicas: persistent run == per-phase
    graph replay, replica by replica, after an autotune on the persistent
    path; a 200-timestep run is one launch."""
    model, base = o.globals_for_config(config)
    gl, states, seeds = workloads.boids2d_ensemble(model, base, replicas=10, n_min=300,
                                                   n_max=6000, seed=11)
    fd = np.float32 if model.float_bytes == 4 else np.float64
    states = [{k: v.astype(fd) for k, v in s.items()} for s in states]
    a = o.Ensemble(model, gl, seeds=seeds)
    a.set_persistent(True)
    a.upload("Boid", states)
    a.autotune(2)
    a.upload("Boid", states)
    a.run(200)
    assert a.last_launch_count() == 1
    b = o.Ensemble(model, gl, seeds=seeds)
    b.upload("Boid", states)
    b.run(200)
    for r, (ra, rb) in enumerate(zip(a.download("Boid"), b.download("Boid"))):
        for k in ra:
            assert np.array_equal(ra[k], rb[k]), (r, k)
    a.close()
    b.close()


def test_persistent_random_steps_equal_per_phase_launches():
    """random() in a step is keyed by the timestep, which the persistent
    kernel counts itself: boids2d_flockers gives the bits of the (eager)
    per-phase path."""
    import sys, os
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from golden_io import load_case
    meta, st = load_case("boids2d_flockers_1000")
    model = o.Model("boids2d_flockers")
    g = model.default_globals()
    tname = model.agent_types[0][0]
    states = [{k: np.ascontiguousarray(v[:n]) for k, v in st.items()} for n in (1000, 500, 300)]
    gl = [g] * 3
    a = o.Ensemble(model, gl, seeds=[5, 6, 7])
    a.set_persistent(True)
    a.upload(tname, states)
    a.run(9)
    b = o.Ensemble(model, gl, seeds=[5, 6, 7])
    b.upload(tname, states)
    b.run(9)
    for ra, rb in zip(a.download(tname), b.download(tname)):
        for k in ra:
            assert np.array_equal(ra[k], rb[k]), k
    a.close()
    b.close()


def test_persistent_barrier_wait_runs_out_and_context_stays_usable():
    """A barrier that waits for one arrival more than the grid has (a flag
    that nothing sets) gives up after its limit: the run returns
    ABL_E_TIMEOUT, no kernel is left running, and the same ensemble then
    computes the right bits."""
    model, base = o.globals_for_config("boids2d_4096")
    gl, states, seeds = workloads.boids2d_ensemble(model, base, replicas=4, n_min=500,
                                                   n_max=3000, seed=2)
    ens = o.Ensemble(model, gl, seeds=seeds)
    ens.set_persistent(True)
    ens.upload("Boid", states)
    ens.inject_barrier_failure(0.2, 1)
    with pytest.raises(o.AblError) as err:
        ens.run(3)
    assert err.value.code == -4
    ens.inject_barrier_failure(0.0, 0)
    ens.upload("Boid", states)
    ens.run(3)
    got = ens.download("Boid")
    for r in range(len(gl)):
        sim = o.Simulation(model, gl[r])
        sim.upload("Boid", states[r])
        sim.run(3)
        want = sim.download("Boid")
        sim.close()
        for k in want:
            assert np.array_equal(got[r][k], want[k]), (r, k)
    ens.close()


def _grazer_replicas(sizes, seed=6):
    model = o.Model("grazers")
    g = model.default_globals()
    W = float(g.get("W"))
    rng = np.random.Generator(np.random.PCG64(seed))
    states = []
    for n in sizes:
        ang = rng.uniform(0, 2 * np.pi, n)
        states.append({
            "Grazer": {"pos": rng.uniform(0, W, (n, 2)), "dir": np.stack([np.cos(ang), np.sin(ang)], 1),
                       "fed": np.zeros(n)},
            "Patch": {"pos": rng.uniform(0, W, (2 * n, 2)), "grass": rng.uniform(0, 1, 2 * n)}})
    return model, [g] * len(sizes), states


@pytest.mark.parametrize("persistent", [False, True])
def test_unstepped_neighbour_type(persistent):
    """A neighbour type that no step changes is binned in the first timestep
    only, so the first timestep's program differs from the later ones (the
    persistent kernel runs ts[0] once, then ts[1], ts[2] in turn); every
    replica gets the bits of its own context."""
    model, gl, states = _grazer_replicas([1500, 600, 2400])
    ens = o.Ensemble(model, gl, seeds=[1, 2, 3])
    ens.set_persistent(persistent)
    for tname in ("Grazer", "Patch"):
        ens.upload(tname, [s[tname] for s in states])
    ens.run(7)
    if persistent:
        assert ens.last_launch_count() == 1
    got = {t: ens.download(t) for t in ("Grazer", "Patch")}
    ens.close()
    for r, st in enumerate(states):
        sim = o.Simulation(model, gl[r])
        sim.set_seed(r + 1)
        for tname in ("Grazer", "Patch"):
            sim.upload(tname, st[tname])
        sim.run(7)
        for tname in ("Grazer", "Patch"):
            want = sim.download(tname)
            for k in want:
                assert np.array_equal(got[tname][r][k], want[k]), (persistent, r, tname, k)
        sim.close()
