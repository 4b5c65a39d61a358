"""predator_prey on the GPU: three agent types, cross-type near loops,
removeCurrent(), add() in step functions, random() from the counter-based
stream and the sequential step, all bit-exact against the CPU oracle's
stated semantics after every timestep."""
import numpy as np
import pytest

import openabl_gb300 as o
from oracle import oracle as O
from pp_setup import case

pytestmark = pytest.mark.gpu


def sim_for(config, state, seed):
    model, g = o.globals_for_config(config)
    sim = o.Simulation(model, g)
    sim.set_seed(seed)
    for t in O.PP_TYPES:
        sim.upload(t, state[t])
    return sim


def assert_same(sim, ref, when):
    got_all = ref.get()
    for t in O.PP_TYPES:
        got = sim.download(t)
        want = got_all[t]
        for k in want:
            assert got[k].shape == want[k].shape, (when, t, k, got[k].shape, want[k].shape)
            assert np.array_equal(got[k], want[k]), (when, t, k)


def test_every_timestep_matches_oracle():
    cfg, state, consts = case("predator_prey_small")
    sim = sim_for("predator_prey_small", state, seed=11)
    ref = O.PredatorPrey(state, consts, seed=11)
    stats = []
    for t in range(30):
        sim.step()
        stats.append(ref.run(1, mode=1)[0])
        assert_same(sim, ref, t)
    rows = [r.split(",") for r in sim.log_text().strip().splitlines()]
    assert len(rows) == 30
    for r, s in zip(rows, stats):
        assert [int(r[0]), int(r[1]), int(r[2])] == s.tolist()
        assert float(r[3]) > 0.0           # getLastExecTime(): seconds of the timestep
    sim.close()
    ref.close()


def test_float_build_every_timestep_matches_oracle():
    """-C use_float=true: the FP32 model against the oracle's float
    restatement (every member and intermediate in float), bit-exact after
    every timestep, with the sequential step's statistics."""
    cfg, state, consts = case("predator_prey_float_small")
    sim = sim_for("predator_prey_float_small", state, seed=11)
    ref = O.PredatorPreyF32(state, consts, seed=11)
    stats = []
    for t in range(30):
        sim.step()
        stats.append(ref.run(1, mode=1)[0])
        assert_same(sim, ref, t)
    rows = [r.split(",") for r in sim.log_text().strip().splitlines()]
    for r, s in zip(rows, stats):
        assert [int(r[0]), int(r[1]), int(r[2])] == s.tolist()
    sim.close()
    ref.close()


def test_reductions():
    cfg, state, consts = case("predator_prey_small")
    sim = sim_for("predator_prey_small", state, seed=1)
    sim.run(5)
    got = sim.download("Grass")
    assert sim.reduce(0, "Prey") == sim.count("Prey")
    assert sim.reduce(1, "Grass", "avail") == int(got["avail"].sum())
    assert sim.reduce(2, "Grass", "dead_cycles", 0) == int((got["dead_cycles"] == 0).sum())
    pred = sim.download("Predator")
    s = sim.reduce(1, "Predator", "pos")
    acc = np.zeros(2)
    for p in pred["pos"]:
        acc = acc + p
    assert np.array_equal(s, acc)
    sim.close()


def test_full_size_matches_oracle():
    cfg, state, consts = case("predator_prey_1m")
    sim = sim_for("predator_prey_1m", state, seed=5)
    ref = O.PredatorPrey(state, consts, seed=5)
    for t in range(2):
        sim.step()
        ref.run(1, mode=1)
        assert_same(sim, ref, t)
    sim.close()
    ref.close()
