"""Every benchmark configuration, at its full size, for its full timestep
count, against the binned CPU oracle.

The oracle is pinned to the reference's own programs at every timestep of
the small golden cases (test_oracle_golden.py); tests/golden/make_full.py
ran it on these workloads and recorded the SHA-256 of the state after every
timestep (full_<config>.json).  Here the CUDA path, through the C ABI,
starts from the same seeded initial state (its hash is checked first) and
must reproduce every one of those hashes: bit-exact, one timestep at a
time, and again at the end of one abl_run over all timesteps (graph
replay).
"""
import json
import os

import pytest

import openabl_gb300 as o
from golden_io import GOLDEN, MEMBERS, full_initial_state, state_digest

pytestmark = pytest.mark.gpu

FULL = ["boids2d_1m", "boids2d_float_1m", "boids3d_1m", "game_of_life_4096", "sugarscape_1m",
        "predator_prey_1m", "predator_prey_float_1m"]


def fixture(config):
    with open(os.path.join(GOLDEN, f"full_{config}.json")) as f:
        return json.load(f)


def start(config):
    state, seed = full_initial_state(config)
    model, g = o.globals_for_config(config)
    sim = o.Simulation(model, g)
    if seed is not None:
        sim.set_seed(seed)
    for t in MEMBERS[config]:
        sim.upload(t, state[t])
    return sim, state


def digest(sim, config):
    return state_digest(config, {t: sim.download(t) for t in MEMBERS[config]})


@pytest.mark.parametrize("config", FULL)
def test_full_run_matches_oracle_every_timestep(config):
    fx = fixture(config)
    sim, state = start(config)
    assert state_digest(config, state) == fx["init_sha256"], "initial state differs on this host"
    for t in range(fx["timesteps"]):
        sim.step()
        assert digest(sim, config) == fx["sha256"][t], f"timestep {t + 1}"
    sim.close()


@pytest.mark.parametrize("config", FULL)
def test_full_run_through_graph_replay(config):
    fx = fixture(config)
    sim, _ = start(config)
    sim.run(fx["timesteps"])
    assert digest(sim, config) == fx["sha256"][-1]
    sim.close()
