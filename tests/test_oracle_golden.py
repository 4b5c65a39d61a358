"""The CPU oracle reproduces the reference programs step by step.

The golden hashes were produced by the reference `c` backend's own programs
(tests/golden/make_golden.py); both neighbour-search modes of the oracle must
give the identical packed state after every timestep.
"""
import math

import numpy as np
import pytest

from golden_io import load_case, state_hash
from oracle import oracle as O


def consts(meta):
    p = meta["params"]
    ex = meta["example"]
    if ex in ("circle", "circle3d"):
        n, rho = int(p["num_agents"]), float(p["rho"])
        w = math.sqrt(n / rho) if ex == "circle" else math.pow(n / rho, 1 / 3)
        return dict(r=5.0, k_rep=0.05, k_att=0.01, W=float("%g" % w))
    if ex == "boids2d":
        n, dens = int(p["num_agents"]), float(p["agent_density"])
        return dict(interaction_radius=0.05, separation_radius=0.005, time_scale=0.0005,
                    global_scale=0.15, steer_scale=0.65, collision_scale=0.75, match_scale=1.25,
                    min_pos=0.0, max_pos=float("%g" % math.sqrt(n / dens)))
    if ex == "game_of_life":
        return dict(radius=1.5, size=int(math.sqrt(int(p["num_agents"]))))
    if ex == "boids":
        # examples/boids.abl at its defaults: 5000 agents, agent_density 1000
        return dict(interaction_radius=0.05, separation_radius=0.005, time_scale=0.0005,
                    global_scale=0.15, steer_scale=0.65, collision_scale=0.75, match_scale=1.25,
                    min_pos=0.0, max_pos=float("%g" % (5000 / 1000) ** (1 / 3)))
    raise KeyError(ex)


CASES = ["circle_4000", "circle3d_4000", "boids2d_4096", "game_of_life_64", "boids3d_5000"]


@pytest.mark.parametrize("case", CASES)
def test_reference_init_restated(case):
    meta, state = load_case(case)
    c = consts(meta)
    ex = meta["example"]
    if ex in ("circle", "circle3d"):
        s = O.init_circle(2 if ex == "circle" else 3, meta["agents"], c["W"])
    elif ex == "boids2d":
        s = O.init_boids2d(meta["agents"], c["min_pos"], c["max_pos"])
    elif ex == "boids":
        s = O.init_boids3d(meta["agents"], c["min_pos"], c["max_pos"])
    else:
        s = O.init_game_of_life(c["size"], float(meta["params"]["alive_fraction"]))
    for k in state:
        assert np.array_equal(s[k], state[k]), k


@pytest.mark.parametrize("case", CASES)
def test_binned_oracle_matches_reference_every_step(case):
    meta, state = load_case(case)
    c = consts(meta)
    step = O.STEP[meta["example"]]
    assert state_hash(meta, state) == meta["sha256"][0]
    for t in range(1, meta["timesteps"] + 1):
        state = step(state, c, mode=1)
        assert state_hash(meta, state) == meta["sha256"][t], f"step {t}"


@pytest.mark.parametrize("case", CASES)
def test_brute_force_oracle_matches_reference(case):
    meta, state = load_case(case)
    c = consts(meta)
    step = O.STEP[meta["example"]]
    for t in range(1, 4):
        state = step(state, c, mode=0)
        assert state_hash(meta, state) == meta["sha256"][t], f"step {t}"


@pytest.mark.parametrize("mode", [1, 0])
def test_sugarscape_oracle_matches_reference(mode):
    """sugarscape 100 x 100: the oracle's four step functions with the
    reference's double buffer reproduce every golden hash (binned), or the
    first three timesteps (brute force)."""
    meta, state = load_case("sugarscape_10000")
    sim = O.Sugarscape(state, radius=1.5, grid_width=100.0, mode=mode)
    assert state_hash(meta, sim.cur) == meta["sha256"][0]
    T = meta["timesteps"] if mode == 1 else 3
    for t in range(1, T + 1):
        assert state_hash(meta, sim.step()) == meta["sha256"][t], f"step {t}"


@pytest.mark.parametrize("mode", [1, 0])
def test_flockers_oracle_matches_single_thread_reference(mode):
    """boids2d_flockers (random() inside the step), recorded from the
    reference program on one thread: the oracle's init draws main()'s agents
    from the xorshift stream, and its steps continue that stream agent by
    agent; every timestep's state hashes like the reference's."""
    meta, state = load_case("boids2d_flockers_1000")
    c = dict(interaction_radius=10.0, steer_scale=0.1, collision_scale=400.0, match_scale=1.0,
             randomness_scale=0.05, momentum_scale=1.0, time_scale=0.7,
             max_pos=float("%g" % math.sqrt(1000 / 0.004)))
    s = O.init_boids2d(meta["agents"], 0.0, c["max_pos"])
    for k in state:
        assert np.array_equal(s[k], state[k]), k
    T = meta["timesteps"] if mode == 1 else 3
    for t in range(1, T + 1):
        s = O.flockers_step(s, c, mode=mode)
        assert state_hash(meta, s) == meta["sha256"][t], f"step {t}"


@pytest.mark.parametrize("mode", [1, 0])
def test_boids2d_fp32_oracle_matches_reference(mode):
    """boids2d built with LIBABL_USE_FLOAT (-C use_float=true): the oracle's
    single-precision restatement reproduces the reference's FP32 program every
    timestep (binned), or the first three (brute force)."""
    meta, state = load_case("boids2d_4096_float")
    c = consts(dict(meta, example="boids2d"))
    s = state
    T = meta["timesteps"] if mode == 1 else 3
    for t in range(1, T + 1):
        s = O.boids2d_step_f32(s, c, mode=mode)
        assert state_hash(meta, s) == meta["sha256"][t], f"step {t}"
