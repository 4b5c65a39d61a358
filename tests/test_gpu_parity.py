"""GPU parity: the CUDA path, through the C ABI, against the reference.

* Golden cases: the packed state after EVERY timestep must hash to the value
  recorded from the reference `c` backend's own program (bit-exact), both
  when stepping one timestep at a time and through abl_run's graph replay.
* Full-size cases: bit-exact against the binned CPU oracle (itself pinned to
  the reference by test_oracle_golden.py) on the benchmark workloads.
"""
import numpy as np
import pytest

import openabl_gb300 as o
from golden_io import load_case, state_hash
from oracle import oracle as O
from openabl_gb300 import workloads

pytestmark = pytest.mark.gpu

GOLDEN = [("circle_4000", "Point"), ("circle3d_4000", "Point"), ("boids2d_4096", "Boid"),
          ("game_of_life_64", "Cell"), ("boids3d_5000", "Boid"), ("sugarscape_10000", "Agent")]


def make_sim(config):
    model, g = o.globals_for_config(config)
    return o.Simulation(model, g)


@pytest.mark.parametrize("case,agent", GOLDEN)
def test_every_timestep_matches_reference(case, agent):
    meta, state = load_case(case)
    sim = make_sim(case)
    sim.upload(agent, state)
    assert state_hash(meta, sim.download(agent)) == meta["sha256"][0]
    for t in range(1, meta["timesteps"] + 1):
        sim.step()
        assert state_hash(meta, sim.download(agent)) == meta["sha256"][t], f"timestep {t}"
    sim.close()


@pytest.mark.parametrize("case,agent", GOLDEN)
def test_graph_replay_matches_reference(case, agent):
    meta, state = load_case(case)
    sim = make_sim(case)
    sim.upload(agent, state)
    T = meta["timesteps"]
    sim.run(7)                      # odd split: eager + graph pairs + eager
    assert state_hash(meta, sim.download(agent)) == meta["sha256"][7]
    sim.run(T - 7)
    assert state_hash(meta, sim.download(agent)) == meta["sha256"][T]
    assert sim.last_launch_count() > 0
    sim.close()


FLOAT_GOLDEN = [("boids2d_4096_float", "boids2d_float_4096", "Boid"),
                ("circle_4000_float", "circle_float_4000", "Point"),
                ("circle3d_4000_float", "circle3d_float_4000", "Point")]


@pytest.mark.parametrize("case,config,agent", FLOAT_GOLDEN)
def test_use_float_matches_reference_every_timestep(case, config, agent):
    """-C use_float=true: the reference `c` program built with
    LIBABL_USE_FLOAT (float agents, double literals) against the generated
    FP32 model, bit-exact after every timestep, one timestep at a time and
    through graph replay."""
    meta, state = load_case(case)
    sim = make_sim(config)
    sim.upload(agent, state)
    for t in range(1, meta["timesteps"] + 1):
        sim.step()
        assert state_hash(meta, sim.download(agent)) == meta["sha256"][t], f"timestep {t}"
    sim.close()
    sim = make_sim(config)
    sim.upload(agent, state)
    sim.run(meta["timesteps"])
    assert state_hash(meta, sim.download(agent)) == meta["sha256"][meta["timesteps"]]
    sim.close()


def boids_consts(g):
    return {k: g.get(k) for k in O.BOIDS2D_KEYS}


def test_boids2d_1m_matches_oracle():
    model, g = o.globals_for_config("boids2d_1m")
    state = workloads.boids2d(g.get("num_agents"), g.get("max_pos"), seed=0)
    sim = o.Simulation(model, g)
    sim.upload("Boid", state)
    c = boids_consts(g)
    ref = state
    for t in range(3):
        sim.step()
        ref = O.boids2d_step(ref, c, mode=1)
        got = sim.download("Boid")
        for k in ("pos", "velocity"):
            assert np.array_equal(got[k], ref[k]), (t, k)
    sim.close()


def test_boids3d_1m_matches_oracle():
    """The 3D bench workload (1,048,576 boids, ~9 per interaction cell)
    against the oracle's restatement of examples/boids.abl."""
    model, g = o.globals_for_config("boids3d_1m")
    state = workloads.boids3d(g.get("num_agents"), g.get("max_pos"), seed=0)
    sim = o.Simulation(model, g)
    sim.upload("Boid", state)
    c = boids_consts(g)
    ref = state
    for t in range(2):
        sim.step()
        ref = O.boids3d_step(ref, c, mode=1)
        got = sim.download("Boid")
        for k in ("pos", "velocity"):
            assert np.array_equal(got[k], ref[k]), (t, k)
    sim.close()


def test_sugarscape_1m_matches_oracle():
    """The sugarscape bench workload (1024 x 1024 grid agents, kept
    neighbour lists) against the oracle's restatement with the reference's
    double buffer."""
    model, g = o.globals_for_config("sugarscape_1m")
    state = workloads.sugarscape(g.get("grid_width"), g.get("occupiedFrac"), seed=0)
    sim = o.Simulation(model, g)
    sim.upload("Agent", state)
    ref = O.Sugarscape(state, radius=g.get("radius"), grid_width=float(g.get("grid_width")))
    for t in range(3):
        sim.step()
        want = ref.step()
        got = sim.download("Agent")
        for k in want:
            assert np.array_equal(got[k], want[k]), (t, k)
    sim.close()


def test_game_of_life_4096_matches_oracle():
    model, g = o.globals_for_config("game_of_life_4096")
    state = workloads.game_of_life(g.get("size"), 0.5, seed=0)
    sim = o.Simulation(model, g)
    sim.upload("Cell", state)
    c = {"radius": g.get("radius"), "size": g.get("size")}
    ref = state
    for t in range(2):
        sim.step()
        ref = O.game_of_life_step(ref, c, mode=1)
        got = sim.download("Cell")
        assert np.array_equal(got["alive"], ref["alive"]), t
        assert np.array_equal(got["pos"], ref["pos"]), t
    sim.close()


def test_integer_count_division_is_ieee_division():
    """Step kernels divide by neighbour counts with a two-term reciprocal
    table (abl::div_int); every quotient must equal IEEE a / n bit for bit,
    here for 2e5 operands per n over n = -3..1027 (~2e8 quotients)."""
    checked, bad = o.runtime.check_int_division(seed=7, per_n=200000)
    assert checked == 200000 * 1031
    assert bad == 0


def test_budget_exhaustion_is_reported():
    model, g = o.globals_for_config("boids2d_4096")
    meta, state = load_case("boids2d_4096")
    sim = o.Simulation(model, g, hbm_budget=64 * 1024)
    with pytest.raises(o.AblError) as e:
        sim.upload("Boid", state)
        sim.step()
    assert e.value.code == -2
    sim.close()


def test_nonfinite_position_is_reported():
    model, g = o.globals_for_config("boids2d_4096")
    meta, state = load_case("boids2d_4096")
    state = {k: v.copy() for k, v in state.items()}
    state["pos"][17, 0] = np.nan
    sim = o.Simulation(model, g)
    sim.upload("Boid", state)
    with pytest.raises(o.AblError) as e:
        sim.step()
    assert e.value.code == -5
    sim.close()
