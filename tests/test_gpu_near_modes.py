"""Ordered near loops give the same results whichever way the neighbours are
gathered.

The runtime can feed an ordered `near` loop (one whose body depends on the
visiting order, reference src/backend/CPrinter.cpp:148-173) from the cells'
own runs sorted per agent, from row lists merged on the fly (2D), or from
whole per-cell neighbourhood lists, and it may hand a block's agents to its
threads by neighbour count.  Every combination must reproduce the reference
`c` backend bit for bit (golden hashes), and the clustered case -- thousands
of agents in a few cells, so neighbour counts far exceed what a thread keeps
in shared memory and row lists exceed the single-thread merge -- must match
the CPU oracle.
"""
import numpy as np
import pytest

import openabl_gb300 as o
from golden_io import load_case, state_hash
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MODES = [o.Simulation.NEAR_RUNS, o.Simulation.NEAR_ROWS, o.Simulation.NEAR_LISTS,
         o.Simulation.NEAR_BLOCK]
CASES = [("circle_4000", "circle_4000", "Point"), ("circle3d_4000", "circle3d_4000", "Point"),
         ("boids2d_4096", "boids2d_4096", "Boid"),
         ("boids2d_4096_float", "boids2d_float_4096", "Boid"),
         ("boids3d_5000", "boids3d_5000", "Boid"), ("sugarscape_10000", "sugarscape_10000", "Agent")]


@pytest.mark.parametrize("balance", [0, 1])
@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("case,config,agent", CASES)
def test_modes_match_reference(case, config, agent, mode, balance):
    meta, state = load_case(case)
    model, g = o.globals_for_config(config)
    sim = o.Simulation(model, g)
    sim.set_near_mode(mode)
    sim.set_balance(balance)
    sim.upload(agent, state)
    sim.step()
    assert state_hash(meta, sim.download(agent)) == meta["sha256"][1]
    T = meta["timesteps"]
    sim.run(T - 1)
    assert state_hash(meta, sim.download(agent)) == meta["sha256"][T]
    sim.close()


@pytest.mark.parametrize("mode", [o.Simulation.NEAR_AUTO] + MODES)
def test_clustered_boids_match_oracle(mode):
    """6000 boids in a 0.08 x 0.08 square (cells 0.05 wide): ~4700
    neighbours per agent and row lists of ~6000 entries."""
    model, g = o.globals_for_config("boids2d_4096")
    n = 6000
    rng = np.random.default_rng(11)
    state = {"pos": 0.5 + 0.08 * rng.random((n, 2)),
             "velocity": rng.uniform(-1.0, 1.0, (n, 2))}
    sim = o.Simulation(model, g)
    sim.set_near_mode(mode)
    sim.upload("Boid", state)
    c = {k: g.get(k) for k in O.BOIDS2D_KEYS}
    ref = state
    for t in range(2):
        sim.step()
        ref = O.boids2d_step(ref, c, mode=1)
        got = sim.download("Boid")
        for k in ("pos", "velocity"):
            assert np.array_equal(got[k], ref[k]), (t, k)
    sim.close()


@pytest.mark.parametrize("balance", [0, 1])
@pytest.mark.parametrize("mode", [o.Simulation.NEAR_AUTO, o.Simulation.NEAR_BLOCK,
                                  o.Simulation.NEAR_ROWS])
def test_mixed_density_boids_match_oracle(mode, balance):
    """Uneven density in one domain: a sparse background (~8 agents per
    cell), a dense band (~60 per cell: most agents have more neighbours than
    a thread keeps in shared memory, so the loop refills from the block's
    lists) and a tight cluster (whose blocks' lists exceed the shared-memory
    budget and are gathered per agent instead)."""
    model, g = o.globals_for_config("boids2d_4096")
    L = g.get("max_pos")
    rng = np.random.default_rng(5)
    sparse = rng.random((3000, 2)) * L
    band = np.column_stack([rng.random(2500) * L, 0.30 + 0.05 * rng.random(2500)])
    cluster = 0.8 + 0.04 * rng.random((1500, 2))
    pos = np.concatenate([sparse, band, cluster])
    perm = rng.permutation(len(pos))        # ids unrelated to position
    state = {"pos": np.ascontiguousarray(pos[perm]),
             "velocity": rng.uniform(-1.0, 1.0, (len(pos), 2))}
    sim = o.Simulation(model, g)
    sim.set_near_mode(mode)
    sim.set_balance(balance)
    sim.upload("Boid", state)
    c = {k: g.get(k) for k in O.BOIDS2D_KEYS}
    ref = state
    for t in range(2):
        sim.step()
        ref = O.boids2d_step(ref, c, mode=1)
        got = sim.download("Boid")
        for k in ("pos", "velocity"):
            assert np.array_equal(got[k], ref[k]), (t, k)
    sim.close()
