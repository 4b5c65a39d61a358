"""Kept neighbour lists give the same results as searching the grid.

When no step function moves agents of a type (game_of_life's cells,
sugarscape's grid agents), the runtime finds each agent's in-radius
neighbours once per binning and reads them at every timestep
(abl_set_near_cache, on by default).  The reference visits every agent and
skips those farther than the radius (src/backend/CPrinter.cpp:160-170), so
the kept lists must hold exactly those, in ascending index for ordered loops.
Checked here: the golden hashes of the reference `c` backend with the lists
on and off and in every gathering mode; an upload of moved agents after
graph replays (the lists must be rebuilt, not replayed); neighbourhoods
longer than a thread's shared-memory column; and neighbourhoods too long to
keep (the step then searches the grid).
"""
import numpy as np
import pytest

import openabl_gb300 as o
from golden_io import load_case, state_hash
from openabl_gb300 import workloads

pytestmark = pytest.mark.gpu

CASES = [("game_of_life_64", "game_of_life_64", "Cell"),
         ("sugarscape_10000", "sugarscape_10000", "Agent")]


@pytest.mark.parametrize("cache", [1, 0])
@pytest.mark.parametrize("mode", [o.Simulation.NEAR_AUTO, o.Simulation.NEAR_RUNS,
                                  o.Simulation.NEAR_LISTS])
@pytest.mark.parametrize("case,config,agent", CASES)
def test_kept_lists_match_reference(case, config, agent, mode, cache):
    meta, state = load_case(case)
    model, g = o.globals_for_config(config)
    sim = o.Simulation(model, g)
    sim.set_near_mode(mode)
    sim.set_near_cache(cache)
    sim.upload(agent, state)
    sim.step()
    assert state_hash(meta, sim.download(agent)) == meta["sha256"][1]
    T = meta["timesteps"]
    sim.run(T - 1)
    assert state_hash(meta, sim.download(agent)) == meta["sha256"][T]
    sim.close()


def run_pair(config, agent, states, steps):
    """Runs the same uploads on two simulations, lists kept and not, and
    returns both final states."""
    out = []
    for cache in (1, 0):
        model, g = o.globals_for_config(config)
        sim = o.Simulation(model, g)
        sim.set_near_cache(cache)
        for state in states:
            sim.upload(agent, state)
            sim.run(steps)
        out.append(sim.download(agent))
        sim.close()
    return out


def assert_same(a, b):
    assert a.keys() == b.keys()
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_upload_of_moved_agents_rebuilds_lists():
    """Six timesteps (replayed from graphs that read the kept lists), then an
    upload of the same number of cells in reversed index order: the buffers
    stay, the lists must not."""
    a = workloads.game_of_life(64, 0.5, seed=3)
    b = {k: np.ascontiguousarray(v[::-1]) for k, v in a.items()}
    b["alive"] = workloads.game_of_life(64, 0.5, seed=4)["alive"]
    kept, searched = run_pair("game_of_life_64", "Cell", [a, b], 6)
    assert_same(kept, searched)


def test_long_ordered_lists():
    """sugarscape with its grid agents packed 0.4 apart: ~44 neighbours
    each, more than a thread's shared-memory column (32), so the ordered
    loops refill from the kept lists."""
    state = workloads.sugarscape(100, 0.3, seed=5)
    state["pos"] = np.ascontiguousarray(state["pos"] * 0.4)
    kept, searched = run_pair("sugarscape_10000", "Agent", [state], 5)
    assert_same(kept, searched)


def test_lists_too_long_to_keep():
    """3000 cells inside one radius: every agent neighbours every other (9
    million pairs), more than the runtime keeps; the step searches the
    grid."""
    rng = np.random.default_rng(8)
    n = 3000
    state = {"pos": np.ascontiguousarray(10.0 + rng.random((n, 2))),
             "alive": (rng.random(n) < 0.5).astype(np.uint8)}
    kept, searched = run_pair("game_of_life_64", "Cell", [state], 3)
    assert_same(kept, searched)


def test_lists_beyond_the_budget_are_not_kept():
    """With an HBM budget that holds the simulation but not the lists, the
    lists are given up (no error) and the step searches the grid."""
    model, g = o.globals_for_config("game_of_life_64")
    state = workloads.game_of_life(64, 0.5, seed=9)
    a = o.Simulation(model, g)
    a.set_near_cache(0)
    a.upload("Cell", state)
    a.run(5)
    used = a.memory_used()
    want = a.download("Cell")
    a.close()
    b = o.Simulation(model, g, hbm_budget=used + 4096)
    b.upload("Cell", state)
    b.run(5)
    assert_same(b.download("Cell"), want)
    b.close()
