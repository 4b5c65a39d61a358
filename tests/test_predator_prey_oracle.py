"""The predator_prey oracle: binned and brute-force neighbour search agree
(populations, removals, births and the sequential step's statistics)."""
import numpy as np

from oracle import oracle as O
from pp_setup import case


def test_binned_matches_brute_force():
    cfg, state, consts = case("predator_prey_small")
    a = O.PredatorPrey(state, consts, seed=7)
    b = O.PredatorPrey(state, consts, seed=7)
    sa = a.run(4, mode=1)
    sb = b.run(4, mode=0)
    assert np.array_equal(sa, sb)
    ga, gb = a.get(), b.get()
    for t in O.PP_TYPES:
        for k in ga[t]:
            assert np.array_equal(ga[t][k], gb[t][k]), (t, k)
    a.close()
    b.close()


def test_population_changes_happen():
    cfg, state, consts = case("predator_prey_small")
    a = O.PredatorPrey(state, consts, seed=3)
    stats = a.run(40, mode=1)
    prey, pred, grass = stats[:, 0], stats[:, 1], stats[:, 2]
    assert len(set(prey.tolist())) > 1 and grass.min() < len(state["Grass"]["pos"])
    a.close()
