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


def test_float_build_binned_matches_brute_force():
    cfg, state, consts = case("predator_prey_float_small")
    assert state["Prey"]["pos"].dtype == np.float32
    a = O.PredatorPreyF32(state, consts, seed=7)
    b = O.PredatorPreyF32(state, consts, seed=7)
    sa = a.run(4, mode=1)
    sb = b.run(4, mode=0)
    assert np.array_equal(sa, sb)
    ga, gb = a.get(), b.get()
    for t in O.PP_TYPES:
        for k in ga[t]:
            assert ga[t][k].dtype == gb[t][k].dtype
            assert np.array_equal(ga[t][k], gb[t][k]), (t, k)
    a.close()
    b.close()


def test_float_build_computes_in_float():
    """The float restatement is not the double one rounded at the end: after
    a few timesteps the two differ, and the float one's state is float32."""
    cfg, state, consts = case("predator_prey_small")
    _, state32, _ = case("predator_prey_float_small")
    a = O.PredatorPrey(state, consts, seed=7)
    b = O.PredatorPreyF32(state32, consts, seed=7)
    a.run(3, mode=1)
    b.run(3, mode=1)
    ga, gb = a.get(), b.get()
    assert gb["Prey"]["pos"].dtype == np.float32
    n = min(len(ga["Predator"]["pos"]), len(gb["Predator"]["pos"]))
    assert not np.array_equal(ga["Predator"]["pos"][:n].astype(np.float32),
                              gb["Predator"]["pos"][:n])
    a.close()
    b.close()


def test_population_changes_happen():
    cfg, state, consts = case("predator_prey_small")
    a = O.PredatorPrey(state, consts, seed=3)
    stats = a.run(40, mode=1)
    prey, pred, grass = stats[:, 0], stats[:, 1], stats[:, 2]
    assert len(set(prey.tolist())) > 1 and grass.min() < len(state["Grass"]["pos"])
    a.close()
