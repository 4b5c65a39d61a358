"""Checkpoint and resume (abl_save_state / abl_load_state).

The reference has no resume, and its save() prints %f, which loses bits.
A run resumed from a checkpoint must equal the uninterrupted run bit for
bit, including:
- the double buffer's older values, which step functions that write a member
  on one branch only leave visible (the `kinds` test model);
- populations changed by removeCurrent() and add();
- random() keyed by the timestep (predator_prey);
- the sequential xorshift stream (boids2d_flockers in sequential mode).
"""
import numpy as np
import pytest

import openabl_gb300 as o
from oracle import oracle as O
from openabl_gb300 import workloads
from pp_setup import case

pytestmark = pytest.mark.gpu


def assert_same(a, b):
    assert a.keys() == b.keys()
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def kinds_state(n=3000, seed=2):
    rng = np.random.default_rng(seed)
    return {"pos": rng.random((n, 2)) * 60.0, "kind": rng.integers(0, 3, n).astype(np.int32),
            "score": np.zeros(n)}


def check_resume(make, types, tmp_path, before=7, after=9):
    """`make()` returns a simulation with its initial state uploaded."""
    a = make()
    a.run(before)
    ckpt = tmp_path / "state.bin"
    a.save_state(ckpt)
    a.run(after)
    want = {t: a.download(t) for t in types}
    a.close()
    b = make()
    b.run(3)  # some other history, replaced by the checkpoint
    b.load_state(ckpt)
    b.run(after)
    for t in types:
        assert_same(b.download(t), want[t])
    b.close()


def test_resume_keeps_the_double_buffer(tmp_path):
    def make():
        model = o.Model("kinds")
        sim = o.Simulation(model, model.default_globals())
        sim.upload("Cell", kinds_state())
        return sim
    check_resume(make, ["Cell"], tmp_path)


def test_resume_predator_prey(tmp_path):
    cfg, state, consts = case("predator_prey_small")

    def make():
        model, g = o.globals_for_config("predator_prey_small")
        sim = o.Simulation(model, g)
        sim.set_seed(5)
        for t in O.PP_TYPES:
            sim.upload(t, state[t])
        return sim
    check_resume(make, list(O.PP_TYPES), tmp_path)


def test_resume_sequential_random(tmp_path):
    def make():
        model = o.Model("boids2d_flockers")
        g = model.default_globals()
        sim = o.Simulation(model, g)
        rng = np.random.default_rng(4)
        n = 500
        sim.upload("Boid", {"pos": rng.random((n, 2)) * 100.0,
                            "velocity": rng.uniform(-1, 1, (n, 2))})
        sim.set_serial_random([0x1234, 0x5678])
        return sim
    check_resume(make, ["Boid"], tmp_path, before=4, after=4)


def test_state_of_another_model_is_refused(tmp_path):
    model, g = o.globals_for_config("game_of_life_64")
    a = o.Simulation(model, g)
    a.upload("Cell", workloads.game_of_life(64, 0.5, seed=1))
    a.save_state(tmp_path / "gol.bin")
    a.close()
    b = o.Simulation(o.Model("kinds"), o.Model("kinds").default_globals())
    with pytest.raises(o.AblError) as e:
        b.load_state(tmp_path / "gol.bin")
    assert e.value.code == -10
    with pytest.raises(o.AblError) as e:
        b.load_state(tmp_path / "missing.bin")
    assert e.value.code == -10
    b.close()


def test_truncated_state_leaves_the_context_unchanged(tmp_path):
    """A file cut short is refused before anything is applied: the context
    keeps its own globals, agents and timestep."""
    model, g = o.globals_for_config("game_of_life_64")
    a = o.Simulation(model, g)
    a.upload("Cell", workloads.game_of_life(64, 0.5, seed=1))
    a.run(2)
    a.save_state(tmp_path / "full.bin")
    a.close()
    data = (tmp_path / "full.bin").read_bytes()
    (tmp_path / "cut.bin").write_bytes(data[: len(data) - 100])
    (tmp_path / "long.bin").write_bytes(data + b"\0")

    b = o.Simulation(model, g)
    b.upload("Cell", workloads.game_of_life(64, 0.5, seed=7))
    b.run(3)
    before = b.download("Cell")
    for bad in ("cut.bin", "long.bin"):
        with pytest.raises(o.AblError) as e:
            b.load_state(tmp_path / bad)
        assert e.value.code == -10
        assert_same(b.download("Cell"), before)
    b.run(1)
    c = o.Simulation(model, g)
    c.upload("Cell", workloads.game_of_life(64, 0.5, seed=7))
    c.run(4)
    assert_same(b.download("Cell"), c.download("Cell"))
    b.close()
    c.close()
