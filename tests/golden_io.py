"""Readers for the golden fixtures in tests/golden (see make_golden.py)."""
import hashlib
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_case(name):
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        meta = json.load(f)
    dt = record_dtype(meta)
    raw = open(os.path.join(GOLDEN, name + "_init.bin"), "rb").read()
    init = np.frombuffer(raw, dtype=dt)
    state = {n: np.ascontiguousarray(init[n]) for n, _, _ in meta["layout"]}
    return meta, state


def record_dtype(meta):
    return np.dtype([(n, d, tuple(s)) for n, d, s in meta["layout"]])


def pack(meta, state):
    dt = record_dtype(meta)
    n = len(next(iter(state.values())))
    rec = np.zeros(n, dtype=dt)
    for name, _, _ in meta["layout"]:
        rec[name] = state[name]
    return rec.tobytes()


def state_hash(meta, state):
    return hashlib.sha256(pack(meta, state)).hexdigest()


# Member order of the full-size fixtures (full_<config>.json, make_full.py):
# per configuration, agent type -> members, in the model's declaration order.
_BOID = {"Boid": ["pos", "velocity"]}
_ANIMAL = ["pos", "dir", "steer", "life"]
MEMBERS = {
    "boids2d_1m": _BOID,
    "boids2d_float_1m": _BOID,
    "boids3d_1m": _BOID,
    "game_of_life_4096": {"Cell": ["pos", "alive"]},
    "sugarscape_1m": {"Agent": ["pos", "target_pos", "agent_id", "state", "sugar_level",
                                "metabolism", "env_sugar_level", "max_env_sugar_level"]},
    "predator_prey_1m": {"Predator": _ANIMAL, "Prey": _ANIMAL,
                         "Grass": ["pos", "dead_cycles", "avail"]},
}
MEMBERS["predator_prey_float_1m"] = MEMBERS["predator_prey_1m"]


def _canonical(a):
    a = np.asarray(a)
    if a.dtype.kind == "f":
        return np.ascontiguousarray(a, dtype="<f%d" % a.dtype.itemsize)
    if a.dtype.kind in "iu" and a.dtype.itemsize == 4:
        return np.ascontiguousarray(a, dtype="<i4")
    if a.dtype.kind in "ub" and a.dtype.itemsize == 1:
        return np.ascontiguousarray(a, dtype="u1")
    raise TypeError(f"unexpected member dtype {a.dtype}")


def state_digest(config, state):
    """SHA-256 over every agent type of `state` ({type: {member: array}}):
    the type's agent count (int64) and then each member column's bytes, in
    MEMBERS order."""
    h = hashlib.sha256()
    for t, members in MEMBERS[config].items():
        cols = state[t]
        h.update(np.int64(len(cols[members[0]])).tobytes())
        for m in members:
            h.update(_canonical(cols[m]).tobytes())
    return h.hexdigest()


def full_initial_state(config):
    """The seeded initial state of a full-size fixture (workloads.py, seed 0),
    as {type: {member: array}}, and the random() seed of the run (or None)."""
    import openabl_gb300 as o
    from openabl_gb300 import workloads
    g = o.configs()[config]["globals"]
    if config in ("boids2d_1m", "boids2d_float_1m", "boids3d_1m"):
        gen = workloads.boids3d if config == "boids3d_1m" else workloads.boids2d
        st = gen(int(g["num_agents"]), float(g["max_pos"]), seed=0)
        if config == "boids2d_float_1m":
            st = {k: v.astype(np.float32) for k, v in st.items()}
        return {"Boid": st}, None
    if config == "game_of_life_4096":
        return {"Cell": workloads.game_of_life(int(g["size"]), float(g["alive_fraction"]),
                                               seed=0)}, None
    if config == "sugarscape_1m":
        return {"Agent": workloads.sugarscape(int(g["grid_width"]), float(g["occupiedFrac"]),
                                              seed=0)}, None
    if config in ("predator_prey_1m", "predator_prey_float_1m"):
        n = int(g["num_agents"])
        n_pred = int(float(g["predator_fraction"]) * n)
        n_prey = int(float(g["prey_fraction"]) * n)
        st = workloads.predator_prey(n_pred, n_prey, n - n_pred - n_prey, float(g["env_size"]),
                                     int(g["GAIN_FROM_FOOD_PREDATOR"]),
                                     int(g["GAIN_FROM_FOOD_PREY"]), seed=0)
        if config == "predator_prey_float_1m":
            st = {t: {k: (v.astype(np.float32) if v.dtype.kind == "f" else v)
                      for k, v in d.items()} for t, d in st.items()}
        return st, 5
    raise KeyError(config)
