"""Per-timestep fixtures of the benchmark workloads at their full size and
full timestep count, made with the binned CPU oracle.

    python tests/golden/make_full.py [config ...]

The oracle (oracle/abl_oracle.c) is pinned to the reference's own programs
at every timestep of the small golden cases (tests/test_oracle_golden.py);
this script runs it on the benchmark configurations -- too large for the
reference's O(N^2) loop -- and records, for each,
  full_<config>.json   the initial state's hash and the SHA-256 of the state
                       after every timestep 1..T
The initial states come from openabl_gb300/workloads.py with the seed
recorded in the file.  Those generators use only correctly rounded
arithmetic, so every host builds the same initial bits; the GPU tests check
the initial hash before stepping.  The hash of a state is `state_digest`
below: the SHA-256 of each member column's little-endian bytes, in the
order of `MEMBERS`, type after type.
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
REPO = os.path.dirname(TESTS)
for p in (REPO, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)

from golden_io import MEMBERS, full_initial_state, state_digest  # noqa: E402
from oracle import oracle as O  # noqa: E402


def _cfg(name):
    with open(os.path.join(REPO, "openabl_gb300", "generated", "configs.json")) as f:
        return json.load(f)[name]["globals"]


def stepper(name, state, seed):
    """The oracle's timestep for configuration `name`, from `state`."""
    g = _cfg(name)
    if name in ("boids2d_1m", "boids2d_float_1m", "boids3d_1m"):
        c = {k: g[k] for k in O.BOIDS2D_KEYS}
        f = {"boids2d_1m": O.boids2d_step, "boids2d_float_1m": O.boids2d_step_f32,
             "boids3d_1m": O.boids3d_step}[name]
        return lambda s: {"Boid": f(s["Boid"], c, mode=1)}
    if name == "game_of_life_4096":
        c = {"radius": g["radius"], "size": g["size"]}
        return lambda s: {"Cell": O.game_of_life_step(s["Cell"], c, mode=1)}
    if name == "sugarscape_1m":
        sim = O.Sugarscape(state["Agent"], radius=g["radius"], grid_width=float(g["grid_width"]))
        return lambda s: {"Agent": sim.step()}
    if name.startswith("predator_prey"):
        consts = {k: g[k] for k in O.PP_DPARAMS + O.PP_IPARAMS}
        cls = O.PredatorPreyF32 if name.endswith("float_1m") else O.PredatorPrey
        ref = cls(state, consts, seed=seed)

        def step(_):
            ref.run(1, mode=1)
            return ref.get()
        return step
    raise KeyError(name)


# config -> timesteps
CASES = {"boids2d_1m": 100, "boids2d_float_1m": 100, "boids3d_1m": 100,
         "game_of_life_4096": 100, "sugarscape_1m": 100, "predator_prey_1m": 500,
         "predator_prey_float_1m": 500}


def make(name):
    T = CASES[name]
    t0 = time.time()
    state, seed = full_initial_state(name)
    step = stepper(name, state, seed)
    out = {"config": name, "workload_seed": 0, "random_seed": seed, "timesteps": T,
           "members": {t: MEMBERS[name][t] for t in state},
           "init_sha256": state_digest(name, state), "sha256": [],
           "source": "binned CPU oracle (oracle/abl_oracle.c, mode 1), x86-64, "
                     "gcc -O2 -std=c99 -ffp-contract=off"}
    for t in range(T):
        state = step(state)
        out["sha256"].append(state_digest(name, state))
        if t % 10 == 9:
            print(f"{name}: timestep {t + 1}/{T}, {time.time() - t0:.0f} s", flush=True)
    out["oracle_seconds"] = round(time.time() - t0, 1)
    with open(os.path.join(HERE, f"full_{name}.json"), "w") as f:
        json.dump(out, f, indent=0)
    print(name, "done in", out["oracle_seconds"], "s", flush=True)


if __name__ == "__main__":
    for n in sys.argv[1:] or list(CASES):
        make(n)
