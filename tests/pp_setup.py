"""Shared set-up of predator_prey cases for the tests."""
import openabl_gb300 as o
from openabl_gb300 import workloads
from oracle import oracle as O


def case(config, seed=0):
    cfg = o.configs()[config]
    g = cfg["globals"]
    n = int(g["num_agents"])
    n_pred = int(float(g["predator_fraction"]) * n)
    n_prey = int(float(g["prey_fraction"]) * n)
    n_grass = n - n_pred - n_prey
    state = workloads.predator_prey(n_pred, n_prey, n_grass, float(g["env_size"]),
                                    int(g["GAIN_FROM_FOOD_PREDATOR"]),
                                    int(g["GAIN_FROM_FOOD_PREY"]), seed=seed)
    if cfg["model"].endswith("_float"):
        state = {t: {k: (v.astype("float32") if v.dtype.kind == "f" else v)
                     for k, v in d.items()} for t, d in state.items()}
    consts = {k: g[k] for k in O.PP_DPARAMS + O.PP_IPARAMS}
    return cfg, state, consts
