"""Seeded synthetic initial states for the benchmark configurations.

They replace the examples' own main() initialisation (which draws from the
reference's fixed-seed xorshift stream) with the distributions the
benchmark configurations specify; the same arrays are loaded into the GPU
path and into the CPU oracle.
"""
import numpy as np


def unit_vectors(rng, n, dim):
    """n directions uniform on the circle (dim 2) or sphere (dim 3): points
    drawn uniformly in the cube [-1, 1)^dim, kept when inside the unit ball
    (and not within 1e-6 of the centre), divided by their length.  Only
    correctly rounded operations (+, *, /, sqrt) are used, so every host
    builds the same bits from the same seed (sin/cos/log differ by an ulp
    between math libraries)."""
    out = np.empty((0, dim))
    while len(out) < n:
        m = int((n - len(out)) * (1.3 if dim == 2 else 2.0)) + 64
        c = rng.uniform(-1.0, 1.0, size=(m, dim))
        r2 = c[:, 0] * c[:, 0] + c[:, 1] * c[:, 1]
        if dim == 3:
            r2 = r2 + c[:, 2] * c[:, 2]
        keep = (r2 <= 1.0) & (r2 > 1e-12)
        out = np.concatenate([out, c[keep] / np.sqrt(r2[keep])[:, None]])
    return np.ascontiguousarray(out[:n])


def boids2d(n, max_pos, seed=0, vmax=1.0):
    """Positions uniform in [0, max_pos)^2; velocity directions uniform on the
    circle with speed uniform in [0.5, 1] * vmax (the speed cap of
    examples/boids2d.abl:98-101 is 1)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = rng.uniform(0.0, max_pos, size=(n, 2))
    d = unit_vectors(rng, n, 2)
    speed = rng.uniform(0.5, 1.0, size=n) * vmax
    vel = d * speed[:, None]
    return {"pos": np.ascontiguousarray(pos), "velocity": np.ascontiguousarray(vel)}


def circle(n, W, dim=2, seed=0):
    """Positions uniform in [0, W)^dim."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return {"pos": np.ascontiguousarray(rng.uniform(0.0, W, size=(n, dim)))}


def game_of_life(size, alive_fraction=0.5, seed=0):
    """One cell agent at (x + 0.5, y + 0.5) per grid point, x-major as in
    examples/game_of_life.abl:63-75; each alive with probability alive_fraction."""
    rng = np.random.Generator(np.random.PCG64(seed))
    x, y = np.meshgrid(np.arange(size, dtype=np.float64), np.arange(size, dtype=np.float64),
                       indexing="ij")
    pos = np.stack([x.ravel() + 0.5, y.ravel() + 0.5], axis=1)
    alive = (rng.uniform(size=size * size) < alive_fraction).astype(np.uint8)
    return {"pos": np.ascontiguousarray(pos), "alive": alive}


def predator_prey(n_pred, n_prey, n_grass, env_size, gain_pred=35, gain_prey=60, seed=0):
    """Uniform positions in [0, env_size)^2 for all three types; animals get a
    heading uniform on the circle (examples/predator_prey.abl:87-90 draws it
    as (sin phi, cos phi); here it is drawn without sin/cos so that every
    host builds the same bits) and zero steer, as :316-333 initialise them,
    and life GAIN_FROM_FOOD + an integer uniform in [0, 10]; grass starts
    available."""
    rng = np.random.Generator(np.random.PCG64(seed))

    def animals(n, gain):
        pos = rng.uniform(0.0, env_size, size=(n, 2))
        return {"pos": pos,
                "dir": unit_vectors(rng, n, 2),
                "steer": np.zeros((n, 2)),
                "life": (gain + rng.integers(0, 11, size=n)).astype(np.int32)}

    grass = {"pos": rng.uniform(0.0, env_size, size=(n_grass, 2)),
             "dead_cycles": np.zeros(n_grass, np.int32),
             "avail": np.ones(n_grass, np.uint8)}
    return {"Predator": animals(n_pred, gain_pred), "Prey": animals(n_prey, gain_prey),
            "Grass": grass}


def boids2d_ensemble(model, base_globals, replicas=256, n_min=1000, n_max=200000,
                     weight_spread=0.2, seed=0, agent_density=3200.0):
    """Parameter points for an ensemble of boids2d replicas: agent counts
    log-uniform in [n_min, n_max]; steer_scale, match_scale and
    collision_scale (the cohesion, alignment and separation weights of
    examples/boids2d.abl:27-29) uniform within +-weight_spread of the file's
    values; the domain side max_pos = sqrt(n / agent_density) printed to six
    significant digits as the compiler folds it; one seed per replica.
    Returns (globals list, states, seeds)."""
    import math
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = np.exp(rng.uniform(np.log(n_min), np.log(n_max), size=replicas)).astype(np.int64)
    globals_list, states = [], []
    seeds = rng.integers(0, 2**63, size=replicas, dtype=np.uint64)
    for r in range(replicas):
        g = model.default_globals()
        for name in ("interaction_radius", "separation_radius", "time_scale", "global_scale",
                     "min_pos"):
            g.set(name, base_globals.get(name))
        for name in ("steer_scale", "match_scale", "collision_scale"):
            g.set(name, base_globals.get(name) * (1.0 + rng.uniform(-weight_spread, weight_spread)))
        n = int(counts[r])
        max_pos = float("%g" % math.sqrt(n / agent_density))
        g.set("num_agents", n)
        g.set("agent_density", agent_density)
        g.set("max_pos", max_pos)
        globals_list.append(g)
        states.append(boids2d(n, max_pos, seed=int(seeds[r] % (2**31))))
    return globals_list, states, seeds


def _g6(x):
    """A folded constant as the compiler prints it: six significant digits."""
    return float("%g" % x)


def served_job(model_name, n, precision, seed):
    """Globals and initial state for one served job of `n` agents.

    The derived globals are the ones the compiler folds for
    `-P num_agents=n` (in double, the `param float` densities dividing as
    floats; results printed to six significant digits -- checked against the
    compiler's own output in tests/test_library_cpu.py):
      circle             W = sqrt(n / rho) with the file's rho = 0.05
      circle3d           W = cbrt(n / rho) with rho = 0.01 (the file's 0.05 puts
                         ~200 agents inside every interaction sphere)
      boids2d            max_pos = sqrt(n / agent_density), agent_density = 3200.0
      predator_prey      env_size = sqrt(n / 1600) * SPACE_MULT; prey and
                         predator fractions 0.4 and 0.1.
    """
    import math
    from . import runtime as R
    name = model_name + ("_float" if precision == "fp32" else "")
    model = R.Model(name)
    g = model.default_globals()
    fd = np.float32 if model.float_bytes == 4 else np.float64
    if model_name in ("circle", "circle3d"):
        rho = 0.05 if model_name == "circle" else 0.01
        w = _g6(math.sqrt(n / rho) if model_name == "circle" else float(np.cbrt(n / rho)))
        g.set("rho", rho)
        g.set("num_agents", n)
        g.set("W", w)
        st = circle(n, w, dim=2 if model_name == "circle" else 3, seed=seed)
        state = {"Point": {"pos": st["pos"].astype(fd)}}
    elif model_name == "boids2d":
        mp = _g6(math.sqrt(n / 3200.0))
        g.set("num_agents", n)
        g.set("agent_density", 3200.0)
        g.set("max_pos", mp)
        st = boids2d(n, mp, seed=seed)
        state = {"Boid": {k: v.astype(fd) for k, v in st.items()}}
    elif model_name == "predator_prey":
        env = _g6(math.sqrt(n / 1600.0) * 1.0)
        g.set("num_agents", n)
        g.set("prey_fraction", 0.4)
        g.set("predator_fraction", 0.1)
        g.set("env_size", env)
        n_pred, n_prey = int(0.1 * n), int(0.4 * n)
        st = predator_prey(n_pred, n_prey, n - n_pred - n_prey, env, seed=seed)
        state = {t: {k: (v.astype(fd) if v.dtype.kind == "f" else v) for k, v in d.items()}
                 for t, d in st.items()}
    else:
        raise KeyError(model_name)
    return model, g, state


def serving_stream(jobs=100, rate=200.0, n_min=1000, n_max=1000000, steps_min=50,
                   steps_max=1000, seed=0,
                   models=("circle", "circle3d", "boids2d", "predator_prey")):
    """A Poisson stream of jobs: (arrival time, model, agents, timesteps,
    precision, seed), agents log-uniform in [n_min, n_max], timesteps uniform
    in [steps_min, steps_max], FP32/FP64 with equal probability."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out = []
    for k in range(jobs):
        t += rng.exponential(1.0 / rate)
        m = models[int(rng.integers(0, len(models)))]
        n = int(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        if m == "predator_prey":
            n = max(n, 1600)
        steps = int(rng.integers(steps_min, steps_max + 1))
        prec = "fp32" if rng.uniform() < 0.5 else "fp64"
        out.append((t, m, n, steps, prec, int(rng.integers(0, 2**31))))
    return out


def boids3d(n, max_pos, seed=0, vmax=1.0):
    """examples/boids.abl in 3D: positions uniform in [0, max_pos)^3;
    velocity directions uniform on the sphere with speed uniform in
    [0.5, 1] * vmax."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = rng.uniform(0.0, max_pos, size=(n, 3))
    d = unit_vectors(rng, n, 3)
    vel = d * (rng.uniform(0.5, 1.0, size=n) * vmax)[:, None]
    return {"pos": np.ascontiguousarray(pos), "velocity": np.ascontiguousarray(vel)}


def sugarscape(grid_width, occupied_frac=0.1, seed=0, gmax=50, min_sugar=1, max_sugar=10):
    """examples/sugarscape.abl: one agent per grid point at (x + 0.5, y + 0.5),
    ids x-major (main() loops x, then y); occupied with probability
    occupied_frac (state 1, sugar level uniform in [min_sugar, max_sugar],
    metabolism 1), else unoccupied (state 0); the cell's capacity is
    calc_max_env_sugar_level(x, y): two Gaussian hills of height gmax at
    (0.25, 0.25) and (0.75, 0.75) * grid_width with variance
    0.025 * grid_width^2, each term added to an int (truncation), distances
    as libabl's dist (float-rounded square root); the sugar level starts
    uniform in [0, capacity]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    w = grid_width
    x, y = np.meshgrid(np.arange(w, dtype=np.float64), np.arange(w, dtype=np.float64),
                       indexing="ij")
    x, y = x.ravel(), y.ravel()
    var = 0.025 * w * w
    cap = np.zeros(w * w, dtype=np.int64)
    for c in (0.25 * w, 0.75 * w):
        d2 = (x - c) * (x - c) + (y - c) * (y - c)
        d = np.sqrt(d2.astype(np.float32)).astype(np.float64)
        cap = np.trunc(cap + gmax * np.exp(-d * d / (2 * var))).astype(np.int64)
    occupied = rng.uniform(size=w * w) < occupied_frac
    sugar = np.where(occupied, rng.integers(min_sugar, max_sugar + 1, size=w * w), 0)
    env = rng.integers(0, cap + 1)
    return {"pos": np.ascontiguousarray(np.stack([x + 0.5, y + 0.5], axis=1)),
            "target_pos": np.zeros((w * w, 2)),
            "agent_id": np.arange(w * w, dtype=np.int32),
            "state": occupied.astype(np.int32),
            "sugar_level": sugar.astype(np.int32),
            "metabolism": occupied.astype(np.int32),
            "env_sugar_level": env.astype(np.int32),
            "max_env_sugar_level": cap.astype(np.int32)}
