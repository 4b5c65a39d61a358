"""ctypes front end of the CPU oracle (abl_oracle.c) — test infrastructure.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module.  It builds liboracle.so with oracle/Makefile on first use.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_d = ctypes.c_double
_l = ctypes.c_long
_i = ctypes.c_int
_p = ctypes.c_void_p


def build():
    subprocess.check_call(["make", "-s", "-C", HERE])


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        srcs = [os.path.join(HERE, f) for f in ("abl_oracle.c", "abl_oracle_pp.h")]
        if not os.path.exists(path) or (os.path.getmtime(path)
                                        < max(os.path.getmtime(f) for f in srcs)):
            build()
        L = ctypes.CDLL(path)
        L.oracle_random_float.restype = _d
        L.oracle_random_float.argtypes = [_d, _d]
        L.oracle_random_int.restype = _i
        L.oracle_random_int.argtypes = [_i, _i]
        L.oracle_init_circle.argtypes = [_i, _l, _d, _p]
        L.oracle_init_boids2d.argtypes = [_l, _d, _d, _p, _p]
        L.oracle_init_game_of_life.argtypes = [_i, _d, _p, _p]
        L.oracle_circle_step.argtypes = [_i, _l, _p, _p, _d, _d, _d, _d, _p, _p, _i, _i, _l, _l]
        L.oracle_boids2d_step.argtypes = [_l, _p, _p, _p, _p, _p, _i, _i, _l, _l]
        L.oracle_init_boids3d.argtypes = [_l, _d, _d, _p, _p]
        L.oracle_devinit_boids2d.argtypes = [_l, _d, _d, _p, _p]
        L.oracle_sugarscape_step.argtypes = [_i, _l, _p, _p, _d, _d, _i, _i]
        L.oracle_flockers_step.argtypes = [_l, _p, _p, _p, _p, _p, _i]
        L.oracle_boids2d_step_f32.argtypes = [_l, _p, _p, _p, _p, _p, _i, _i]
        L.oracle_boids3d_step.argtypes = [_l, _p, _p, _p, _p, _p, _i, _i, _l, _l]
        L.oracle_game_of_life_step.argtypes = [_l, _p, _p, _p, _p, _d, _d, _i, _i, _l, _l]
        _LIB = L
    return _LIB


def _ptr(a):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.c_void_p)


def rng_reset():
    lib().oracle_rng_reset()


def init_circle(dim, n, W):
    rng_reset()
    pos = np.zeros((n, dim), np.float64)
    lib().oracle_init_circle(dim, n, W, _ptr(pos))
    return {"pos": pos}


def init_boids2d(n, min_pos, max_pos):
    rng_reset()
    pos = np.zeros((n, 2), np.float64)
    vel = np.zeros((n, 2), np.float64)
    lib().oracle_init_boids2d(n, min_pos, max_pos, _ptr(pos), _ptr(vel))
    return {"pos": pos, "velocity": vel}


def init_game_of_life(size, alive_fraction):
    rng_reset()
    n = size * size
    pos = np.zeros((n, 2), np.float64)
    alive = np.zeros(n, np.uint8)
    lib().oracle_init_game_of_life(size, alive_fraction, _ptr(pos), _ptr(alive))
    return {"pos": pos, "alive": alive}


def _range(n, first, count):
    if count is None:
        count = n - first
    return first, count


def circle_step(state, c, mode=1, nthreads=0, first=0, count=None):
    """One move_point step.  `c` holds the printed constants r, k_rep, k_att, W."""
    pos = np.ascontiguousarray(state["pos"])
    n, dim = pos.shape
    out = pos.copy()
    emin = np.zeros(3)
    emax = np.full(3, c["W"])
    first, count = _range(n, first, count)
    lib().oracle_circle_step(dim, n, _ptr(pos), _ptr(out), c["r"], c["k_rep"], c["k_att"],
                             c["W"], _ptr(emin), _ptr(emax), mode, nthreads, first, count)
    return {"pos": out}


BOIDS2D_KEYS = ("interaction_radius", "separation_radius", "time_scale", "global_scale",
                "steer_scale", "collision_scale", "match_scale", "min_pos", "max_pos")


def boids2d_step(state, c, mode=1, nthreads=0, first=0, count=None):
    pos = np.ascontiguousarray(state["pos"])
    vel = np.ascontiguousarray(state["velocity"])
    n = pos.shape[0]
    po, vo = pos.copy(), vel.copy()
    p = np.array([c[k] for k in BOIDS2D_KEYS] + [0.0], np.float64)
    first, count = _range(n, first, count)
    lib().oracle_boids2d_step(n, _ptr(pos), _ptr(vel), _ptr(po), _ptr(vo), _ptr(p), mode,
                              nthreads, first, count)
    return {"pos": po, "velocity": vo}


def devinit_boids2d(n, min_pos, max_pos):
    """boids2d's main() loop as the device initialisation kernel draws it
    (-C cuda.device_init=true; counter-based stream, see abl_oracle.c)."""
    pos = np.zeros((n, 2), np.float64)
    vel = np.zeros((n, 2), np.float64)
    lib().oracle_devinit_boids2d(n, min_pos, max_pos, _ptr(pos), _ptr(vel))
    return {"pos": pos, "velocity": vel}


def init_boids3d(n, min_pos, max_pos):
    """examples/boids.abl's main(): positions and velocities from the reference stream."""
    rng_reset()
    pos = np.zeros((n, 3), np.float64)
    vel = np.zeros((n, 3), np.float64)
    lib().oracle_init_boids3d(n, min_pos, max_pos, _ptr(pos), _ptr(vel))
    return {"pos": pos, "velocity": vel}


def boids3d_step(state, c, mode=1, nthreads=0, first=0, count=None):
    """One timestep of examples/boids.abl (boids in 3D); constants as BOIDS2D_KEYS."""
    pos = np.ascontiguousarray(state["pos"])
    vel = np.ascontiguousarray(state["velocity"])
    n = pos.shape[0]
    po, vo = pos.copy(), vel.copy()
    p = np.array([c[k] for k in BOIDS2D_KEYS] + [0.0], np.float64)
    first, count = _range(n, first, count)
    lib().oracle_boids3d_step(n, _ptr(pos), _ptr(vel), _ptr(po), _ptr(vo), _ptr(p), mode,
                              nthreads, first, count)
    return {"pos": po, "velocity": vo}


def game_of_life_step(state, c, mode=1, nthreads=0, first=0, count=None):
    pos = np.ascontiguousarray(state["pos"])
    alive = np.ascontiguousarray(state["alive"], dtype=np.uint8)
    n = pos.shape[0]
    po, ao = pos.copy(), alive.copy()
    first, count = _range(n, first, count)
    lib().oracle_game_of_life_step(n, _ptr(pos), _ptr(alive), _ptr(po), _ptr(ao), c["radius"],
                                   float(c["size"]), mode, nthreads, first, count)
    return {"pos": po, "alive": ao}


def boids2d_step_f32(state, c, mode=1, nthreads=0):
    """One timestep of examples/boids2d.abl as built with LIBABL_USE_FLOAT:
    float32 state, constants rounded to float like the printed globals."""
    pos = np.ascontiguousarray(state["pos"], dtype=np.float32)
    vel = np.ascontiguousarray(state["velocity"], dtype=np.float32)
    n = pos.shape[0]
    po, vo = pos.copy(), vel.copy()
    p = np.array([c[k] for k in BOIDS2D_KEYS] + [0.0], np.float32)
    lib().oracle_boids2d_step_f32(n, _ptr(pos), _ptr(vel), _ptr(po), _ptr(vo), _ptr(p), mode,
                                  nthreads)
    return {"pos": po, "velocity": vo}


FLOCKERS_KEYS = ("interaction_radius", "steer_scale", "collision_scale", "match_scale",
                 "randomness_scale", "momentum_scale", "time_scale", "max_pos")


def flockers_step(state, c, mode=1):
    """One timestep of examples/boids2d_flockers.abl as the reference runs it
    on one thread: random() continues the oracle's xorshift stream (reset by
    the init_* functions), agent by agent."""
    pos = np.ascontiguousarray(state["pos"])
    vel = np.ascontiguousarray(state["velocity"])
    n = pos.shape[0]
    po, vo = pos.copy(), vel.copy()
    p = np.array([c[k] for k in FLOCKERS_KEYS] + [0.0], np.float64)
    lib().oracle_flockers_step(n, _ptr(pos), _ptr(vel), _ptr(po), _ptr(vo), _ptr(p), mode)
    return {"pos": po, "velocity": vo}


SUGARSCAPE_MEMBERS = ("pos", "target_pos", "agent_id", "state", "sugar_level", "metabolism",
                      "env_sugar_level", "max_env_sugar_level")


class _SgCols(ctypes.Structure):
    _fields_ = [(m, ctypes.c_void_p) for m in SUGARSCAPE_MEMBERS]


def _sg_cols(state):
    return _SgCols(*[state[m].ctypes.data for m in SUGARSCAPE_MEMBERS])


class Sugarscape:
    """examples/sugarscape.abl's simulate loop with the reference's double
    buffer (src/backend/CPrinter.cpp:189-233): the buffer a step function
    writes starts as a copy of the population and keeps, in the members the
    step does not assign, what it held two swaps before."""

    def __init__(self, state, radius=1.5, grid_width=100.0, mode=1, nthreads=0):
        self.cur = {m: np.array(state[m], copy=True, order="C") for m in SUGARSCAPE_MEMBERS}
        self.dbuf = {m: v.copy() for m, v in self.cur.items()}
        self.radius, self.grid_width = float(radius), float(grid_width)
        self.mode, self.nthreads = mode, nthreads

    def step(self):
        n = len(self.cur["state"])
        for k in range(4):
            a, b = _sg_cols(self.cur), _sg_cols(self.dbuf)
            lib().oracle_sugarscape_step(k, n, ctypes.byref(a), ctypes.byref(b), self.radius,
                                         self.grid_width, self.mode, self.nthreads)
            self.cur, self.dbuf = self.dbuf, self.cur
        return self.cur


STEP = {"circle": circle_step, "circle3d": circle_step, "boids2d": boids2d_step,
        "game_of_life": game_of_life_step, "boids": boids3d_step}


# ------------------------------------------------------------ predator_prey

PP_TYPES = ("Predator", "Prey", "Grass")
PP_DPARAMS = ("PRED_PREY_INTERACTION_RADIUS", "PREY_GROUP_COHESION_RADIUS",
              "SAME_SPECIES_AVOIDANCE_RADIUS", "GRASS_EAT_DISTANCE", "PRED_KILL_DISTANCE",
              "DELTA_TIME", "PRED_SPEED_ADVANTAGE", "SPACE_MULT", "REPRODUCE_PREY_PROB",
              "REPRODUCE_PREDATOR_PROB", "env_size")
PP_IPARAMS = ("GAIN_FROM_FOOD_PREDATOR", "GAIN_FROM_FOOD_PREY", "GRASS_REGROW_CYCLES")


class PredatorPrey:
    """The predator_prey restatement (abl_oracle.c) over a population dict
    {type name: {member: array}} and the printed constants `c`; FP64 build."""

    SUFFIX = ""
    REAL = np.float64

    def _fn(self, name):
        return getattr(lib(), name + self.SUFFIX)

    def __init__(self, state, c, seed=0):
        create = self._fn("oracle_pp_create")
        create.restype = ctypes.c_void_p
        create.argtypes = [_p, _p, ctypes.c_uint64, _p, _p, _p, _p, _p, _p, _p]
        self._fn("oracle_pp_destroy").argtypes = [_p]
        self._fn("oracle_pp_count").restype = _l
        self._fn("oracle_pp_count").argtypes = [_p, _i]
        self._fn("oracle_pp_get").argtypes = [_p, _i, _p, _p, _p, _p, _p, _p]
        self._fn("oracle_pp_run").argtypes = [_p, _i, _i, _i, _p]
        self._keep = []
        dp = np.array([float(c[k]) for k in PP_DPARAMS], np.float64)
        ip = np.array([int(c[k]) for k in PP_IPARAMS], np.int32)
        n = np.array([len(state[t]["pos"]) for t in PP_TYPES], np.int64)
        R = self.REAL

        def arr(a, dt):
            a = np.ascontiguousarray(a, dtype=dt)
            self._keep.append(a)
            return a.ctypes.data

        pos = (ctypes.c_void_p * 3)(*[arr(state[t]["pos"], R) for t in PP_TYPES])
        dirs = (ctypes.c_void_p * 2)(*[arr(state[t]["dir"], R) for t in PP_TYPES[:2]])
        steer = (ctypes.c_void_p * 2)(*[arr(state[t]["steer"], R) for t in PP_TYPES[:2]])
        life = (ctypes.c_void_p * 2)(*[arr(state[t]["life"], np.int32) for t in PP_TYPES[:2]])
        self.h = create(_ptr(dp), _ptr(ip), seed, _ptr(n), pos, dirs, steer, life,
                        arr(state["Grass"]["dead_cycles"], np.int32),
                        arr(state["Grass"]["avail"], np.uint8))

    def run(self, timesteps, mode=1, nthreads=0):
        stats = np.zeros((timesteps, 3), np.int32)
        self._fn("oracle_pp_run")(self.h, timesteps, mode, nthreads, _ptr(stats))
        return stats

    def get(self):
        out = {}
        R = self.REAL
        for k, t in enumerate(PP_TYPES):
            n = self._fn("oracle_pp_count")(self.h, k)
            pos = np.zeros((n, 2), R)
            if t == "Grass":
                dc = np.zeros(n, np.int32)
                av = np.zeros(n, np.uint8)
                self._fn("oracle_pp_get")(self.h, k, _ptr(pos), None, None, None, _ptr(dc),
                                          _ptr(av))
                out[t] = {"pos": pos, "dead_cycles": dc, "avail": av}
            else:
                d, s = np.zeros((n, 2), R), np.zeros((n, 2), R)
                life = np.zeros(n, np.int32)
                self._fn("oracle_pp_get")(self.h, k, _ptr(pos), _ptr(d), _ptr(s), _ptr(life),
                                          None, None)
                out[t] = {"pos": pos, "dir": d, "steer": s, "life": life}
        return out

    def close(self):
        if self.h:
            self._fn("oracle_pp_destroy")(self.h)
            self.h = None


class PredatorPreyF32(PredatorPrey):
    """The same restatement as the use_float build computes it: every member,
    printed constant and intermediate in float (abl_oracle_pp.h)."""

    SUFFIX = "_f32"
    REAL = np.float32
