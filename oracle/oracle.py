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
        if not os.path.exists(path) or (os.path.getmtime(path)
                                        < os.path.getmtime(os.path.join(HERE, "abl_oracle.c"))):
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


def game_of_life_step(state, c, mode=1, nthreads=0, first=0, count=None):
    pos = np.ascontiguousarray(state["pos"])
    alive = np.ascontiguousarray(state["alive"], dtype=np.uint8)
    n = pos.shape[0]
    po, ao = pos.copy(), alive.copy()
    first, count = _range(n, first, count)
    lib().oracle_game_of_life_step(n, _ptr(pos), _ptr(alive), _ptr(po), _ptr(ao), c["radius"],
                                   float(c["size"]), mode, nthreads, first, count)
    return {"pos": po, "alive": ao}


STEP = {"circle": circle_step, "circle3d": circle_step, "boids2d": boids2d_step,
        "game_of_life": game_of_life_step}
