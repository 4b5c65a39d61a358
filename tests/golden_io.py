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
