"""The mixed-precision form (-C cuda.precision=mixed): near-loop sums of
neighbour members in FP32, everything else in FP64.

Its results are not the reference's bits, so it is checked against the FP64
oracle (itself pinned to the reference) with a stated tolerance: after every
timestep, every agent's position within 1e-5 of the domain side and every
velocity within 1e-5 of the FP64 value -- the precision target the form is
built for (trajectory error <= 1e-5 relative to FP64 after 100 timesteps).
Positions are compared up to the domain's periodic image (boundPosition
wraps an agent leaving the domain to the opposite side).  The form must also
repeat itself exactly: one timestep at a time and graph replay give the
same bits.
"""
import numpy as np
import pytest

import openabl_gb300 as o
from golden_io import load_case
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-5


def rel_pos_err(a, b, L):
    d = np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))
    return (np.minimum(d, np.abs(L - d)).max(axis=1) / L).max()


@pytest.mark.parametrize("config,case,step", [
    ("boids2d_mixed_4096", "boids2d_4096", O.boids2d_step),
    ("boids3d_mixed_5000", "boids3d_5000", O.boids3d_step)])
def test_mixed_within_tolerance_of_fp64_every_timestep(config, case, step):
    meta, state = load_case(case)
    model, g = o.globals_for_config(config)
    c = {k: g.get(k) for k in O.BOIDS2D_KEYS}
    L = g.get("max_pos") - g.get("min_pos")
    sim = o.Simulation(model, g)
    sim.upload("Boid", state)
    ref = state
    worst = 0.0
    for t in range(100):
        sim.step()
        ref = step(ref, c, mode=1)
        got = sim.download("Boid")
        ep = rel_pos_err(got["pos"], ref["pos"], L)
        ev = np.abs(got["velocity"] - ref["velocity"]).max()
        worst = max(worst, ep)
        assert ep <= TOL and ev <= TOL, (t + 1, ep, ev)
    # not bit-identical to FP64: the sums really run in FP32
    assert not np.array_equal(got["velocity"], ref["velocity"])
    sim.close()


def test_mixed_repeats_exactly_through_graph_replay():
    meta, state = load_case("boids2d_4096")
    model, g = o.globals_for_config("boids2d_mixed_4096")
    a = o.Simulation(model, g)
    a.upload("Boid", state)
    for _ in range(20):
        a.step()
    b = o.Simulation(model, g)
    b.upload("Boid", state)
    b.run(20)
    x, y = a.download("Boid"), b.download("Boid")
    for k in x:
        assert np.array_equal(x[k], y[k]), k
    a.close()
    b.close()


def test_mixed_models_are_refused_where_float_copies_are_missing():
    """The ensemble and the allocation-free timestep do not build the float
    copies the FP32 sums read, so they refuse mixed models."""
    model, g = o.globals_for_config("boids2d_mixed_4096")
    with pytest.raises(o.AblError) as e:
        o.Ensemble(model, [g, g])
    assert e.value.code == -6
