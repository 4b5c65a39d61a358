"""abl_step_noalloc: one timestep without any device allocation.

Some callers cannot allocate device memory while they run -- code embedded in
another framework's memory pool, or a loop that must not allocate once it has
started.  For them the library exports abl_step_noalloc, which runs one
timestep on device buffers the caller provides and keeps every temporary in a
fixed static device array.  This test drives it through the C ABI on
caller-owned device buffers and checks that two calls in a row (in -> out,
then out -> in) produce, bit for bit, the states that the regular entry points
(abl_upload / abl_step / abl_download) produce after one and two timesteps.
The file sorts last so that a stop-at-first-failure run has already run every
other test; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import openabl_gb300 as o
from golden_io import load_case

pytestmark = pytest.mark.gpu

CASES = [("boids2d_4096", "Boid"), ("game_of_life_64", "Cell"), ("circle_4000", "Point"),
         ("circle3d_4000", "Point")]


def _entry():
    L = o.library()
    f = L.abl_step_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                  ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                  ctypes.c_size_t, ctypes.c_void_p]
    return f


def _device_columns(torch, model, state):
    cols = []
    for name, vt in model.agent_types[0][1]:
        dt, _ = o.runtime.member_dtype(vt, 8)
        cols.append(torch.from_numpy(np.array(state[name], dtype=dt)).cuda())
    return cols


def _ptrs(cols):
    return (ctypes.c_void_p * len(cols))(*[c.data_ptr() for c in cols])


@pytest.mark.parametrize("case,agent", CASES)
def test_noalloc_matches_regular_entry_points_two_calls(case, agent):
    torch = pytest.importorskip("torch")
    meta, state = load_case(case)
    model, g = o.globals_for_config(case)

    # Regular path: context-owned memory.
    sim = o.Simulation(model, g)
    sim.upload(agent, state)
    expected = []
    for _ in range(2):
        sim.step()
        expected.append(sim.download(agent))
    sim.close()

    # Allocation-free path on caller-owned buffers A (input) and B (output).
    a = _device_columns(torch, model, state)
    b = _device_columns(torch, model, state)  # out starts as a copy, like the double buffer
    torch.cuda.synchronize()
    step = _entry()
    n = len(state[model.agent_types[0][1][0][0]])
    rc = step(model.ptr, ctypes.addressof(g.buf), model.globals_size, _ptrs(a), _ptrs(b), n, None)
    assert rc == 0, o.library().abl_strerror(rc)
    rc = step(model.ptr, ctypes.addressof(g.buf), model.globals_size, _ptrs(b), _ptrs(a), n, None)
    assert rc == 0, o.library().abl_strerror(rc)
    torch.cuda.synchronize()
    for got_cols, want in ((b, expected[0]), (a, expected[1])):
        for (name, _), col in zip(model.agent_types[0][1], got_cols):
            assert np.array_equal(col.cpu().numpy(), want[name]), name


def test_noalloc_rejects_problems_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    model, g = o.globals_for_config("boids2d_4096")
    step = _entry()
    n = 131072 + 1
    dummy = torch.zeros(16, dtype=torch.float64, device="cuda")
    cols = (ctypes.c_void_p * 2)(dummy.data_ptr(), dummy.data_ptr())
    rc = step(model.ptr, ctypes.addressof(g.buf), model.globals_size, cols, cols, n, None)
    assert rc == -9
    assert b"scratch" in o.library().abl_strerror(rc)


def test_noalloc_rejects_3d_problems_whose_lists_do_not_fit():
    """In 3D the neighbourhood lists take about 300 bytes per agent, so the
    fixed array runs out well below the agent limit (near 90,000 agents)."""
    torch = pytest.importorskip("torch")
    model, g = o.globals_for_config("circle3d_4000")
    step = _entry()
    dummy = torch.zeros(16, dtype=torch.float64, device="cuda")
    cols = (ctypes.c_void_p * 1)(dummy.data_ptr())
    rc = step(model.ptr, ctypes.addressof(g.buf), model.globals_size, cols, cols, 120000, None)
    assert rc == -9


def test_noalloc_refuses_models_it_cannot_step_without_allocating():
    """random() in a step (its stream is keyed by a timestep this entry point
    does not take) and several agent types are refused before any GPU work."""
    torch = pytest.importorskip("torch")
    step = _entry()
    dummy = torch.zeros(16, dtype=torch.float64, device="cuda")
    cols = (ctypes.c_void_p * 16)(*([dummy.data_ptr()] * 16))
    for name in ("boids2d_flockers", "predator_prey"):
        model = o.Model(name)
        g = model.default_globals()
        rc = step(model.ptr, ctypes.addressof(g.buf), model.globals_size, cols, cols, 4, None)
        assert rc == -6, name
