"""The C-ABI library loads on a machine without a GPU and exports every
entry point that include/openabl_cuda.h declares; the model descriptors
compiled into it are readable (no compute call is made here)."""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for f in sorted(os.listdir(os.path.join(REPO, "include"))):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(REPO, "include", f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^[A-Za-z_][\w\s\*]*?\b(abl_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from openabl_gb300 import build_lib
    build_lib.build()
    return ctypes.CDLL(build_lib.LIB)


def test_every_declared_entry_point_is_exported(lib):
    names = declared_functions()
    assert "abl_create" in names and "abl_run" in names
    for n in names:
        assert hasattr(lib, n), n


def test_model_descriptors(lib):
    import openabl_gb300 as o
    for name, agent, members in [("circle", "Point", ["pos"]), ("boids2d", "Boid",
                                 ["pos", "velocity"]), ("game_of_life", "Cell", ["pos", "alive"]),
                                 ("circle3d", "Point", ["pos"])]:
        m = o.Model(name)
        assert m.agent_types[0][0] == agent
        assert [x[0] for x in m.agent_types[0][1]] == members


def test_config_globals_are_the_printed_constants():
    import openabl_gb300 as o
    _, g = o.globals_for_config("boids2d_1m")
    assert g.get("max_pos") == 18.1019      # sqrt(1048576 / 3200.0) printed to 6 digits
    assert g.get("num_agents") == 1048576
    _, g = o.globals_for_config("circle_4000")
    assert g.get("W") == 200.0
