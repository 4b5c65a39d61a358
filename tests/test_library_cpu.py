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


def test_served_job_globals_match_compiler_folding():
    """The serving helper derives per-job globals the way the compiler folds
    them; configs.json holds what the compiler printed for these -P values."""
    import openabl_gb300 as o
    from openabl_gb300 import workloads
    cfg = o.configs()
    for name, key in [("boids2d_1m", "max_pos"), ("boids2d_4096", "max_pos"),
                      ("predator_prey_1m", "env_size"), ("predator_prey_small", "env_size")]:
        c = cfg[name]
        n = int(c["globals"]["num_agents"])
        _, g, _ = workloads.served_job(c["model"].replace("_float", ""), n, "fp64", 0)
        assert g.get(key) == float(c["globals"][key]), name


def test_every_error_code_has_its_own_text(lib):
    """abl_strerror (no GPU needed) names every ABL_E_* code the header
    defines, each differently."""
    src = open(os.path.join(REPO, "include", "openabl_cuda.h")).read()
    codes = {n: int(v) for n, v in re.findall(r"#define (ABL_E_\w+) (-\d+)", src)}
    assert "ABL_E_IO" in codes and len(codes) >= 10
    lib.abl_strerror.restype = ctypes.c_char_p
    lib.abl_strerror.argtypes = [ctypes.c_int]
    texts = {n: lib.abl_strerror(v).decode() for n, v in codes.items()}
    unknown = lib.abl_strerror(-999).decode()
    for n, t in texts.items():
        assert t and t != unknown, n
    assert len(set(texts.values())) == len(texts)


@pytest.mark.parametrize("name", ["kinds", "boids2d_flockers", "ants", "keratinocyte",
                                  "boids3d", "sugarscape"])
def test_more_models_are_compiled_in(lib, name):
    import openabl_gb300 as o
    m = o.Model(name)
    assert m.agent_types
