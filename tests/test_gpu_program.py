"""Whole generated programs as a drop-in for the reference's.

`OpenABL -b cuda` writes <model>.cu (openabl_gb300/generated/ holds the
generator's output for each model): kernels plus the program's main(), which
initialises the agents on the host from the reference's xorshift stream
(asset/c/libabl.c:8-39), runs the simulate loop on the GPU through the C ABI
and writes the result with save() (libabl.c:215-231).  Here each program is
built with the backend's build.sh line (-DABL_STANDALONE_MAIN, -fmad=false)
and run in an empty directory; the file its save() writes must equal, byte
for byte, the file the reference `c` program writes at the same (default)
parameters (tests/golden/programs.json, made by make_golden.py).
"""
import hashlib
import json
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(REPO, "openabl_gb300", "csrc")
GEN = os.path.join(REPO, "openabl_gb300", "generated")
INC = os.path.join(REPO, "include")
PROGRAMS = json.load(open(os.path.join(REPO, "tests", "golden", "programs.json")))

# The cuda backend's build.sh line (openabl_gb300/backend/CudaBackend.cpp).
NVCC = [shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc", "-gencode",
        "arch=compute_103a,code=sm_103a", "-O3", "-fmad=false", "-Xcompiler",
        "-ffp-contract=off", "-std=c++17",
        "-diag-suppress", "177", "-DABL_STANDALONE_MAIN", "-I", CSRC, "-I", INC]


def build_program(model, runtime_objects, tmp_path, defines=()):
    """The two compilations of build.sh: the model file for its kernels, host
    code and main(), and (models with an ensemble form) again with
    ABL_PERSIST for the persistent ensemble kernel; then the link."""
    src = os.path.join(GEN, model + ".cu")
    objs = [str(tmp_path / (model + ".o"))]
    subprocess.check_call(NVCC + list(defines) + ["-c", src, "-o", objs[0]])
    with open(src) as f:
        if "#ifdef ABL_PERSIST" in f.read():
            objs.append(str(tmp_path / (model + ".persist.o")))
            subprocess.check_call(NVCC + ["-DABL_PERSIST", "-c", src, "-o", objs[1]])
    exe = str(tmp_path / "main")
    subprocess.check_call(NVCC[:3] + objs + runtime_objects + ["-o", exe])
    return exe


@pytest.fixture(scope="module")
def runtime_objects(tmp_path_factory):
    d = tmp_path_factory.mktemp("abl_program_runtime")
    objs = []
    for src in ("abl_runtime.cu", "abl_host.cpp"):
        obj = str(d / (src + ".o"))
        subprocess.check_call(NVCC + ["-c", os.path.join(CSRC, src), "-o", obj])
        objs.append(obj)
    return objs


@pytest.mark.gpu
@pytest.mark.parametrize("model", sorted(PROGRAMS))
def test_generated_program_writes_the_reference_output(model, runtime_objects, tmp_path):
    want = PROGRAMS[model]
    # Programs drawing random numbers in steps were recorded on one thread;
    # -DABL_SERIAL_RANDOM continues the host stream in the same order.
    serial = ["-DABL_SERIAL_RANDOM"] if want.get("serial_random") else []
    exe = build_program(model, runtime_objects, tmp_path, serial)
    run_dir = tmp_path / "run"
    run_dir.mkdir()
    subprocess.run([exe], cwd=run_dir, check=True, stdout=subprocess.DEVNULL, timeout=300)
    assert sorted(os.listdir(run_dir)) == [want["file"]]
    data = (run_dir / want["file"]).read_bytes()
    assert len(data) == want["bytes"]
    assert hashlib.sha256(data).hexdigest() == want["sha256"]


@pytest.mark.gpu
def test_device_initialised_program_matches_the_oracle(runtime_objects, tmp_path):
    """`-C cuda.device_init=true`: boids2d's main() loop `for (int i :
    0..num_agents) add(Boid{...})` runs as a kernel drawing from the
    counter-based stream (so results differ from the reference's host init
    by design).  The oracle restates those draws (oracle_devinit_boids2d) and
    the 100 timesteps that follow; the file the program writes must equal,
    byte for byte, the oracle's state written in save()'s JSON layout
    (asset/c/libabl.c:46-124).  Two runs of the program write the same file."""
    import numpy as np
    import openabl_gb300 as o
    from oracle import oracle as O
    exe = build_program("boids2d_devinit", runtime_objects, tmp_path)
    outs = []
    for k in range(2):
        run_dir = tmp_path / f"run{k}"
        run_dir.mkdir()
        subprocess.run([exe], cwd=run_dir, check=True, stdout=subprocess.DEVNULL, timeout=300)
        outs.append((run_dir / "boids.out").read_bytes())
    assert outs[0] == outs[1]
    g = o.Model("boids2d").default_globals()
    n = g.get("num_agents")
    state = O.devinit_boids2d(n, g.get("min_pos"), g.get("max_pos"))
    c = {k: g.get(k) for k in O.BOIDS2D_KEYS}
    for _ in range(g.get("num_timesteps")):
        state = O.boids2d_step(state, c, mode=1)
    want = '{"Boid":[' + ",\n".join(
        '{"pos":[%f,%f],"velocity":[%f,%f]}' % (p[0], p[1], v[0], v[1])
        for p, v in zip(state["pos"], state["velocity"])) + "]}"
    assert outs[0].decode() == want


# Models that call random() inside step functions.  The reference draws those
# numbers from one xorshift stream shared by all OpenMP threads
# (asset/c/libabl.c:8-39), so its own runs differ from one another; the cuda
# backend draws from a counter-based stream keyed by agent, step and draw, so
# a run repeats exactly.  Each program runs twice here: the files it writes
# must match (keratinocyte's log.csv without its timing column), and they
# must hold the populations the models keep.
UNPINNED = {"ants": "ants.out", "boids2d_flockers": "boids.out", "keratinocyte": "log.csv"}
# (ants and boids2d_flockers are also pinned in their sequential mode, above,
# against the reference programs run on one thread)


def run_program(exe, run_dir):
    run_dir.mkdir()
    subprocess.run([exe], cwd=run_dir, check=True, stdout=subprocess.DEVNULL, timeout=300)
    return sorted(os.listdir(run_dir))


@pytest.mark.gpu
@pytest.mark.parametrize("model", sorted(UNPINNED))
def test_programs_with_random_steps_repeat_exactly(model, runtime_objects, tmp_path):
    exe = build_program(model, runtime_objects, tmp_path)
    out = UNPINNED[model]
    texts = []
    for r in ("a", "b"):
        assert run_program(exe, tmp_path / r) == [out]
        texts.append((tmp_path / r / out).read_text())
    if model == "keratinocyte":
        rows = [[line.split(",") for line in t.splitlines()] for t in texts]
        assert len(rows[0]) == 100  # one line per timestep
        assert [r[:-1] for r in rows[0]] == [r[:-1] for r in rows[1]]
        assert all(sum(int(v) for v in r[:-1]) > 0 for r in rows[0])
    else:
        assert texts[0] == texts[1]
        data = json.loads(texts[0])
        n = {"ants": None, "boids2d_flockers": 1000}[model]
        if n is not None:
            assert sum(len(v) for v in data.values()) == n
