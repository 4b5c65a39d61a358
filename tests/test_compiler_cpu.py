"""The OpenABL compiler with the `cuda` backend plugged in (CPU only).

These tests need an OpenABL source tree (the compiler is built from it by
openabl_gb300/backend/Makefile with the hand-written front end in place of
the flex/bison output); they are skipped where none is present.

- The reference's lint goldens (test.sh:34-52): `--lint-only` on every
  test/*.abl that has a .exp file prints exactly the expected errors,
  compared with `diff -b` as test.sh does.  This pins the hand-written
  parser: every error message carries the line the bison parser would
  have recorded.
- The reference's example smoke test (test.sh:55-93) for `-b cuda`: every
  example either generates code or is refused with exit code 2 (a
  BackendError, which test.sh counts as a skip).
- The model sources compiled into the library are what the generator
  prints today (openabl_gb300/generated/regenerate.py writes them).
"""
import glob
import json
import os
import shutil
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# The OpenABL source tree: $OPENABL_REF, else a `reference` directory beside
# this repository.
REF = os.environ.get("OPENABL_REF") or os.path.join(os.path.dirname(REPO), "reference")
COMPILER = os.path.join(REPO, "_build", "compiler", "openabl")
GEN = os.path.join(REPO, "openabl_gb300", "generated")

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")),
                                reason="no OpenABL source tree to build the compiler from")


@pytest.fixture(scope="module")
def compiler():
    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "openabl_gb300", "backend"),
                           "-j8", f"REF={REF}"], stdout=subprocess.DEVNULL)
    return COMPILER


def _lint_cases():
    if not os.path.isdir(os.path.join(REF, "test")):
        return []
    return sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(REF, "test", "*.abl"))
                  if os.path.exists(f[:-4] + ".exp"))


@pytest.mark.parametrize("case", _lint_cases())
def test_lint_golden(compiler, case, tmp_path):
    src = os.path.join(REF, "test", case + ".abl")
    out = tmp_path / (case + ".out")
    with open(out, "w") as f:
        subprocess.run([compiler, "-A", os.path.join(REF, "asset"), "--lint-only", "-i", src],
                       stderr=f, stdout=subprocess.DEVNULL)
    r = subprocess.run(["diff", "-b", str(out), os.path.join(REF, "test", case + ".exp")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout


def _examples():
    return sorted(os.path.basename(f)[:-4]
                  for f in glob.glob(os.path.join(REF, "examples", "*.abl")))


@pytest.mark.parametrize("example", _examples())
def test_example_generates_or_is_refused(compiler, example, tmp_path):
    r = subprocess.run([compiler, "-A", os.path.join(REF, "asset"), "-i",
                        os.path.join(REF, "examples", example + ".abl"), "-o", str(tmp_path),
                        "-b", "cuda", "-C", f"cuda.model={example}"],
                       capture_output=True, text=True)
    assert r.returncode in (0, 2), r.stdout + r.stderr
    if r.returncode == 0:
        for f in (example + ".cu", example + ".globals.json", "build.sh", "run.sh",
                  "abl_runtime.cu", "openabl_cuda.h"):
            assert (tmp_path / f).exists(), f
        json.load(open(tmp_path / (example + ".globals.json")))


def test_unsupported_feature_exits_with_backend_error(compiler, tmp_path):
    # A near() radius read from the agent: no single cell size serves the
    # loop, so the cuda backend refuses the model (exit 2, main.cpp:270-274).
    r = subprocess.run([compiler, "-A", os.path.join(REF, "asset"), "-i",
                        os.path.join(REPO, "tests", "models", "agent_radius.abl"), "-o",
                        str(tmp_path), "-b", "cuda"], capture_output=True, text=True)
    assert r.returncode == 2
    assert "radius" in r.stdout + r.stderr


@pytest.mark.parametrize("example,accepted", [("boids2d", True), ("predator_prey", True),
                                              ("game_of_life", False), ("sugarscape", False)])
def test_device_init_takes_independent_add_loops_only(compiler, example, accepted, tmp_path):
    """-C cuda.device_init=true turns main()'s `for (int i : a..b) add(T{...})`
    loops into kernels; a main() that builds agents any other way (nested
    loops, a running counter) is refused with the plugin's exit code 2."""
    r = subprocess.run([compiler, "-A", os.path.join(REF, "asset"), "-i",
                        os.path.join(REF, "examples", example + ".abl"), "-o", str(tmp_path),
                        "-b", "cuda", "-C", f"cuda.model={example}", "-C", "cuda.device_init=true"],
                       capture_output=True, text=True)
    assert r.returncode == (0 if accepted else 2), r.stdout + r.stderr
    if accepted:
        src = (tmp_path / (example + ".cu")).read_text()
        assert "__global__ void abl_init_0(" in src and "abl_reserve(ctx" in src


def test_committed_model_sources_are_current(compiler):
    sys.path.insert(0, GEN)
    import regenerate
    for model, (example, config) in regenerate.MODELS.items():
        out = regenerate.run_compiler(model, {})
        with open(os.path.join(out, model + ".cu")) as f:
            now = f.read()
        shutil.rmtree(out)
        with open(os.path.join(GEN, model + ".cu")) as f:
            committed = f.read()
        assert now == committed, f"{model}.cu differs from the generator's output"
    configs = json.load(open(os.path.join(GEN, "configs.json")))
    for name, (model, params) in regenerate.CONFIGS.items():
        out = regenerate.run_compiler(model, params)
        with open(os.path.join(out, model + ".globals.json")) as f:
            manifest = json.load(f)
        shutil.rmtree(out)
        assert configs[name]["globals"] == manifest["globals"], name


def test_seed_option_keys_random_in_steps(compiler, tmp_path):
    """-C cuda.seed=N: the generated program keys random() in steps by N."""
    r = subprocess.run([compiler, "-A", os.path.join(REF, "asset"), "-i",
                        os.path.join(REF, "examples", "boids2d_flockers.abl"), "-o", str(tmp_path),
                        "-b", "cuda", "-C", "cuda.model=flockers", "-C", "cuda.seed=42"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    src = (tmp_path / "flockers.cu").read_text()
    assert 'abl_check(abl_set_seed(ctx, 42ull), "abl_set_seed");' in src


def test_constant_arrays_and_local_radius(compiler, tmp_path):
    """Constant arrays become fixed-size fields of the globals block with the
    reference's initialisers; a near() radius held in a step-local variable of
    globals (keratinocyte's `float radius = 125;`) stands for its value."""
    r = subprocess.run([compiler, "-A", os.path.join(REF, "asset"), "-i",
                        os.path.join(REPO, "tests", "models", "kinds.abl"), "-o",
                        str(tmp_path / "kinds"), "-b", "cuda", "-C", "cuda.model=kinds"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    src = (tmp_path / "kinds" / "kinds.cu").read_text()
    assert "float WEIGHT[3];" in src and "int NEXT_KIND[3];" in src
    assert "abl_G.WEIGHT[nx->kind]" in src
    r = subprocess.run([compiler, "-A", os.path.join(REF, "asset"), "-i",
                        os.path.join(REF, "examples", "keratinocyte.abl"), "-o",
                        str(tmp_path / "ker"), "-b", "cuda", "-C", "cuda.model=keratinocyte"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    src = (tmp_path / "ker" / "keratinocyte.cu").read_text()
    # the host's radius function and the presorted phase use the initialiser
    assert "return (double) (((double) (125.0)));" in src


def step_descriptor(model, step):
    """The fields of a generated step descriptor (abl_step_desc), by name."""
    src = open(os.path.join(REPO, "openabl_gb300", "generated", model + ".cu")).read()
    line = next(l for l in src.splitlines() if l.strip().startswith('{"%s",' % step))
    f = [x.strip() for x in line.strip().strip("{},").split(",")]
    names = ["name", "agent_type", "near_type", "ordered", "radius", "near_members",
             "out_written", "launch", "uses_remove", "add_type", "out_copy", "launch_ens",
             "uses_rng", "presorted", "out_changed", "near_cacheable"]
    return dict(zip(names, f))


@pytest.mark.parametrize("model,step,changed,cacheable", [
    # out.pos = in.pos is not a change: game_of_life's positions never move
    ("game_of_life", "step_move", "2u", "1"),
    ("boids2d", "update_boid", "3u", "1"),
    # sugarscape's agents sit on the grid; the step writes state and target
    ("sugarscape", "movement_request", "10u", "1"),
    ("kinds", "mix", "6u", "1"),
    # no near loop
    ("predator_prey", "prey_move", "11u", "0"),
])
def test_step_descriptors(model, step, changed, cacheable):
    """The analysis behind static positions and kept neighbour lists: which
    members a step may change, and whether its near loop is centred on its own
    agent with a radius of globals."""
    d = step_descriptor(model, step)
    if changed is not None:
        assert d["out_changed"] == changed
    assert d["near_cacheable"] == cacheable


def test_runtime_settings_options(compiler, tmp_path):
    """-C cuda.near_mode / cuda.near_cache / cuda.balance become calls in the
    generated main(); an unknown mode is refused with exit 2."""
    base = [compiler, "-A", os.path.join(REF, "asset"), "-i",
            os.path.join(REF, "examples", "boids2d.abl"), "-b", "cuda", "-C", "cuda.model=b"]
    r = subprocess.run(base + ["-o", str(tmp_path / "a"), "-C", "cuda.near_mode=lists",
                               "-C", "cuda.near_cache=false", "-C", "cuda.balance=false"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    src = (tmp_path / "a" / "b.cu").read_text()
    assert 'abl_check(abl_set_near_mode(ctx, 3), "abl_set_near_mode");' in src
    assert 'abl_check(abl_set_near_cache(ctx, 0), "abl_set_near_cache");' in src
    assert 'abl_check(abl_set_balance(ctx, 0), "abl_set_balance");' in src
    r = subprocess.run(base + ["-o", str(tmp_path / "b"), "-C", "cuda.near_mode=fastest"],
                       capture_output=True, text=True)
    assert r.returncode == 2
