"""Builds the reference `c` backend programs used to pin the oracle.

Test infrastructure, run only where the reference tree is present.  For each
case below it
  1. builds the OpenABL compiler from the reference sources (see
     openabl_gb300/backend/Makefile),
  2. runs `openabl -b c` on the reference example with the case's -P/-C
     values, producing the reference's own main.c (src/backend/CBackend.cpp),
  3. inserts one call `abl_ref_dump(&agents, agents_info);` after the
     `dyn_array tmp;` line that opens every timestep
     (src/backend/CPrinter.cpp:191-194) and compiles main.c with the
     reference's build line (CBackend.cpp:21-27) plus `-Dsave=abl_ref_save`,
     the reference's asset/c/libabl.c and oracle/ref_harness.c,
  4. leaves the program in oracle/_ref/<case>/main (git-ignored).

PROGRAMS are built unmodified (no dump hook, the example's default
parameters) into oracle/_ref/prog_<model>/main: their save() output files
are the reference results that the whole `-b cuda` program must reproduce.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
# The OpenABL source tree: $OPENABL_REF, else a `reference` directory beside
# this repository.
REF = os.environ.get("OPENABL_REF") or os.path.join(os.path.dirname(REPO), "reference")
OUT = os.path.join(HERE, "_ref")
COMPILER = os.path.join(REPO, "_build", "compiler", "openabl")

# name -> (example, -P params, -C config)
CASES = {
    "circle_4000": ("circle", {"num_agents": "4000", "rho": "0.1", "num_timesteps": "100"}, {}),
    "circle3d_4000": ("circle3d", {"num_agents": "4000", "rho": "0.01", "num_timesteps": "50"}, {}),
    "boids2d_4096": ("boids2d", {"num_agents": "4096", "agent_density": "3200.0",
                                 "num_timesteps": "100"}, {}),
    "game_of_life_64": ("game_of_life", {"num_agents": "4096", "alive_fraction": "0.5",
                                         "num_timesteps": "100"}, {}),
    "boids2d_4096_float": ("boids2d", {"num_agents": "4096", "agent_density": "3200.0",
                                       "num_timesteps": "100"}, {"use_float": "true"}),
    "circle_4000_float": ("circle", {"num_agents": "4000", "rho": "0.1", "num_timesteps": "100"},
                          {"use_float": "true"}),
    "circle3d_4000_float": ("circle3d", {"num_agents": "4000", "rho": "0.01",
                                         "num_timesteps": "50"}, {"use_float": "true"}),
    "boids3d_5000": ("boids", {"num_timesteps": "100"}, {}),
    "sugarscape_10000": ("sugarscape", {"num_timesteps": "100"}, {}),
    # random() inside the step: recorded on one OpenMP thread (SERIAL_RANDOM)
    "boids2d_flockers_1000": ("boids2d_flockers", {"num_timesteps": "50"}, {}),
}

# model -> (example, -C config): whole reference programs at default parameters
PROGRAMS = {
    "circle": ("circle", {}),
    "circle3d": ("circle3d", {}),
    "boids2d": ("boids2d", {}),
    "game_of_life": ("game_of_life", {}),
    "boids2d_float": ("boids2d", {"use_float": "true"}),
    "circle_float": ("circle", {"use_float": "true"}),
    "circle3d_float": ("circle3d", {"use_float": "true"}),
    "boids3d": ("boids", {}),
    # a model of this repository's tests (constant arrays, a member written
    # on one branch only)
    "kinds": ("tests/models/kinds", {}),
    # a model of this repository's tests: a near loop over another agent
    # type whose agents no step changes
    "grazers": ("tests/models/grazers", {}),
    # random() inside the step: run on one OpenMP thread, so its draws come
    # from the xorshift stream in agent order (SERIAL_RANDOM)
    "boids2d_flockers": ("boids2d_flockers", {}),
    # random() and randomInt() inside ant_act (serial, as boids2d_flockers)
    "ants": ("ants", {}),
}

# Programs whose reference run uses one thread and whose cuda build continues
# the host stream in steps (-DABL_SERIAL_RANDOM).
SERIAL_RANDOM = {"boids2d_flockers", "boids2d_flockers_1000", "ants"}


def model_path(example):
    """An example of the reference tree, or a model path within this repository."""
    if "/" in example:
        return os.path.join(REPO, example + ".abl")
    return os.path.join(REF, "examples", example + ".abl")


def build_compiler():
    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "openabl_gb300", "backend"),
                           "-j8", f"REF={REF}"])


def build_case(name):
    example, params, config = CASES[name]
    d = os.path.join(OUT, name)
    os.makedirs(d, exist_ok=True)
    cmd = [COMPILER, "-A", os.path.join(REF, "asset"), "-i",
           os.path.join(REF, "examples", example + ".abl"), "-o", d, "-b", "c"]
    for k, v in params.items():
        cmd += ["-P", f"{k}={v}"]
    for k, v in config.items():
        cmd += ["-C", f"{k}={v}"]
    subprocess.check_call(cmd)
    src = open(os.path.join(d, "main.c")).read()
    marker = "dyn_array tmp;"
    assert src.count(marker) == 1, "unexpected simulate loop shape"
    src = src.replace(marker, marker + " abl_ref_dump(&agents, agents_info);")
    src = src.replace('#include "libabl.h"',
                      '#include "libabl.h"\nvoid abl_ref_dump(void *, const agent_info *);', 1)
    with open(os.path.join(d, "main_dump.c"), "w") as f:
        f.write(src)
    use_float = config.get("use_float") == "true"
    fl = ["-DLIBABL_USE_FLOAT=1"] if use_float else []
    asset_c = os.path.join(REF, "asset", "c")
    # Reference build line: gcc -O2 -std=c99 [-DLIBABL_USE_FLOAT=1] main.c libabl.c -lm -fopenmp
    subprocess.check_call(["gcc", "-O2", "-std=c99", *fl, "-Dsave=abl_ref_save", "-I", asset_c,
                           "-c", os.path.join(d, "main_dump.c"), "-o", os.path.join(d, "main.o"),
                           "-fopenmp"])
    subprocess.check_call(["gcc", "-O2", "-std=c99", *fl, "-I", asset_c, "-c",
                           os.path.join(asset_c, "libabl.c"), "-o", os.path.join(d, "libabl.o")])
    subprocess.check_call(["gcc", "-O2", "-std=c99", *fl, "-I", asset_c, "-c",
                           os.path.join(HERE, "ref_harness.c"), "-o", os.path.join(d, "harness.o")])
    subprocess.check_call(["gcc", os.path.join(d, "main.o"), os.path.join(d, "libabl.o"),
                           os.path.join(d, "harness.o"), "-lm", "-fopenmp", "-o",
                           os.path.join(d, "main")])
    return os.path.join(d, "main")


def build_program(model):
    """The reference compiler's unmodified `c` output for `model` at default
    parameters, compiled with the build line of CBackend.cpp:21-27."""
    example, config = PROGRAMS[model]
    d = os.path.join(OUT, "prog_" + model)
    os.makedirs(d, exist_ok=True)
    cmd = [COMPILER, "-A", os.path.join(REF, "asset"), "-i", model_path(example), "-o", d,
           "-b", "c"]
    for k, v in config.items():
        cmd += ["-C", f"{k}={v}"]
    subprocess.check_call(cmd)
    fl = ["-DLIBABL_USE_FLOAT=1"] if config.get("use_float") == "true" else []
    subprocess.check_call(["gcc", "-O2", "-std=c99", *fl, os.path.join(d, "main.c"),
                           os.path.join(d, "libabl.c"), "-lm", "-fopenmp", "-o",
                           os.path.join(d, "main")])
    return os.path.join(d, "main")


def main(argv):
    if not os.path.isdir(REF):
        print("reference tree not present; nothing to build")
        return 0
    build_compiler()
    names = argv[1:] or list(CASES)
    for n in names:
        print("built", build_case(n))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
