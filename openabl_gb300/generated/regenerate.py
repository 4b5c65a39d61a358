"""Regenerates the model sources in this directory with `OpenABL -b cuda`.

The code generator is a plugin of the OpenABL compiler, whose sources live in
an OpenABL tree; it runs where such a tree is available (set OPENABL_REF):
    python openabl_gb300/generated/regenerate.py
For every model below it runs the compiler with `-b cuda -C cuda.model=NAME`
and keeps NAME.cu; for every named configuration it records the folded
globals that the compiler printed for those -P values (configs.json), so that
hosts which drive the runtime directly can set up exactly that configuration.
The build compiles the files kept here; it does not need the compiler.
"""
import json
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
REPO = os.path.dirname(PKG)
# The OpenABL source tree: $OPENABL_REF, else a `reference` directory beside
# this repository.
REF = os.environ.get("OPENABL_REF") or os.path.join(os.path.dirname(REPO), "reference")
COMPILER = os.path.join(REPO, "_build", "compiler", "openabl")

# model name -> (example file, -C config)
MODELS = {
    "circle": ("circle.abl", {}),
    "circle3d": ("circle3d.abl", {}),
    "boids2d": ("boids2d.abl", {}),
    "game_of_life": ("game_of_life.abl", {}),
    "boids2d_float": ("boids2d.abl", {"use_float": "true"}),
    "predator_prey": ("predator_prey.abl", {}),
    "circle_float": ("circle.abl", {"use_float": "true"}),
    "circle3d_float": ("circle3d.abl", {"use_float": "true"}),
    "predator_prey_float": ("predator_prey.abl", {"use_float": "true"}),
    "boids3d": ("boids.abl", {}),
    # near-loop sums in FP32, everything else FP64 (-C cuda.precision=mixed)
    "boids2d_mixed": ("boids2d.abl", {"cuda.precision": "mixed"}),
    "boids3d_mixed": ("boids.abl", {"cuda.precision": "mixed"}),
    "sugarscape": ("sugarscape.abl", {}),
    # main()'s add() loop as a kernel (-C cuda.device_init=true)
    "boids2d_devinit": ("boids2d.abl", {"cuda.device_init": "true"}),
    # a model of this repository's tests: constant arrays
    "kinds": ("tests/models/kinds.abl", {}),
    # a model of this repository's tests: a neighbour type no step changes
    "grazers": ("tests/models/grazers.abl", {}),
    # random() inside steps: runs are reproducible, the reference's are not
    "ants": ("ants.abl", {}),
    "boids2d_flockers": ("boids2d_flockers.abl", {}),
    "keratinocyte": ("keratinocyte.abl", {}),
}

# configuration name -> (model, -P params)
CONFIGS = {
    "circle_4000": ("circle", {"num_agents": "4000", "rho": "0.1", "num_timesteps": "100"}),
    "circle3d_4000": ("circle3d", {"num_agents": "4000", "rho": "0.01", "num_timesteps": "50"}),
    "boids2d_4096": ("boids2d", {"num_agents": "4096", "agent_density": "3200.0",
                                 "num_timesteps": "100"}),
    "boids2d_1m": ("boids2d", {"num_agents": "1048576", "agent_density": "3200.0",
                               "num_timesteps": "100"}),
    "boids2d_float_4096": ("boids2d_float", {"num_agents": "4096", "agent_density": "3200.0",
                                             "num_timesteps": "100"}),
    "boids2d_float_1m": ("boids2d_float", {"num_agents": "1048576", "agent_density": "3200.0",
                                           "num_timesteps": "100"}),
    "boids2d_mixed_4096": ("boids2d_mixed", {"num_agents": "4096", "agent_density": "3200.0",
                                             "num_timesteps": "100"}),
    "boids2d_mixed_1m": ("boids2d_mixed", {"num_agents": "1048576", "agent_density": "3200.0",
                                           "num_timesteps": "100"}),
    "circle_float_4000": ("circle_float", {"num_agents": "4000", "rho": "0.1",
                                           "num_timesteps": "100"}),
    "circle3d_float_4000": ("circle3d_float", {"num_agents": "4000", "rho": "0.01",
                                               "num_timesteps": "50"}),
    "game_of_life_64": ("game_of_life", {"num_agents": "4096", "alive_fraction": "0.5",
                                         "num_timesteps": "100"}),
    "game_of_life_4096": ("game_of_life", {"num_agents": "16777216", "alive_fraction": "0.5",
                                           "num_timesteps": "100"}),
    # 800,000 prey and 200,000 predators (and 1,000,000 grass) at the file's
    # density of 1600 agents per unit area.
    "predator_prey_1m": ("predator_prey", {"num_agents": "2000000", "prey_fraction": "0.4",
                                           "predator_fraction": "0.1", "num_timesteps": "500"}),
    "predator_prey_small": ("predator_prey", {"num_agents": "20000", "prey_fraction": "0.4",
                                              "predator_fraction": "0.1", "num_timesteps": "50"}),
    "predator_prey_float_1m": ("predator_prey_float", {"num_agents": "2000000",
                                                       "prey_fraction": "0.4",
                                                       "predator_fraction": "0.1",
                                                       "num_timesteps": "500"}),
    "predator_prey_float_small": ("predator_prey_float", {"num_agents": "20000",
                                                          "prey_fraction": "0.4",
                                                          "predator_fraction": "0.1",
                                                          "num_timesteps": "50"}),
    # examples/boids.abl (3D) at its defaults: 5,000 agents, agent_density 1000.
    "boids3d_5000": ("boids3d", {"num_timesteps": "100"}),
    "boids3d_mixed_5000": ("boids3d_mixed", {"num_timesteps": "100"}),
    # 1,048,576 agents at 16 per unit volume: ~9 agents per interaction cell.
    "boids3d_1m": ("boids3d", {"num_agents": "1048576", "agent_density": "16",
                               "interaction_radius": "0.8", "separation_radius": "0.08",
                               "num_timesteps": "100"}),
    # examples/sugarscape.abl at its defaults: a 100 x 100 grid.
    "sugarscape_10000": ("sugarscape", {"num_timesteps": "100"}),
    "sugarscape_1m": ("sugarscape", {"num_agents": "1048576", "num_timesteps": "100"}),
}


def run_compiler(model, params):
    example, config = MODELS[model]
    out = tempfile.mkdtemp(prefix="abl_gen_")
    src = os.path.join(REPO, example) if "/" in example else os.path.join(REF, "examples", example)
    cmd = [COMPILER, "-A", os.path.join(REF, "asset"), "-i", src, "-o", out, "-b", "cuda",
           "-C", f"cuda.model={model}"]
    for k, v in config.items():
        cmd += ["-C", f"{k}={v}"]
    for k, v in params.items():
        cmd += ["-P", f"{k}={v}"]
    subprocess.check_call(cmd)
    return out


def main():
    subprocess.check_call(["make", "-s", "-C", os.path.join(PKG, "backend"), "-j8", f"REF={REF}"])
    for model, (example, config) in MODELS.items():
        out = run_compiler(model, {})
        with open(os.path.join(out, model + ".cu")) as f:
            src = f.read()
        shutil.rmtree(out)
        with open(os.path.join(HERE, model + ".cu"), "w") as f:
            f.write(src)
        print("generated", model)
    configs = {}
    for name, (model, params) in CONFIGS.items():
        out = run_compiler(model, params)
        with open(os.path.join(out, model + ".globals.json")) as f:
            manifest = json.load(f)
        shutil.rmtree(out)
        configs[name] = {"model": model, "params": params, "globals": manifest["globals"]}
    with open(os.path.join(HERE, "configs.json"), "w") as f:
        json.dump(configs, f, indent=1)
    with open(os.path.join(HERE, "registry.cpp"), "w") as f:
        f.write("// Models compiled into libopenabl_cuda (written by regenerate.py).\n")
        f.write('#include "abl_model.h"\n\nextern "C" {\n')
        for model in MODELS:
            f.write(f"const abl_model_desc *abl_model_desc_{model}(void);\n")
        f.write("extern const abl_model_desc *const abl_builtin_models[];\n")
        f.write("const abl_model_desc *const abl_builtin_models[] = {\n")
        for model in MODELS:
            f.write(f"    abl_model_desc_{model}(),\n")
        f.write("    nullptr};\n}\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
