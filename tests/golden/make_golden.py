"""Regenerates the golden fixtures in this directory from the reference itself.

Runs where the reference tree is present (it is read at build time only):
  python tests/golden/make_golden.py
For every case of oracle/build_ref.py it builds the reference `c` program
(the reference compiler's own output, compiled with the reference libabl.c),
runs it with the per-timestep dump hook, and writes
  <case>.json       model, parameters, record layout, SHA-256 of the packed
                    state at every timestep 0..T
  <case>_init.bin   the packed initial state (agent records, members in
                    declaration order, no padding)
It also builds the unmodified reference programs of build_ref.PROGRAMS
(default parameters), runs each in an empty directory and records the file
its save() writes in
  programs.json     per model: output file name, size and SHA-256
The GPU and oracle tests compare against these files; nothing reads the
reference tree at test time.
"""
import hashlib
import json
import os
import struct
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import build_ref  # noqa: E402

# Record layouts of the example agents (member, dtype, shape), FP64 build.
LAYOUTS = {
    "circle": [("pos", "<f8", (2,))],
    "circle3d": [("pos", "<f8", (3,))],
    "boids2d": [("pos", "<f8", (2,)), ("velocity", "<f8", (2,))],
    "game_of_life": [("pos", "<f8", (2,)), ("alive", "u1", ())],
    "boids": [("pos", "<f8", (3,)), ("velocity", "<f8", (3,))],
    "boids2d_flockers": [("pos", "<f8", (2,)), ("velocity", "<f8", (2,))],
    "sugarscape": [("pos", "<f8", (2,)), ("target_pos", "<f8", (2,)), ("agent_id", "<i4", ()),
                   ("state", "<i4", ()), ("sugar_level", "<i4", ()), ("metabolism", "<i4", ()),
                   ("env_sugar_level", "<i4", ()), ("max_env_sugar_level", "<i4", ())],
}


def layout(example, use_float):
    lay = LAYOUTS[example]
    if use_float:
        lay = [(n, "<f4" if d == "<f8" else d, s) for n, d, s in lay]
    return lay


def read_dump(path, lay):
    dt = np.dtype([(n, d, s) for n, d, s in lay])
    b = open(path, "rb").read()
    off, out = 0, []
    while off < len(b):
        n = struct.unpack_from("<Q", b, off)[0]
        off += 8
        out.append(np.frombuffer(b, dtype=dt, count=n, offset=off))
        off += n * dt.itemsize
    return out


def main():
    build_ref.build_compiler()
    for name, (example, params, config) in build_ref.CASES.items():
        exe = build_ref.build_case(name)
        d = os.path.dirname(exe)
        dump = os.path.join(d, "dump.bin")
        threads = 1 if name in build_ref.SERIAL_RANDOM else os.cpu_count()
        env = dict(os.environ, ABL_DUMP=dump, OMP_NUM_THREADS=str(threads))
        subprocess.check_call([exe], cwd=d, env=env)
        use_float = config.get("use_float") == "true"
        lay = layout(example, use_float)
        states = read_dump(dump, lay)
        hashes = [hashlib.sha256(s.tobytes()).hexdigest() for s in states]
        with open(os.path.join(HERE, name + "_init.bin"), "wb") as f:
            f.write(states[0].tobytes())
        meta = {
            "case": name,
            "example": example,
            "params": params,
            "config": config,
            "layout": [[n, dt, list(s)] for n, dt, s in lay],
            "agents": int(len(states[0])),
            "timesteps": len(states) - 1,
            "sha256": hashes,
            "source": "reference c backend (OpenABL -b c) + asset/c/libabl.c, gcc -O2 -std=c99 "
                      "-fopenmp on x86-64" + (", OMP_NUM_THREADS=1" if threads == 1 else ""),
        }
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(meta, f, indent=1)
        print(name, len(states) - 1, "steps")
    programs = {}
    for model, (example, config) in build_ref.PROGRAMS.items():
        exe = build_ref.build_program(model)
        run_dir = os.path.join(os.path.dirname(exe), "run")
        os.makedirs(run_dir, exist_ok=True)
        for f in os.listdir(run_dir):
            os.remove(os.path.join(run_dir, f))
        serial = model in build_ref.SERIAL_RANDOM
        threads = 1 if serial else os.cpu_count()
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        subprocess.check_call([exe], cwd=run_dir, env=env, stdout=subprocess.DEVNULL)
        (out,) = os.listdir(run_dir)
        data = open(os.path.join(run_dir, out), "rb").read()
        programs[model] = {"example": example, "config": config, "file": out,
                           "bytes": len(data), "sha256": hashlib.sha256(data).hexdigest(),
                           "serial_random": serial,
                           "source": "reference c backend program at default parameters "
                                     "(OpenABL -b c, gcc -O2 -std=c99 -fopenmp, x86-64, "
                                     f"OMP_NUM_THREADS={'1' if serial else 'all cores'})"}
        print(model, out, len(data), "bytes")
    with open(os.path.join(HERE, "programs.json"), "w") as f:
        json.dump(programs, f, indent=1)


if __name__ == "__main__":
    main()
