"""Registers the `cuda` backend with OpenABL's benchmark harness.

The reference harness (bench/bench.py:21-37) keeps its backends and their
default agent ranges in two literals, `default_backends` and
`default_agent_ranges`.  A maintainer adds `cuda` to both; this module makes
that change for a tree it does not own: it writes a copy of bench/bench.py
with the two entries added (and the epilog line that lists the range) next
to a copy of bench/openabl.py, in a directory laid out like the OpenABL tree
(`bench/`, with `examples/`, `asset/` and the `OpenABL` binary linked beside
it), so that

    python -m openabl_gb300.bench_integration --ref <OpenABL tree> \\
        --compiler _build/compiler/openabl --out <dir>
    python <dir>/bench/bench.py -b cuda -m circle,boids2d -r results

runs the reference sweep (agent counts doubling from 250, 100 timesteps,
`Execution time:` parsed by bench/openabl.py:57-62) on the `cuda` backend.
Every other line of the harness is the reference's own.
"""
import argparse
import os
import re
import shutil
import sys

CUDA_RANGE = (250, 1024000)


def patch_bench(text, rng=CUDA_RANGE):
    """bench/bench.py with `cuda` in default_backends and default_agent_ranges.
    Raises ValueError when an anchor is missing (the harness has changed)."""
    m = re.search(r"default_backends\s*=\s*\[", text)
    if not m:
        raise ValueError("default_backends list not found")
    text = text[:m.end()] + "\n    'cuda'," + text[m.end():]
    m = re.search(r"default_agent_ranges\s*=\s*\{", text)
    if not m:
        raise ValueError("default_agent_ranges dict not found")
    text = text[:m.end()] + "\n    'cuda': (%d, %d)," % rng + text[m.end():]
    m = re.search(r"Default agent ranges:\n", text)
    if m:
        text = text[:m.end()] + "    * cuda:     %d-%d\n" % rng + text[m.end():]
    return text


def install(ref, compiler, out):
    """Lays out `out` as an OpenABL tree whose bench/ knows `cuda`."""
    os.makedirs(os.path.join(out, "bench"), exist_ok=True)
    with open(os.path.join(ref, "bench", "bench.py")) as f:
        patched = patch_bench(f.read())
    with open(os.path.join(out, "bench", "bench.py"), "w") as f:
        f.write(patched)
    shutil.copy(os.path.join(ref, "bench", "openabl.py"), os.path.join(out, "bench", "openabl.py"))
    for name in ("examples", "asset"):
        dst = os.path.join(out, name)
        if not os.path.lexists(dst):
            os.symlink(os.path.abspath(os.path.join(ref, name)), dst)
    exe = os.path.join(out, "OpenABL")
    if os.path.lexists(exe):
        os.remove(exe)
    os.symlink(os.path.abspath(compiler), exe)
    return os.path.join(out, "bench", "bench.py")


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--ref", required=True, help="OpenABL source tree")
    ap.add_argument("--compiler", required=True, help="OpenABL binary with the cuda backend")
    ap.add_argument("--out", required=True, help="directory to lay out")
    a = ap.parse_args(argv)
    print(install(a.ref, a.compiler, a.out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
