"""The `cuda` backend registered with the reference benchmark harness
(openabl_gb300/bench_integration.py, bench/bench.py:21-37).

The harness is laid out from the reference tree with `cuda` added to its
default backends and agent ranges, then run with `-b cuda` and no `-n`, so
the sweep takes the added default range.  The OpenABL binary here is a
stand-in that records its arguments and prints the driver's
"Execution time: Xs" line (src/main.cpp:300-309), so the check needs no
GPU: every sweep point must invoke `-b cuda` with the doubled agent counts
and 100 timesteps, and the results file must hold the parsed times.
"""
import os
import subprocess
import sys

import pytest

from openabl_gb300 import bench_integration as BI

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("OPENABL_REF") or os.path.join(os.path.dirname(REPO), "reference")

pytestmark = pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "bench", "bench.py")),
                                reason="no OpenABL tree with bench/")


def test_patch_adds_cuda_and_keeps_the_rest():
    src = open(os.path.join(REF, "bench", "bench.py")).read()
    out = BI.patch_bench(src)
    added = [l for l in out.splitlines() if l not in src.splitlines()]
    assert added == ["    'cuda',", "    'cuda': (250, 1024000),", "    * cuda:     250-1024000"]
    with pytest.raises(ValueError):
        BI.patch_bench("print('no harness here')")


def test_reference_sweep_runs_the_cuda_backend(tmp_path):
    log = tmp_path / "calls.txt"
    fake = tmp_path / "fake_openabl.sh"
    fake.write_text("#!/bin/sh\necho \"$@\" >> %s\necho 'Execution time: 0.25s'\n" % log)
    fake.chmod(0o755)
    bench = BI.install(REF, str(fake), str(tmp_path / "tree"))
    res = tmp_path / "results"
    subprocess.run([sys.executable, bench, "-b", "cuda", "-m", "circle", "-r", str(res)],
                   check=True, capture_output=True, timeout=120)
    calls = log.read_text().splitlines()
    counts = [250 * 2 ** k for k in range(13)]          # 250 .. 1,024,000, doubling
    assert len(calls) == len(counts)
    for c, n in zip(calls, counts):
        a = c.split()
        assert a[a.index("-b") + 1] == "cuda"
        assert a[a.index("-i") + 1].endswith("examples/circle.abl")
        ps = {a[i + 1] for i, x in enumerate(a) if x == "-P"}
        assert ps == {"num_timesteps=100", f"num_agents={n}"}
    rows = (res / "bench_circle_cuda.txt").read_text().splitlines()
    assert rows[0] == "n,t" and rows[1:] == [f"{n},0.25" for n in counts]
