"""Builds libopenabl_cuda.so in-tree for sm_103a (runtime + generated models).

    python -m openabl_gb300.build_lib     (or __graft_entry__.build())

Translation units are compiled in parallel with nvcc; objects go to
openabl_gb300/_build/, the library to openabl_gb300/libopenabl_cuda.so.
Device code is compiled with -fmad=false (no FMA contraction, as the
reference's `gcc -std=c99` build) and IEEE division and square root.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
GEN = os.path.join(PKG, "generated")
INC = os.path.join(REPO, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libopenabl_cuda.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true",
                     "-prec-sqrt=true", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-diag-suppress", "177", "-I", CSRC, "-I", INC]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build openabl_gb300")
    return path


def sources():
    """(source, defines) pairs.  A model with a persistent ensemble kernel is
    compiled a second time with ABL_PERSIST, which builds only that kernel
    (with plain instead of read-only loads) into an object of its own."""
    srcs = [os.path.join(CSRC, "abl_runtime.cu"), os.path.join(CSRC, "abl_host.cpp"),
            os.path.join(CSRC, "abl_diag.cu"), os.path.join(CSRC, "abl_serve.cpp"),
            os.path.join(GEN, "registry.cpp")]
    models = sorted(os.path.join(GEN, f) for f in os.listdir(GEN) if f.endswith(".cu"))
    out = [(s, ()) for s in srcs + models]
    for m in models:
        with open(m) as f:
            if "#ifdef ABL_PERSIST\nextern \"C\" int abl_persist_launch_" in f.read():
                out.append((m, ("-DABL_PERSIST",)))
    return out


def _deps_mtime():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INC, f)
                                                                  for f in os.listdir(INC)]
    return max(os.path.getmtime(f) for f in files)


def _compile(item):
    src, defines = item
    tag = ".persist" if defines else ""
    obj = os.path.join(BUILD, os.path.basename(src) + tag + ".o")
    if (os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src)
            and os.path.getmtime(obj) >= _deps_mtime()):
        return obj
    lang = ["-x", "cu"] if src.endswith((".cu", "registry.cpp")) else ["-Xcompiler", "-pthread"]
    cmd = [nvcc()] + NVCC_FLAGS + list(defines) + lang + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-ldl",
                                                              "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
