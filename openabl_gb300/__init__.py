"""OpenABL on GB300: the `-b cuda` backend's device runtime and its hosts.

    openabl_gb300/backend     `-b cuda` code generator (OpenABL compiler plugin, C++)
    openabl_gb300/frontend    hand-written ABL parser used to build the compiler here
    openabl_gb300/csrc        device runtime (CUDA, C ABI in include/openabl_cuda.h)
    openabl_gb300/generated   `-b cuda` output for the example models
    openabl_gb300/runtime.py  Python host over the C ABI
"""
from .runtime import (AblError, Ensemble, Globals, Model, Server, Simulation, configs,  # noqa: F401
                      globals_for_config, library)
