"""Python host for the OpenABL CUDA runtime, through its C ABI.

The reference drives a simulation from a generated C program
(src/backend/CPrinter.cpp:189-233).  This module offers the same steps to a
Python caller -- build the population, run `simulate` for T timesteps, read it
back -- by calling the C entry points of include/openabl_cuda.h with ctypes.
No computation happens here: every step runs in libopenabl_cuda.so on the GPU,
and a missing library or GPU is an error, never a fallback.

Agent state is a dict member name -> numpy array (float2 members as (n, 2),
float3 as (n, 3), float as (n,), int as int32, bool as uint8).
"""
import ctypes
import json
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libopenabl_cuda.so")
CONFIGS_PATH = os.path.join(PKG, "generated", "configs.json")

ABL_T_BOOL, ABL_T_INT, ABL_T_FLOAT, ABL_T_FLOAT2, ABL_T_FLOAT3 = 1, 2, 3, 5, 6

_lib = None


class AblError(RuntimeError):
    def __init__(self, code, what):
        msg = _load().abl_strerror(code).decode() if _lib is not None else str(code)
        super().__init__(f"{what}: {msg} ({code})")
        self.code = code


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with "
                               "`python -m openabl_gb300.build_lib`")
        L = ctypes.CDLL(LIB_PATH)
        vp, i, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
        L.abl_model_lookup.restype = vp
        L.abl_model_lookup.argtypes = [ctypes.c_char_p]
        L.abl_model_num_agent_types.argtypes = [vp]
        L.abl_model_agent_name.restype = ctypes.c_char_p
        L.abl_model_agent_name.argtypes = [vp, i]
        L.abl_model_num_members.argtypes = [vp, i]
        L.abl_model_member.argtypes = [vp, i, i, ctypes.POINTER(ctypes.c_char_p),
                                       ctypes.POINTER(ctypes.c_int)]
        L.abl_model_globals_size.restype = sz
        L.abl_model_globals_size.argtypes = [vp]
        L.abl_model_globals_default.argtypes = [vp, vp]
        L.abl_model_global.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(sz),
                                       ctypes.POINTER(ctypes.c_int)]
        L.abl_create.argtypes = [vp, sz, ctypes.POINTER(vp)]
        L.abl_set_globals.argtypes = [vp, vp, sz]
        L.abl_upload.argtypes = [vp, i, ctypes.POINTER(vp), sz]
        L.abl_step.argtypes = [vp]
        L.abl_run.argtypes = [vp, i]
        L.abl_count.argtypes = [vp, i, ctypes.POINTER(sz)]
        L.abl_download.argtypes = [vp, i, ctypes.POINTER(vp), ctypes.POINTER(sz)]
        L.abl_reduce.argtypes = [vp, i, i, i, vp]
        L.abl_last_exec_time.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
        L.abl_memory_used.argtypes = [vp, ctypes.POINTER(sz)]
        L.abl_last_launch_count.argtypes = [vp, ctypes.POINTER(ctypes.c_long)]
        L.abl_destroy.argtypes = [vp]
        L.abl_strerror.restype = ctypes.c_char_p
        L.abl_strerror.argtypes = [i]
        _lib = L
    return _lib


def library():
    return _load()


def fp64_rates():
    """Measured FP64 FMA / add / multiply instruction rates (per lane, per s)."""
    L = _load()
    d = ctypes.c_double
    L.abl_diag_fp64_rates.argtypes = [ctypes.POINTER(d)] * 3
    a, b, c = d(), d(), d()
    _check(L.abl_diag_fp64_rates(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
           "abl_diag_fp64_rates")
    return a.value, b.value, c.value


def fp64_add_as_fma_rate():
    """Measured rate of FP64 additions issued as fma(x, 1.0, y), per lane, per s."""
    L = _load()
    d = ctypes.c_double
    L.abl_diag_fp64_add_as_fma_rate.argtypes = [ctypes.POINTER(d)]
    a = d()
    _check(L.abl_diag_fp64_add_as_fma_rate(ctypes.byref(a)), "abl_diag_fp64_add_as_fma_rate")
    return a.value


def check_int_division(seed=1, per_n=200000):
    """Device check of the step kernels' division by an int count against
    IEEE division: returns (quotients compared, quotients that differ)."""
    L = _load()
    u = ctypes.c_ulonglong
    L.abl_diag_check_int_division.argtypes = [u, ctypes.c_long, ctypes.POINTER(u),
                                              ctypes.POINTER(u)]
    checked, bad = u(), u()
    _check(L.abl_diag_check_int_division(seed, per_n, ctypes.byref(checked), ctypes.byref(bad)),
           "abl_diag_check_int_division")
    return checked.value, bad.value


def _check(code, what):
    if code != 0:
        raise AblError(code, what)


def configs():
    with open(CONFIGS_PATH) as f:
        return json.load(f)


class Model:
    """A model compiled into the library by `-b cuda` (its descriptor)."""

    def __init__(self, name):
        L = _load()
        self.name = name
        self.ptr = L.abl_model_lookup(name.encode())
        if not self.ptr:
            raise KeyError(f"model {name!r} is not compiled into {LIB_PATH}")
        self.agent_types = []
        for t in range(L.abl_model_num_agent_types(self.ptr)):
            members = []
            for m in range(L.abl_model_num_members(self.ptr, t)):
                nm, vt = ctypes.c_char_p(), ctypes.c_int()
                _check(L.abl_model_member(self.ptr, t, m, ctypes.byref(nm), ctypes.byref(vt)),
                       "abl_model_member")
                members.append((nm.value.decode(), vt.value))
            self.agent_types.append((L.abl_model_agent_name(self.ptr, t).decode(), members))
        self.globals_size = L.abl_model_globals_size(self.ptr)
        L.abl_model_float_bytes.argtypes = [ctypes.c_void_p]
        self.float_bytes = L.abl_model_float_bytes(self.ptr)

    def type_id(self, name):
        for k, (n, _) in enumerate(self.agent_types):
            if n == name:
                return k
        raise KeyError(name)

    def default_globals(self):
        buf = (ctypes.c_ubyte * self.globals_size)()
        _check(_load().abl_model_globals_default(self.ptr, buf), "abl_model_globals_default")
        return Globals(self, buf)


class Globals:
    """The model's globals block, addressable by name."""

    def __init__(self, model, buf):
        self.model = model
        self.buf = buf
        self.float_bytes = model.float_bytes

    def _slot(self, name):
        off, vt = ctypes.c_size_t(), ctypes.c_int()
        _check(_load().abl_model_global(self.model.ptr, name.encode(), ctypes.byref(off),
                                        ctypes.byref(vt)), f"unknown global {name!r}")
        return off.value, vt.value

    def set(self, name, value):
        off, vt = self._slot(name)
        base = ctypes.addressof(self.buf) + off
        fdt = ctypes.c_float if self.float_bytes == 4 else ctypes.c_double
        if vt == ABL_T_BOOL:
            ctypes.c_bool.from_address(base).value = bool(value)
        elif vt == ABL_T_INT:
            ctypes.c_int.from_address(base).value = int(value)
        elif vt == ABL_T_FLOAT:
            fdt.from_address(base).value = float(value)
        else:
            comps = 2 if vt == ABL_T_FLOAT2 else 3
            vals = list(value) if hasattr(value, "__len__") else [value] * comps
            for k in range(comps):
                fdt.from_address(base + k * ctypes.sizeof(fdt)).value = float(vals[k])

    def get(self, name):
        off, vt = self._slot(name)
        base = ctypes.addressof(self.buf) + off
        fdt = ctypes.c_float if self.float_bytes == 4 else ctypes.c_double
        if vt == ABL_T_BOOL:
            return ctypes.c_bool.from_address(base).value
        if vt == ABL_T_INT:
            return ctypes.c_int.from_address(base).value
        if vt == ABL_T_FLOAT:
            return fdt.from_address(base).value
        comps = 2 if vt == ABL_T_FLOAT2 else 3
        return [fdt.from_address(base + k * ctypes.sizeof(fdt)).value for k in range(comps)]

    def update(self, values):
        for k, v in values.items():
            if isinstance(v, str):
                v = json.loads(v) if v not in ("true", "false") else v == "true"
            self.set(k, v)
        return self


def globals_for_config(config_name):
    cfg = configs()[config_name]
    model = Model(cfg["model"])
    g = model.default_globals().update(cfg["globals"])
    return model, g


def member_dtype(vt, float_bytes):
    fd = np.float32 if float_bytes == 4 else np.float64
    return {ABL_T_BOOL: (np.uint8, ()), ABL_T_INT: (np.int32, ()), ABL_T_FLOAT: (fd, ()),
            ABL_T_FLOAT2: (fd, (2,)), ABL_T_FLOAT3: (fd, (3,))}[vt]


class Simulation:
    """One runtime context: device-resident agents of one model."""

    def __init__(self, model, globals_=None, hbm_budget=0):
        L = _load()
        self.model = model if isinstance(model, Model) else Model(model)
        self.globals = globals_ if globals_ is not None else self.model.default_globals()
        self.ctx = ctypes.c_void_p()
        _check(L.abl_create(self.model.ptr, hbm_budget, ctypes.byref(self.ctx)), "abl_create")
        _check(L.abl_set_globals(self.ctx, self.globals.buf, self.model.globals_size),
               "abl_set_globals")

    def close(self):
        if self.ctx:
            _load().abl_destroy(self.ctx)
            self.ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _members(self, type_id):
        return self.model.agent_types[type_id][1]

    def upload(self, type_name, state):
        tid = self.model.type_id(type_name)
        members = self._members(tid)
        n = None
        keep, ptrs = [], []
        for nm, vt in members:
            dt, shape = member_dtype(vt, self.globals.float_bytes)
            a = np.ascontiguousarray(state[nm], dtype=dt)
            if n is None:
                n = a.shape[0]
            assert a.shape == (n,) + shape, (nm, a.shape)
            keep.append(a)
            ptrs.append(a.ctypes.data_as(ctypes.c_void_p))
        arr = (ctypes.c_void_p * len(ptrs))(*[p.value for p in ptrs])
        _check(_load().abl_upload(self.ctx, tid, arr, n), "abl_upload")

    def run(self, timesteps):
        _check(_load().abl_run(self.ctx, int(timesteps)), "abl_run")

    def step(self):
        _check(_load().abl_step(self.ctx), "abl_step")

    def count(self, type_name):
        n = ctypes.c_size_t()
        _check(_load().abl_count(self.ctx, self.model.type_id(type_name), ctypes.byref(n)),
               "abl_count")
        return n.value

    def download(self, type_name, out=None):
        """Copies the agents of `type_name` to the host.  `out` may supply the
        destination arrays (e.g. pinned buffers); they must be large enough."""
        tid = self.model.type_id(type_name)
        n = self.count(type_name)
        ptrs = []
        if out is None:
            out = {}
            for nm, vt in self._members(tid):
                dt, shape = member_dtype(vt, self.globals.float_bytes)
                out[nm] = np.empty((n,) + shape, dtype=dt)
        for nm, vt in self._members(tid):
            a = out[nm]
            assert a.flags["C_CONTIGUOUS"] and a.shape[0] >= n
            ptrs.append(a.ctypes.data)
        arr = (ctypes.c_void_p * len(ptrs))(*ptrs)
        cap = ctypes.c_size_t(n)
        _check(_load().abl_download(self.ctx, tid, arr, ctypes.byref(cap)), "abl_download")
        return out

    def last_exec_time(self):
        s = ctypes.c_double()
        _check(_load().abl_last_exec_time(self.ctx, ctypes.byref(s)), "abl_last_exec_time")
        return s.value

    def memory_used(self):
        b = ctypes.c_size_t()
        _check(_load().abl_memory_used(self.ctx, ctypes.byref(b)), "abl_memory_used")
        return b.value

    def set_serial_random(self, state):
        """random() in steps continues the xorshift128+ stream `state` (two
        uint64) in agent order, as the reference does on one thread; None
        returns to the counter-based streams (abl_set_serial_random)."""
        L = _load()
        L.abl_set_serial_random.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        if state is None:
            _check(L.abl_set_serial_random(self.ctx, None), "abl_set_serial_random")
            return
        arr = (ctypes.c_uint64 * 2)(*[int(v) for v in state])
        _check(L.abl_set_serial_random(self.ctx, ctypes.cast(arr, ctypes.c_void_p)),
               "abl_set_serial_random")

    def save_state(self, path):
        """Checkpoint: the whole state, both buffers, bit for bit (abl_save_state)."""
        L = _load()
        L.abl_save_state.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        _check(L.abl_save_state(self.ctx, os.fsencode(str(path))), "abl_save_state")

    def load_state(self, path):
        """Resume from a checkpoint of the same model (abl_load_state)."""
        L = _load()
        L.abl_load_state.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        _check(L.abl_load_state(self.ctx, os.fsencode(str(path))), "abl_load_state")

    def set_seed(self, seed):
        L = _load()
        L.abl_set_seed.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        _check(L.abl_set_seed(self.ctx, int(seed)), "abl_set_seed")

    def log_text(self):
        """Rows written by log_csv() in the model's sequential step."""
        L = _load()
        L.abl_log_text.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t,
                                   ctypes.POINTER(ctypes.c_size_t)]
        n = ctypes.c_size_t()
        _check(L.abl_log_text(self.ctx, None, 0, ctypes.byref(n)), "abl_log_text")
        buf = ctypes.create_string_buffer(n.value + 1)
        _check(L.abl_log_text(self.ctx, buf, n.value + 1, None), "abl_log_text")
        return buf.value.decode()

    def reduce(self, kind, type_name, member=None, value=None):
        """count / sum / count-equal of the sequential-step builtins."""
        L = _load()
        tid = self.model.type_id(type_name)
        midx = 0
        vt = None
        if member is not None:
            names = [m for m, _ in self._members(tid)]
            midx = names.index(member)
            vt = self._members(tid)[midx][1]
        buf = (ctypes.c_ubyte * 32)()
        if value is not None:
            dt, shape = member_dtype(vt, self.globals.float_bytes)
            v = np.ascontiguousarray(np.array(value, dtype=dt).reshape(shape))
            ctypes.memmove(buf, v.ctypes.data, v.nbytes)
        _check(L.abl_reduce(self.ctx, kind, tid, midx, buf), "abl_reduce")
        if kind in (0, 2) or vt in (ABL_T_BOOL, ABL_T_INT):
            return ctypes.c_int.from_buffer(buf).value
        dt, shape = member_dtype(vt, self.globals.float_bytes)
        return np.frombuffer(bytes(buf), dtype=dt, count=int(np.prod(shape) or 1)).copy()

    def set_profiling(self, enable=True):
        L = _load()
        L.abl_set_profiling.argtypes = [ctypes.c_void_p, ctypes.c_int]
        _check(L.abl_set_profiling(self.ctx, 1 if enable else 0), "abl_set_profiling")

    NEAR_AUTO, NEAR_RUNS, NEAR_ROWS, NEAR_LISTS, NEAR_BLOCK = 0, 1, 2, 3, 4

    def set_near_mode(self, mode):
        """How ordered near loops gather neighbours (results are identical in every mode)."""
        L = _load()
        L.abl_set_near_mode.argtypes = [ctypes.c_void_p, ctypes.c_int]
        _check(L.abl_set_near_mode(self.ctx, int(mode)), "abl_set_near_mode")

    def set_near_cache(self, enable=True):
        """Keep each agent's neighbour list across timesteps where positions
        never change (abl_set_near_cache); results are identical either way."""
        L = _load()
        L.abl_set_near_cache.argtypes = [ctypes.c_void_p, ctypes.c_int]
        _check(L.abl_set_near_cache(self.ctx, 1 if enable else 0), "abl_set_near_cache")

    def set_balance(self, enable=True):
        """Hand each block's agents to threads by neighbour count (ordered near loops)."""
        L = _load()
        L.abl_set_balance.argtypes = [ctypes.c_void_p, ctypes.c_int]
        _check(L.abl_set_balance(self.ctx, 1 if enable else 0), "abl_set_balance")

    def step_kernel_time(self, step=0):
        """(total seconds, launches) of a step function's kernel while profiling."""
        L = _load()
        L.abl_step_kernel_time.argtypes = [ctypes.c_void_p, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_long)]
        s, n = ctypes.c_double(), ctypes.c_long()
        _check(L.abl_step_kernel_time(self.ctx, step, ctypes.byref(s), ctypes.byref(n)),
               "abl_step_kernel_time")
        return s.value, n.value

    def last_launch_count(self):
        c = ctypes.c_long()
        _check(_load().abl_last_launch_count(self.ctx, ctypes.byref(c)), "abl_last_launch_count")
        return c.value


class Ensemble:
    """Replicas of one model run together (abl_ensemble_* in the C ABI).

    `globals_list` holds one Globals block per replica (its parameter point);
    states are uploaded and downloaded as one list of per-replica dicts.  A
    run is one launch per phase for all replicas (graph replay), or with
    set_persistent() one cooperative launch for all its timesteps."""

    def __init__(self, model, globals_list, seeds=None, hbm_budget=0):
        L = _load()
        vp = ctypes.c_void_p
        L.abl_ensemble_create.argtypes = [vp, ctypes.c_int, vp, vp, ctypes.c_size_t,
                                          ctypes.POINTER(vp)]
        L.abl_ensemble_upload.argtypes = [vp, ctypes.c_int, vp, ctypes.POINTER(vp)]
        L.abl_ensemble_run.argtypes = [vp, ctypes.c_int]
        L.abl_ensemble_download.argtypes = [vp, ctypes.c_int, vp, ctypes.POINTER(vp)]
        L.abl_ensemble_set_tuning.argtypes = [vp, ctypes.c_int, ctypes.c_double, ctypes.c_int]
        L.abl_ensemble_set_tiling.argtypes = [vp, ctypes.c_int]
        L.abl_ensemble_get_tuning.argtypes = [vp, ctypes.POINTER(ctypes.c_int),
                                              ctypes.POINTER(ctypes.c_double),
                                              ctypes.POINTER(ctypes.c_int),
                                              ctypes.POINTER(ctypes.c_int)]
        L.abl_ensemble_autotune.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                            ctypes.POINTER(ctypes.c_double),
                                            ctypes.POINTER(ctypes.c_int)]
        L.abl_ensemble_last_exec_time.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
        L.abl_ensemble_last_launch_count.argtypes = [vp, ctypes.POINTER(ctypes.c_long)]
        L.abl_ensemble_set_persistent.argtypes = [vp, ctypes.c_int]
        L.abl_ensemble_persistent_blocks.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
        L.abl_ensemble_phase_times.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                               ctypes.POINTER(ctypes.c_int)]
        L.abl_diag_ensemble_barrier.argtypes = [vp, ctypes.c_double, ctypes.c_int]
        L.abl_ensemble_destroy.argtypes = [vp]
        self.model = model if isinstance(model, Model) else Model(model)
        self.replicas = len(globals_list)
        self.float_bytes = self.model.float_bytes
        blob = b"".join(bytes(g.buf) for g in globals_list)
        self._gbuf = ctypes.create_string_buffer(blob, len(blob))
        sd = None
        if seeds is not None:
            self._seeds = np.ascontiguousarray(seeds, dtype=np.uint64)
            sd = self._seeds.ctypes.data
        self.e = ctypes.c_void_p()
        _check(L.abl_ensemble_create(self.model.ptr, self.replicas, self._gbuf, sd, hbm_budget,
                                     ctypes.byref(self.e)), "abl_ensemble_create")

    def upload(self, type_name, states):
        tid = self.model.type_id(type_name)
        members = self.model.agent_types[tid][1]
        counts = np.array([len(s[members[0][0]]) for s in states], np.uint64)
        keep = []
        for nm, vt in members:
            dt, _ = member_dtype(vt, self.float_bytes)
            keep.append(np.ascontiguousarray(np.concatenate([np.asarray(s[nm], dt)
                                                             for s in states])))
        arr = (ctypes.c_void_p * len(keep))(*[a.ctypes.data for a in keep])
        _check(_load().abl_ensemble_upload(self.e, tid, counts.ctypes.data, arr),
               "abl_ensemble_upload")

    def run(self, timesteps):
        _check(_load().abl_ensemble_run(self.e, int(timesteps)), "abl_ensemble_run")

    def download(self, type_name):
        tid = self.model.type_id(type_name)
        members = self.model.agent_types[tid][1]
        counts = np.zeros(self.replicas, np.uint64)
        _check(_load().abl_ensemble_download(self.e, tid, counts.ctypes.data, None),
               "abl_ensemble_download")
        total = int(counts.sum())
        cols = {}
        for nm, vt in members:
            dt, shape = member_dtype(vt, self.float_bytes)
            cols[nm] = np.empty((total,) + shape, dt)
        arr = (ctypes.c_void_p * len(members))(*[cols[nm].ctypes.data for nm, _ in members])
        _check(_load().abl_ensemble_download(self.e, tid, None, arr), "abl_ensemble_download")
        out, base = [], 0
        for c in counts.astype(np.int64):
            out.append({nm: cols[nm][base:base + c] for nm, _ in members})
            base += c
        return out

    def set_tuning(self, block, cell_factor, visit_sorted):
        _check(_load().abl_ensemble_set_tuning(self.e, block, cell_factor, visit_sorted),
               "abl_ensemble_set_tuning")

    def set_tiling(self, entries):
        """Block tiling of ordered 2D near loops: shared-memory list entries per
        block (0: none); results do not depend on it."""
        _check(_load().abl_ensemble_set_tiling(self.e, int(entries)), "abl_ensemble_set_tiling")

    def tuning(self):
        b, f, v, t = ctypes.c_int(), ctypes.c_double(), ctypes.c_int(), ctypes.c_int()
        _check(_load().abl_ensemble_get_tuning(self.e, ctypes.byref(b), ctypes.byref(f),
                                               ctypes.byref(v), ctypes.byref(t)),
               "abl_ensemble_get_tuning")
        return {"block": b.value, "cell_factor": f.value, "visit_sorted": v.value,
                "tiling_entries": t.value}

    def autotune(self, trial_timesteps=3):
        b, f, v = ctypes.c_int(), ctypes.c_double(), ctypes.c_int()
        _check(_load().abl_ensemble_autotune(self.e, trial_timesteps, ctypes.byref(b),
                                             ctypes.byref(f), ctypes.byref(v)),
               "abl_ensemble_autotune")
        return self.tuning()

    def last_exec_time(self):
        s = ctypes.c_double()
        _check(_load().abl_ensemble_last_exec_time(self.e, ctypes.byref(s)), "exec time")
        return s.value

    def last_launch_count(self):
        c = ctypes.c_long()
        _check(_load().abl_ensemble_last_launch_count(self.e, ctypes.byref(c)), "launches")
        return c.value

    def set_persistent(self, enable=True):
        """Every timestep of a run in one cooperative launch (grid barriers
        between the phases); results do not depend on it."""
        _check(_load().abl_ensemble_set_persistent(self.e, int(bool(enable))),
               "abl_ensemble_set_persistent")

    def persistent_blocks(self):
        c = ctypes.c_int()
        _check(_load().abl_ensemble_persistent_blocks(self.e, ctypes.byref(c)),
               "abl_ensemble_persistent_blocks")
        return c.value

    def phase_times(self, cap=64):
        """Durations (s) of the first phases of the last persistent run."""
        buf = (ctypes.c_double * cap)()
        n = ctypes.c_int()
        _check(_load().abl_ensemble_phase_times(self.e, buf, cap, ctypes.byref(n)),
               "abl_ensemble_phase_times")
        return list(buf[:n.value])

    def inject_barrier_failure(self, limit_seconds, extra_arrivals):
        """Failure injection (abl_diag_ensemble_barrier): barrier waits give up
        after limit_seconds; with extra_arrivals=1 no barrier completes."""
        _check(_load().abl_diag_ensemble_barrier(self.e, float(limit_seconds),
                                                 int(extra_arrivals)),
               "abl_diag_ensemble_barrier")

    def close(self):
        if self.e:
            _load().abl_ensemble_destroy(self.e)
            self.e = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _JobDesc(ctypes.Structure):
    _fields_ = [("model", ctypes.c_void_p), ("globals", ctypes.c_void_p),
                ("seed", ctypes.c_uint64), ("timesteps", ctypes.c_int),
                ("counts", ctypes.c_void_p), ("cols", ctypes.c_void_p)]


class Server:
    """Continuous-batching simulation server (abl_server_* in the C ABI)."""

    def __init__(self, slots=8, hbm_budget=0):
        L = _load()
        vp = ctypes.c_void_p
        L.abl_server_create.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.POINTER(vp)]
        L.abl_server_submit.argtypes = [vp, ctypes.POINTER(_JobDesc), ctypes.POINTER(ctypes.c_long)]
        L.abl_server_wait.argtypes = [vp, ctypes.c_long, ctypes.c_double]
        L.abl_server_job_info.argtypes = [vp, ctypes.c_long, ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.c_double)]
        L.abl_server_result.argtypes = [vp, ctypes.c_long, ctypes.c_int, vp,
                                        ctypes.POINTER(ctypes.c_size_t)]
        L.abl_server_release.argtypes = [vp, ctypes.c_long]
        L.abl_server_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_int),
                                       ctypes.POINTER(ctypes.c_int),
                                       ctypes.POINTER(ctypes.c_size_t)]
        L.abl_server_destroy.argtypes = [vp]
        L.abl_server_set_batching.argtypes = [vp, ctypes.c_int, ctypes.c_long]
        self.s = ctypes.c_void_p()
        _check(L.abl_server_create(slots, hbm_budget, ctypes.byref(self.s)), "abl_server_create")
        self.models = {}

    def set_batching(self, max_jobs=64, max_agents=65536):
        """Small jobs of one model run as the replicas of one ensemble
        (max_jobs=1: off)."""
        _check(_load().abl_server_set_batching(self.s, int(max_jobs), int(max_agents)),
               "abl_server_set_batching")

    def submit(self, model, globals_, state, timesteps, seed=0):
        """`state`: {type name: {member: array}}; returns the job id."""
        model = model if isinstance(model, Model) else Model(model)
        self.models_for = getattr(self, "models_for", {})
        keep = []
        counts = np.zeros(len(model.agent_types), np.uint64)
        per_type = []
        for t, (tname, members) in enumerate(model.agent_types):
            st = state.get(tname, {})
            n = len(st[members[0][0]]) if st else 0
            counts[t] = n
            ptrs = []
            for nm, vt in members:
                dt, shape = member_dtype(vt, model.float_bytes)
                a = np.ascontiguousarray(st[nm], dtype=dt) if n else np.zeros((1,) + shape, dt)
                keep.append(a)
                ptrs.append(a.ctypes.data)
            arr = (ctypes.c_void_p * len(ptrs))(*ptrs)
            keep.append(arr)
            per_type.append(ctypes.cast(arr, ctypes.c_void_p).value)
        tarr = (ctypes.c_void_p * len(per_type))(*per_type)
        jd = _JobDesc(model.ptr, ctypes.addressof(globals_.buf), int(seed), int(timesteps),
                      counts.ctypes.data, ctypes.cast(tarr, ctypes.c_void_p).value)
        jid = ctypes.c_long()
        _check(_load().abl_server_submit(self.s, ctypes.byref(jd), ctypes.byref(jid)),
               "abl_server_submit")
        self.models_for[jid.value] = model
        return jid.value

    def wait(self, job_id, timeout=600.0):
        _check(_load().abl_server_wait(self.s, job_id, timeout), "abl_server_wait")

    def info(self, job_id):
        st = ctypes.c_int()
        t = (ctypes.c_double * 4)()
        _check(_load().abl_server_job_info(self.s, job_id, ctypes.byref(st), t), "job_info")
        return {"status": st.value, "submit": t[0], "admit": t[1], "done": t[2],
                "exec_s": t[3]}

    def result(self, job_id):
        model = self.models_for[job_id]
        out = {}
        for t, (tname, members) in enumerate(model.agent_types):
            n = ctypes.c_size_t(0)
            _check(_load().abl_server_result(self.s, job_id, t, None, ctypes.byref(n)), "result")
            cols = {}
            for nm, vt in members:
                dt, shape = member_dtype(vt, model.float_bytes)
                cols[nm] = np.empty((n.value,) + shape, dt)
            arr = (ctypes.c_void_p * len(members))(*[cols[nm].ctypes.data for nm, _ in members])
            _check(_load().abl_server_result(self.s, job_id, t, arr, ctypes.byref(n)), "result")
            out[tname] = cols
        return out

    def release(self, job_id):
        _check(_load().abl_server_release(self.s, job_id), "release")

    def close(self):
        if self.s:
            _load().abl_server_destroy(self.s)
            self.s = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
