"""ctypes bindings of libsagesim_gb300.so (the C ABI in include/sagesim_gb300.h).

There is no fallback: if the library is missing it is built with nvcc, and if
that fails the import error says why. Every wrapper raises SageSimError with
the engine's message when a call returns a non-zero status.
"""
import ctypes
import os
import threading

from . import _build

_lock = threading.Lock()
_lib = None

SG_OK = 0
SG_ERR_INVALID = 1
SG_ERR_BAD_CSR = 2
SG_ERR_CUDA = 3
SG_ERR_OOM = 4
SG_ERR_COMPILE = 5
SG_ERR_BUDGET = 6
SG_ERR_TIMEOUT = 7
SG_ERR_OOB = 8
SG_ERR_NOT_FOUND = 9

SG_I32 = 0
SG_F32 = 1

SG_BUILTIN_SIR_A = 1
SG_BUILTIN_SIR_B = 2
SG_BUILTIN_OPINION = 3

SG_SIR_PULL = 0
SG_SIR_COUNT = 1
SG_SIR_FRONTIER = 2

SG_REQ_QUEUED = 0
SG_REQ_RUNNING = 1
SG_REQ_DONE = 2
SG_REQ_FAILED = 3
SG_REQ_BORROW = 256

SG_GRAPH_ORDERED = 1
SG_GRAPH_SYMMETRIC = 2

_ERRNAMES = {1: "SG_ERR_INVALID", 2: "SG_ERR_BAD_CSR", 3: "SG_ERR_CUDA", 4: "SG_ERR_OOM",
             5: "SG_ERR_COMPILE", 6: "SG_ERR_BUDGET", 7: "SG_ERR_TIMEOUT", 8: "SG_ERR_OOB",
             9: "SG_ERR_NOT_FOUND"}


class SageSimError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code, message):
        super().__init__("%s: %s" % (_ERRNAMES.get(code, str(code)), message))
        self.code = code


class EngineCfg(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("flags", ctypes.c_int32), ("stream", ctypes.c_void_p)]


class BuiltinParams(ctypes.Structure):
    _fields_ = [("builtin", ctypes.c_int32), ("strategy", ctypes.c_int32),
                ("state_prop", ctypes.c_int32), ("aux_prop", ctypes.c_int32),
                ("code_s", ctypes.c_int32), ("code_i", ctypes.c_int32), ("code_r", ctypes.c_int32),
                ("priority", ctypes.c_int32), ("begin", ctypes.c_int64), ("end", ctypes.c_int64),
                ("beta", ctypes.c_double), ("gamma", ctypes.c_double), ("sigma", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [("ticks", ctypes.c_int64), ("agent_ticks", ctypes.c_int64),
                ("edge_visits", ctypes.c_int64), ("device_ms", ctypes.c_double),
                ("kernel_launches", ctypes.c_int64)]


class ScenarioDesc(ctypes.Structure):
    _fields_ = [("n_agents", ctypes.c_int64), ("nnz", ctypes.c_int64),
                ("offsets", ctypes.c_void_p), ("indices", ctypes.c_void_p),
                ("state", ctypes.c_void_p), ("lids", ctypes.c_void_p),
                ("seed", ctypes.c_int64), ("beta", ctypes.c_double), ("gamma", ctypes.c_double),
                ("builtin", ctypes.c_int32), ("code_s", ctypes.c_int32), ("code_i", ctypes.c_int32),
                ("code_r", ctypes.c_int32), ("horizon", ctypes.c_int32), ("flags", ctypes.c_int32)]


class Tune(ctypes.Structure):
    _fields_ = [("strategy", ctypes.c_int32), ("blocks_per_sm", ctypes.c_int32),
                ("thread_row", ctypes.c_int32), ("mega_row", ctypes.c_int32),
                ("count_flavour", ctypes.c_int32), ("us_per_tick", ctypes.c_double)]


class ServerCfg(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("builtin", ctypes.c_int32), ("stream", ctypes.c_void_p),
                ("budget_bytes", ctypes.c_int64), ("agent_slots", ctypes.c_int64),
                ("edge_slots", ctypes.c_int64), ("max_resident", ctypes.c_int32),
                ("flags", ctypes.c_int32)]


_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_U64 = ctypes.c_uint64
_D = ctypes.c_double
_SZ = ctypes.c_size_t
_C = ctypes.c_char_p

# name -> argtypes (all return int status)
SIGNATURES = {
    "sg_engine_create": [ctypes.POINTER(EngineCfg), ctypes.POINTER(_P)],
    "sg_engine_destroy": [_P],
    "sg_last_error": [_P, ctypes.c_char_p, _SZ],
    "sg_set_graph_csr": [_P, _P, _I64, _P, _I64, _I32],
    "sg_set_graph_id_edges": [_P, _P, _I64, _P, _P, _I64, _I32],
    "sg_get_graph_csr": [_P, _P, _P, _P],
    "sg_set_logical_ids": [_P, _P, _I64],
    "sg_set_seed": [_P, _I64],
    "sg_set_globals_f64": [_P, _P, _I32],
    "sg_add_property": [_P, _C, _I32, _I32, _I32, _P, ctypes.POINTER(_I32)],
    "sg_add_array": [_P, _C, _I32, _I32, _I64, _I32, _P, ctypes.POINTER(_I32)],
    "sg_get_tick_history": [_P, _P, _I64, ctypes.POINTER(_I64), ctypes.POINTER(_I64)],
    "sg_set_property": [_P, _I32, _P, _I64, _I64],
    "sg_get_property": [_P, _I32, _P, _I64, _I64],
    "sg_property_device_ptr": [_P, _I32, ctypes.POINTER(_P)],
    "sg_add_builtin_step": [_P, ctypes.POINTER(BuiltinParams), ctypes.POINTER(_I32)],
    "sg_update_builtin_step": [_P, _I32, ctypes.POINTER(BuiltinParams)],
    "sg_compile_step": [_P, _C, _C, _I32, _I64, _I64, _P, _I32, ctypes.POINTER(_I32)],
    "sg_run": [_P, _I64, _I32, _P, ctypes.POINTER(Stats)],
    "sg_run_async": [_P, _I64, _I32, _I32],
    "sg_synchronize": [_P],
    "sg_last_run_active": [_P, _P, _I32],
    "sg_engine_set_tune": [_P, ctypes.POINTER(Tune)],
    "sg_snapshot": [_P],
    "sg_restore": [_P],
    "sg_profile_enable": [_P, _I32],
    "sg_profile_get": [_P, _I32, ctypes.c_char_p, _SZ, ctypes.POINTER(_I64), ctypes.POINTER(_D)],
    "sg_opinion_cosine_check": [_P, _I32, _I32, _P, _P],
    "sg_opinion_noise_check": [_P, _D, _I64, _P, _P, _P, _P, _P, _P],
    "sg_batch_create": [ctypes.POINTER(EngineCfg), ctypes.POINTER(_P)],
    "sg_batch_destroy": [_P],
    "sg_batch_last_error": [_P, ctypes.c_char_p, _SZ],
    "sg_batch_add_scenario": [_P, ctypes.POINTER(ScenarioDesc), ctypes.POINTER(_I32)],
    "sg_batch_commit": [_P],
    "sg_batch_set_tune": [_P, ctypes.POINTER(Tune)],
    "sg_batch_get_tune": [_P, ctypes.POINTER(Tune)],
    "sg_batch_tune": [_P, _I32, ctypes.POINTER(Tune)],
    "sg_batch_run": [_P, _I32, _I32],
    "sg_batch_synchronize": [_P],
    "sg_batch_get_state": [_P, _I32, _P, _I64],
    "sg_batch_scenario_tick": [_P, _I32, ctypes.POINTER(_I64)],
    "sg_batch_info": [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64), ctypes.POINTER(_I64)],
    "sg_batch_snapshot": [_P],
    "sg_batch_restore": [_P],
    "sg_server_create": [ctypes.POINTER(ServerCfg), ctypes.POINTER(_P)],
    "sg_server_destroy": [_P],
    "sg_server_last_error": [_P, ctypes.c_char_p, _SZ],
    "sg_server_submit": [_P, ctypes.POINTER(ScenarioDesc), ctypes.POINTER(_I64)],
    "sg_server_step": [_P, _I32, ctypes.POINTER(_I32)],
    "sg_server_poll": [_P, _I64, ctypes.POINTER(_I32), ctypes.POINTER(_I64)],
    "sg_server_take_result": [_P, _I64, _P, _I64],
    "sg_server_counts": [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64), ctypes.POINTER(_I64),
                         ctypes.POINTER(_I64)],
    "sg_server_set_tune": [_P, ctypes.POINTER(Tune)],
    "sg_sir_run_noalloc": [_P, _P, _P, _I64, _I32, _I64, _I64, _I32, _D, _D, _I32, _I32, _I32, _P],
    "sg_graph_er": [_I64, _D, _U64, _P, _P, ctypes.POINTER(_I64)],
    "sg_graph_ba": [_I64, _I32, _U64, _P, _P, ctypes.POINTER(_I64)],
    "sg_graph_ws": [_I64, _I32, _D, _U64, _P, _P, ctypes.POINTER(_I64)],
    "sg_partition_relabel": [_I64, _P, _P, _I32, _U64, _P, _P],
    "sg_csr_permute": [_I64, _P, _P, _P, _P, _P],
}


def load(build_if_missing=True):
    """Returns the loaded library, building it first if it is absent or stale."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing:
            _build.build()
        if not os.path.exists(path):
            raise ImportError("libsagesim_gb300.so not found at %s (build with "
                              "sagesim_gb300._build.build())" % path)
        lib = ctypes.CDLL(path)
        for name, argtypes in SIGNATURES.items():
            fn = getattr(lib, name, None)
            if fn is None:
                continue
            fn.argtypes = argtypes
            fn.restype = ctypes.c_int
        _lib = lib
        return lib


def last_error(handle, fn="sg_last_error"):
    buf = ctypes.create_string_buffer(4096)
    getattr(load(), fn)(handle, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc, handle=None, fn="sg_last_error"):
    if rc != SG_OK:
        raise SageSimError(rc, last_error(handle, fn))
    return rc
