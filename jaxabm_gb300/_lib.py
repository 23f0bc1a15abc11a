"""ctypes binding of ``libjaxabm_gb300.so`` (the C ABI declared in include/jaxabm_gb300.h).

The library is required: when it is missing or a symbol is absent, loading raises instead
of falling back to any other implementation.  With ``JAXABM_CHECKED=1`` in the
environment the range-checked build (``libjaxabm_gb300_checked.so``, made by
``jaxabm_gb300.build(checked=True)``) is loaded instead.
"""

import ctypes
import os
import threading

from . import trace as _trace
from ._build import CHECKED_LIB_PATH, LIB_PATH

ABM_OK = 0
ABM_ERR_BADARG = 1
ABM_ERR_OOM = 2
ABM_ERR_TIMEOUT = 3
ABM_ERR_BOUNDS = 4
ABM_ERR_UNREGISTERED = 5
ABM_ERR_CUDA = 6
ABM_ERR_WORKSPACE = 7

RNG_LEGACY = 0
RNG_PARTITIONABLE = 1

_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_u64 = ctypes.c_uint64
_f32 = ctypes.c_float
_p = ctypes.c_void_p
_sz = ctypes.c_size_t
_int = ctypes.c_int

# name -> (restype, argtypes); every symbol declared in include/jaxabm_gb300.h
SIGNATURES = {
    "abm_version": (_int, []),
    "abm_status_string": (ctypes.c_char_p, [_int]),
    "abm_last_cuda_error": (ctypes.c_char_p, []),
    "abm_bounds_detail": (ctypes.c_char_p, []),
    "abm_checked_build": (_int, []),
    "abm_device_info": (_int, [_p, _p, _p]),
    "abm_rng_split": (_int, [_p, _i64, _i64, _p, _int, _p]),
    "abm_rng_bits": (_int, [_p, _i64, _i64, _p, _int, _p]),
    "abm_rng_uniform": (_int, [_p, _i64, _i64, _f32, _f32, _p, _int, _p]),
    "abm_rng_normal": (_int, [_p, _i64, _i64, _p, _int, _p]),
    "abm_rng_bernoulli": (_int, [_p, _i64, _i64, _f32, _p, _int, _p]),
    "abm_rng_randint": (_int, [_p, _i64, _i64, _i32, _i32, _p, _int, _p]),
    "abm_keychain": (_int, [_p, _i64, _i32, _i32, _p, _p, _p]),
    "abm_randomwalk_init": (_int, [_p, _p, _i64, _p, _p]),
    "abm_randomwalk_workspace_bytes": (_sz, [_i64, _i32]),
    "abm_randomwalk_run": (_int, [_p, _p, _i64, _p, _i32, _f32, _p, _p, _sz, _p]),
    "abm_randomwalk_init_batch": (_int, [_p, _p, _i64, _i32, _p, _p]),
    "abm_randomwalk_batch_workspace_bytes": (_sz, [_i64, _i32, _i32]),
    "abm_randomwalk_run_batch": (_int, [_p, _p, _i64, _i32, _p, _i32, _p, _p, _p, _sz, _p]),
    "abm_graph_ba_num_edges": (_i64, [_i64, _i32]),
    "abm_graph_barabasi_albert": (_int, [_i64, _i32, _u64, _p, _p, _i64]),
    "abm_graph_random_regular": (_int, [_i64, _i32, _u64, _p, _p, _i64]),
    "abm_csr_workspace_bytes": (_sz, [_i64, _i64]),
    "abm_csr_from_edges": (_int, [_p, _p, _i64, _i64, _p, _p, _p, _p, _sz, _p]),
    "abm_sir_instance_size": (_sz, []),
    "abm_sir_pack": (_int, [_p, _p, _p, _i64, _p, _p, _p, _p, _p, _p, _p]),
    "abm_sir_pack_batch": (_int, [_p, _p, _i32, _p, _p, _p, _p]),
    "abm_sir_count_batch": (_int, [_p, _p, _i32, _p, _p, _p]),
    "abm_copy_segments": (_int, [_i64, _p, _p, _p, _i32, _p]),
    "abm_copy_segments_kernel": (_int, [_p, _i64, _p]),
    "abm_sir_unpack": (_int, [_p, _i64, _p, _p]),
    "abm_sir_changes_bytes": (_sz, [_i64, _i64]),
    "abm_sir_steps": (_int, [_p, _i32, _p, _i32, _p, _i32, _p, _p, _sz, _p]),
    "abm_sir_default_launch": (_int, [_p]),
    "abm_sir_resident_max_agents": (_i32, []),
    "abm_sir_resident_grid": (_i32, [_i32]),
    "abm_sir_resident_scratch_bytes": (_sz, [_i32, _i32]),
    "abm_sir_steps_resident": (_int, [_p, _i32, _p, _i32, _i32, _i32, _p, _p, _p, _sz, _p,
                                       _p]),
    "abm_sir_tile_agents": (_i32, []),
    "abm_sir_hub_degree": (_i32, []),
    "abm_sir_run_workspace_bytes": (_sz, [_i64, _i64]),
    "abm_sir_run": (_int, [_p, _p, _i64, _i64, _p, _p, _i32, _f32, _f32, _p, _p, _sz, _p]),
    "abm_schelling_workspace_bytes": (_sz, [_i64, _i32, _i32]),
    "abm_schelling_place": (_int, [_p, _p, _i64, _i32, _i32, _p, _p, _p, _p]),
    "abm_schelling_run": (_int, [_p, _p, _i64, _i32, _i32, _p, _p, _p, _i32, _i32, _i32, _p, _p,
                                 _sz, _p]),
    "abm_schelling_run_batch": (_int, [_p, _i32, _i32, _i32, _i32, _p]),
    "abm_opinion_run": (_int, [_p, _p, _p, _p, _i64, _i32, _p, _p, _p, _i32, _i32, _p, _p]),
    "abm_opinion_step": (_int, [_p, _p, _p, _p, _i64, _i32, _p, _p, _p, _p]),
    "abm_opinion_sigmoid": (_int, [_p, _p, _i64, _p]),
    "abm_opinion_inv_degree": (_int, [_p, _i64, _p, _p]),
    "abm_opinion_moments_workspace_bytes": (_sz, [_i64, _i32]),
    "abm_opinion_moments": (_int, [_p, _i64, _i32, _p, _p, _sz, _p]),
    "abm_opinion_adjoint_init": (_int, [_p, _i64, _i32, _p, _p, _p]),
    "abm_opinion_grad_workspace_bytes": (_sz, [_i64, _i32]),
    "abm_opinion_adjoint_step": (_int, [_p, _p, _p, _p, _p, _p, _i64, _i32, _p, _p, _p, _p, _sz,
                                        _p]),
    "abm_opinion_grad_reduce": (_int, [_p, _i64, _i32, _p, _p]),
    "abm_select_workspace_bytes": (_sz, [_i64]),
    "abm_select_indices": (_int, [_p, _i64, _p, _p, _p, _sz, _p]),
    "abm_select_where": (_int, [_p, _i32, _p, _i32, _i64, _p, _p, _p, _sz, _p]),
    "abm_select_indices_noalloc": (_int, [_p, _i64, _p, _p, _p]),
    "abm_gather_rows": (_int, [_p, _i64, _i64, _p, _i64, _p, _p]),
    "abm_reduce_workspace_bytes": (_sz, [_i64]),
    "abm_reduce_f32": (_int, [_p, _i64, _int, _p, _p, _sz, _p]),
}


class AbmError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, status, where, detail=""):
        self.status = status
        msg = f"{where}: {status_string(status)} (status {status})"
        if detail:
            msg += f": {detail}"
        super().__init__(msg)


_lib = None
_lock = threading.Lock()


def load(path=None):
    """Load the shared library (once) and bind every declared symbol."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or default_path()
        if not os.path.exists(p):
            raise RuntimeError(
                f"{os.path.basename(p)} is not built: call jaxabm_gb300.build() "
                "(needs nvcc); there is no non-CUDA implementation of the engine")
        lib = ctypes.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)  # AttributeError if the symbol is missing
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


def default_path():
    """The library ``load()`` opens: the range-checked build when ``JAXABM_CHECKED`` is set
    to a non-zero value, else the normal one."""
    if os.environ.get("JAXABM_CHECKED", "0") not in ("", "0"):
        return CHECKED_LIB_PATH
    return LIB_PATH


def status_string(status):
    try:
        return load().abm_status_string(int(status)).decode()
    except Exception:  # library not loadable: still give a readable error
        return {0: "ok", 1: "bad argument", 2: "out of device memory", 3: "device wait timed out",
                4: "index out of bounds", 5: "no step kernel registered", 6: "CUDA error",
                7: "workspace too small"}.get(int(status), "unknown status")


def check(status, where):
    if status != ABM_OK:
        detail = ""
        if status == ABM_ERR_CUDA:
            detail = load().abm_last_cuda_error().decode()
        elif status == ABM_ERR_BOUNDS:
            detail = load().abm_bounds_detail().decode()
        raise AbmError(status, where, detail)


def call(name, *args):
    """Call a C-ABI entry point and raise AbmError on a non-zero status (inside an NVTX
    range named after the entry point when tracing is on)."""
    fn = getattr(load(), name)
    if _trace.tracing():
        with _trace.nvtx_range(name):
            check(fn(*args), name)
        return
    check(fn(*args), name)
