"""ctypes binding of libnaivegpu (include/naivegpu.h).

The library is the only compute path: if it is missing this module raises at
import time instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.environ.get("NAIVEGPU_LIB", os.path.join(PKG_DIR, "lib", "libnaivegpu.so"))

ND_OK = 0
ND_NEED_REALLOC = 1
ND_ERR_ARG = -1
ND_ERR_SPEC = -2
ND_ERR_NONFINITE = -3
ND_ERR_RANGE = -4
ND_ERR_CUDA = -5
ND_ERR_NOMEM = -6
ND_ERR_INTERNAL = -7
ND_ERR_OVERFLOW = -8
ND_ERR_NODEVICE = -9

ND_ORDER_REFERENCE = 0
ND_ORDER_SPATIAL = 1
ND_BOX_LEAF = 0
ND_BOX_ATOM = 1
ND_PAIRS_ORDERED = 0
ND_PAIRS_UNORDERED = 1
ND_CRIT_SQUARED = 0
ND_CRIT_SQRT = 1
ND_UNION_BLOCKS = 0
ND_UNION_TREE = 1

GRIDKEY_DTYPE = np.dtype([("min", np.float32, 3), ("max", np.float32, 3),
                          ("left", np.int32), ("skip", np.int32)])
PAIR_DTYPE = np.dtype([("i", np.int32), ("j", np.int32), ("d", np.float32)])


class NDError(RuntimeError):
    """A libnaivegpu call returned an error status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


class SpecError(NDError):
    """SpheresBVHSpecs checks (the reference raises `error()` there)."""


class InexactError(NDError):
    """Coordinate not representable after quantisation (Julia's InexactError)."""


class BVHSpec(ctypes.Structure):
    _fields_ = [("neighbor_distance", ctypes.c_float), ("atom_count", ctypes.c_int32),
                ("leaves_count", ctypes.c_int32), ("branches_count", ctypes.c_int32),
                ("atomsperleaf", ctypes.c_int32)]


class MDParams(ctypes.Structure):
    _fields_ = [("sigma", ctypes.c_double), ("epsilon", ctypes.c_double),
                ("coulomb_k", ctypes.c_double), ("cutoff", ctypes.c_double),
                ("skin", ctypes.c_double), ("dt", ctypes.c_double),
                ("box_lo", ctypes.c_double * 3), ("box_hi", ctypes.c_double * 3),
                ("atomsperleaf", ctypes.c_int32), ("rebuild_every", ctypes.c_int32),
                ("order", ctypes.c_int32), ("max_neighbors", ctypes.c_int32),
                ("resort_every", ctypes.c_int32), ("stage_policy", ctypes.c_int32),
                ("union_search", ctypes.c_int32), ("refit_check_every", ctypes.c_int32),
                ("threads_per_atom", ctypes.c_int32), ("cta_split", ctypes.c_int32)]


class CompatSim(ctypes.Structure):
    """nd_compat_sim: the collector and SimSpec fields simulate! reads."""
    _fields_ = [("min_dim", ctypes.c_float * 3), ("max_dim", ctypes.c_float * 3),
                ("temperature", ctypes.c_float), ("objectnumber", ctypes.c_int64),
                ("stepwidth", ctypes.c_int64), ("duration", ctypes.c_int64),
                ("velocity_dampening", ctypes.c_float)]


class Collector(ctypes.Structure):
    """nd_collector: the GenericRandomCollector fields collect_objects reads."""
    _fields_ = [("objectnumber", ctypes.c_int64), ("min_dim", ctypes.c_float * 3),
                ("max_dim", ctypes.c_float * 3), ("temperature", ctypes.c_float),
                ("randomvelocity", ctypes.c_int32), ("minmass", ctypes.c_float),
                ("maxmass", ctypes.c_float), ("minimumdistance", ctypes.c_float),
                ("mincharge", ctypes.c_float), ("maxcharge", ctypes.c_float)]


class MDDiag(ctypes.Structure):
    """nd_md_diag."""
    _fields_ = [("skin_violations", ctypes.c_int64), ("max_neighbors", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("resorts", ctypes.c_int64),
                ("refits", ctypes.c_int64), ("early_refits", ctypes.c_int64),
                ("resort_kernels", ctypes.c_int64), ("refit_kernels", ctypes.c_int64),
                ("body_kernels", ctypes.c_int64)]


class System(ctypes.Structure):
    """nd_system: one member of a batched ensemble."""
    _fields_ = [("n_atoms", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("sigma", ctypes.c_double), ("epsilon", ctypes.c_double),
                ("box_lo", ctypes.c_double * 3), ("box_hi", ctypes.c_double * 3)]


class AdjSpec(ctypes.Structure):
    """nd_adj_spec: differentiable trajectory and histogram loss."""
    _fields_ = [("steps", ctypes.c_int32), ("checkpoint_every", ctypes.c_int32),
                ("bins", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("r_max", ctypes.c_double), ("width", ctypes.c_double),
                ("r_switch", ctypes.c_double)]


_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_u64 = ctypes.c_uint64
_vp = ctypes.c_void_p
_f = ctypes.c_float
_d = ctypes.c_double
_pp = ctypes.POINTER(ctypes.c_void_p)

# name -> (restype, argtypes); every symbol declared in include/naivegpu.h
SIGNATURES = {
    "nd_ctx_create": (_i32, [_pp, _i32]),
    "nd_ctx_destroy": (_i32, [_vp]),
    "nd_last_error": (ctypes.c_char_p, [_vp]),
    "nd_status_string": (ctypes.c_char_p, [_i32]),
    "nd_ctx_stream": (_vp, [_vp]),
    "nd_ctx_device_name": (_i32, [_vp, ctypes.c_char_p, _i32]),
    "nd_ctx_synchronize": (_i32, [_vp]),
    "nd_ctx_launch_count": (_i64, [_vp]),
    "nd_bvh_spec_init": (_i32, [ctypes.POINTER(BVHSpec), _f, _i32, _i32]),
    "nd_morton_codes_dev": (_i32, [_vp, _vp, _i32, _i32, _vp]),
    "nd_sortperm_dev": (_i32, [_vp, _vp, _i32, _vp]),
    "nd_tree": (_i32, [_vp, _vp, ctypes.POINTER(BVHSpec), _i32, _i32, _vp, _i64, _vp, _vp, _vp,
                       _vp]),
    "nd_leaf_pairs": (_i32, [_vp, _vp, ctypes.POINTER(BVHSpec), _i32, _i32, _vp, _vp, _vp, _i64,
                             ctypes.POINTER(_i64)]),
    "nd_leaf_pairs_refresh": (_i32, [_vp, _vp, ctypes.POINTER(BVHSpec), _vp, _vp, _i32, _vp, _i64,
                                     _vp, _vp, _vp, _vp, _i64, ctypes.POINTER(_i64)]),
    "nd_leaf_pairs_dev": (_i32, [_vp, _vp, ctypes.POINTER(BVHSpec), _i32, _i32, _vp, _vp, _vp,
                                 _i64, ctypes.POINTER(_i64)]),
    "nd_simd_leaf_pairs": (_i32, [_vp, _vp, ctypes.POINTER(BVHSpec), _i32, _i32, _vp, _vp, _vp,
                                  _i64, ctypes.POINTER(_i64)]),
    "nd_atom_pairs": (_i32, [_vp, _vp, ctypes.POINTER(BVHSpec), _i32, _vp, _vp, _vp, _i64,
                             ctypes.POINTER(_i64)]),
    "nd_pair_hash_dev": (_i32, [_vp, _vp, _vp, _vp, _i64, ctypes.POINTER(_u64)]),
    "nd_leaf_pairs_noalloc_dev": (_i32, [_vp, ctypes.POINTER(BVHSpec), _i32, _i32, _vp, _vp, _vp,
                                         _i64, ctypes.POINTER(_i64), _vp]),
    "nd_forces_pairs": (_i32, [_vp, ctypes.POINTER(MDParams), _i32, _vp, _vp, _vp, _vp, _i64,
                               _vp, ctypes.POINTER(_d)]),
    "nd_forces": (_i32, [_vp, ctypes.POINTER(MDParams), _i32, _vp, _vp, _vp,
                         ctypes.POINTER(_d)]),
    "nd_compat_force_lennardjones": (_i32, [_vp, _i32, _vp, _vp, _vp, _i64, _vp]),
    "nd_compat_force_coulomb": (_i32, [_vp, _i32, _vp, _vp, _vp, _i64, _vp, _vp]),
    "nd_compat_simulate": (_i32, [_vp, ctypes.POINTER(CompatSim), _i32, _vp, _vp, _vp, _vp, _vp,
                                  _vp]),
    "nd_collect_objects": (_i32, [_vp, ctypes.POINTER(Collector), ctypes.c_uint64, _vp, _vp, _vp,
                                  _vp, _vp]),
    "nd_md_create": (_i32, [_vp, ctypes.POINTER(MDParams), _i32, _vp, _vp, _vp, _vp, _pp]),
    "nd_md_create_dev": (_i32, [_vp, ctypes.POINTER(MDParams), _i32, _vp, _vp, _vp, _vp, _pp]),
    "nd_md_destroy": (_i32, [_vp]),
    "nd_md_run": (_i32, [_vp, _i64]),
    "nd_md_sync": (_i32, [_vp]),
    "nd_md_get": (_i32, [_vp, _vp, _vp, _vp]),
    "nd_md_get_dev": (_i32, [_vp, _vp, _vp, _vp]),
    "nd_md_energy": (_i32, [_vp, ctypes.POINTER(_d), ctypes.POINTER(_d)]),
    "nd_md_stats": (_i32, [_vp, ctypes.POINTER(_i64), ctypes.POINTER(_i64), ctypes.POINTER(_i64),
                           ctypes.POINTER(_i32)]),
    "nd_md_launches_per_run": (_i64, [_vp, _i64]),
    "nd_md_step_times": (_i32, [_vp, _i32, _vp]),
    "nd_batch_create": (_i32, [_vp, ctypes.POINTER(MDParams), _i32, ctypes.POINTER(System), _vp,
                               _vp, _vp, _vp, _pp]),
    "nd_batch_create_dev": (_i32, [_vp, ctypes.POINTER(MDParams), _i32, ctypes.POINTER(System),
                                   _vp, _vp, _vp, _vp, _pp]),
    "nd_batch_energies": (_i32, [_vp, _vp, _vp]),
    "nd_md_autotune": (_i32, [_vp, ctypes.POINTER(MDParams), _i32, _i32, ctypes.POINTER(System),
                              _vp, _vp, _vp, _vp, _i32, ctypes.POINTER(MDParams),
                              ctypes.POINTER(_d)]),
    "nd_md_diagnostics": (_i32, [_vp, ctypes.POINTER(MDDiag)]),
    "nd_simulate_diagnostics": (_i32, [_vp, ctypes.POINTER(MDDiag)]),
    "nd_md_list_pairs": (_i32, [_vp, _vp, _vp, _vp, _i64, ctypes.POINTER(_i64)]),
    "nd_md_set_thermostat": (_i32, [_vp, _d, _d, _i32]),
    "nd_md_set_log": (_i32, [_vp, _i32, _i32]),
    "nd_md_log_count": (_i32, [_vp, ctypes.POINTER(_i64)]),
    "nd_md_log_read": (_i32, [_vp, _i64, _i64, _vp]),
    "nd_simulate": (_i32, [_vp, ctypes.POINTER(MDParams), _i32, _vp, _vp, _vp, _vp, _vp, _i64]),
    "nd_adj_create": (_i32, [_vp, ctypes.POINTER(MDParams), _i32, _vp, _vp, _vp, _vp,
                             ctypes.POINTER(AdjSpec), _pp]),
    "nd_adj_destroy": (_i32, [_vp]),
    "nd_adj_set_params": (_i32, [_vp, _d, _d]),
    "nd_adj_set_target": (_i32, [_vp, _vp]),
    "nd_adj_forward": (_i32, [_vp, _vp, ctypes.POINTER(_d)]),
    "nd_adj_backward": (_i32, [_vp, _vp, _vp, ctypes.POINTER(_d), ctypes.POINTER(_d)]),
    "nd_adj_final": (_i32, [_vp, _vp]),
    "nd_adj_times": (_i32, [_vp, ctypes.POINTER(_f), ctypes.POINTER(_f)]),
    "nd_synth_uniform": (_i32, [_u64, _i32, _d, _d, _vp]),
    "nd_synth_uniform_mindist": (_i32, [_u64, _i32, _d, _d, _vp]),
    "nd_synth_clusters": (_i32, [_u64, _i32, _i32, _d, _d, _d, _vp]),
    "nd_synth_normal": (_i32, [_u64, _i64, _d, _vp]),
    "nd_synth_charges": (_i32, [_u64, _i32, _vp]),
}

_lock = threading.Lock()
_lib = None


def lib():
    """Load libnaivegpu.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(
                    f"libnaivegpu.so not found at {LIB_PATH}; build it with "
                    "`python naivedynamics.jl_gb300/build.py` (no CPU fallback exists)")
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def status_string(st: int) -> str:
    return lib().nd_status_string(st).decode()


def raise_for(st: int, ctx=None, what: str = ""):
    if st in (ND_OK,):
        return
    msg = status_string(st)
    if ctx is not None:
        detail = lib().nd_last_error(ctx).decode()
        if detail:
            msg = f"{msg}: {detail}"
    if what:
        msg = f"{what}: {msg}"
    if st == ND_ERR_SPEC:
        raise SpecError(st, msg)
    if st in (ND_ERR_NONFINITE, ND_ERR_RANGE):
        raise InexactError(st, msg)
    raise NDError(st, msg)


def ptr(a) -> int | None:
    """Address of a numpy array (host), a torch tensor or an int (device)."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if hasattr(a, "data_ptr"):
        return int(a.data_ptr())
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return int(a.ctypes.data)
    raise TypeError(f"cannot take the address of {type(a)}")


class Context:
    """One CUDA device + stream (nd_ctx)."""

    def __init__(self, device: int = 0):
        h = ctypes.c_void_p()
        st = lib().nd_ctx_create(ctypes.byref(h), device)
        raise_for(st, None, "nd_ctx_create")
        self.handle = h.value
        self.device = device

    def close(self):
        if getattr(self, "handle", None):
            lib().nd_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return int(lib().nd_ctx_stream(self.handle) or 0)

    def synchronize(self):
        raise_for(lib().nd_ctx_synchronize(self.handle), self.handle, "synchronize")

    def launch_count(self) -> int:
        return int(lib().nd_ctx_launch_count(self.handle))

    def device_name(self) -> str:
        buf = ctypes.create_string_buffer(256)
        raise_for(lib().nd_ctx_device_name(self.handle, buf, 256), self.handle, "device name")
        return buf.value.decode()

    def check(self, st: int, what: str = ""):
        raise_for(st, self.handle, what)


_default: dict[int, Context] = {}


def default_context(device: int = 0) -> Context:
    with _lock:
        c = _default.get(device)
    if c is None:
        c = Context(device)
        with _lock:
            _default[device] = c
    return c
