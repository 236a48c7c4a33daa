"""ctypes binding of the C ABI declared in include/cunusht_gb300.h.

The shared library is built in-tree (``python -m cunusht_gb300.build`` or
``__graft_entry__.build()``).  There is no fallback: if the library is missing
or fails to load, importing the transformer raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcunusht_gb300.so")

OK = 0
NSTAGE = 11
STAGES = ["leg_synth", "theta_fwd", "phi_fwd", "interp", "spread", "phi_adj", "theta_adj", "leg_adj",
          "ptg_leg", "ptg_ring", "ptg_rot"]
F64 = 0
F32 = 1
PREC_AUTO, PREC_FP64, PREC_MIXED = 0, 1, 2

# every symbol the header declares, with its ctypes signature
_vp = ctypes.c_void_p
_i = ctypes.c_int
_d = ctypes.c_double
_i64 = ctypes.c_int64
SIGNATURES = {
    "cunusht_last_error": (ctypes.c_char_p, []),
    "cunusht_version": (_i, []),
    "cunusht_plan_create": (_i, [ctypes.POINTER(_vp), _i, _d, _i, _i, _i, _vp, _vp, _vp, _vp]),
    "cunusht_plan_destroy": (_i, [_vp]),
    "cunusht_plan_info": (_i, [_vp, _vp, _i]),
    "cunusht_plan_set_profiling": (_i, [_vp, _i]),
    "cunusht_plan_force_split": (_i, [_vp, _i]),
    "cunusht_plan_set_ring_transform": (_i, [_vp, _i]),
    "cunusht_plan_ring_transform": (_i, [_vp]),
    "cunusht_plan_set_mmax": (_i, [_vp, _i]),
    "cunusht_plan_set_tensor_cores": (_i, [_vp, _i]),
    "cunusht_plan_set_start_states": (_i, [_vp, _i, _i, _i]),
    "cunusht_plan_set_spreading": (_i, [_vp, _i, _i, _i64]),
    "cunusht_plan_device_status": (_i, [_vp, ctypes.POINTER(_i)]),
    "cunusht_tc_selftest": (_i, [_i, _i, _i, ctypes.POINTER(_d), ctypes.POINTER(_i)]),
    "cunusht_dlm2A": (_i, [_vp, _vp, _vp, _i, _vp, _vp]),
    "cunusht_server_create": (_i, [ctypes.POINTER(_vp), _d, _i]),
    "cunusht_server_set_policy": (_i, [_vp, _i, _i, _i]),
    "cunusht_server_submit": (_i, [_vp, _i, _i, _i, _d, _i, _vp, _vp, _vp, _vp, ctypes.POINTER(_i64)]),
    "cunusht_server_poll": (_i, [_vp, _vp, _i, ctypes.POINTER(_i), ctypes.POINTER(_i)]),
    "cunusht_server_stats": (_i, [_vp, _vp, _i]),
    "cunusht_server_prewarm": (_i, [_vp, _i, _i, _d, _i, ctypes.POINTER(_i)]),
    "cunusht_server_destroy": (_i, [_vp]),
    "cunusht_delensing_batch": (_i, [_vp, _i, _i, _i, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp]),
    "cunusht_synth_points": (_i, [_vp, _i, _i, _vp, _i, _vp, _i64, _i, _vp, _vp, _vp]),
    "cunusht_plan_stage_times": (_i, [_vp, _vp, _vp, _i]),
    "cunusht_plan_reserve_batch": (_i, [_vp, _i]),
    "cunusht_lensing_batch": (_i, [_vp, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp]),
    "cunusht_nusht2d2": (_i, [_vp, _i, _i, _vp, _i, _vp, _i64, _i, _vp, _vp, _i, _vp]),
    "cunusht_nusht2d1": (_i, [_vp, _i, _i, _vp, _i, _vp, _i64, _i, _vp, _vp, _i, _vp]),
    "cunusht_dlm2pointing": (_i, [_vp, _vp, _vp, _i, _vp, _vp, _vp]),
    "cunusht_synthesis": (_i, [_vp, _i, _i, _vp, _i, _vp, _vp]),
    "cunusht_lensing_vjp_dlm": (_i, [_vp, _i, _vp, _i, _vp, _i, _vp, _vp, _vp]),
    "cunusht_adjoint_synthesis": (_i, [_vp, _i, _i, _vp, _vp, _i, _vp]),
    "cunusht_analysis": (_i, [_vp, _i, _i, _vp, _vp, _vp, _i, _vp]),
    "cunusht_pointing": (_i, [_i, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp]),
    "cunusht_doubling": (_i, [_vp, _i64, _i64, _i, _i, _i, _vp, _vp]),
    "cunusht_adjoint_doubling": (_i, [_vp, _i64, _i64, _i, _i, _vp, _vp]),
    "cunusht_synthesis_noalloc": (_i, [_i, _i, _i, _vp, _i, _vp, _vp, _i, _vp, _vp]),
}


class CunushtError(RuntimeError):
    """A C-ABI call returned a non-zero status."""


_lib = None


def load():
    """Load the library once; raise ImportError when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"cunusht_gb300 CUDA library not found at {LIB_PATH}; build it with "
            "`python -m cunusht_gb300.build` (there is no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int):
    if rc != OK:
        msg = load().cunusht_last_error().decode(errors="replace")
        raise CunushtError(f"cunusht error {rc}: {msg}")
