"""ctypes binding of ``libttgb300.so`` (the C ABI declared in include/ttgb300.h).

The library is required: there is no CPU fallback. ``lib()`` raises when the shared object is
missing or cannot be loaded (build it with ``python -m torchtt_gb300.build``).
"""
import ctypes
import os

from .errors import GB300Error, InvalidArguments

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libttgb300.so")

TTGB_OK = 0
TTGB_ERR_INVALID = 1
TTGB_ERR_CUDA = 2
TTGB_ERR_NUMERICAL = 3
TTGB_ERR_OOM = 5

c_i32, c_i64, c_dbl, c_u64, c_vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_uint64, ctypes.c_void_p
c_dp = ctypes.POINTER(ctypes.c_double)


class TTDesc(ctypes.Structure):
    _fields_ = [("d", c_i32), ("rows", ctypes.POINTER(c_i64)), ("cols", ctypes.POINTER(c_i64)),
                ("ranks", ctypes.POINTER(c_i64)), ("cores", ctypes.POINTER(c_vp))]


class AmenParams(ctypes.Structure):
    _fields_ = [("nswp", c_i32), ("eps", c_dbl), ("rmax", c_i64), ("max_full", c_i64),
                ("kickrank", c_i32), ("kick2", c_i32), ("local_iterations", c_i32),
                ("resets", c_i32), ("verbose", c_i32), ("preconditioner", c_i32), ("seed", c_u64),
                ("profile", c_i32), ("precision", c_i32), ("lowp_engine", c_i32),
                ("a_structure", c_i32), ("fp64_engine", c_i32), ("strict_eps", c_i32)]

PRECISION = {"fp64": 0, "mixed": 1}


class Stats(ctypes.Structure):
    _fields_ = [("sweeps", c_i32), ("converged", c_i32), ("max_res", c_dbl),
                ("local_solves", c_i64), ("direct_solves", c_i64), ("gmres_iterations", c_i64),
                ("matvecs", c_i64), ("matvec_flops", c_dbl), ("phi_flops", c_dbl),
                ("other_flops", c_dbl), ("host_syncs", c_i64), ("contract_ms", c_dbl),
                ("contract_launches", c_i64), ("contract_flops", c_dbl),
                ("lowp_matvecs", c_i64), ("lowp_flops", c_dbl), ("refinements", c_i64),
                ("phase_ms", c_dbl * 12), ("lowp_ms", c_dbl), ("lowp_launches", c_i64),
                ("lowp_gemm_flops", c_dbl), ("krylov_ms", c_dbl), ("krylov_launches", c_i64),
                ("krylov_bytes", c_dbl), ("krylov_traffic_bytes", c_dbl),
                ("gmres_syncs", c_i64), ("gmres_overrun", c_i64), ("gmres_reorth", c_i64)]

    PHASES = ("bwd_z", "bwd_qr", "bwd_phi", "fwd_setup", "local_solve", "svd", "rank_search",
              "fwd_z", "enrichment", "fwd_phi", "other")

    def as_dict(self):
        out = {k: getattr(self, k) for k, _ in self._fields_ if k != "phase_ms"}
        out["phase_ms"] = {n: self.phase_ms[i] for i, n in enumerate(self.PHASES)}
        return out


# name -> (restype, argtypes)
_SIGS = {
    "ttgb_default_params": (None, [ctypes.POINTER(AmenParams)]),
    "ttgb_amen_solve": (c_i32, [ctypes.POINTER(TTDesc), ctypes.POINTER(TTDesc), ctypes.POINTER(TTDesc),
                                ctypes.POINTER(TTDesc), ctypes.POINTER(AmenParams), c_vp,
                                ctypes.POINTER(c_vp)]),
    "ttgb_solution_dims": (c_i32, [c_vp, ctypes.POINTER(c_i32), ctypes.POINTER(c_i64)]),
    "ttgb_solution_stats": (c_i32, [c_vp, ctypes.POINTER(Stats)]),
    "ttgb_solution_core": (c_vp, [c_vp, c_i32]),
    "ttgb_solution_copy_core": (c_i32, [c_vp, c_i32, c_vp, c_i32, c_vp]),
    "ttgb_solution_free": (None, [c_vp]),
    "ttgb_local_product": (c_i32, [c_i64] * 8 + [c_vp] * 5 + [c_i32, c_vp]),
    "ttgb_local_product_noalloc": (c_i32, [c_i64] * 8 + [c_vp] * 5 + [c_i32, c_vp]),
    "ttgb_local_product_lowp": (c_i32, [c_i64] * 8 + [c_vp] * 5 + [c_i32, c_vp]),
    "ttgb_phi_fwd_A": (c_i32, [c_i64] * 8 + [c_vp] * 5 + [c_vp]),
    "ttgb_phi_bck_A": (c_i32, [c_i64] * 8 + [c_vp] * 5 + [c_vp]),
    "ttgb_phi_fwd_rhs": (c_i32, [c_i64] * 5 + [c_vp] * 4 + [c_vp]),
    "ttgb_phi_bck_rhs": (c_i32, [c_i64] * 5 + [c_vp] * 4 + [c_vp]),
    "ttgb_qr": (c_i32, [c_vp, c_i64, c_i64, c_i64, c_vp, c_vp, c_vp]),
    "ttgb_svd": (c_i32, [c_vp, c_i64, c_i64, c_i64, c_vp, c_vp, c_vp, c_vp]),
    "ttgb_local_gmres": (c_i32, [c_i64] * 5 + [c_vp] * 5 + [c_i32, c_dbl, c_i32, c_i32,
                                                          ctypes.POINTER(c_i32), ctypes.POINTER(c_i32), c_vp]),
    "ttgb_server_create": (c_i32, [c_i32, c_i64, ctypes.POINTER(c_vp)]),
    "ttgb_server_submit": (c_i32, [c_vp, ctypes.POINTER(TTDesc), ctypes.POINTER(TTDesc),
                                   ctypes.POINTER(TTDesc), ctypes.POINTER(AmenParams),
                                   ctypes.POINTER(c_i64)]),
    "ttgb_server_wait": (c_i32, [c_vp, c_i64, c_dbl, ctypes.POINTER(c_vp), ctypes.POINTER(c_dbl),
                                 ctypes.POINTER(c_dbl)]),
    "ttgb_server_stats": (c_i32, [c_vp, ctypes.POINTER(c_i64), ctypes.POINTER(c_i64),
                                  ctypes.POINTER(c_i32), ctypes.POINTER(c_i32)]),
    "ttgb_server_destroy": (None, [c_vp]),
    "ttgb_dmrg_matvec": (c_i32, [ctypes.POINTER(TTDesc), ctypes.POINTER(TTDesc), ctypes.POINTER(TTDesc),
                                 c_i32, c_dbl, c_i64, c_i32, ctypes.c_uint64, c_i32, c_vp,
                                 ctypes.POINTER(c_vp)]),
    "ttgb_amen_mv": (c_i32, [ctypes.POINTER(TTDesc), ctypes.POINTER(TTDesc), ctypes.POINTER(TTDesc),
                             c_i32, c_dbl, c_i64, c_i32, c_i32, ctypes.c_uint64, c_i32, c_vp,
                             ctypes.POINTER(c_vp)]),
    "ttgb_tt_matvec": (c_i32, [ctypes.POINTER(TTDesc), ctypes.POINTER(TTDesc), c_vp, ctypes.POINTER(c_vp)]),
    "ttgb_tt_norm": (c_i32, [ctypes.POINTER(TTDesc), ctypes.POINTER(c_dbl), c_vp]),
    "ttgb_tt_round": (c_i32, [ctypes.POINTER(TTDesc), c_dbl, c_i64, c_vp, ctypes.POINTER(c_vp)]),
    "ttgb_launch_count": (c_i64, []),
    "ttgb_autotune": (c_i32, [c_i32]),
    "ttgb_autotune_classes": (c_i64, []),
    "ttgb_calibrate_fma": (c_i32, [c_i32, ctypes.POINTER(c_dbl)]),
    "ttgb_last_error": (ctypes.c_char_p, []),
    "ttgb_version": (c_i32, []),
    "ttgb_server_memory": (c_i32, [c_vp, ctypes.POINTER(c_i64), ctypes.POINTER(c_i64),
                                   ctypes.POINTER(c_i64)]),
    "ttgb_footprint": (c_i32, [ctypes.POINTER(TTDesc), ctypes.POINTER(TTDesc), ctypes.POINTER(TTDesc),
                               ctypes.POINTER(AmenParams), ctypes.POINTER(c_i64)]),
    "ttgb_pool_usage": (c_i32, [ctypes.POINTER(c_i64), ctypes.POINTER(c_i64), c_i32]),
}

EXPORTED = tuple(_SIGS)

_lib = None


def lib():
    """Load (once) and return the CDLL with declared signatures."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise GB300Error("libttgb300.so is not built (run `python -m torchtt_gb300.build`); "
                             "the GB300 solver has no CPU fallback")
        handle = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def check(status):
    """Raise the matching exception for a non-zero status code."""
    if status == TTGB_OK:
        return
    msg = lib().ttgb_last_error().decode(errors="replace")
    if status == TTGB_ERR_INVALID:
        raise InvalidArguments(msg)
    raise GB300Error("ttgb status %d: %s" % (status, msg))
