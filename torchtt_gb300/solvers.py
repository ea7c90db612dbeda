"""``amen_solve``: the AMEn linear solve in the TT format on one GB300.

The signature is the reference's ``torchtt.solvers.amen_solve`` (``torchtt/solvers.py:211``) plus
the backend selection: ``backend='gb300'`` (the default here) runs the solve in ``libttgb300.so``.
Argument checks and their exceptions follow ``torchtt/solvers.py:259-282``. As in the reference's
native path (``cpp/amen_solve.h:122``), ``trunc_norm``, ``local_solver`` and ``band_diagonal`` do not
change the algorithm.

Inputs may live on the CPU or on a CUDA device; CPU cores are copied to the GPU and the solution
is returned on the device of ``b``'s cores, with the class of ``b`` (so a reference ``torchtt.TT``
goes in and comes out). The computation itself never runs on the CPU.
"""
import ctypes

import torch

from . import _lib
from .errors import IncompatibleTypes, InvalidArguments, ShapeMismatch
from .tt import TT

_PREC = {None: 0, "c": 1, "r": 2}


def _is_tt(x):
    return hasattr(x, "cores") and hasattr(x, "is_ttm")


def _rows(x):
    """Row mode sizes of a TT-matrix (``x.M`` when the class has it, else from the cores)."""
    M = getattr(x, "M", None)
    return [int(m) for m in M] if M is not None else [int(c.shape[1]) for c in x.cores]


def _cols(x):
    """Column mode sizes of a TT-matrix, or the mode sizes of a TT-vector (``x.N`` or the cores)."""
    N = getattr(x, "N", None)
    if N is not None:
        return [int(n) for n in N]
    return [int(c.shape[2] if x.is_ttm else c.shape[1]) for c in x.cores]


def _desc(cores, matrix, keep):
    """Build a ttgb_tt descriptor for device tensors; `keep` holds the ctypes arrays alive."""
    d = len(cores)
    ranks = [int(cores[0].shape[0])] + [int(c.shape[-1]) for c in cores]
    cols = [int(c.shape[2] if matrix else c.shape[1]) for c in cores]
    rows = [int(c.shape[1]) for c in cores] if matrix else None
    arr_cols = (_lib.c_i64 * d)(*cols)
    arr_ranks = (_lib.c_i64 * (d + 1))(*ranks)
    arr_rows = (_lib.c_i64 * d)(*rows) if matrix else None
    arr_cores = (_lib.c_vp * d)(*[c.data_ptr() for c in cores])
    keep.extend([arr_cols, arr_ranks, arr_rows, arr_cores])
    desc = _lib.TTDesc(d, ctypes.cast(arr_rows, ctypes.POINTER(_lib.c_i64)) if matrix else None,
                       ctypes.cast(arr_cols, ctypes.POINTER(_lib.c_i64)),
                       ctypes.cast(arr_ranks, ctypes.POINTER(_lib.c_i64)),
                       ctypes.cast(arr_cores, ctypes.POINTER(_lib.c_vp)))
    keep.append(desc)
    return desc


def _prep(cores, device):
    return [c.detach().to(device=device, dtype=torch.float64).contiguous() for c in cores]


def solve_cores(A_cores, b_cores, x0_cores=None, z0_cores=None, nswp=22, eps=1e-10, rmax=32768,
                max_full=500, kickrank=4, kick2=0, local_iterations=40, resets=2, verbose=False,
                preconditioner=0, seed=1, stream=None, precision="fp64", profile=False,
                engine="auto", a_structure=True, fp64_engine="auto", strict_eps=False):
    """Native solve on lists of CUDA float64 cores; returns ``(x_cores, stats_dict)``.

    This is the thin layer over ``ttgb_amen_solve`` (include/ttgb300.h); ``amen_solve`` below adds
    the reference's argument handling on top.
    """
    L = _lib.lib()
    keep = []
    dA = _desc(A_cores, True, keep)
    db = _desc(b_cores, False, keep)
    dx = _desc(x0_cores, False, keep) if x0_cores else None
    dz = _desc(z0_cores, False, keep) if z0_cores else None
    p = make_params(nswp=nswp, eps=eps, rmax=rmax, max_full=max_full, kickrank=kickrank,
                    kick2=kick2, local_iterations=local_iterations, resets=resets, verbose=verbose,
                    preconditioner=preconditioner, seed=seed, precision=precision, profile=profile,
                    engine=engine, a_structure=a_structure, fp64_engine=fp64_engine,
                    strict_eps=strict_eps)
    if stream is None:
        stream = torch.cuda.current_stream(A_cores[0].device)
    handle = _lib.c_vp()
    _lib.check(L.ttgb_amen_solve(ctypes.byref(dA), ctypes.byref(db),
                                 ctypes.byref(dx) if dx is not None else None,
                                 ctypes.byref(dz) if dz is not None else None,
                                 ctypes.byref(p), ctypes.c_void_p(stream.cuda_stream),
                                 ctypes.byref(handle)))
    return fetch_solution(handle, [int(c.shape[2]) for c in A_cores], A_cores[0].device, stream)


def fetch_solution(handle, modes, device, stream):
    """Copies the cores of a library-owned solution into new CUDA tensors, frees the handle and
    returns ``(cores, stats)``."""
    L = _lib.lib()
    try:
        d = len(modes)
        dd = _lib.c_i32()
        ranks = (_lib.c_i64 * (d + 1))()
        _lib.check(L.ttgb_solution_dims(handle, ctypes.byref(dd), ranks))
        st = _lib.Stats()
        _lib.check(L.ttgb_solution_stats(handle, ctypes.byref(st)))
        out = []
        for k in range(d):
            t = torch.empty((ranks[k], modes[k], ranks[k + 1]), dtype=torch.float64, device=device)
            _lib.check(L.ttgb_solution_copy_core(handle, k, ctypes.c_void_p(t.data_ptr()), 0,
                                                 ctypes.c_void_p(stream.cuda_stream)))
            out.append(t)
        stream.synchronize()
    finally:
        L.ttgb_solution_free(handle)
    stats = st.as_dict()
    stats["ranks"] = [int(r) for r in ranks]
    return out, stats


def make_params(nswp=22, eps=1e-10, rmax=32768, max_full=500, kickrank=4, kick2=0,
                local_iterations=40, resets=2, verbose=False, preconditioner=0, seed=1,
                precision="fp64", profile=False, engine="auto", a_structure=True,
                fp64_engine="auto", strict_eps=False):
    """A ``ttgb_amen_params`` structure from keyword arguments (defaults of the reference).
    ``a_structure=False`` forces the dense contraction of the A cores; ``fp64_engine`` is
    'auto' (double-float FP64 products on the mixed path), 'native' or 'df'; ``strict_eps``
    runs the sweeps at eps / 4 so that the true residual ends at or below eps (the reference's
    rule bounds the local residuals only, and its true residual can end a few times above eps)."""
    p = _lib.AmenParams()
    _lib.lib().ttgb_default_params(ctypes.byref(p))
    p.nswp, p.eps, p.rmax, p.max_full = int(nswp), float(eps), int(rmax), int(max_full)
    p.kickrank, p.kick2 = int(kickrank), int(kick2)
    p.local_iterations, p.resets = int(local_iterations), int(resets)
    p.verbose, p.preconditioner, p.seed = int(bool(verbose)), int(preconditioner), int(seed)
    if precision not in _lib.PRECISION:
        raise InvalidArguments("precision must be 'fp64' or 'mixed'")
    p.precision = _lib.PRECISION[precision]
    p.profile = int(bool(profile))
    engines = {"auto": 0, "fp32": 1, "tc": 2}
    if engine not in engines:
        raise InvalidArguments("engine must be 'auto', 'fp32' or 'tc'")
    p.lowp_engine = engines[engine]
    p.a_structure = int(bool(a_structure))
    engines64 = {"auto": 0, "native": 1, "df": 2}
    if fp64_engine not in engines64:
        raise InvalidArguments("fp64_engine must be 'auto', 'native' or 'df'")
    p.fp64_engine = engines64[fp64_engine]
    p.strict_eps = int(bool(strict_eps))
    return p


def amen_solve(A, b, nswp=22, x0=None, eps=1e-10, rmax=32768, max_full=500, kickrank=4, kick2=0,
               trunc_norm='res', local_solver=1, local_iterations=40, resets=2, verbose=False,
               preconditioner=None, use_cpp=True, band_diagonal=-1, use_single_precision=False,
               backend='gb300', seed=1, z0=None, return_stats=False, precision=None,
               engine='auto', strict_eps=False):
    """Solve the multilinear system A x = b in the TT format with AMEn on the GPU.

    Arguments are those of ``torchtt.solvers.amen_solve`` (``torchtt/solvers.py:211``), with the same
    defaults and checks, plus:

    * ``backend``: ``'gb300'`` (this library);
    * ``seed``: seed of the counter-based RNG that draws the initial enrichment cores;
    * ``z0``: optional list of initial enrichment cores of ranks ``[1, kickrank+kick2, ..., 1]``
      (replays a given random start exactly);
    * ``return_stats``: also return a dict of solver statistics;
    * ``precision``: ``'fp64'`` (the reference's arithmetic) or ``'mixed'`` (low-precision local
      GMRES operator inside FP64 iterative refinement). ``use_single_precision=True``, the
      reference's own mixed mode (``torchtt/solvers.py:469-496``), selects ``'mixed'``;
    * ``engine``: low-precision contraction engine of the mixed path, ``'auto'`` (tcgen05 when
      available), ``'tc'`` (tcgen05 3xTF32 tensor cores) or ``'fp32'`` (FP32 CUDA cores);
    * ``strict_eps``: the sweeps solve, truncate and stop at eps / 4, so that the true relative
      residual ends at or below eps (the reference's tolerance, the default, bounds only the local
      residuals, and its true residual can end a few times above eps).
    """
    # argument checks of torchtt/solvers.py:259-266
    if not (_is_tt(A) and _is_tt(b)):
        raise InvalidArguments('A and b must be TT instances.')
    if not (A.is_ttm and not b.is_ttm):
        raise IncompatibleTypes('A must be TT-matrix and b must be vector.')
    if _rows(A) != _cols(A):
        raise ShapeMismatch('A is not quadratic.')
    if _cols(A) != _cols(b):
        raise ShapeMismatch('Dimension mismatch.')
    if preconditioner not in _PREC:
        raise InvalidArguments("Invalid preconditioner.")
    if backend != 'gb300':
        raise InvalidArguments("Unknown backend %r (this package provides 'gb300')." % (backend,))
    if not torch.cuda.is_available():
        raise RuntimeError("The gb300 backend needs a CUDA device; it has no CPU fallback.")
    out_device = b.cores[0].device
    out_dtype = b.cores[0].dtype
    dev = out_device if out_device.type == "cuda" else torch.device("cuda", torch.cuda.current_device())
    Ac = _prep(A.cores, dev)
    bc = _prep(b.cores, dev)
    xc = _prep(x0.cores, dev) if x0 is not None else None
    zc = _prep(z0, dev) if z0 is not None else None
    cores, stats = solve_cores(Ac, bc, xc, zc, nswp=nswp, eps=eps, rmax=rmax, max_full=max_full,
                               kickrank=kickrank, kick2=kick2, local_iterations=local_iterations,
                               resets=resets, verbose=verbose, preconditioner=_PREC[preconditioner],
                               seed=seed, engine=engine, strict_eps=strict_eps,
                               precision=precision or ("mixed" if use_single_precision else "fp64"))
    cores = [c.to(device=out_device, dtype=out_dtype) for c in cores]
    cls = type(b) if _is_tt(b) else TT
    try:
        x = cls(cores)
    except Exception:
        x = TT(cores)
    return (x, stats) if return_stats else x
