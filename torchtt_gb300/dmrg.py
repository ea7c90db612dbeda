"""Fast TT matvec by two-site DMRG on the GPU.

Reference: ``torchtt.dmrg_matvec`` / ``torchttcpp.dmrg_mv`` (``torchtt/_dmrg.py:22-45``,
``cpp/dmrg_mv.h:23-230``). ``y ~ A x`` is computed to relative accuracy ``eps`` without forming the
product's full-rank TT: the sweeps build y's cores directly from two-site blocks of A x, truncated
by SVD. The random start and rank kicks come from a counter-based RNG seeded by ``seed`` (the
reference draws them from the global torch RNG).
"""
import ctypes

import torch

from . import _lib
from .errors import IncompatibleTypes, ShapeMismatch
from .solvers import _desc, _is_tt, fetch_solution
from .tt import TT


def dmrg_matvec(A, x, y0=None, nswp=20, eps=1e-12, rmax=32768, kickrank=4, verb=False,
                use_cpp=True, seed=1):
    """``y = A x`` in the TT format by DMRG; returns a TT on the device of ``x``'s cores."""
    if not (_is_tt(A) and _is_tt(x)) or not A.is_ttm or x.is_ttm:
        raise IncompatibleTypes("A must be a TT-matrix and x a TT-vector.")
    if list(A.N) != list(x.N):
        raise ShapeMismatch("Shapes are incompatible.")
    if not torch.cuda.is_available():
        raise RuntimeError("The gb300 backend needs a CUDA device; it has no CPU fallback.")
    out_device = x.cores[0].device
    dev = out_device if out_device.type == "cuda" else torch.device("cuda", torch.cuda.current_device())
    prep = lambda cs: [c.detach().to(device=dev, dtype=torch.float64).contiguous() for c in cs]
    Ac, xc = prep(A.cores), prep(x.cores)
    keep = []
    dA, dx = _desc(Ac, True, keep), _desc(xc, False, keep)
    dy = _desc(prep(y0.cores), False, keep) if y0 is not None else None
    stream = torch.cuda.current_stream(dev)
    h = _lib.c_vp()
    _lib.check(_lib.lib().ttgb_dmrg_matvec(ctypes.byref(dA), ctypes.byref(dx),
                                           ctypes.byref(dy) if dy is not None else None,
                                           int(nswp), float(eps), int(rmax), int(kickrank),
                                           int(seed), int(bool(verb)),
                                           ctypes.c_void_p(stream.cuda_stream), ctypes.byref(h)))
    cores, _ = fetch_solution(h, [int(c.shape[1]) for c in Ac], dev, stream)
    return TT([c.to(out_device) for c in cores])
