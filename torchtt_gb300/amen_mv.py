"""TT products by AMEn on the GPU: ``amen_mv`` (TT-matrix x TT-vector) and ``amen_mm``
(TT-matrix x TT-matrix).

Reference: ``torchtt.amen_mv`` / ``torchtt.amen_mm`` (``torchtt/_amen.py:55-125``, the sweep of
``_amen_mm_python``, ``:126-410``). The product is built core by core as the projection of A b onto
the current interfaces, truncated to ``eps`` and enriched with the projected residual, so it never
forms the full-rank product. ``amen_mm`` computes A B as ``(A (x) I) vec(B)``: the operator cores
gain a diagonal factor over B's column mode, which the structured A stage applies from its
nonzeros. Random directions come from a counter-based RNG seeded by ``seed``.
"""
import ctypes

import torch

from . import _lib
from .errors import IncompatibleTypes, InvalidArguments, ShapeMismatch
from .solvers import _desc, _is_tt, fetch_solution
from .tt import TT


def _run(Ac, bc, x0c, nswp, eps, rmax, kickrank, kick2, seed, verbose, dev):
    keep = []
    dA, db = _desc(Ac, True, keep), _desc(bc, False, keep)
    dx = _desc(x0c, False, keep) if x0c is not None else None
    stream = torch.cuda.current_stream(dev)
    h = _lib.c_vp()
    _lib.check(_lib.lib().ttgb_amen_mv(ctypes.byref(dA), ctypes.byref(db),
                                       ctypes.byref(dx) if dx is not None else None, int(nswp),
                                       float(eps), int(rmax), int(kickrank), int(kick2), int(seed),
                                       int(bool(verbose)), ctypes.c_void_p(stream.cuda_stream),
                                       ctypes.byref(h)))
    cores, _ = fetch_solution(h, [int(c.shape[1]) for c in Ac], dev, stream)
    return cores


def _device(t):
    if not torch.cuda.is_available():
        raise RuntimeError("The gb300 backend needs a CUDA device; it has no CPU fallback.")
    d0 = t.cores[0].device
    return d0 if d0.type == "cuda" else torch.device("cuda", torch.cuda.current_device())


def amen_mv(A, b, nswp=22, x0=None, eps=1e-10, rmax=1024, kickrank=4, kick2=0, verbose=False,
            use_cpp=True, seed=1):
    """``A @ b`` for a TT-matrix A and a TT-vector b by AMEn; returns a TT on the device of ``b``."""
    if not (_is_tt(A) and _is_tt(b)):
        raise InvalidArguments('A and b must be TT instances.')
    if not (A.is_ttm and not b.is_ttm):
        raise IncompatibleTypes('A must be TT-matrix and b must be vector.')
    if list(A.N) != list(b.N):
        raise ShapeMismatch('Dimension mismatch.')
    dev = _device(b)
    prep = lambda cs: [c.detach().to(device=dev, dtype=torch.float64).contiguous() for c in cs]
    cores = _run(prep(A.cores), prep(b.cores), prep(x0.cores) if x0 is not None else None, nswp,
                 eps, rmax, kickrank, kick2, seed, verbose, dev)
    return TT([c.to(b.cores[0].device) for c in cores])


def amen_mm(A, B, nswp=22, X0=None, eps=1e-10, rmax=1024, kickrank=4, kick2=0, verbose=False,
            seed=1, max_core_entries=1 << 26):
    """``A @ B`` for TT-matrices A (M x K) and B (K x N) by AMEn on ``(A (x) I_N) vec(B)``; returns
    a TT-matrix (M x N) on the device of ``B``. The operator cores hold rA M N K N rA' entries,
    bounded by ``max_core_entries``."""
    if not (_is_tt(A) and _is_tt(B)) or not (A.is_ttm and B.is_ttm):
        raise IncompatibleTypes('A and B must be TT-matrices.')
    if list(A.N) != list(B.M):
        raise ShapeMismatch('Dimension mismatch.')
    dev = _device(B)
    Ns = list(B.N)
    Ak = []
    for a, n in zip(A.cores, Ns):
        a = a.detach().to(device=dev, dtype=torch.float64)
        ra, m, k, rA = a.shape
        if ra * m * n * k * n * rA > max_core_entries:
            raise InvalidArguments("amen_mm: operator core too large for the (A x I) form.")
        eye = torch.eye(n, dtype=torch.float64, device=dev)
        Ak.append(torch.einsum('amkA,np->amnkpA', a, eye).reshape(ra, m * n, k * n, rA).contiguous())
    bv = [c.detach().to(device=dev, dtype=torch.float64).reshape(c.shape[0], -1, c.shape[-1]).contiguous()
          for c in B.cores]
    x0 = None
    if X0 is not None:
        x0 = [c.detach().to(device=dev, dtype=torch.float64).reshape(c.shape[0], -1, c.shape[-1]).contiguous()
              for c in X0.cores]
    cores = _run(Ak, bv, x0, nswp, eps, rmax, kickrank, kick2, seed, verbose, dev)
    out = [c.reshape(c.shape[0], m, n, c.shape[-1]).to(B.cores[0].device)
           for c, m, n in zip(cores, A.M, Ns)]
    return TT(out)
