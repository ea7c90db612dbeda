"""Elementwise division in the TT format, x = b / a, by AMEn on the GPU.

Reference: ``amen_divide`` (``torchtt/_division.py:76-398``), used by ``TT.__truediv__`` and
``TT.__rtruediv__`` (``torchtt/_tt_base.py:900-975``). The reference runs its AMEn skeleton with the
elementwise product by ``a`` as the operator. Here the operator is the diagonal TT-matrix
``diag(a)`` (core k holds ``a_k[s, m, S]`` on the diagonal ``m = n``) solved by the library's AMEn;
its cores are ``1/n`` dense, so the structured A stage applies them from their nonzeros. The
reference's defaults are kept: ``rmax`` 100 and the all-ones start of rank 2.
"""
import torch

from .errors import IncompatibleTypes, InvalidArguments, ShapeMismatch
from .solvers import _is_tt, solve_cores

_PREC = {None: 0, "c": 1, "r": 2}


def diag_ttm(a_cores):
    """Cores of the TT-matrix diag(a) for the TT-vector cores ``a_cores`` (r x n x r')."""
    out = []
    for c in a_cores:
        r, n, R = c.shape
        D = torch.zeros((r, n, n, R), dtype=c.dtype, device=c.device)
        idx = torch.arange(n, device=c.device)
        D[:, idx, idx, :] = c
        out.append(D)
    return out


def amen_divide(a, b, nswp=22, x0=None, eps=1e-10, rmax=100, max_full=500, kickrank=4, kick2=0,
                trunc_norm='res', local_iterations=40, resets=2, verbose=False, preconditioner=None,
                precision='fp64', seed=1):
    """Solves ``a * x = b`` elementwise for TT tensors (or TT-matrices) ``a`` and ``b`` of the same
    shape; returns the list of cores of ``x`` (as the reference does), on the device of ``b``'s
    cores. ``rmax`` is an integer rank cap. ``trunc_norm`` is accepted and, as in the reference's
    native paths, does not change the algorithm."""
    if not (_is_tt(a) and _is_tt(b)):
        raise InvalidArguments('a and b must be TT instances.')
    if a.is_ttm != b.is_ttm:
        raise IncompatibleTypes('Operands should be either TT or TTM.')
    if list(a.N) != list(b.N) or (a.is_ttm and list(a.M) != list(b.M)):
        raise ShapeMismatch('Both operands should have the same shape.')
    if preconditioner not in _PREC:
        raise InvalidArguments("Invalid preconditioner.")
    if isinstance(rmax, (list, tuple)):
        raise InvalidArguments("rmax must be an integer here.")
    if not torch.cuda.is_available():
        raise RuntimeError("The gb300 backend needs a CUDA device; it has no CPU fallback.")
    out_device = b.cores[0].device
    dev = out_device if out_device.type == "cuda" else torch.device("cuda", torch.cuda.current_device())
    flat = lambda cs: [c.detach().to(device=dev, dtype=torch.float64).reshape(c.shape[0], -1, c.shape[-1])
                       .contiguous() for c in cs]
    ac, bc = flat(a.cores), flat(b.cores)
    modes = [c.shape[1] for c in bc]
    d = len(modes)
    if x0 is None:   # the reference's start: all ones of rank 2 (torchtt/_division.py:91-93)
        rx = [1] + [2] * (d - 1) + [1]
        xc = [torch.ones((rx[k], modes[k], rx[k + 1]), dtype=torch.float64, device=dev) for k in range(d)]
    else:
        xc = flat(x0.cores)
    cores, _ = solve_cores(diag_ttm(ac), bc, xc, nswp=nswp, eps=eps, rmax=int(rmax),
                           max_full=max_full, kickrank=kickrank, kick2=kick2,
                           local_iterations=local_iterations, resets=resets, verbose=verbose,
                           preconditioner=_PREC[preconditioner], seed=seed, precision=precision)
    shapes = [tuple(c.shape[1:-1]) for c in b.cores]
    return [c.reshape((c.shape[0],) + sh + (c.shape[-1],)).to(out_device) for c, sh in zip(cores, shapes)]
