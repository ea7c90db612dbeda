"""The tensor-train type at the solver boundary.

``TT`` mirrors the parts of the reference's ``torchtt.TT`` (``torchtt/_tt_base.py:18-229``) that
the AMEn path uses: construction from a list of cores with the same rank checks and errors, the
``cores``/``N``/``M``/``R``/``is_ttm`` properties, device moves, the algebra the reference's
tests apply to a solution (``A @ x``, ``x - b``, ``.norm()``; ``tests/test_solvers.py:19``) and
``round``. ``@``, ``norm`` and ``round`` run on the GPU through the library; ``+``/``-`` only
concatenate cores.
The solver also accepts the reference's own ``torchtt.TT`` objects (anything with ``cores`` and
``is_ttm``) and returns an object of the same class as ``b``.
"""
import torch

from .errors import IncompatibleTypes, InvalidArguments, RankMismatch, ShapeMismatch


class TT:
    def __init__(self, cores):
        if not isinstance(cores, (list, tuple)) or len(cores) == 0:
            raise InvalidArguments("TT expects a non-empty list of cores.")
        cores = list(cores)
        R = [cores[0].shape[0]]
        N, M = [], []
        for i, c in enumerate(cores):   # torchtt/_tt_base.py:123-161
            s = c.shape
            if s[0] != R[-1]:
                raise RankMismatch("Ranks of the given cores do not match: for core number %d previous "
                                   "rank is %d and and current rank is %d." % (i, R[-1], s[0]))
            if len(s) == 3:
                R.append(s[2]); N.append(s[1])
            elif len(s) == 4:
                R.append(s[3]); M.append(s[1]); N.append(s[2])
            else:
                raise InvalidArguments("Invalid input: TT-cores have to be either 4d or 3d.")
        if R[0] != 1 or R[-1] != 1 or (len(M) != 0 and len(M) != len(N)):
            raise InvalidArguments("Check the ranks and the mode size.")
        self.cores = cores
        self._R = [int(r) for r in R]
        self._N = [int(n) for n in N]
        self._M = [int(m) for m in M]
        self._is_ttm = len(M) == len(N)

    # -- properties ------------------------------------------------------------------------
    @property
    def is_ttm(self):
        return self._is_ttm

    @property
    def N(self):
        return list(self._N)

    @property
    def M(self):
        if not self._is_ttm:
            raise IncompatibleTypes("The field is_ttm is defined only for TT matrices.")
        return list(self._M)

    @property
    def R(self):
        return list(self._R)

    @property
    def shape(self):
        return [(m, n) for m, n in zip(self._M, self._N)] if self._is_ttm else list(self._N)

    def __repr__(self):
        kind = "TT-matrix" if self._is_ttm else "TT"
        return "%s with sizes %s, ranks %s, device %s" % (kind, self.shape, self._R, self.cores[0].device)

    # -- device / dtype ----------------------------------------------------------------------
    def to(self, device=None, dtype=None):
        return TT([c.to(device=device, dtype=dtype) for c in self.cores])

    def cuda(self, device=None):
        return TT([c.cuda(device) for c in self.cores])

    def cpu(self):
        return TT([c.cpu() for c in self.cores])

    def clone(self):
        return TT([c.clone() for c in self.cores])

    # -- algebra used to check solutions ------------------------------------------------------
    def __matmul__(self, other):
        """TT-matrix @ TT-vector core by core (torchtt/_tt_base.py:807-817): ranks multiply. Runs
        on the GPU (``ttgb_tt_matvec``); the result lives on the device of ``other``'s cores."""
        import ctypes
        from . import _lib
        from .solvers import _desc, fetch_solution
        if not (self._is_ttm and not other.is_ttm):
            raise IncompatibleTypes("Only TT-matrix @ TT-vector is supported here.")
        if self._N != list(other.N):
            raise ShapeMismatch("Shapes are incompatible.")
        Ac, dev = self._device_cores()
        xc = [c.detach().to(device=dev, dtype=torch.float64).contiguous() for c in other.cores]
        keep = []
        dA, dx = _desc(Ac, True, keep), _desc(xc, False, keep)
        stream = torch.cuda.current_stream(dev)
        h = _lib.c_vp()
        _lib.check(_lib.lib().ttgb_tt_matvec(ctypes.byref(dA), ctypes.byref(dx),
                                             ctypes.c_void_p(stream.cuda_stream), ctypes.byref(h)))
        out, _ = fetch_solution(h, list(self._M), dev, stream)
        return TT([c.to(other.cores[0].device) for c in out])

    def _combine(self, other, beta):
        if self._is_ttm or other.is_ttm:
            raise IncompatibleTypes("Only TT-vectors can be added here.")
        if self._N != list(other.N):
            raise ShapeMismatch("Shapes are incompatible.")
        d = len(self.cores)
        a_c, b_c = self.cores, list(other.cores)
        if d == 1:
            return TT([a_c[0] + beta * b_c[0]])
        out = []
        for k in range(d):
            a, b = a_c[k], b_c[k]
            if k == 0:
                out.append(torch.cat([a, beta * b], dim=2))
            elif k == d - 1:
                out.append(torch.cat([a, b], dim=0))
            else:
                c = torch.zeros((a.shape[0] + b.shape[0], a.shape[1], a.shape[2] + b.shape[2]),
                                dtype=a.dtype, device=a.device)
                c[:a.shape[0], :, :a.shape[2]] = a
                c[a.shape[0]:, :, a.shape[2]:] = b
                out.append(c)
        return TT(out)

    def __add__(self, other):
        return self._combine(other, 1.0)

    def __sub__(self, other):
        return self._combine(other, -1.0)

    def __mul__(self, alpha):
        return TT([self.cores[0] * alpha] + self.cores[1:])

    __rmul__ = __mul__

    def __truediv__(self, other):
        """``self / other``: by a scalar, or elementwise by a TT of the same shape through AMEn on
        the GPU with the reference's fixed settings (50 sweeps, eps 1e-12, rmax 500;
        torchtt/_tt_base.py:900-934)."""
        if isinstance(other, (int, float)) or (torch.is_tensor(other) and other.numel() == 1):
            return TT([self.cores[0] / other] + self.cores[1:])
        if isinstance(other, TT) or (hasattr(other, "cores") and hasattr(other, "is_ttm")):
            from .division import amen_divide
            return TT(amen_divide(other, self, 50, None, 1e-12, 500))
        raise InvalidArguments("Operand not permitted. A TT-object can be divided only with scalars.")

    def __rtruediv__(self, other):
        """``scalar / self`` elementwise through AMEn on the GPU (torchtt/_tt_base.py:936-966)."""
        if isinstance(other, (int, float)) or (torch.is_tensor(other) and other.numel() == 1):
            from .division import amen_divide
            ones = TT([torch.ones((1,) + tuple(c.shape[1:-1]) + (1,), dtype=c.dtype, device=c.device)
                       for c in self.cores])
            ones.cores[0] = ones.cores[0] * other
            return TT(amen_divide(self, ones, 50, None, 1e-12, 500))
        raise InvalidArguments("The first operand must be int, float or 1d torch.tensor.")

    def _device_cores(self):
        """The cores as contiguous CUDA float64 tensors (copied to the current GPU if needed)."""
        if not torch.cuda.is_available():
            raise RuntimeError("TT products, norms and rounding run on the GPU; no CUDA device is "
                               "available.")
        dev = self.cores[0].device if self.cores[0].is_cuda else \
            torch.device("cuda", torch.cuda.current_device())
        return [c.detach().to(device=dev, dtype=torch.float64).contiguous() for c in self.cores], dev

    def norm(self):
        """Frobenius norm (torchtt/_tt_base.py:1021-1051), computed on the GPU by a QR sweep
        (``ttgb_tt_norm``); returns a 0-d float64 tensor on the device of the cores."""
        import ctypes
        from . import _lib
        from .solvers import _desc
        cores, dev = self._device_cores()
        keep = []
        desc = _desc(cores, self._is_ttm, keep)
        out = ctypes.c_double()
        stream = torch.cuda.current_stream(dev)
        _lib.check(_lib.lib().ttgb_tt_norm(ctypes.byref(desc), ctypes.byref(out),
                                           ctypes.c_void_p(stream.cuda_stream)))
        return torch.tensor(out.value, dtype=torch.float64, device=self.cores[0].device)

    def round(self, eps=1e-12, rmax=2**62):
        """TT rounding to relative accuracy ``eps`` with rank cap ``rmax`` (torchtt/_tt_base.py:
        1427-1450, round_tt in torchtt/_decomposition.py:169-228) on the GPU (``ttgb_tt_round``).
        Returns a new TT on the device of the cores."""
        import ctypes
        from . import _lib
        from .solvers import _desc, fetch_solution
        if isinstance(rmax, (list, tuple)):
            raise InvalidArguments("rmax must be an integer here.")
        cores, dev = self._device_cores()
        keep = []
        desc = _desc(cores, self._is_ttm, keep)
        stream = torch.cuda.current_stream(dev)
        h = _lib.c_vp()
        _lib.check(_lib.lib().ttgb_tt_round(ctypes.byref(desc), float(eps), int(rmax),
                                            ctypes.c_void_p(stream.cuda_stream), ctypes.byref(h)))
        modes = [m * n for m, n in zip(self._M, self._N)] if self._is_ttm else list(self._N)
        out, _ = fetch_solution(h, modes, dev, stream)
        if self._is_ttm:
            out = [c.reshape(c.shape[0], m, n, c.shape[2]) for c, m, n in zip(out, self._M, self._N)]
        return TT([c.to(self.cores[0].device) for c in out])

    def full(self):
        t = self.cores[0]
        for c in self.cores[1:]:
            t = torch.tensordot(t, c, dims=([t.dim() - 1], [0]))
        return t.reshape(t.shape[1:-1])
