"""Kernel-level operations of the AMEn path on CUDA float64 tensors, through the C ABI.

Each function mirrors one reference helper (cited) and runs the library's kernel on the current
CUDA stream. Shapes follow the reference's tensor layouts.
"""
import ctypes

import torch

from . import _lib


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream(dev):
    return ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def _dev64(*ts):
    for t in ts:
        if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
            raise ValueError("expected contiguous CUDA float64 tensors")


def local_product(Phi_right, Phi_left, coreA, core):
    """y[l,m,L] = sum Phi_left[l,s,r] coreA[s,m,n,S] Phi_right[L,S,R] core[r,n,R]
    (reference: local_product, cpp/amen_solve.h:17-27). ``core`` may carry a leading batch dim."""
    batched = core.dim() == 4
    x = core if batched else core.unsqueeze(0)
    _dev64(Phi_right, Phi_left, coreA, x)
    rl, s, r = Phi_left.shape
    s2, m, n, S = coreA.shape
    RL, S2, R = Phi_right.shape
    nb = x.shape[0]
    assert s2 == s and S2 == S and x.shape[1:] == (r, n, R)
    y = torch.empty((nb, rl, m, RL), dtype=torch.float64, device=x.device)
    _lib.check(_lib.lib().ttgb_local_product(rl, s, r, m, n, S, RL, R, _ptr(Phi_left), _ptr(coreA),
                                             _ptr(Phi_right), _ptr(x), _ptr(y), nb, _stream(x.device)))
    return y if batched else y[0]


def compute_phi_fwd_A(Phi_now, core_left, core_A, core_right):
    """Phi_next[L,S,R] (reference: compute_phi_fwd_A, cpp/amen_solve.h:58-68)."""
    _dev64(Phi_now, core_left, core_A, core_right)
    l, M, L = core_left.shape
    s, _, N, S = core_A.shape
    r, _, R = core_right.shape
    out = torch.empty((L, S, R), dtype=torch.float64, device=core_A.device)
    _lib.check(_lib.lib().ttgb_phi_fwd_A(l, L, s, S, r, R, M, N, _ptr(Phi_now), _ptr(core_left),
                                         _ptr(core_A), _ptr(core_right), _ptr(out), _stream(out.device)))
    return out


def compute_phi_bck_A(Phi_now, core_left, core_A, core_right):
    """Phi[l,s,r] (reference: compute_phi_bck_A, cpp/amen_solve.h:38-47)."""
    _dev64(Phi_now, core_left, core_A, core_right)
    l, M, L = core_left.shape
    s, _, N, S = core_A.shape
    r, _, R = core_right.shape
    out = torch.empty((l, s, r), dtype=torch.float64, device=core_A.device)
    _lib.check(_lib.lib().ttgb_phi_bck_A(l, L, s, S, r, R, M, N, _ptr(Phi_now), _ptr(core_left),
                                         _ptr(core_A), _ptr(core_right), _ptr(out), _stream(out.device)))
    return out


def compute_phi_fwd_rhs(Phi_now, core_rhs, core):
    """Phi_next[B,R] (reference: compute_phi_fwd_rhs, cpp/amen_solve.h:93-98)."""
    _dev64(Phi_now, core_rhs, core)
    b, n, B = core_rhs.shape
    r, _, R = core.shape
    out = torch.empty((B, R), dtype=torch.float64, device=core.device)
    _lib.check(_lib.lib().ttgb_phi_fwd_rhs(b, B, r, R, n, _ptr(Phi_now), _ptr(core_rhs), _ptr(core),
                                           _ptr(out), _stream(out.device)))
    return out


def compute_phi_bck_rhs(Phi_now, core_b, core):
    """Phi[b,r] (reference: compute_phi_bck_rhs, cpp/amen_solve.h:78-83)."""
    _dev64(Phi_now, core_b, core)
    b, n, B = core_b.shape
    r, _, R = core.shape
    out = torch.empty((b, r), dtype=torch.float64, device=core.device)
    _lib.check(_lib.lib().ttgb_phi_bck_rhs(b, B, r, R, n, _ptr(Phi_now), _ptr(core_b), _ptr(core),
                                           _ptr(out), _stream(out.device)))
    return out


def qr(mat):
    """Thin QR of a (m x n) CUDA float64 matrix (reference: at::linalg_qr, reduced mode)."""
    m, n = mat.shape
    a = mat.t().contiguous()                 # column-major storage of mat
    k = min(m, n)
    q = torch.empty((k, m), dtype=torch.float64, device=mat.device)   # column-major m x k
    r = torch.empty((n, k), dtype=torch.float64, device=mat.device)   # column-major k x n
    _lib.check(_lib.lib().ttgb_qr(_ptr(a), m, m, n, _ptr(q), _ptr(r), _stream(mat.device)))
    return q.t(), r.t()


def svd(mat):
    """Thin SVD of a (m x n) CUDA float64 matrix: U, S, Vh (reference: at::linalg_svd(.., false))."""
    m, n = mat.shape
    a = mat.t().contiguous()
    k = min(m, n)
    u = torch.empty((k, m), dtype=torch.float64, device=mat.device)
    s = torch.empty((k,), dtype=torch.float64, device=mat.device)
    vh = torch.empty((n, k), dtype=torch.float64, device=mat.device)
    _lib.check(_lib.lib().ttgb_svd(_ptr(a), m, m, n, _ptr(u), _ptr(s), _ptr(vh), _stream(mat.device)))
    return u.t(), s, vh.t()


def local_gmres(Phi_left, coreA, Phi_right, rhs, iters=40, threshold=1e-10, resets=2, prec=0):
    """GMRES on the local AMEn operator (reference: gmres, cpp/gmres.h:146-161, on AMENsolveMV).
    Returns ``(x, flag, nit)``; ``rhs`` has shape r x n x R."""
    _dev64(Phi_left, coreA, Phi_right, rhs)
    r, s, _ = Phi_left.shape
    _, n, _, S = coreA.shape
    R = Phi_right.shape[0]
    x = torch.empty_like(rhs)
    flag = _lib.c_i32()
    nit = _lib.c_i32()
    _lib.check(_lib.lib().ttgb_local_gmres(r, s, n, S, R, _ptr(Phi_left), _ptr(coreA), _ptr(Phi_right),
                                           _ptr(rhs), _ptr(x), int(iters), float(threshold), int(resets),
                                           int(prec), ctypes.byref(flag), ctypes.byref(nit),
                                           _stream(rhs.device)))
    return x, flag.value, nit.value


ENGINE_FP32 = 1
ENGINE_TC = 2
ENGINE_DF = 3


def local_product_lowp(Phi_right, Phi_left, coreA, core, engine=ENGINE_TC):
    """The local product with a low-precision engine (FP32 CUDA cores or tcgen05 3xTF32),
    FP64 in and out: the operator of the mixed path's inner GMRES. ``ENGINE_DF`` runs the mixed
    path's FP64-class products instead (double-float arithmetic on the FP32 pipe)."""
    _dev64(Phi_right, Phi_left, coreA, core)
    rl, s, r = Phi_left.shape
    _, m, n, S = coreA.shape
    RL, _, R = Phi_right.shape
    y = torch.empty((rl, m, RL), dtype=torch.float64, device=core.device)
    _lib.check(_lib.lib().ttgb_local_product_lowp(rl, s, r, m, n, S, RL, R, _ptr(Phi_left), _ptr(coreA),
                                                  _ptr(Phi_right), _ptr(core), _ptr(y), int(engine),
                                                  _stream(core.device)))
    return y


def calibrate_fma(dtype="fp64"):
    """Measured peak of this GPU's FMA pipe in TFLOP/s for ``dtype`` 'fp64' or 'fp32'
    (independent FMA chains on every SM; about 0.2 s)."""
    out = ctypes.c_double()
    _lib.check(_lib.lib().ttgb_calibrate_fma({"fp64": 0, "fp32": 1}[dtype], ctypes.byref(out)))
    return out.value


def autotune(mode=None):
    """Tile autotuner of the contraction engine: ``True`` on, ``False`` off (occupancy heuristic),
    ``None`` only queries. Returns the previous state and the number of recorded shape classes."""
    L = _lib.lib()
    prev = L.ttgb_autotune(-1 if mode is None else int(bool(mode)))
    return bool(prev), int(L.ttgb_autotune_classes())
