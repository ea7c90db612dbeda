"""Batched / served AMEn solves on one GPU.

``Server`` wraps the library's request server (``ttgb_server_*`` in include/ttgb300.h): up to
``slots`` solves run concurrently, each on its own CUDA stream and host thread, so their kernels
overlap on the device; requests are admitted FIFO as a slot frees and their estimated HBM footprint
fits the budget (continuous batching). Each request keeps its inputs resident until it completes
and reports its queue and run latency.

    with Server(slots=8) as srv:
        ids = [srv.submit(A, b, eps=1e-8, precision="mixed", seed=i) for i, (A, b) in enumerate(reqs)]
        results = [srv.result(i) for i in ids]     # (TT, stats) with stats["queue_ms"], ["run_ms"]
"""
import ctypes

import torch

from . import _lib
from .solvers import _desc, _is_tt, _prep, fetch_solution, make_params
from .tt import TT

_PREC = {None: 0, "c": 1, "r": 2}


class Server:
    def __init__(self, slots=8, mem_budget_bytes=0, device=None):
        if not torch.cuda.is_available():
            raise RuntimeError("the gb300 server needs a CUDA device")
        if isinstance(device, torch.device):
            self.device = device
        else:
            self.device = torch.device("cuda", torch.cuda.current_device() if device is None else int(device))
        torch.cuda.set_device(self.device)
        self._L = _lib.lib()
        h = _lib.c_vp()
        _lib.check(self._L.ttgb_server_create(int(slots), int(mem_budget_bytes), ctypes.byref(h)))
        self._h = h
        self._inflight = {}   # id -> (input tensors and descriptors kept alive, modes, output class)

    def submit(self, A, b, x0=None, preconditioner=None, **params):
        """Queues A x = b; returns the request id. Keyword arguments as ``amen_solve`` plus
        ``precision``, ``engine``, ``seed``."""
        if not (_is_tt(A) and _is_tt(b)):
            raise TypeError("A and b must be TT instances")
        Ac = _prep(A.cores, self.device)
        bc = _prep(b.cores, self.device)
        xc = _prep(x0.cores, self.device) if x0 is not None else None
        keep = [Ac, bc, xc]
        dA = _desc(Ac, True, keep)
        db = _desc(bc, False, keep)
        dx = _desc(xc, False, keep) if xc else None
        p = make_params(preconditioner=_PREC[preconditioner], **params)
        keep.append(p)
        torch.cuda.current_stream(self.device).synchronize()   # inputs resident before workers read
        rid = _lib.c_i64()
        _lib.check(self._L.ttgb_server_submit(self._h, ctypes.byref(dA), ctypes.byref(db),
                                              ctypes.byref(dx) if dx is not None else None,
                                              ctypes.byref(p), ctypes.byref(rid)))
        out_cls = type(b) if _is_tt(b) else TT
        self._inflight[rid.value] = (keep, [int(c.shape[2]) for c in Ac], out_cls, b.cores[0].device)
        return rid.value

    def result(self, rid, timeout=None):
        """Waits for request ``rid``; returns ``(x, stats)`` (``x`` of the class of ``b``, on the device
        of ``b``) with the latencies in ``stats['queue_ms']`` and ``stats['run_ms']``."""
        keep, modes, cls, out_dev = self._inflight[rid]
        sol = _lib.c_vp()
        qms, rms = ctypes.c_double(), ctypes.c_double()
        st = self._L.ttgb_server_wait(self._h, int(rid), -1.0 if timeout is None else float(timeout),
                                      ctypes.byref(sol), ctypes.byref(qms), ctypes.byref(rms))
        if st == 6:   # still running
            raise TimeoutError("request %d still running" % rid)
        del self._inflight[rid]
        _lib.check(st)
        cores, stats = fetch_solution(sol, modes, self.device, torch.cuda.current_stream(self.device))
        stats["queue_ms"] = qms.value
        stats["run_ms"] = rms.value
        cores = [c.to(out_dev) for c in cores]
        try:
            x = cls(cores)
        except Exception:
            x = TT(cores)
        return x, stats

    def stats(self):
        sub, comp = _lib.c_i64(), _lib.c_i64()
        run, peak = _lib.c_i32(), _lib.c_i32()
        _lib.check(self._L.ttgb_server_stats(self._h, ctypes.byref(sub), ctypes.byref(comp),
                                             ctypes.byref(run), ctypes.byref(peak)))
        return {"submitted": sub.value, "completed": comp.value, "running": run.value,
                "peak_running": peak.value}

    def memory(self):
        """Admission accounting: ``budget``, ``in_use`` (bytes reserved by running requests) and
        ``peak_in_use`` (the most reserved at once so far)."""
        b, u, pk = _lib.c_i64(), _lib.c_i64(), _lib.c_i64()
        _lib.check(self._L.ttgb_server_memory(self._h, ctypes.byref(b), ctypes.byref(u), ctypes.byref(pk)))
        return {"budget": b.value, "in_use": u.value, "peak_in_use": pk.value}

    def close(self):
        if self._h:
            self._L.ttgb_server_destroy(self._h)
            self._h = None
            self._inflight.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def footprint(A, b, x0=None, preconditioner=None, **params):
    """Upper bound of the device bytes one solve of A x = b allocates (the server's admission unit,
    ``ttgb_footprint``): every core, interface and workspace at the largest rank the solve can
    reach, rank(x0) + nswp (kickrank + kick2), capped by rmax and the mode sizes."""
    keep = []
    dev = b.cores[0].device if b.cores[0].is_cuda else torch.device("cuda", torch.cuda.current_device())
    Ac, bc = _prep(A.cores, dev), _prep(b.cores, dev)
    xc = _prep(x0.cores, dev) if x0 is not None else None
    dA, db = _desc(Ac, True, keep), _desc(bc, False, keep)
    dx = _desc(xc, False, keep) if xc else None
    p = make_params(preconditioner=_PREC[preconditioner], **params)
    out = _lib.c_i64()
    _lib.check(_lib.lib().ttgb_footprint(ctypes.byref(dA), ctypes.byref(db),
                                         ctypes.byref(dx) if dx is not None else None,
                                         ctypes.byref(p), ctypes.byref(out)))
    return out.value


def pool_usage(reset_high=False):
    """Bytes the library holds in the device's default memory pool now and at most since the last
    reset: ``(used_now, used_high)``."""
    now, high = _lib.c_i64(), _lib.c_i64()
    _lib.check(_lib.lib().ttgb_pool_usage(ctypes.byref(now), ctypes.byref(high), int(bool(reset_high))))
    return now.value, high.value
