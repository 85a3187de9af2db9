"""pnfft_gb300 -- PNFFT's nonequispaced FFT hot path on one NVIDIA GB300.

The product is the C-ABI library libpnfft_gb300.so (include/pnfft.h,
include/pnfft_gb300.h).  This package is a thin Python view of it:

  * ``Plan`` mirrors a pnfft plan + nodes pair over host (numpy) arrays, the
    way the reference's C callers use the library (pnfft_init_guru,
    pnfft_init_nodes, pnfft_set_*, pnfft_trafo, pnfft_adj);
  * ``Plan.trafo_device`` / ``Plan.adj_device`` run on device-resident torch
    tensors through the zero-copy extension (no host copies);
  * ``pnfft_gb300.autograd`` wraps trafo as a torch.autograd.Function.

Every call goes through the CUDA library; a missing library or GPU raises.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import *  # noqa: F401,F403  (flag constants)

__all__ = ["Plan", "PnfftError", "load", "last_error", "device_count"]

load = _lib.load
last_error = _lib.last_error


def device_count():
    return load().pnfft_gb300_device_count()


def _pd(v):
    return (ctypes.c_ssize_t * 3)(*[int(a) for a in v])


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class PnfftError(RuntimeError):
    pass


def _stream_handle(stream):
    """cudaStream_t of a torch stream; torch's default stream (handle 0) is the
    legacy default stream, passed as cudaStreamLegacy (0x1) because a NULL
    stream selects the plan's own stream."""
    h = stream.cuda_stream
    return h if h else 0x1


def _check(rc=0, what="pnfft"):
    msg = last_error()
    if rc != 0 or msg:
        load().pnfft_gb300_clear_error()
        raise PnfftError(f"{what}: {msg or 'error'}")


class Plan:
    """One pnfft plan (1x1x1 mesh) with one nodes object.

    N, n: 3 sizes (n defaults to 2N); m: window cutoff; flags: PNFFT plan flags
    (window, interlacing, ik, intpol tables, transposed f_hat...); c2r: real
    plan; precision: "fp64" or "fp32" (FP32-mixed).
    """

    def __init__(self, N, n=None, m=6, flags=0, x_max=0.5, c2r=False, precision="fp64", M=0):
        L = load()
        L.pnfft_gb300_clear_error()
        self.N = tuple(int(v) for v in N)
        self.n = tuple(int(v) for v in (n if n is not None else [2 * v for v in N]))
        self.m = int(m)
        self.c2r = bool(c2r)
        xm = np.ascontiguousarray(np.broadcast_to(np.asarray(x_max, dtype=np.float64), (3,)))
        init = L.pnfft_init_guru_c2r if self.c2r else L.pnfft_init_guru
        self._p = init(3, _pd(self.N), _pd(self.n), _dp(xm), self.m, ctypes.c_uint(flags), PFFT_ESTIMATE,
                       MPI_COMM_WORLD)
        if not self._p:
            _check(-1, "pnfft_init_guru")
        self.set_precision(precision)
        lN, lNs = (ctypes.c_ssize_t * 3)(), (ctypes.c_ssize_t * 3)()
        lo, up = (ctypes.c_double * 3)(), (ctypes.c_double * 3)()
        ls = L.pnfft_local_size_guru_c2r if self.c2r else L.pnfft_local_size_guru
        ls(3, _pd(self.N), _pd(self.n), _dp(xm), self.m, MPI_COMM_WORLD, ctypes.c_uint(flags), lN, lNs, lo, up)
        self.local_N = tuple(lN)
        self.local_N_start = tuple(lNs)
        self.lower_border = tuple(lo)
        self.upper_border = tuple(up)
        self.flags = L.pnfft_get_pnfft_flags(self._p)
        self._nodes = L.pnfft_init_nodes(0, 0)
        self._M = 0
        self._keep = []

    # ------------------------------------------------------------------
    def close(self):
        L = load()
        if getattr(self, "_nodes", None):
            L.pnfft_free_nodes(self._nodes, 0)
            self._nodes = None
        if getattr(self, "_p", None):
            L.pnfft_finalize(self._p, 0)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._p

    @property
    def transposed(self):
        return bool(self.flags & TRANSPOSED_F_HAT)

    @property
    def fhat_shape(self):
        a, b, c = self.local_N
        return (b, c, a) if self.transposed else (a, b, c)

    def set_precision(self, precision):
        code = {"fp64": GB300_FP64, "fp32": GB300_FP32_MIXED, "fp32-mixed": GB300_FP32_MIXED}[precision]
        _check(load().pnfft_gb300_set_precision(self._p, code), "set_precision")
        self.precision = precision

    def b(self):
        b0, b1, b2 = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        load().pnfft_get_b(self._p, ctypes.byref(b0), ctypes.byref(b1), ctypes.byref(b2))
        return (b0.value, b1.value, b2.value)

    def set_b(self, b0, b1, b2):
        load().pnfft_set_b(b0, b1, b2, self._p)

    def psi(self, dim, x):
        return load().pnfft_psi(self._p, dim, x)

    def dpsi(self, dim, x):
        return load().pnfft_dpsi(self._p, dim, x)

    def ddpsi(self, dim, x):
        return load().pnfft_ddpsi(self._p, dim, x)

    def phi_hat(self, dim, k):
        return load().pnfft_phi_hat(self._p, dim, k)

    def inv_phi_hat(self, dim, k):
        return load().pnfft_inv_phi_hat(self._p, dim, k)

    def stage_ms(self, adjoint=False):
        out = (ctypes.c_double * TIMER_LENGTH)()
        load().pnfft_gb300_last_stage_ms(self._p, 1 if adjoint else 0, out)
        return list(out)

    def timers(self, adjoint=False):
        L = load()
        t = (L.pnfft_get_timer_adj if adjoint else L.pnfft_get_timer_trafo)(self._p)
        v = [t[i] for i in range(TIMER_LENGTH)]
        L.pnfft_timer_free(t)
        return v

    # ------------------------------------------------------------------
    def _nodes_for(self, M):
        L = load()
        if M != self._M:
            L.pnfft_free_nodes(self._nodes, 0)
            self._nodes = L.pnfft_init_nodes(M, 0)
            self._M = M
        return self._nodes

    def _out(self, M, comps):
        dt = np.float64 if self.c2r else np.complex128
        return np.zeros((M, comps) if comps > 1 else M, dtype=dt)

    def trafo(self, x, f_hat, compute_flags=COMPUTE_F, f=None, grad=None, hess=None):
        """pnfft_trafo on host arrays; returns (f, grad_f, hessian_f)."""
        L = load()
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        M = x.shape[0]
        nd = self._nodes_for(M)
        fh = np.ascontiguousarray(f_hat, dtype=np.complex128).reshape(-1)
        if fh.size != int(np.prod(self.local_N)):
            raise ValueError(f"f_hat has {fh.size} entries, plan expects {int(np.prod(self.local_N))}")
        if compute_flags & COMPUTE_F and f is None:
            f = self._out(M, 1)
        if compute_flags & COMPUTE_GRAD_F and grad is None:
            grad = self._out(M, 3)
        if compute_flags & COMPUTE_HESSIAN_F and hess is None:
            hess = self._out(M, 6)
        L.pnfft_set_x(x.ctypes.data, nd)
        L.pnfft_set_f(f.ctypes.data if f is not None else None, nd)
        L.pnfft_set_grad_f(grad.ctypes.data if grad is not None else None, nd)
        L.pnfft_set_hessian_f(hess.ctypes.data if hess is not None else None, nd)
        L.pnfft_set_f_hat(fh.ctypes.data, self._p)
        L.pnfft_gb300_clear_error()
        L.pnfft_trafo(self._p, nd, ctypes.c_uint(compute_flags))
        _check(0, "pnfft_trafo")
        return f, grad, hess

    def adj(self, x, f=None, grad=None, compute_flags=COMPUTE_F, f_hat=None):
        """pnfft_adj on host arrays; returns f_hat (flattened, plan layout)."""
        L = load()
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        M = x.shape[0]
        nd = self._nodes_for(M)
        dt = np.float64 if self.c2r else np.complex128
        if f is not None:
            f = np.ascontiguousarray(f, dtype=dt).reshape(-1)
        if grad is not None:
            grad = np.ascontiguousarray(grad, dtype=dt).reshape(-1, 3)
        size = int(np.prod(self.local_N))
        if f_hat is None:
            f_hat = np.zeros(size, dtype=np.complex128)
        L.pnfft_set_x(x.ctypes.data, nd)
        L.pnfft_set_f(f.ctypes.data if f is not None else None, nd)
        L.pnfft_set_grad_f(grad.ctypes.data if grad is not None else None, nd)
        L.pnfft_set_f_hat(f_hat.ctypes.data, self._p)
        L.pnfft_gb300_clear_error()
        L.pnfft_adj(self._p, nd, ctypes.c_uint(compute_flags))
        _check(0, "pnfft_adj")
        return f_hat

    # ------------------------------------------------------------------
    # device-resident (zero-copy) entry points over torch tensors
    def _bind_device(self, x, f, grad, hess, f_hat, stream):
        L = load()
        M = x.shape[0]
        nd = self._nodes_for(M)
        ptr = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        L.pnfft_gb300_set_device_arrays(nd, ptr(x), ptr(f), ptr(grad), ptr(hess))
        L.pnfft_gb300_set_device_f_hat(self._p, ptr(f_hat))
        L.pnfft_gb300_set_stream(self._p, stream)
        return nd

    def _unbind_device(self):
        L = load()
        L.pnfft_gb300_set_device_arrays(self._nodes, None, None, None, None)
        L.pnfft_gb300_set_device_f_hat(self._p, None)

    def set_conv_method(self, method):
        """Both directions: 0 line kernels (default); 1 one thread per node; 2 the
        FP32-mixed B one warp per node over 8x8x8 tiles and B^T with the window
        that moves by copies; 3 as 2 with groups of nodes for f alone."""
        _check(load().pnfft_gb300_set_conv_method(self._p, int(method)), "set_conv_method")

    def tuning(self):
        """(interpolation method, spreading method, nodes per line sub-problem)."""
        t = (ctypes.c_int * 3)()
        _check(load().pnfft_gb300_get_tuning(self._p, t), "get_tuning")
        return tuple(t)

    def set_tuning(self, tuning):
        """Restore a tuning() triple."""
        t = (ctypes.c_int * 3)(*[int(v) for v in tuning])
        _check(load().pnfft_gb300_set_tuning(self._p, t), "set_tuning")

    def autotune_device(self, x, f_hat, trafo_flags=COMPUTE_F, adj_flags=COMPUTE_F, reps=2):
        """pnfft_gb300_autotune on CUDA tensors: times the kernel families and the
        line sub-problem size on the nodes x for a trafo with trafo_flags and an
        adjoint with adj_flags (0: not used) and keeps the fastest; returns
        tuning().  The transforms run on scratch node arrays and a copy of
        f_hat; the arguments are left unchanged."""
        import torch
        dt = torch.float64 if self.c2r else torch.complex128
        M = x.shape[0]
        grad = (trafo_flags | adj_flags) & COMPUTE_GRAD_F
        fo = torch.zeros(M, dtype=dt, device=x.device)
        go = torch.zeros(M, 3, dtype=dt, device=x.device) if grad else None
        ho = torch.zeros(M, 6, dtype=dt, device=x.device) if trafo_flags & COMPUTE_HESSIAN_F else None
        fh = f_hat.clone()
        s = _stream_handle(torch.cuda.current_stream(x.device))
        L = load()
        nd = self._bind_device(x, fo, go, ho, fh, s)
        L.pnfft_gb300_clear_error()
        rc = L.pnfft_gb300_autotune(self._p, nd, ctypes.c_uint(trafo_flags), ctypes.c_uint(adj_flags), int(reps))
        self.synchronize()
        _check(rc, "pnfft_gb300_autotune")
        return self.tuning()

    CONV_KERNELS = {0: "none", 1: "group", 2: "tile", 3: "line", 4: "generic"}

    def conv_kernel(self, adjoint=False):
        """Kernel family of the last B (or B^T with adjoint=True): "group",
        "tile", "line", "generic" or "none"."""
        return self.CONV_KERNELS.get(load().pnfft_gb300_get_conv_kernel(self._p, int(bool(adjoint))), "?")

    def trafo_device(self, x, f_hat, compute_flags=COMPUTE_F, f=None, grad=None, hess=None, stream=None,
                     fixed_nodes=False):
        """pnfft_trafo on CUDA tensors: x (M,3) float64, f_hat complex128 in the
        plan layout; outputs complex128 (c2c) or float64 (c2r).  Runs on
        `stream` (a torch.cuda.Stream, default: current) without host sync."""
        import torch
        dt = torch.float64 if self.c2r else torch.complex128
        M = x.shape[0]
        if compute_flags & COMPUTE_F and f is None:
            f = torch.empty(M, dtype=dt, device=x.device)
        if compute_flags & COMPUTE_GRAD_F and grad is None:
            grad = torch.empty(M, 3, dtype=dt, device=x.device)
        if compute_flags & COMPUTE_HESSIAN_F and hess is None:
            hess = torch.empty(M, 6, dtype=dt, device=x.device)
        s = _stream_handle(stream or torch.cuda.current_stream(x.device))
        nd = self._bind_device(x, f, grad, hess, f_hat, s)
        L = load()
        if fixed_nodes:
            L.pnfft_gb300_nodes_set_fixed(nd, 1) if not getattr(self, "_fixed", False) else None
            self._fixed = True
        L.pnfft_gb300_clear_error()
        L.pnfft_trafo(self._p, nd, ctypes.c_uint(compute_flags))
        _check(0, "pnfft_trafo")
        return f, grad, hess

    def adj_device(self, x, f=None, grad=None, compute_flags=COMPUTE_F, f_hat=None, stream=None, fixed_nodes=False):
        """pnfft_adj on CUDA tensors; returns f_hat (complex128, plan layout)."""
        import torch
        if f_hat is None:
            f_hat = torch.empty(int(np.prod(self.local_N)), dtype=torch.complex128, device=x.device)
        s = _stream_handle(stream or torch.cuda.current_stream(x.device))
        nd = self._bind_device(x, f, grad, None, f_hat, s)
        L = load()
        if fixed_nodes:
            L.pnfft_gb300_nodes_set_fixed(nd, 1) if not getattr(self, "_fixed", False) else None
            self._fixed = True
        L.pnfft_gb300_clear_error()
        L.pnfft_adj(self._p, nd, ctypes.c_uint(compute_flags))
        _check(0, "pnfft_adj")
        return f_hat

    def synchronize(self):
        _check(load().pnfft_gb300_synchronize(self._p), "synchronize")

    # ------------------------------------------------------------------
    def sort_nodes(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        pairs = np.zeros(2 * x.shape[0], dtype=np.int64)
        rc = load().pnfft_gb300_sort_nodes(self._p, x.shape[0], _dp(x),
                                           pairs.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)))
        _check(rc, "sort_nodes")
        return pairs.reshape(-1, 2)

    def node_index(self, x, interlaced=0):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        u = np.zeros((x.shape[0], 3), dtype=np.int64)
        rc = load().pnfft_gb300_node_index(self._p, x.shape[0], _dp(x), interlaced,
                                           u.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)))
        _check(rc, "node_index")
        return u
