"""The reference PNFFT itself, driven through its own public C API --
TEST INFRASTRUCTURE ONLY.

oracle/build_ref.py compiles the reference's C sources unmodified against
single-process stand-ins for MPI, PFFT and GSL (oracle/refbuild/) into
oracle/_ref/libpnfft_ref.so.  RefPlan calls pnfft_init_guru, pnfft_init_nodes,
pnfft_trafo and pnfft_adj of that library (api/pnfft.h:51-275) exactly as a C
caller would, on a 1x1x1 mesh, c2c, without PNFFT_TRANSPOSED_F_HAT.  The tests
use it to pin the oracle restatement (pnfft_oracle.c) to the reference; the
product never loads it.  available() is False where the reference tree was not
present at build time (then no library exists).
"""
import ctypes
import os

import numpy as np

from . import build_ref

MALLOC_X, MALLOC_F, MALLOC_GRAD_F, MALLOC_HESSIAN_F = 1, 2, 4, 8
MALLOC_F_HAT = 1 << 6
PFFT_ESTIMATE = 1 << 4  # the stand-in's value (oracle/refbuild/pfft.h)
MPI_COMM_WORLD = 1

_lib = None


def available():
    return build_ref.available() or os.path.exists(build_ref.LIB)


def lib():
    global _lib
    if _lib is None:
        path = build_ref.build()
        if not path or not os.path.exists(path):
            raise RuntimeError("the reference build oracle/_ref/libpnfft_ref.so is not available")
        L = ctypes.CDLL(path, mode=os.RTLD_LOCAL)
        P, D, I, U, SS = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_uint, ctypes.c_ssize_t
        PS = ctypes.POINTER(ctypes.c_ssize_t)
        L.pnfft_init.argtypes = []
        L.pnfft_init_guru.restype = P
        L.pnfft_init_guru.argtypes = [I, PS, PS, D, I, U, U, I]
        L.pnfft_init_nodes.restype = P
        L.pnfft_init_nodes.argtypes = [SS, U]
        for name in ("pnfft_get_x", "pnfft_get_f", "pnfft_get_grad_f", "pnfft_get_hessian_f"):
            getattr(L, name).restype = P
            getattr(L, name).argtypes = [P]
        L.pnfft_get_f_hat.restype = P
        L.pnfft_get_f_hat.argtypes = [P]
        L.pnfft_trafo.argtypes = [P, P, U]
        L.pnfft_adj.argtypes = [P, P, U]
        L.pnfft_precompute_psi.argtypes = [P, P, U]
        L.pnfft_free_nodes.argtypes = [P, U]
        L.pnfft_finalize.argtypes = [P, U]
        L.pnfft_init()
        _lib = L
    return _lib


def _view(ptr, count):
    return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_double)), (count,))


class RefPlan:
    """pnfft_init_guru(3, N, n, x_max = 0.5, m, flags | PNFFT_MALLOC_F_HAT, ...) of the reference."""

    def __init__(self, N, n=None, m=6, flags=0):
        L = lib()
        self.N = tuple(int(v) for v in N)
        self.n = tuple(int(v) for v in (n if n is not None else [2 * v for v in N]))
        Nc = (ctypes.c_ssize_t * 3)(*self.N)
        nc = (ctypes.c_ssize_t * 3)(*self.n)
        xm = (ctypes.c_double * 3)(0.5, 0.5, 0.5)
        self._p = L.pnfft_init_guru(3, Nc, nc, xm, int(m), ctypes.c_uint(flags | MALLOC_F_HAT),
                                    ctypes.c_uint(PFFT_ESTIMATE), MPI_COMM_WORLD)
        if not self._p:
            raise RuntimeError("pnfft_init_guru of the reference returned NULL")
        self.size = int(np.prod(self.N))

    def _nodes(self, x):
        L = lib()
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        M = x.shape[0]
        nd = L.pnfft_init_nodes(M, ctypes.c_uint(MALLOC_X | MALLOC_F | MALLOC_GRAD_F | MALLOC_HESSIAN_F))
        _view(L.pnfft_get_x(nd), 3 * M)[:] = x.ravel()
        return nd, M

    def trafo(self, x, f_hat, cflags=1, precompute=0):
        """f, grad_f, hessian_f of pnfft_trafo (zeros where not computed)."""
        L = lib()
        nd, M = self._nodes(x)
        _view(L.pnfft_get_f_hat(self._p), 2 * self.size)[:] = np.ascontiguousarray(f_hat, np.complex128).view(
            np.float64)
        if precompute:
            L.pnfft_precompute_psi(self._p, nd, ctypes.c_uint(precompute))
        L.pnfft_trafo(self._p, nd, ctypes.c_uint(cflags))
        f = _view(L.pnfft_get_f(nd), 2 * M).copy().view(np.complex128)
        g = _view(L.pnfft_get_grad_f(nd), 6 * M).copy().view(np.complex128).reshape(M, 3)
        h = _view(L.pnfft_get_hessian_f(nd), 12 * M).copy().view(np.complex128).reshape(M, 6)
        L.pnfft_free_nodes(nd, ctypes.c_uint(MALLOC_X | MALLOC_F | MALLOC_GRAD_F | MALLOC_HESSIAN_F))
        return f, g, h

    def adj(self, x, f, grad=None, cflags=1):
        """f_hat of pnfft_adj."""
        L = lib()
        nd, M = self._nodes(x)
        _view(L.pnfft_get_f(nd), 2 * M)[:] = np.ascontiguousarray(f, np.complex128).view(np.float64)
        if grad is not None:
            _view(L.pnfft_get_grad_f(nd), 6 * M)[:] = np.ascontiguousarray(grad, np.complex128).view(
                np.float64).ravel()
        L.pnfft_adj(self._p, nd, ctypes.c_uint(cflags))
        out = _view(L.pnfft_get_f_hat(self._p), 2 * self.size).copy().view(np.complex128)
        L.pnfft_free_nodes(nd, ctypes.c_uint(MALLOC_X | MALLOC_F | MALLOC_GRAD_F | MALLOC_HESSIAN_F))
        return out

    def close(self):
        if self._p:
            lib().pnfft_finalize(self._p, ctypes.c_uint(MALLOC_F_HAT))
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
