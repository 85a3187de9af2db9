"""CPU oracle of the PNFFT hot path (FP64) -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and the CPU legs of bench.py may import
this module; the product never does.  The arithmetic lives in
oracle/pnfft_oracle.c (a restatement of the reference's kernel/ code, see the
header of that file); this module restates the orchestration of
api/api-basic.c (trafo 100-244, adj 249-378) and performs the F step with
scipy.fft in place of PFFT.

Conventions (single process, 1x1x1 mesh):
  f_hat: N0 x N1 x N2 complex, k_t = i_t - N_t/2 (PNFFT_TRANSPOSED_F_HAT:
         N1 x N2 x N0); c2r plans store k2 in [-N2/2, 0] (N2/2+1 planes).
  x:     M x 3 float64 in [-0.5, 0.5).
  f:     M complex (c2c) or M real (c2r); grad_f M x 3; hessian_f M x 6
         ordered xx, xy, xz, yy, yz, zz.
"""
import ctypes
import os
import numpy as np
import scipy.fft

from . import build as _build

# plan flags, api/pnfft.h:302-334
PRE_PHI_HAT = 1 << 0
FAST_GAUSSIAN = 1 << 1
PRE_CONST_PSI = 1 << 2
PRE_LIN_PSI = 1 << 3
PRE_QUAD_PSI = 1 << 4
PRE_CUB_PSI = 1 << 5
MALLOC_F_HAT = 1 << 6
INTERLACED = 1 << 8
TRANSPOSED_F_HAT = 1 << 11
DIFF_IK = 1 << 12
WINDOW_KAISER_BESSEL = 0
WINDOW_GAUSSIAN = 1 << 13
WINDOW_BSPLINE = 1 << 14
WINDOW_SINC_POWER = 1 << 15
WINDOW_BESSEL_I0 = 1 << 16
WINDOW_GAUSSIAN_T = (1 << 17) | (1 << 13)
SORT_NODES = 1 << 18
# compute flags, api/pnfft.h:383-390
COMPUTE_F = 1 << 0
COMPUTE_GRAD_F = 1 << 1
COMPUTE_HESSIAN_F = 1 << 2
COMPUTE_DIRECT = 1 << 3
COMPUTE_ACCUMULATED = 1 << 4
OMIT_DECONV = 1 << 5
OMIT_FFT = 1 << 6
OMIT_CONV = 1 << 7

_lib = None
_I64P = ctypes.POINTER(ctypes.c_int64)
_DP = ctypes.POINTER(ctypes.c_double)
_VP = ctypes.c_void_p


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        L.or_plan_create.restype = _VP
        L.or_plan_create.argtypes = [_I64P, _I64P, ctypes.c_int, ctypes.c_uint, ctypes.c_int]
        L.or_plan_destroy.argtypes = [_VP]
        for name in ("or_psi", "or_dpsi", "or_ddpsi"):
            getattr(L, name).restype = ctypes.c_double
            getattr(L, name).argtypes = [_VP, ctypes.c_int, ctypes.c_double]
        for name in ("or_phi_hat", "or_inv_phi_hat"):
            getattr(L, name).restype = ctypes.c_double
            getattr(L, name).argtypes = [_VP, ctypes.c_int, ctypes.c_int64]
        L.or_get_b.restype = ctypes.c_double
        L.or_get_b.argtypes = [_VP, ctypes.c_int]
        L.or_set_b.argtypes = [_VP, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.or_get_flags.restype = ctypes.c_uint
        L.or_get_flags.argtypes = [_VP]
        L.or_intpol_K.restype = ctypes.c_int64
        L.or_intpol_K.argtypes = [_VP]
        L.or_intpol_order.restype = ctypes.c_int
        L.or_intpol_order.argtypes = [_VP]
        L.or_bessel_i0.restype = ctypes.c_double
        L.or_bessel_i0.argtypes = [ctypes.c_double]
        L.or_bessel_i1.restype = ctypes.c_double
        L.or_bessel_i1.argtypes = [ctypes.c_double]
        L.or_re_erf_complex.restype = ctypes.c_double
        L.or_re_erf_complex.argtypes = [ctypes.c_double, ctypes.c_double]
        L.or_bspline.restype = ctypes.c_double
        L.or_bspline.argtypes = [ctypes.c_int, ctypes.c_double]
        L.or_window_tensor.argtypes = [_VP, _DP, ctypes.c_int, _DP, _DP, _DP]
        L.or_node_index.argtypes = [_VP, ctypes.c_int64, _DP, ctypes.c_int, _I64P, _DP]
        L.or_trafo_B.argtypes = [_VP, ctypes.c_int64, _DP, _VP, _DP, _DP, _DP, ctypes.c_int64, ctypes.c_int64,
                                 ctypes.c_int, ctypes.c_int, ctypes.c_uint, ctypes.c_int]
        L.or_adjoint_B.argtypes = [_VP, ctypes.c_int64, _DP, _DP, _DP, ctypes.c_int64, ctypes.c_int64,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_uint, _VP, ctypes.c_int]
        L.or_trafo_D.argtypes = [_VP, _I64P, _I64P, _VP, ctypes.c_int, _VP]
        L.or_adjoint_D.argtypes = [_VP, _I64P, _I64P, _VP, ctypes.c_int, _VP]
        for name in ("or_trafo_scale_ik", "or_trafo_scale_ik2", "or_adjoint_scale_ik"):
            getattr(L, name).argtypes = [_VP, _I64P, _I64P, _VP, ctypes.c_int, _VP]
        L.or_ndft_trafo.argtypes = [_VP, _I64P, _I64P, ctypes.c_int64, _DP, _VP, _DP, _DP, _DP, ctypes.c_uint,
                                    ctypes.c_int]
        L.or_ndft_adj.argtypes = [_VP, _I64P, _I64P, ctypes.c_int64, _DP, _DP, _DP, ctypes.c_uint, _VP,
                                  ctypes.c_int]
        L.or_sort_nodes.argtypes = [_VP, ctypes.c_int64, _DP, _I64P]
        L.or_ndft_adj_lattice.argtypes = [ctypes.c_int64, _DP, _DP, ctypes.c_int, _I64P, ctypes.c_int, _I64P,
                                          ctypes.c_int, _I64P, _VP, ctypes.c_int]
        L.or_srand.argtypes = [ctypes.c_uint]
        L.or_init_x_3d_adv.argtypes = [_DP, _DP, _DP, ctypes.c_int64, _DP]
        L.or_init_f.argtypes = [ctypes.c_int64, _DP]
        L.or_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a, kind=_DP):
    if a is None:
        return None
    return a.ctypes.data_as(kind)


def _v(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _i64(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.int64))


class OraclePlan:
    """A 1x1x1 PNFFT plan restated on the CPU (FP64)."""

    def __init__(self, N, n=None, m=6, flags=0, c2r=False, nthreads=0):
        self.N = tuple(int(v) for v in N)
        self.n = tuple(int(v) for v in (n if n is not None else [2 * v for v in N]))
        self.m = int(m)
        self.c2r = bool(c2r)
        self.nthreads = int(nthreads)
        L = lib()
        self._h = L.or_plan_create(_p(_i64(self.N), _I64P), _p(_i64(self.n), _I64P), self.m, ctypes.c_uint(flags),
                                   int(self.c2r))
        self.flags = L.or_get_flags(self._h)
        self.cutoff = 2 * self.m + 1
        # local block of f_hat in (axis0, axis1, axis2) order
        if self.c2r:
            self.local_N = (self.N[0], self.N[1], self.N[2] // 2 + 1)
        else:
            self.local_N = self.N
        self.local_N_start = (-(self.N[0] // 2), -(self.N[1] // 2), -(self.N[2] // 2))
        self._Nl = _i64(self.local_N)
        self._ks = _i64(self.local_N_start)

    def __del__(self):
        try:
            lib().or_plan_destroy(self._h)
        except Exception:
            pass

    # --- scalar helpers ---------------------------------------------------
    @property
    def transposed(self):
        return bool(self.flags & TRANSPOSED_F_HAT)

    @property
    def fhat_shape(self):
        a, b, c = self.local_N
        return (b, c, a) if self.transposed else (a, b, c)

    def b(self):
        return tuple(lib().or_get_b(self._h, t) for t in range(3))

    def set_b(self, b0, b1, b2):
        lib().or_set_b(self._h, b0, b1, b2)

    def psi(self, dim, x):
        return lib().or_psi(self._h, dim, x)

    def dpsi(self, dim, x):
        return lib().or_dpsi(self._h, dim, x)

    def ddpsi(self, dim, x):
        return lib().or_ddpsi(self._h, dim, x)

    def phi_hat(self, dim, k):
        return lib().or_phi_hat(self._h, dim, k)

    def inv_phi_hat(self, dim, k):
        return lib().or_inv_phi_hat(self._h, dim, k)

    def window_tensor(self, xj, interlaced=0, deriv=0):
        xj = np.ascontiguousarray(xj, dtype=np.float64)
        c = self.cutoff
        psi = np.zeros(3 * c)
        d = np.zeros(3 * c) if deriv >= 1 else None
        dd = np.zeros(3 * c) if deriv >= 2 else None
        lib().or_window_tensor(self._h, _p(xj), interlaced, _p(psi), _p(d), _p(dd))
        return psi, d, dd

    def node_index(self, x, interlaced=0):
        x = np.ascontiguousarray(x, dtype=np.float64)
        M = x.shape[0]
        u = np.zeros((M, 3), dtype=np.int64)
        fnx = np.zeros((M, 3))
        lib().or_node_index(self._h, M, _p(x), interlaced, _p(u, _I64P), _p(fnx))
        return u, fnx

    def sort_nodes(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        M = x.shape[0]
        pairs = np.zeros(2 * M, dtype=np.int64)
        lib().or_sort_nodes(self._h, M, _p(x), _p(pairs, _I64P))
        return pairs.reshape(M, 2)

    # --- F: zero-pad + FFT (PFFT stand-in) --------------------------------
    def _to_cube(self, g):
        """f_hat layout -> (axis0, axis1, axis2) array."""
        if self.transposed:
            return np.ascontiguousarray(g.reshape(self.fhat_shape).transpose(2, 0, 1))
        return g.reshape(self.fhat_shape)

    def _from_cube(self, c):
        if self.transposed:
            return np.ascontiguousarray(c.transpose(1, 2, 0)).reshape(-1)
        return np.ascontiguousarray(c).reshape(-1)

    def _idx(self):
        return [(np.arange(self.local_N[t]) + self.local_N_start[t]) % self.n[t] for t in range(3)]

    def _c2r_mask(self):
        """Weights turning the stored half spectrum into the c2c spectrum whose
        real part is the c2r result: 1 at k=0 (real part only), 2 on the
        non-redundant set, 0 on is_hermitian points (ndft-parallel.c:356-374,
        564-588)."""
        k = [np.arange(self.local_N[t]) + self.local_N_start[t] for t in range(3)]
        k0, k1, k2 = np.meshgrid(*k, indexing="ij")
        N0, N1, N2 = self.N
        e0 = (k0 == 0) | (k0 == -N0 // 2)
        e1 = (k1 == 0) | (k1 == -N1 // 2)
        e2 = (k2 == 0) | (k2 == -N2 // 2)
        herm = (e0 & e1 & e2) | ((k1 > 0) & e2) | ((k0 > 0) & e1 & e2)
        w = np.where(herm, 0.0, 2.0)
        zero = (k0 == 0) & (k1 == 0) & (k2 == 0)
        return w, zero

    def forward_F(self, g1):
        cube = self._to_cube(g1)
        if self.c2r:
            w, zero = self._c2r_mask()
            cube = cube * w
            cube = np.where(zero, np.real(self._to_cube(g1)) + 0j, cube)
        grid = np.zeros(self.n, dtype=np.complex128)
        i0, i1, i2 = self._idx()
        grid[np.ix_(i0, i1, i2)] = cube
        grid = scipy.fft.fftn(grid, workers=self.nthreads if self.nthreads > 0 else -1)
        if self.c2r:
            return np.ascontiguousarray(grid.real)
        return grid

    def adjoint_F(self, grid):
        if self.c2r:
            grid = grid.astype(np.complex128)
        full = scipy.fft.ifftn(grid, norm="forward", workers=self.nthreads if self.nthreads > 0 else -1)
        i0, i1, i2 = self._idx()
        return self._from_cube(full[np.ix_(i0, i1, i2)])

    # --- D, B, B^T ---------------------------------------------------------
    def trafo_D(self, f_hat, interlaced):
        out = np.zeros(int(np.prod(self.local_N)), dtype=np.complex128)
        fh = np.ascontiguousarray(f_hat, dtype=np.complex128).reshape(-1)
        lib().or_trafo_D(self._h, _p(self._Nl, _I64P), _p(self._ks, _I64P), _v(fh), interlaced, _v(out))
        return out

    def adjoint_D(self, g1, interlaced, f_hat):
        g = np.ascontiguousarray(g1, dtype=np.complex128).copy()
        lib().or_adjoint_D(self._h, _p(self._Nl, _I64P), _p(self._ks, _I64P), _v(g), interlaced, _v(f_hat))

    def _ik(self, name, src, dim, dst):
        getattr(lib(), name)(self._h, _p(self._Nl, _I64P), _p(self._ks, _I64P), _v(src), dim, _v(dst))

    def trafo_B(self, x, grid, f=None, grad=None, hess=None, offset=0, stride=1, use_il=0, il=0, cflags=COMPUTE_F):
        grid = np.ascontiguousarray(grid)
        lib().or_trafo_B(self._h, x.shape[0], _p(x), _v(grid), _p(f), _p(grad), _p(hess), offset, stride, use_il, il,
                         ctypes.c_uint(cflags), self.nthreads)

    def adjoint_B(self, x, f=None, grad=None, offset=0, stride=1, use_il=0, il=0, cflags=COMPUTE_F):
        dt = np.float64 if self.c2r else np.complex128
        grid = np.zeros(self.n, dtype=dt)
        lib().or_adjoint_B(self._h, x.shape[0], _p(x), _p(f), _p(grad), offset, stride, use_il, il,
                           ctypes.c_uint(cflags), _v(grid), self.nthreads)
        return grid

    # --- the transforms (api/api-basic.c) -----------------------------------
    def _outs(self, M, cflags, f, grad, hess):
        dt = np.float64 if self.c2r else np.complex128
        if (cflags & COMPUTE_F) and f is None:
            f = np.zeros(M, dtype=dt)
        if (cflags & COMPUTE_GRAD_F) and grad is None:
            grad = np.zeros((M, 3), dtype=dt)
        if (cflags & COMPUTE_HESSIAN_F) and hess is None:
            hess = np.zeros((M, 6), dtype=dt)
        return f, grad, hess

    @staticmethod
    def _rv(a):
        """complex array -> float64 view (interleaved), or the real array."""
        if a is None:
            return None
        return a.view(np.float64) if np.iscomplexobj(a) else a

    def trafo(self, x, f_hat, cflags=COMPUTE_F, f=None, grad=None, hess=None):
        """pnfft_trafo, api-basic.c:199-244; returns (f, grad_f, hessian_f)."""
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        M = x.shape[0]
        f, grad, hess = self._outs(M, cflags, f, grad, hess)
        if (not cflags & COMPUTE_ACCUMULATED) and (not cflags & OMIT_CONV):  # 210-222
            for a in (f, grad, hess):
                if a is not None:
                    a[...] = 0
        fhat = np.ascontiguousarray(f_hat, dtype=np.complex128).reshape(-1)
        if cflags & COMPUTE_DIRECT:  # 224-231 -> trafo_A, which zeroes its outputs (400-414)
            for a in (f, grad, hess):
                if a is not None:
                    a[...] = 0
            lib().or_ndft_trafo(self._h, _p(self._Nl, _I64P), _p(self._ks, _I64P), M, _p(x), _v(fhat),
                                _p(self._rv(f)), _p(self._rv(grad)), _p(self._rv(hess)), ctypes.c_uint(cflags),
                                self.nthreads)
            return f, grad, hess
        passes = [(1, 0), (1, 1)] if self.flags & INTERLACED else [(0, 0)]
        for use_il, il in passes:
            self._trafo_pass(x, fhat, cflags, f, grad, hess, use_il, il)
        return f, grad, hess

    def _trafo_pass(self, x, fhat, cflags, f, grad, hess, use_il, il):
        g1 = self.trafo_D(fhat, il) if not cflags & OMIT_DECONV else np.zeros(int(np.prod(self.local_N)), complex)
        rv = self._rv
        if self.flags & DIFF_IK:  # trafo_F_and_B_ik_complex_input, 100-167
            buf = g1.copy()
            if cflags & COMPUTE_F:
                grid = self.forward_F(g1)
                if not cflags & OMIT_CONV:
                    self.trafo_B(x, grid, f=rv(f), use_il=use_il, il=il, cflags=COMPUTE_F)
            if cflags & COMPUTE_GRAD_F:
                for dim in range(3):
                    g = np.zeros_like(buf)
                    self._ik("or_trafo_scale_ik", buf, dim, g)
                    grid = self.forward_F(g)
                    self.trafo_B(x, grid, f=rv(grad), offset=dim, stride=3, use_il=use_il, il=il, cflags=COMPUTE_F)
            if cflags & COMPUTE_HESSIAN_F:
                for dim in range(6):
                    g = np.zeros_like(buf)
                    self._ik("or_trafo_scale_ik2", buf, dim, g)
                    grid = self.forward_F(g)
                    self.trafo_B(x, grid, f=rv(hess), offset=dim, stride=6, use_il=use_il, il=il, cflags=COMPUTE_F)
        else:
            grid = self.forward_F(g1)
            if not cflags & OMIT_CONV:
                self.trafo_B(x, grid, f=rv(f), grad=rv(grad), hess=rv(hess), use_il=use_il, il=il,
                             cflags=cflags & (COMPUTE_F | COMPUTE_GRAD_F | COMPUTE_HESSIAN_F))

    def adj(self, x, f=None, grad=None, cflags=COMPUTE_F, f_hat=None):
        """pnfft_adj, api-basic.c:344-378; returns f_hat (accumulated into the
        given array when COMPUTE_ACCUMULATED)."""
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        M = x.shape[0]
        size = int(np.prod(self.local_N))
        if f_hat is None:
            f_hat = np.zeros(size, dtype=np.complex128)
        else:
            f_hat = np.ascontiguousarray(f_hat, dtype=np.complex128).reshape(-1)
        if not cflags & COMPUTE_ACCUMULATED:
            f_hat[...] = 0
        dt = np.float64 if self.c2r else np.complex128
        f = None if f is None else np.ascontiguousarray(f, dtype=dt).reshape(-1)
        grad = None if grad is None else np.ascontiguousarray(grad, dtype=dt).reshape(-1, 3)
        rv = self._rv
        if cflags & COMPUTE_DIRECT:
            lib().or_ndft_adj(self._h, _p(self._Nl, _I64P), _p(self._ks, _I64P), M, _p(x), _p(rv(f)), _p(rv(grad)),
                              ctypes.c_uint(cflags), _v(f_hat), self.nthreads)
            return f_hat
        passes = [(1, 0), (1, 1)] if self.flags & INTERLACED else [(0, 0)]
        for use_il, il in passes:
            if self.flags & DIFF_IK:  # adjoint_B_and_F_ik_complex_input, 249-305
                buf = np.zeros(size, dtype=np.complex128)
                if cflags & COMPUTE_F:
                    grid = self.adjoint_B(x, f=rv(f), use_il=use_il, il=il, cflags=COMPUTE_F)
                    buf += self.adjoint_F(grid)
                if cflags & COMPUTE_GRAD_F:
                    for dim in range(3):
                        grid = self.adjoint_B(x, f=rv(grad), offset=dim, stride=3, use_il=use_il, il=il,
                                              cflags=COMPUTE_F)
                        g = self.adjoint_F(grid)
                        self._ik("or_adjoint_scale_ik", g, dim, buf)
                g1 = buf
            else:
                grid = self.adjoint_B(x, f=rv(f), grad=rv(grad), use_il=use_il, il=il,
                                      cflags=cflags & (COMPUTE_F | COMPUTE_GRAD_F))
                g1 = self.adjoint_F(grid)
            if not cflags & OMIT_DECONV:
                self.adjoint_D(g1, il, f_hat)
        return f_hat


def ndft_adj_lattice(x, f, k0, k1, k2, nthreads=0):
    """FP64 adjoint NDFT (ndft-parallel.c:617-722, c2c, f only) at the
    frequencies (k0[i0], k1[i1], k2[i2]) of a lattice, summed over all nodes;
    returns a len(k0) x len(k1) x len(k2) complex array."""
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
    f = np.ascontiguousarray(f, dtype=np.complex128).reshape(-1)
    ks = [np.ascontiguousarray(k, dtype=np.int64) for k in (k0, k1, k2)]
    out = np.zeros((len(ks[0]), len(ks[1]), len(ks[2])), dtype=np.complex128)
    lib().or_ndft_adj_lattice(x.shape[0], _p(x), _p(f.view(np.float64)), len(ks[0]), _p(ks[0], _I64P), len(ks[1]),
                              _p(ks[1], _I64P), len(ks[2]), _p(ks[2], _I64P), _v(out), nthreads)
    return out


# --- reference input generators (glibc rand) --------------------------------
def srand(seed):
    lib().or_srand(seed)


def init_x_3d_adv(lo, up, x_max, M):
    x = np.zeros((M, 3))
    lib().or_init_x_3d_adv(_p(np.asarray(lo, float)), _p(np.asarray(up, float)), _p(np.asarray(x_max, float)), M,
                           _p(x))
    return x


def init_f(M):
    d = np.zeros(2 * M)
    lib().or_init_f(M, _p(d))
    return d.view(np.complex128)


def bessel_i0(x):
    return lib().or_bessel_i0(x)


def bessel_i1(x):
    return lib().or_bessel_i1(x)


def re_erf_complex(a, y):
    return lib().or_re_erf_complex(a, y)


def bspline(p, x):
    return lib().or_bspline(p, x)


def num_threads():
    return lib().or_num_threads()
