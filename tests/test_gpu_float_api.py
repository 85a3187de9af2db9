"""The single-precision API pnfftf_* through the C ABI on float host arrays:
trafo (f, grad) and adj against the FP64 oracle at FP32 accuracy, the c2r
form, and COMPUTE_ACCUMULATED on float outputs."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

P, U, I, S = ctypes.c_void_p, ctypes.c_uint, ctypes.c_int, ctypes.c_ssize_t


def _bind(L):
    sig = {"pnfftf_init_guru": (P, [I, P, P, P, I, U, U, I]), "pnfftf_init_guru_c2r": (P, [I, P, P, P, I, U, U, I]),
           "pnfftf_init_nodes": (P, [S, U]), "pnfftf_get_x": (P, [P]), "pnfftf_get_f": (P, [P]),
           "pnfftf_get_grad_f": (P, [P]), "pnfftf_get_f_hat": (P, [P]), "pnfftf_trafo": (None, [P, P, U]),
           "pnfftf_adj": (None, [P, P, U]), "pnfftf_finalize": (None, [P, U]), "pnfftf_free_nodes": (None, [P, U])}
    for k, (r, a) in sig.items():
        getattr(L, k).restype = r
        getattr(L, k).argtypes = a


def _view(ptr, n):
    return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_float)), (n,))


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("c2r", [False, True])
def test_float_api_trafo_adj(lib, oracle, c2r):
    if lib.device_count() == 0:
        pytest.fail("no CUDA device visible for a -m gpu test")
    L = lib.load()
    _bind(L)
    rng = np.random.default_rng(71)
    N, M, m = (16, 16, 16), 1500, 6
    Nc = (ctypes.c_ssize_t * 3)(*N)
    nc = (ctypes.c_ssize_t * 3)(*[2 * v for v in N])
    xm = (ctypes.c_float * 3)(0.5, 0.5, 0.5)
    init = L.pnfftf_init_guru_c2r if c2r else L.pnfftf_init_guru
    p = init(3, Nc, nc, xm, m, lib.MALLOC_F_HAT, lib.PFFT_ESTIMATE, lib.MPI_COMM_WORLD)
    nd = L.pnfftf_init_nodes(M, lib.MALLOC_X | lib.MALLOC_F | lib.MALLOC_GRAD_F)
    o = oracle.OraclePlan(N, m=m, c2r=c2r)
    nfh = int(np.prod(o.local_N))
    tu = 1 if c2r else 2
    x = rng.uniform(-0.5, 0.5, (M, 3)).astype(np.float32)
    _view(L.pnfftf_get_x(nd), 3 * M)[:] = x.ravel()
    fh = (rng.standard_normal(nfh) + 1j * rng.standard_normal(nfh)).astype(np.complex64)
    _view(L.pnfftf_get_f_hat(p), 2 * nfh)[:] = fh.view(np.float32)
    L.pnfftf_trafo(p, nd, lib.COMPUTE_F | lib.COMPUTE_GRAD_F)
    f = _view(L.pnfftf_get_f(nd), tu * M).copy()
    g = _view(L.pnfftf_get_grad_f(nd), 3 * tu * M).copy()
    x64 = x.astype(np.float64)
    wf, wg, _ = o.trafo(x64, fh.astype(np.complex128), lib.COMPUTE_F | lib.COMPUTE_GRAD_F)
    if c2r:
        assert _rel(f, wf) < 1e-6 and _rel(g, wg.ravel()) < 1e-6
    else:
        assert _rel(f.view(np.complex64), wf) < 1e-6 and _rel(g.view(np.complex64), wg.ravel()) < 1e-6
    # accumulated trafo adds to the float outputs
    L.pnfftf_trafo(p, nd, lib.COMPUTE_F | lib.COMPUTE_ACCUMULATED)
    f2 = _view(L.pnfftf_get_f(nd), tu * M).copy()
    assert _rel(f2, 2 * f) < 1e-6
    # adj of real or complex f
    fv = rng.standard_normal(M).astype(np.float32) if c2r else \
        (rng.standard_normal(M) + 1j * rng.standard_normal(M)).astype(np.complex64)
    _view(L.pnfftf_get_f(nd), tu * M)[:] = fv.view(np.float32)
    L.pnfftf_adj(p, nd, lib.COMPUTE_F)
    a = _view(L.pnfftf_get_f_hat(p), 2 * nfh).copy().view(np.complex64)
    wa = o.adj(x64, fv.astype(np.float64 if c2r else np.complex128))
    assert _rel(a, wa) < 1e-6
    L.pnfftf_free_nodes(nd, lib.FREE_X | lib.FREE_F | lib.FREE_GRAD_F)
    L.pnfftf_finalize(p, lib.FREE_F_HAT)


def test_float_api_hessian_grad_adj_fixed_nodes(lib, oracle):
    """Hessian output, the adjoint of gradient inputs accumulated onto f_hat,
    fixed nodes (pnfftf_precompute_psi) whose x array is then replaced by
    pnfftf_set_x (the binning must follow the new array), and M = 0."""
    if lib.device_count() == 0:
        pytest.fail("no CUDA device visible for a -m gpu test")
    L = lib.load()
    _bind(L)
    L.pnfftf_precompute_psi.argtypes = [P, P, U]
    L.pnfftf_set_x.argtypes = [P, P]
    L.pnfftf_get_hessian_f.restype = P
    L.pnfftf_get_hessian_f.argtypes = [P]
    rng = np.random.default_rng(72)
    N, M, m = (16, 16, 16), 2000, 5
    Nc = (ctypes.c_ssize_t * 3)(*N)
    nc = (ctypes.c_ssize_t * 3)(*[2 * v for v in N])
    xm = (ctypes.c_float * 3)(0.5, 0.5, 0.5)
    p = L.pnfftf_init_guru(3, Nc, nc, xm, m, lib.MALLOC_F_HAT, lib.PFFT_ESTIMATE, lib.MPI_COMM_WORLD)
    nd = L.pnfftf_init_nodes(M, lib.MALLOC_X | lib.MALLOC_F | lib.MALLOC_GRAD_F | lib.MALLOC_HESSIAN_F)
    o = oracle.OraclePlan(N, m=m)
    nfh = int(np.prod(N))
    x = rng.uniform(-0.5, 0.5, (M, 3)).astype(np.float32)
    _view(L.pnfftf_get_x(nd), 3 * M)[:] = x.ravel()
    L.pnfftf_precompute_psi(p, nd, 1 << 1)  # PNFFT_PRE_PSI
    fh = (rng.standard_normal(nfh) + 1j * rng.standard_normal(nfh)).astype(np.complex64)
    _view(L.pnfftf_get_f_hat(p), 2 * nfh)[:] = fh.view(np.float32)
    flags = lib.COMPUTE_GRAD_F | lib.COMPUTE_HESSIAN_F
    L.pnfftf_trafo(p, nd, flags)
    g = _view(L.pnfftf_get_grad_f(nd), 6 * M).copy().view(np.complex64)
    h = _view(L.pnfftf_get_hessian_f(nd), 12 * M).copy().view(np.complex64)
    _, wg, wh = o.trafo(x.astype(np.float64), fh.astype(np.complex128), flags)
    assert _rel(g, wg.ravel()) < 1e-6 and _rel(h, wh.ravel()) < 1e-6
    # adjoint of f, then of grad inputs accumulated
    fv = (rng.standard_normal(M) + 1j * rng.standard_normal(M)).astype(np.complex64)
    gv = (rng.standard_normal((M, 3)) + 1j * rng.standard_normal((M, 3))).astype(np.complex64)
    _view(L.pnfftf_get_f(nd), 2 * M)[:] = fv.view(np.float32)
    _view(L.pnfftf_get_grad_f(nd), 6 * M)[:] = gv.view(np.float32).ravel()
    L.pnfftf_adj(p, nd, lib.COMPUTE_F)
    L.pnfftf_adj(p, nd, lib.COMPUTE_GRAD_F | lib.COMPUTE_ACCUMULATED)
    a = _view(L.pnfftf_get_f_hat(p), 2 * nfh).copy().view(np.complex64)
    x64 = x.astype(np.float64)
    wa = o.adj(x64, fv.astype(np.complex128)) + o.adj(x64, None, gv.astype(np.complex128), lib.COMPUTE_GRAD_F)
    assert _rel(a, wa.ravel()) < 1e-6
    # a new x array on the fixed nodes: the transform follows it
    x2 = np.ascontiguousarray(rng.uniform(-0.5, 0.5, (M, 3)).astype(np.float32))
    L.pnfftf_set_x(x2.ctypes.data, nd)
    _view(L.pnfftf_get_f_hat(p), 2 * nfh)[:] = fh.view(np.float32)
    L.pnfftf_trafo(p, nd, lib.COMPUTE_F)
    f = _view(L.pnfftf_get_f(nd), 2 * M).copy().view(np.complex64)
    wf, _, _ = o.trafo(x2.astype(np.float64), fh.astype(np.complex128), lib.COMPUTE_F)
    assert _rel(f, wf) < 1e-6
    L.pnfftf_set_x(None, nd)
    L.pnfftf_free_nodes(nd, lib.FREE_F | lib.FREE_GRAD_F | lib.FREE_HESSIAN_F)
    # M = 0: nothing to do, f_hat of the adjoint is zero
    n0 = L.pnfftf_init_nodes(0, lib.MALLOC_X | lib.MALLOC_F)
    L.pnfftf_adj(p, n0, lib.COMPUTE_F)
    assert not np.any(_view(L.pnfftf_get_f_hat(p), 2 * nfh))
    L.pnfftf_free_nodes(n0, lib.FREE_X | lib.FREE_F)
    L.pnfftf_finalize(p, lib.FREE_F_HAT)
