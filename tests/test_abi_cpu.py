"""The C ABI of libpnfft_gb300 without a GPU: the library builds and loads,
exports every entry point include/*.h declares, and its host-side plan logic
(window shape b, window values and Fourier coefficients, local sizes, flag
handling, argument parsing) agrees with the oracle.  No transform runs here;
on a machine without a GPU a transform must fail loudly (no CPU fallback)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WINDOWS = [0, 1 << 13, 1 << 14, 1 << 15, 1 << 16, (1 << 17) | (1 << 13)]


def declared_functions():
    names = set()
    for h in ("pnfft.h", "pnfft_gb300.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(pnfft_[A-Za-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return names


def test_conv_kernel_query_before_any_transform(lib):
    # no B / B^T launched yet; conv methods outside 0..3 are refused
    p = lib.Plan((8, 8, 8), m=3)
    assert p.conv_kernel() == "none" and p.conv_kernel(adjoint=True) == "none"
    with pytest.raises(lib.PnfftError):
        p.set_conv_method(4)
    p.set_conv_method(2)
    assert lib.load().pnfft_gb300_get_conv_method(p._p) == 2
    p.close()


def test_exports_every_declared_symbol(lib):
    L = lib.load()
    names = declared_functions()
    assert len(names) > 90
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing
    # and the Python binding covers the same set
    from pnfft_gb300._lib import SIGNATURES
    assert names == set(SIGNATURES), names ^ set(SIGNATURES)


@pytest.mark.parametrize("win", WINDOWS)
@pytest.mark.parametrize("m", [3, 6])
def test_window_values_match_oracle(lib, oracle, win, m):
    N, n = (16, 20, 24), (32, 40, 50)
    p = lib.Plan(N, n, m=m, flags=win)
    o = oracle.OraclePlan(N, n, m=m, flags=win)
    np.testing.assert_allclose(p.b(), o.b(), rtol=1e-15)
    rng = np.random.default_rng(m + win % 97)
    for t in range(3):
        for x in rng.uniform(-(m + 1.0) / n[t], (m + 1.0) / n[t], 25):
            for fn in ("psi", "dpsi", "ddpsi"):
                a, b = getattr(p, fn)(t, x), getattr(o, fn)(t, x)
                assert abs(a - b) <= 1e-12 * max(abs(b), 1e-3 * abs(o.psi(t, 0.0)) * n[t] ** 2), (fn, t, x, a, b)
        for k in range(-N[t] // 2, N[t] // 2):
            a, b = p.phi_hat(t, k), o.phi_hat(t, k)
            assert abs(a - b) <= 1e-13 * abs(b) + 1e-300, (k, a, b)
            a, b = p.inv_phi_hat(t, k), o.inv_phi_hat(t, k)
            assert abs(a - b) <= 1e-13 * abs(b) + 1e-300, (k, a, b)
    p.close()


def test_local_sizes_and_getters(lib):
    L = lib.load()
    N = (ctypes.c_ssize_t * 3)(16, 8, 12)
    ln, ls = (ctypes.c_ssize_t * 3)(), (ctypes.c_ssize_t * 3)()
    lo, up = (ctypes.c_double * 3)(), (ctypes.c_double * 3)()
    L.pnfft_local_size_3d(N, lib.MPI_COMM_WORLD, 0, ln, ls, lo, up)
    assert list(ln) == [16, 8, 12] and list(ls) == [-8, -4, -6]
    assert list(lo) == [-0.5] * 3 and list(up) == [0.5] * 3
    L.pnfft_local_size_3d_c2r(N, lib.MPI_COMM_WORLD, 0, ln, ls, lo, up)
    assert list(ln) == [16, 8, 7] and list(ls) == [-8, -4, -6]
    # x_max < 0.5 prunes the FFT output (api-guru.c:195-218)
    n = (ctypes.c_ssize_t * 3)(32, 16, 24)
    xm = (ctypes.c_double * 3)(0.25, 0.5, 0.1)
    L.pnfft_local_size_guru(3, N, n, xm, 3, lib.MPI_COMM_WORLD, 0, ln, ls, lo, up)
    assert list(lo) == [-0.25, -0.5, -0.1] and list(up) == [0.25, 0.5, 0.1]
    p = L.pnfft_init_guru(3, N, n, xm, 3, ctypes.c_uint(lib.MALLOC_F_HAT | lib.PRE_LIN_PSI), 0, lib.MPI_COMM_WORLD)
    assert p
    assert L.pnfft_get_d(p) == 3 and L.pnfft_get_m(p) == 3
    f = L.pnfft_get_pnfft_flags(p)
    assert f & lib.PRE_CONST_PSI and f & lib.FAST_GAUSSIAN  # api-guru.c:152-155 promotion
    got = (ctypes.c_ssize_t * 3)()
    L.pnfft_get_n(p, got)
    assert list(got) == [32, 16, 24]
    xmo = (ctypes.c_double * 3)()
    L.pnfft_get_x_max(p, xmo)
    assert list(xmo) == [0.25, 0.5, 0.1]
    assert L.pnfft_get_f_hat(p)
    L.pnfft_finalize(p, lib.FREE_F_HAT)


def test_invalid_plans_return_null(lib):
    L = lib.load()
    N = (ctypes.c_ssize_t * 3)(8, 8, 8)
    assert not L.pnfft_init_adv(2, N, 0, 0, lib.MPI_COMM_WORLD)
    assert "d != 3" in lib.last_error()
    n = (ctypes.c_ssize_t * 3)(4, 8, 8)
    xm = (ctypes.c_double * 3)(0.5, 0.5, 0.5)
    assert not L.pnfft_init_guru(3, N, n, xm, 4, 0, 0, lib.MPI_COMM_WORLD)
    np3 = (ctypes.c_int * 3)(2, 1, 1)
    out = ctypes.c_int()
    assert L.pnfft_create_procmesh(3, lib.MPI_COMM_WORLD, np3, ctypes.byref(out)) == 1
    np3 = (ctypes.c_int * 3)(1, 1, 1)
    assert L.pnfft_create_procmesh(3, lib.MPI_COMM_WORLD, np3, ctypes.byref(out)) == 0
    assert out.value == lib.MPI_COMM_WORLD
    # FP32-mixed refuses radial windows that overflow FP32 (b*m >= 80)
    n = (ctypes.c_ssize_t * 3)(64, 64, 64)
    N = (ctypes.c_ssize_t * 3)(32, 32, 32)
    assert not L.pnfft_init_guru(3, N, n, xm, 17, lib.GB300_FP32, 0, lib.MPI_COMM_WORLD)
    assert "overflows FP32" in lib.last_error()
    p = L.pnfft_init_guru(3, N, n, xm, 17, 0, 0, lib.MPI_COMM_WORLD)
    assert p and L.pnfft_gb300_set_precision(p, 1) == -1
    L.pnfft_finalize(p, 0)
    p = L.pnfft_init_guru(3, N, n, xm, 16, lib.GB300_FP32, 0, lib.MPI_COMM_WORLD)
    assert p and L.pnfft_gb300_get_precision(p) == 1
    L.pnfft_finalize(p, 0)


def test_rand_generators_match_oracle(lib, oracle):
    L = lib.load()
    libc = ctypes.CDLL(None)
    lo = (ctypes.c_double * 3)(-0.5, -0.5, -0.5)
    up = (ctypes.c_double * 3)(0.5, 0.5, 0.5)
    x = (ctypes.c_double * 30)()
    libc.srand(3)
    L.pnfft_init_x_3d(lo, up, 10, x)
    oracle.srand(3)
    xo = oracle.init_x_3d_adv([-0.5] * 3, [0.5] * 3, [0.5] * 3, 10)
    np.testing.assert_array_equal(np.array(list(x)), xo.ravel())


def test_check_init_parameters(lib):
    L = lib.load()
    args = [b"prog", b"-pnfft_N", b"8", b"10", b"12", b"-pnfft_m", b"4", b"-pnfft_window", b"1", b"-pnfft_interlaced",
            b"1", b"-pnfft_intpol", b"3", b"-pnfft_compute_hessian_f", b"0"]
    argv = (ctypes.c_char_p * len(args))(*args)
    N, n, M = (ctypes.c_ssize_t * 3)(), (ctypes.c_ssize_t * 3)(), ctypes.c_ssize_t()
    m = ctypes.c_int()
    pf, cf = ctypes.c_uint(), ctypes.c_uint()
    xm = (ctypes.c_double * 3)()
    npr = (ctypes.c_int * 3)()
    cd, dbg = ctypes.c_int(0), ctypes.c_int(0)
    L.pnfft_check_init_parameters(len(args), argv, N, n, ctypes.byref(M), ctypes.byref(m), ctypes.byref(pf),
                                  ctypes.byref(cf), xm, npr, ctypes.byref(cd), ctypes.byref(dbg))
    assert list(N) == [8, 10, 12] and list(n) == [16, 20, 24] and m.value == 4 and M.value == 960
    assert pf.value == lib.WINDOW_BSPLINE | lib.INTERLACED | lib.PRE_CUB_PSI
    assert cf.value == lib.COMPUTE_F | lib.COMPUTE_GRAD_F


def test_no_gpu_fails_loudly(lib):
    if lib.device_count() > 0:
        pytest.skip("a GPU is present")
    p = lib.Plan((8, 8, 8), m=3)
    x = np.zeros((4, 3))
    with pytest.raises(lib.PnfftError, match="no CUDA device"):
        p.trafo(x, np.zeros(512, complex))


def test_float_api_exports_and_generators(lib):
    # the single-precision instantiation pnfftf_* (api/pnfft.h:287)
    L = lib.load()
    src = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "pnfftf.h")).read(), flags=re.S)
    names = set(re.findall(r"\b(pnfftf_[A-Za-z0-9_]+)\s*\(", src))
    assert len(names) > 80
    assert not [n for n in sorted(names) if not hasattr(L, n)]
    # pnfftf_init_x_3d with R = float (api-adv.c:35-86): (float)rand()/RAND_MAX below 1,
    # then (up - lo) * t + lo in float, against the same expressions in numpy float32
    libc = ctypes.CDLL(None)
    f3 = ctypes.c_float * 3
    lo, up = f3(-0.5, -0.25, -0.5), f3(0.5, 0.25, 0.125)
    x = (ctypes.c_float * 60)()
    fn = L.pnfftf_init_x_3d
    fn.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float), ctypes.c_ssize_t,
                   ctypes.POINTER(ctypes.c_float)]
    fn.restype = None
    libc.srand(7)
    fn(lo, up, 20, x)
    libc.srand(7)
    want = []
    for _ in range(20):
        for t in range(3):
            while True:
                while True:
                    v = np.float32(libc.rand()) / np.float32(2147483647)
                    if v < np.float32(1.0):
                        break
                v = (np.float32(up[t]) - np.float32(lo[t])) * v + np.float32(lo[t])
                if not (v < -np.float32(0.5) or np.float32(0.5) <= v):
                    break
            want.append(v)
    np.testing.assert_array_equal(np.array(list(x), dtype=np.float32), np.array(want, dtype=np.float32))
    # pnfftf_init_f: 100.0 * (float)rand() / RAND_MAX in double, rounded to float
    f = (ctypes.c_float * 20)()
    L.pnfftf_init_f.argtypes = [ctypes.c_ssize_t, ctypes.c_void_p]
    L.pnfftf_init_f.restype = None
    libc.srand(8)
    L.pnfftf_init_f(10, f)
    libc.srand(8)
    want = [np.float32(100.0 * float(np.float32(libc.rand())) / 2147483647) for _ in range(20)]
    np.testing.assert_array_equal(np.array(list(f), dtype=np.float32), np.array(want, dtype=np.float32))
    # plan getters and window values agree with the double plan
    N = (ctypes.c_ssize_t * 3)(8, 10, 12)
    n = (ctypes.c_ssize_t * 3)(16, 20, 24)
    L.pnfftf_init_guru.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                   ctypes.c_uint, ctypes.c_uint, ctypes.c_int]
    L.pnfftf_init_guru.restype = ctypes.c_void_p
    p = L.pnfftf_init_guru(3, N, n, f3(0.5, 0.5, 0.5), 4, lib.MALLOC_F_HAT, lib.PFFT_ESTIMATE, lib.MPI_COMM_WORLD)
    assert p
    for name in ("pnfftf_get_m", "pnfftf_get_d"):
        getattr(L, name).argtypes = [ctypes.c_void_p]
    assert L.pnfftf_get_m(p) == 4 and L.pnfftf_get_d(p) == 3
    L.pnfftf_gb300_double_plan.argtypes = [ctypes.c_void_p]
    L.pnfftf_gb300_double_plan.restype = ctypes.c_void_p
    dp = L.pnfftf_gb300_double_plan(p)
    assert L.pnfft_gb300_get_precision(dp) == lib.GB300_FP32_MIXED
    L.pnfftf_psi.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_float]
    L.pnfftf_psi.restype = ctypes.c_float
    for xv in (0.0, 0.03, -0.07):
        assert L.pnfftf_psi(p, 1, xv) == np.float32(L.pnfft_psi(dp, 1, float(np.float32(xv))))
    L.pnfftf_finalize.argtypes = [ctypes.c_void_p, ctypes.c_uint]
    L.pnfftf_finalize(p, lib.FREE_F_HAT)


def test_batch_and_tuning_host_logic(lib):
    """pnfft_gb300_batch_begin / _end and the tuning setters without a GPU:
    a batch cannot be opened twice or closed unopened, an empty batch closes
    with no deferred calls, and invalid tunings are refused."""
    L = lib.load()
    L.pnfft_gb300_clear_error()
    assert L.pnfft_gb300_batch_end() != 0  # nothing open
    L.pnfft_gb300_clear_error()
    assert L.pnfft_gb300_batch_begin(None) != 0  # a stream is required
    L.pnfft_gb300_clear_error()
    assert L.pnfft_gb300_batch_begin(0x1) == 0
    assert L.pnfft_gb300_batch_begin(0x1) != 0  # already open
    L.pnfft_gb300_clear_error()
    assert L.pnfft_gb300_batch_end() == 0
    d, n = ctypes.c_int(-1), ctypes.c_int(-1)
    assert L.pnfft_gb300_batch_stats(ctypes.byref(d), ctypes.byref(n)) == 0
    assert (d.value, n.value) == (0, 0)
    p = lib.Plan((8, 8, 8), m=3, precision="fp32")
    assert p.tuning() == (0, 0, 512)
    p.set_tuning((2, 0, 256))
    assert p.tuning() == (2, 0, 256)
    for bad in [(4, 0, 512), (0, -1, 512), (0, 0, 48), (0, 0, 8192)]:
        with pytest.raises(lib.PnfftError):
            p.set_tuning(bad)
    assert p.tuning() == (2, 0, 256)
    p.close()
