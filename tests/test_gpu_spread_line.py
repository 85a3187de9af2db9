"""The FP32-mixed spreading of f along lines with a rotating register window.

k_spread_line_f (conv method 0, the default for the FP32-mixed adjoint of f
alone) matches the oracle within the FP32-mixed tolerance in every window,
cutoff and mode, and the spreading of method 2 (the register window that
moves by copies) on the same FP32 data within its own rounding.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WINDOWS = {
    "kaiser_bessel": 0,
    "gaussian": 1 << 13,
    "bspline": 1 << 14,
    "sinc_power": 1 << 15,
    "bessel_i0": 1 << 16,
    "gaussian_t": (1 << 17) | (1 << 13),
}


def rel(a, b):
    d = np.linalg.norm((np.asarray(a) - np.asarray(b)).ravel())
    nb = np.linalg.norm(np.asarray(b).ravel())
    return d / nb if nb > 0 else d


@pytest.fixture(scope="module")
def gpu(lib):
    if lib.device_count() == 0:
        pytest.fail("no CUDA device visible for a -m gpu test")
    return lib


@pytest.mark.parametrize("win", list(WINDOWS))
@pytest.mark.parametrize("m", [2, 3, 4, 5, 6])
def test_spread_line_all_windows_and_cutoffs(gpu, oracle, win, m):
    N = (16, 16, 16)
    rng = np.random.default_rng(300 + m)
    x = rng.uniform(-0.5, 0.5, (3000, 3))
    f = rng.standard_normal(3000) + 1j * rng.standard_normal(3000)
    p = gpu.Plan(N, m=m, flags=WINDOWS[win], precision="fp32")
    o = oracle.OraclePlan(N, m=m, flags=WINDOWS[win])
    got = p.adj(x, f)
    assert p.conv_kernel(adjoint=True) == "line"
    assert rel(got, o.adj(x, f)) < 1e-6


@pytest.mark.parametrize("case", ["interlaced", "pre_lin_psi", "pre_cub_psi", "accumulated", "c2r", "odd_grid",
                                  "small_odd_grid", "clustered", "dense_flush", "boundary_nodes", "sigma_1p5",
                                  "diff_ik"])
def test_spread_line_variants(gpu, oracle, case):
    rng = np.random.default_rng(9)
    N, n, m, flags, c2r, fh0 = (16, 16, 16), None, 6, 0, False, None
    M = 4000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    tol = 1e-6
    cflags = 1
    if case == "interlaced":
        flags = gpu.INTERLACED
    elif case == "pre_lin_psi":
        flags = gpu.PRE_LIN_PSI
    elif case == "pre_cub_psi":
        flags = gpu.PRE_CUB_PSI
    elif case == "accumulated":
        fh0 = rng.standard_normal(4096) + 1j * rng.standard_normal(4096)
        cflags |= gpu.COMPUTE_ACCUMULATED
    elif case == "c2r":
        c2r = True
    elif case == "odd_grid":
        N = (12, 18, 14)  # n = 24 x 36 x 28: n2 not a multiple of 4 (scalar commits)
    elif case == "small_odd_grid":
        N, n, m = (6, 5, 7), (10, 9, 13), 3  # windows wider than the grid; sigma < 2
        tol = 3e-6
    elif case == "clustered":
        x = np.concatenate([x[:500], 0.1 + 0.001 * rng.standard_normal((6000, 3)),
                            -0.3 + 0.0004 * rng.standard_normal((3000, 3))])
    elif case == "dense_flush":
        # thousands of nodes in one slab: the complete commit every 256 nodes
        x = np.concatenate([x[:200], np.tile([[0.1, 0.2, 0.3]], (3000, 1)) + 1e-5 * rng.standard_normal((3000, 3))])
    elif case == "boundary_nodes":
        g = np.arange(-16, 16) / 32.0
        x = np.stack(np.meshgrid(g, g[::3], g[::2], indexing="ij"), -1).reshape(-1, 3)
        x = np.concatenate([x, np.full((64, 3), -0.5), np.full((64, 3), 0.5 - 2.0 ** -40)])
    elif case == "sigma_1p5":
        # oversampling 1.5 on odd grids: D^T multiplies the FP32 rounding of
        # the grid by 1/phi_hat, large at the edge of the spectrum, and the
        # float atomics' order varies between calls: 1.3e-5 to 1.8e-5 measured
        N, n = (16, 8, 12), (24, 12, 18)
        tol = 3e-5
    elif case == "diff_ik":
        flags = gpu.DIFF_IK
    M = x.shape[0]
    f = rng.standard_normal(M) + (0 if c2r else 1j) * rng.standard_normal(M)
    p = gpu.Plan(N, n, m=m, flags=flags, c2r=c2r, precision="fp32")
    o = oracle.OraclePlan(N, n, m=m, flags=flags, c2r=c2r)
    kw = {} if fh0 is None else {"f_hat": fh0[:int(np.prod(p.local_N))].copy()}
    got = p.adj(x, f, None, cflags, **kw)
    assert p.conv_kernel(adjoint=True) == "line"
    kw = {} if fh0 is None else {"f_hat": fh0[:int(np.prod(p.local_N))].copy()}
    want = o.adj(x, f, None, cflags, **kw)
    q = gpu.Plan(N, n, m=m, flags=flags, c2r=c2r, precision="fp32")
    q.set_conv_method(2)
    kw = {} if fh0 is None else {"f_hat": fh0[:int(np.prod(p.local_N))].copy()}
    prev = q.adj(x, f, None, cflags, **kw)
    # the FP32-mixed bound, or the FP32 error of the previous kernel on the same
    # case where that is larger (constant-table windows, a dense cluster, sigma
    # 1.5), with a margin for the order of the float atomics, which varies
    # between calls
    assert rel(got, want) < max(tol, 1.5 * rel(prev, want))
    assert rel(got, prev) < max(tol, 2.5 * rel(prev, want))


def test_spread_repeatable_to_rounding(gpu):
    # the commits are float atomics: repeated calls agree to FP32 rounding
    N = (32, 32, 32)
    rng = np.random.default_rng(11)
    x = rng.uniform(-0.5, 0.5, (50000, 3))
    f = rng.standard_normal(50000) + 1j * rng.standard_normal(50000)
    p = gpu.Plan(N, m=6, precision="fp32")
    a = p.adj(x, f).copy()
    b = p.adj(x, f)
    assert rel(a, b) < 1e-6
