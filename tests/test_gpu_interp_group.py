"""The FP32-mixed interpolation of f alone: lines and groups.

By default (conv method 0) the FP32-mixed trafo with f only interpolates
along lines of tiles (k_interp_line, the transpose of the spreading); it
matches the oracle within the FP32-mixed tolerance in every window, cutoff
and mode, and repeated calls give the same bits.
Conv method 3 interpolates the nodes of one 2x2x4 block of stencil corners
in groups of up to four per warp when there are enough of them (half a
node per block or more).  Its sums are the ones of the one-node-per-warp
kernel term by term, so method 3 and method 2 (one node per warp) give the
same bits.
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


def spectrum(rng, p):
    S = int(np.prod(p.local_N))
    return rng.standard_normal(S) + 1j * rng.standard_normal(S)


def both_methods(gpu, N, x, m, flags=0, c2r=False, cflags=1, f0=None, seed=0, methods=(3, 2)):
    """trafo (f only) with the grouped kernel and with one node per warp."""
    out = []
    for method in methods:
        p = gpu.Plan(N, m=m, flags=flags, precision="fp32", c2r=c2r)
        p.set_conv_method(method)
        fh = spectrum(np.random.default_rng(seed), p)
        kw = {} if f0 is None else {"f": f0.copy()}
        out.append(p.trafo(x, fh, cflags, **kw)[0].copy())
        p.close()
    return out


@pytest.mark.parametrize("win", list(WINDOWS))
@pytest.mark.parametrize("m", [2, 3, 4, 5, 6, 7])  # m = 7: cutoff 15 is not grouped
def test_grouped_same_bits_as_per_node(gpu, win, m):
    N = (16, 16, 16)  # n = 32^3: 64 tiles, 2048 corner blocks
    x = np.random.default_rng(100 + m).uniform(-0.5, 0.5, (3000, 3))
    a, b = both_methods(gpu, N, x, m, flags=WINDOWS[win], seed=m)
    assert np.isfinite(a).all()
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("case", ["interlaced", "pre_lin_psi", "pre_cub_psi", "accumulated", "c2r", "odd_grid",
                                  "clustered", "boundary_nodes"])
def test_grouped_same_bits_variants(gpu, case):
    rng = np.random.default_rng(7)
    N, m, flags, c2r, f0 = (16, 16, 16), 6, 0, False, None
    M = 4000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    if case == "interlaced":
        flags = gpu.INTERLACED
    elif case == "pre_lin_psi":
        flags = gpu.PRE_LIN_PSI
    elif case == "pre_cub_psi":
        flags = gpu.PRE_CUB_PSI
    elif case == "accumulated":
        f0 = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    elif case == "c2r":
        c2r = True
        f0 = None
    elif case == "odd_grid":
        N = (12, 18, 14)  # n = 24 x 36 x 28: tiles that wrap
    elif case == "clustered":
        # dense clusters: sub-problems of 1024 nodes split blocks and groups
        x = np.concatenate([x[:500], 0.1 + 0.001 * rng.standard_normal((6000, 3)),
                            -0.3 + 0.0004 * rng.standard_normal((3000, 3))])
    elif case == "boundary_nodes":
        # nodes on cell boundaries and at the ends of the torus
        g = np.arange(-16, 16) / 32.0
        x = np.stack(np.meshgrid(g, g[::3], g[::2], indexing="ij"), -1).reshape(-1, 3)
        x = np.concatenate([x, np.full((64, 3), -0.5), np.full((64, 3), 0.5 - 2.0 ** -40)])
    cflags = 1 | (gpu.COMPUTE_ACCUMULATED if f0 is not None else 0)
    a, b = both_methods(gpu, N, x, m, flags=flags, c2r=c2r, cflags=cflags, f0=f0, seed=3)
    assert np.isfinite(a).all()
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("method", [0, 3], ids=["line", "group"])
@pytest.mark.parametrize("win", ["kaiser_bessel", "bessel_i0", "bspline"])
def test_grouped_and_line_vs_oracle(gpu, oracle, win, method):
    N = (16, 16, 16)
    rng = np.random.default_rng(21)
    x = rng.uniform(-0.5, 0.5, (3000, 3))
    p = gpu.Plan(N, m=6, flags=WINDOWS[win], precision="fp32")
    p.set_conv_method(method)
    o = oracle.OraclePlan(N, m=6, flags=WINDOWS[win])
    fh = spectrum(rng, p)
    assert rel(p.trafo(x, fh)[0], o.trafo(x, fh)[0]) < 1e-6
    assert p.conv_kernel() == ("line" if method == 0 else "group")


@pytest.mark.parametrize("win", list(WINDOWS))
@pytest.mark.parametrize("m", [2, 3, 4, 5, 6])
def test_line_all_windows_and_cutoffs_vs_oracle(gpu, oracle, win, m):
    N = (16, 16, 16)
    rng = np.random.default_rng(200 + m)
    x = rng.uniform(-0.5, 0.5, (3000, 3))
    p = gpu.Plan(N, m=m, flags=WINDOWS[win], precision="fp32")
    o = oracle.OraclePlan(N, m=m, flags=WINDOWS[win])
    fh = spectrum(rng, p)
    got = p.trafo(x, fh)[0]
    assert p.conv_kernel() == "line"
    assert rel(got, o.trafo(x, fh)[0]) < 1e-6
    # the same bits on every call: a node's sum does not depend on the others
    np.testing.assert_array_equal(got, p.trafo(x, fh)[0])


@pytest.mark.parametrize("case", ["interlaced", "pre_lin_psi", "pre_cub_psi", "accumulated", "c2r", "odd_grid",
                                  "small_odd_grid", "clustered", "boundary_nodes", "sigma_1p5"])
def test_line_variants_vs_oracle(gpu, oracle, case):
    rng = np.random.default_rng(8)
    N, n, m, flags, c2r, f0 = (16, 16, 16), None, 6, 0, False, None
    M = 4000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    tol = 1e-6
    if case == "interlaced":
        flags = gpu.INTERLACED
    elif case == "pre_lin_psi":
        flags = gpu.PRE_LIN_PSI
    elif case == "pre_cub_psi":
        flags = gpu.PRE_CUB_PSI
    elif case == "accumulated":
        f0 = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    elif case == "c2r":
        c2r = True
    elif case == "odd_grid":
        N = (12, 18, 14)  # n = 24 x 36 x 28: lines that wrap, n2 not a multiple of 4
    elif case == "small_odd_grid":
        N, n, m = (6, 5, 7), (10, 9, 13), 3  # regions wider than the grid; sigma < 2 amplifies FP32 rounding
        tol = 3e-6
    elif case == "clustered":
        # dense clusters: lines of more than one sub-problem
        x = np.concatenate([x[:500], 0.1 + 0.001 * rng.standard_normal((6000, 3)),
                            -0.3 + 0.0004 * rng.standard_normal((3000, 3))])
    elif case == "boundary_nodes":
        g = np.arange(-16, 16) / 32.0
        x = np.stack(np.meshgrid(g, g[::3], g[::2], indexing="ij"), -1).reshape(-1, 3)
        x = np.concatenate([x, np.full((64, 3), -0.5), np.full((64, 3), 0.5 - 2.0 ** -40)])
    elif case == "sigma_1p5":
        # sigma = 1.5: 1/phi_hat grows towards |k| = N/2, the deconvolved grid
        # values grow and the interpolation sums cancel more, which amplifies
        # the FP32 rounding of every FP32 kernel to a few 1e-6
        N, n = (16, 8, 12), (24, 12, 18)
        tol = 1e-5
    cflags = 1 | (gpu.COMPUTE_ACCUMULATED if f0 is not None else 0)
    p = gpu.Plan(N, n, m=m, flags=flags, c2r=c2r, precision="fp32")
    o = oracle.OraclePlan(N, n, m=m, flags=flags, c2r=c2r)
    fh = spectrum(rng, p)
    kw = {} if f0 is None else {"f": f0.copy()}
    got = p.trafo(x, fh, cflags, **kw)[0]
    assert p.conv_kernel() == "line"
    kw = {} if f0 is None else {"f": f0.copy()}
    want = o.trafo(x, fh, cflags, **kw)[0]
    assert rel(got, want) < tol
    # against the one-node-per-warp kernel on the same FP32 grid: only the
    # kernels' own rounding differs
    q = gpu.Plan(N, n, m=m, flags=flags, c2r=c2r, precision="fp32")
    q.set_conv_method(2)
    kw = {} if f0 is None else {"f": f0.copy()}
    per_node = q.trafo(x, fh, cflags, **kw)[0]
    assert q.conv_kernel() == "tile"
    assert rel(got, per_node) < tol


def test_grouped_kernel_runs(gpu):
    # the kernel family each call launched (pnfft_gb300_get_conv_kernel): lines
    # for f and f + gradient by default and for B^T; groups with method 3 (not
    # with too few nodes per corner block); one warp per node for method 2 and
    # for the Hessian
    N = (16, 16, 16)
    rng = np.random.default_rng(5)
    x = rng.uniform(-0.5, 0.5, (3000, 3))
    f = rng.standard_normal(3000) + 1j * rng.standard_normal(3000)

    def kernel(method, cflags, nodes=x, adjoint=False):
        p = gpu.Plan(N, m=6, precision="fp32")
        p.set_conv_method(method)
        assert p.conv_kernel() == "none"
        if adjoint:
            p.adj(nodes, f[:nodes.shape[0]])
        else:
            p.trafo(nodes, spectrum(np.random.default_rng(1), p), cflags)
        k = p.conv_kernel(adjoint)
        p.close()
        return k

    assert kernel(0, gpu.COMPUTE_F) == "line"
    assert kernel(3, gpu.COMPUTE_F) == "group"
    assert kernel(2, gpu.COMPUTE_F) == "tile"
    assert kernel(1, gpu.COMPUTE_F) == "generic"
    assert kernel(0, gpu.COMPUTE_F | gpu.COMPUTE_GRAD_F) == "line"
    assert kernel(2, gpu.COMPUTE_F | gpu.COMPUTE_GRAD_F) == "tile"
    assert kernel(0, gpu.COMPUTE_HESSIAN_F) == "tile"
    assert kernel(3, gpu.COMPUTE_F, nodes=x[:500]) == "tile"  # 500 nodes on 2048 corner blocks
    assert kernel(0, gpu.COMPUTE_F, adjoint=True) == "line"
    # FP64 plans interpolate one node per warp
    p = gpu.Plan(N, m=6)
    p.trafo(x, spectrum(np.random.default_rng(1), p))
    assert p.conv_kernel() == "tile"
    p.close()


@pytest.mark.parametrize("cflags", [1 | 2, 2], ids=["f_grad", "grad"])
@pytest.mark.parametrize("case", ["kaiser_bessel_m6", "gaussian_m2", "bspline_m4", "sinc_power_m5", "bessel_i0_m3",
                                  "interlaced", "pre_cub_psi", "c2r", "odd_grid", "clustered", "accumulated"])
def test_line_gradient_vs_oracle_and_per_node(gpu, oracle, case, cflags):
    # the FP32-mixed interpolation with the gradient along lines (k_interp_line_g)
    rng = np.random.default_rng(40)
    N, n, m, flags, c2r, acc = (16, 16, 16), None, 6, 0, False, False
    M = 3000
    x = rng.uniform(-0.5, 0.5, (M, 3))
    if "_m" in case:
        win, mm = case.rsplit("_m", 1)
        flags, m = WINDOWS[win], int(mm)
    elif case == "interlaced":
        flags = gpu.INTERLACED
    elif case == "pre_cub_psi":
        flags = gpu.PRE_CUB_PSI
    elif case == "c2r":
        c2r = True
    elif case == "odd_grid":
        N, m = (12, 18, 14), 5
    elif case == "clustered":
        x = np.concatenate([x[:500], 0.1 + 0.001 * rng.standard_normal((5000, 3))])
    elif case == "accumulated":
        acc = True
    M = x.shape[0]
    cf = cflags | (gpu.COMPUTE_ACCUMULATED if acc else 0)
    dt = np.float64 if c2r else np.complex128
    f0 = rng.standard_normal(M).astype(dt) if acc else None
    g0 = rng.standard_normal((M, 3)).astype(dt) if acc else None
    outs = []
    for method in (0, 2):
        p = gpu.Plan(N, n, m=m, flags=flags, c2r=c2r, precision="fp32")
        p.set_conv_method(method)
        fh = spectrum(np.random.default_rng(4), p)
        kw = {} if not acc else {"f": None if f0 is None or not cflags & 1 else f0.copy(), "grad": g0.copy()}
        outs.append(p.trafo(x, fh, cf, **kw))
        assert p.conv_kernel() == ("line" if method == 0 else "tile")
        p.close()
    o = oracle.OraclePlan(N, n, m=m, flags=flags, c2r=c2r)
    kw = {} if not acc else {"f": None if f0 is None or not cflags & 1 else f0.copy(), "grad": g0.copy()}
    want = o.trafo(x, fh, cf, **kw)
    for k in ((0, 1) if cflags & 1 else (1,)):
        assert rel(outs[0][k], want[k]) < 1e-6, (case, k)
        assert rel(outs[0][k], outs[1][k]) < 1e-6, (case, k)
