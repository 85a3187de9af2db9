"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

FP64: every transform variant agrees with the oracle's restatement of the
reference on the same inputs to 1e-12 relative l2 (the FP64 bar); node
indices and the PNFFT_SORT_NODES permutation are bit-exact.
FP32-mixed: within 1e-6 relative l2 of the FP64 NDFT at m = 6 (FP32_TOL, the
bar of the FP32-mixed form for f, grad_f and the adjoint); Hessians, which
are outside that bar, within 5e-6 of the FP64 oracle.
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
FP64_TOL = 1e-12
FP32_TOL = 1e-6


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    d = np.linalg.norm((a - b).ravel())
    nb = np.linalg.norm(b.ravel())
    return d / nb if nb > 0 else d


def case(N, M, seed, c2r=False, local_N=None):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-0.5, 0.5, (M, 3))
    size = int(np.prod(local_N or N))
    fh = rng.standard_normal(size) + 1j * rng.standard_normal(size)
    if c2r:
        f = rng.standard_normal(M)
        g = rng.standard_normal((M, 3))
    else:
        f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
        g = rng.standard_normal((M, 3)) + 1j * rng.standard_normal((M, 3))
    return x, fh, f, g


@pytest.fixture(scope="module")
def gpu(lib):
    if lib.device_count() == 0:
        pytest.fail("no CUDA device visible for a -m gpu test")
    return lib


CF_ALL = 1 | 2 | 4


@pytest.mark.parametrize("win", list(WINDOWS))
def test_fp64_all_windows(gpu, oracle, win):
    N, M = (16, 12, 20), 700
    x, fh, f, g = case(N, M, 1)
    p = gpu.Plan(N, m=4, flags=WINDOWS[win])
    o = oracle.OraclePlan(N, m=4, flags=WINDOWS[win])
    a = p.trafo(x, fh, CF_ALL)
    b = o.trafo(x, fh, CF_ALL)
    for u, v in zip(a, b):
        assert rel(u, v) < FP64_TOL
    fa = p.adj(x, f, g, 1 | 2)
    fb = o.adj(x, f, g, 1 | 2)
    assert rel(fa, fb) < FP64_TOL


@pytest.mark.parametrize("mode", ["plain_m6", "interlaced", "diff_ik", "cub", "const", "quad_real_only",
                                  "transposed", "sigma_1p5", "ik_interlaced", "fast_gaussian"])
def test_fp64_modes(gpu, oracle, mode):
    N, m, n = (16, 16, 16), 6, None
    flags = {"plain_m6": 0, "interlaced": gpu.INTERLACED, "diff_ik": gpu.DIFF_IK, "cub": gpu.PRE_CUB_PSI,
             "const": gpu.PRE_CONST_PSI, "quad_real_only": gpu.PRE_QUAD_PSI, "transposed": gpu.TRANSPOSED_F_HAT,
             "sigma_1p5": 0, "ik_interlaced": gpu.DIFF_IK | gpu.INTERLACED,
             "fast_gaussian": gpu.WINDOW_GAUSSIAN | gpu.FAST_GAUSSIAN}[mode]
    if mode == "sigma_1p5":
        N, n = (16, 8, 12), (24, 12, 18)
    x, fh, f, g = case(N, 500, 2)
    p = gpu.Plan(N, n, m=m, flags=flags)
    o = oracle.OraclePlan(N, n, m=m, flags=flags)
    a = p.trafo(x, fh, CF_ALL)
    b = o.trafo(x, fh, CF_ALL)
    for u, v in zip(a, b):
        assert rel(u, v) < FP64_TOL, mode
    fa = p.adj(x, f, g, 1 | 2)
    fb = o.adj(x, f, g, 1 | 2)
    assert rel(fa, fb) < FP64_TOL


@pytest.mark.parametrize("m", [1, 2, 3, 5, 7, 8, 10])
def test_fp64_cutoffs(gpu, oracle, m):
    N = (8, 8, 12)
    x, fh, f, g = case(N, 300, 3)
    p = gpu.Plan(N, m=m)
    o = oracle.OraclePlan(N, m=m)
    a = p.trafo(x, fh, 1 | 2)
    b = o.trafo(x, fh, 1 | 2)
    assert rel(a[0], b[0]) < FP64_TOL and rel(a[1], b[1]) < FP64_TOL
    assert rel(p.adj(x, f, g, 1 | 2), o.adj(x, f, g, 1 | 2)) < FP64_TOL


@pytest.mark.parametrize("n,m", [((13, 11, 15), 3), ((18, 10, 21), 5), ((9, 12, 7), 2), ((40, 36, 66), 7)])
def test_odd_and_wrapping_grids(gpu, oracle, n, m):
    # odd n2 (scalar commits), n not a multiple of the tile edge, and regions
    # that wrap over grids smaller than the stencil region.  These plans
    # oversample by as little as sigma = n/N = 1 (n = 7, 10 and 9 against N = 7
    # and 8), where 1/phi_hat grows large towards |k| = N/2 and amplifies the
    # FP32 rounding of the grid: the FP32 bound is 3e-6 here
    N = tuple(min(v, 8) for v in n)
    x, fh, f, g = case(N, 700, 4)
    o = oracle.OraclePlan(N, n, m=m)
    want_t = o.trafo(x, fh, 1 | 2)
    want_a = o.adj(x, f, g, 1 | 2)
    for prec, tol in (("fp64", FP64_TOL), ("fp32", 3e-6)):
        p = gpu.Plan(N, n, m=m, precision=prec)
        got_t = p.trafo(x, fh, 1 | 2)
        assert rel(got_t[0], want_t[0]) < tol and rel(got_t[1], want_t[1]) < tol, prec
        assert rel(p.adj(x, f, g, 1 | 2), want_a) < tol, prec


@pytest.mark.parametrize("win", ["kaiser_bessel", "gaussian", "bspline"])
def test_fp64_c2r(gpu, oracle, win):
    N = (8, 12, 16)
    p = gpu.Plan(N, m=5, flags=WINDOWS[win], c2r=True)
    o = oracle.OraclePlan(N, m=5, flags=WINDOWS[win], c2r=True)
    x, fh, f, g = case(N, 400, 4, c2r=True, local_N=p.local_N)
    a = p.trafo(x, fh, CF_ALL)
    b = o.trafo(x, fh, CF_ALL)
    for u, v in zip(a, b):
        assert rel(u, v) < FP64_TOL
    assert rel(p.adj(x, f, g, 1 | 2), o.adj(x, f, g, 1 | 2)) < FP64_TOL


def test_direct_ndft_on_gpu(gpu, oracle):
    N = (8, 10, 12)
    x, fh, f, g = case(N, 200, 5)
    for flags in (0, gpu.TRANSPOSED_F_HAT):
        p = gpu.Plan(N, m=3, flags=flags)
        o = oracle.OraclePlan(N, m=3, flags=flags)
        a = p.trafo(x, fh, CF_ALL | gpu.COMPUTE_DIRECT)
        b = o.trafo(x, fh, CF_ALL | gpu.COMPUTE_DIRECT)
        for u, v in zip(a, b):
            assert rel(u, v) < 1e-12
        assert rel(p.adj(x, f, g, 3 | gpu.COMPUTE_DIRECT), o.adj(x, f, g, 3 | gpu.COMPUTE_DIRECT)) < 1e-12
    pr = gpu.Plan(N, m=3, c2r=True)
    orr = oracle.OraclePlan(N, m=3, c2r=True)
    x, fh, f, g = case(N, 200, 6, c2r=True, local_N=pr.local_N)
    a = pr.trafo(x, fh, CF_ALL | gpu.COMPUTE_DIRECT)
    b = orr.trafo(x, fh, CF_ALL | gpu.COMPUTE_DIRECT)
    for u, v in zip(a, b):
        assert rel(u, v) < 1e-12


def test_check_vs_pfft_identity_gpu(gpu):
    N = (16, 16, 16)
    k = [np.arange(-n // 2, n // 2) for n in N]
    K0, K1, K2 = np.meshgrid(*k, indexing="ij")
    x = np.stack([K0.ravel() / N[0], K1.ravel() / N[1], K2.ravel() / N[2]], 1)
    g = np.arange(int(np.prod(N)))
    fh = 1000.0 / (2 * g + 1) + 1j * 1000.0 / (2 * g + 2)
    for prec, tol in (("fp64", 1e-10), ("fp32", 1e-6)):
        p = gpu.Plan(N, m=6, precision=prec)
        f, _, _ = p.trafo(x, fh)
        back = p.adj(x, f) / np.prod(N)
        assert np.abs(back - fh).max() / np.abs(fh).sum() < tol, prec


def test_node_index_and_sort_bitexact(gpu, oracle):
    rng = np.random.default_rng(9)
    N, n, m = (16, 16, 16), (32, 48, 40), 4
    x = rng.uniform(-0.5, 0.5, (20000, 3))
    # edge nodes: the interval ends, grid points, one ulp around grid points
    edge = np.array([-0.5, 0.0, 0.5 - 2 ** -53, 1 / 32, -1 / 32, 15 / 32, -15 / 32, 3 / 48, 7 / 40])
    edge = np.concatenate([edge, np.nextafter(edge, 1), np.nextafter(edge, -1)])
    edge = edge[(edge >= -0.5) & (edge < 0.5)]
    x[: edge.size * 3].reshape(-1, 3)[:] = 0
    for t in range(3):
        x[t * edge.size:(t + 1) * edge.size, t] = edge
    x[5000:6000] = x[17]
    p = gpu.Plan(N, n, m=m)
    p32 = gpu.Plan(N, n, m=m, precision="fp32")  # integer-only index path
    o = oracle.OraclePlan(N, n, m=m)
    for il in (0, 1):
        want = o.node_index(x, il)[0]
        np.testing.assert_array_equal(p.node_index(x, il), want)
        np.testing.assert_array_equal(p32.node_index(x, il), want)
    # wider coverage of the integer path: many magnitudes, odd grid sizes
    rng2 = np.random.default_rng(10)
    xs = np.concatenate([rng2.uniform(-0.5, 0.5, (4000, 3)),
                         (rng2.uniform(-1, 1, (2000, 3)) * 10.0 ** rng2.integers(-12, 0, (2000, 3))) % 1 - 0.5,
                         rng2.uniform(-1, 1, (2000, 3)) * 10.0 ** rng2.integers(-300, 0, (2000, 3))])
    for nn in [(17, 1023, 1000), (96, 129, 2048)]:
        a = gpu.Plan((8, 8, 8), nn, m=3, precision="fp32")
        np.testing.assert_array_equal(a.node_index(xs), oracle.OraclePlan((8, 8, 8), nn, m=3).node_index(xs)[0])
    np.testing.assert_array_equal(p.sort_nodes(x), o.sort_nodes(x))


def test_fp32_mixed_vs_ndft(gpu, oracle):
    N = (32, 32, 32)
    M = 4096
    rng = np.random.default_rng(12)
    x = rng.uniform(-0.5, 0.5, (M, 3))
    k = [np.arange(-n // 2, n // 2) for n in N]
    K = np.stack(np.meshgrid(*k, indexing="ij"), -1).reshape(-1, 3)
    fh = (rng.standard_normal(K.shape[0]) + 1j * rng.standard_normal(K.shape[0])) / (1 + (K ** 2).sum(1))
    p = gpu.Plan(N, m=6, precision="fp32")
    o = oracle.OraclePlan(N, m=6)
    sub = slice(0, 512)
    f, g, _ = p.trafo(x, fh, 1 | 2)
    fd, gd, _ = o.trafo(x[sub], fh, 1 | 2 | gpu.COMPUTE_DIRECT)
    assert rel(f[sub], fd) < FP32_TOL
    assert rel(g[sub], gd) < FP32_TOL
    fv = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    a = p.adj(x, fv)
    ad = o.adj(x, fv, None, 1 | gpu.COMPUTE_DIRECT)
    assert rel(a, ad) < FP32_TOL


def test_fp32_tiny_and_edge_coordinates(gpu, oracle):
    # coordinates whose product n*x lies below 2^-11 (the whole product is
    # fraction), signed zeros, subnormals and the ends of [-0.5, 0.5)
    N = (16, 16, 16)
    rng = np.random.default_rng(33)
    special = np.array([0.0, -0.0, 1.03e-5, -1.03e-5, 3e-9, -3e-9, 1e-300, -1e-300, 5e-324, -5e-324,
                        -0.5, 0.5 - 2.0 ** -53, 2.0 ** -16, -2.0 ** -16])
    x = rng.uniform(-0.5, 0.5, (3 * special.size, 3))
    for t in range(3):
        x[t * special.size:(t + 1) * special.size, t] = special
    fh = rng.standard_normal(4096) + 1j * rng.standard_normal(4096)
    f = rng.standard_normal(x.shape[0]) + 1j * rng.standard_normal(x.shape[0])
    p = gpu.Plan(N, m=6, precision="fp32")
    o = oracle.OraclePlan(N, m=6)
    got, want = p.trafo(x, fh)[0], o.trafo(x, fh)[0]
    assert np.abs(got - want).max() <= FP32_TOL * np.abs(want).max()
    assert rel(p.adj(x, f), o.adj(x, f)) < FP32_TOL


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("fp32", FP32_TOL)])
def test_coordinates_outside_the_unit_cell(gpu, oracle, prec, tol):
    # the transform is periodic: nodes shifted by whole periods (up to 1e4,
    # where the grid index leaves the one-period range of the wrap and takes
    # the general remainder) give the results of the same nodes in
    # [-0.5, 0.5); the tolerance covers the rounding of x + k in FP64
    N = (16, 16, 16)
    rng = np.random.default_rng(35)
    x0 = rng.uniform(-0.5, 0.5, (1200, 3))
    k = rng.choice(np.array([-10000, -7, -2, -1, 0, 1, 2, 3, 9999]), size=x0.shape)
    x = x0 + k
    xw = x - np.floor(x + 0.5)  # the same points wrapped, after the rounding of x0 + k
    fh = rng.standard_normal(4096) + 1j * rng.standard_normal(4096)
    f = rng.standard_normal(x.shape[0]) + 1j * rng.standard_normal(x.shape[0])
    p = gpu.Plan(N, m=5, precision=prec)
    o = oracle.OraclePlan(N, m=5)
    assert rel(p.trafo(x, fh)[0], o.trafo(xw, fh)[0]) < tol
    assert rel(p.adj(x, f), o.adj(xw, f)) < tol


@pytest.mark.parametrize("win", list(WINDOWS))
def test_fp32_mixed_all_windows_vs_fp64_oracle(gpu, oracle, win):
    # the FP32 windows are evaluated with a compensated argument; against the
    # same algorithm in FP64 every output stays within a few FP32 ulps
    N = (16, 16, 16)
    x, fh, f, g = case(N, 2000, 31)
    p = gpu.Plan(N, m=6, flags=WINDOWS[win], precision="fp32")
    o = oracle.OraclePlan(N, m=6, flags=WINDOWS[win])
    got = p.trafo(x, fh, CF_ALL)
    want = o.trafo(x, fh, CF_ALL)
    for a, b, tol in zip(got, want, (FP32_TOL, FP32_TOL, 5e-6)):
        assert rel(a, b) < tol, (win, rel(a, b))
    assert rel(p.adj(x, f, g, 1 | 2), o.adj(x, f, g, 1 | 2)) < FP32_TOL


def test_accumulated_and_empty(gpu, oracle):
    N = (8, 8, 8)
    x, fh, f, g = case(N, 100, 13)
    p = gpu.Plan(N, m=3)
    o = oracle.OraclePlan(N, m=3)
    f0 = np.arange(100) * (1 + 1j)
    fa, _, _ = p.trafo(x, fh, 1 | gpu.COMPUTE_ACCUMULATED, f=f0.copy())
    fb, _, _ = o.trafo(x, fh, 1 | gpu.COMPUTE_ACCUMULATED, f=f0.copy())
    assert rel(fa, fb) < FP64_TOL
    fh0 = np.ones(512, complex)
    a = p.adj(x, f, None, 1 | gpu.COMPUTE_ACCUMULATED, f_hat=fh0.copy())
    b = o.adj(x, f, None, 1 | gpu.COMPUTE_ACCUMULATED, f_hat=fh0.copy())
    assert rel(a, b) < FP64_TOL
    # no nodes: trafo returns nothing, adj returns zeros
    e = np.zeros((0, 3))
    fe, _, _ = p.trafo(e, fh)
    assert fe.size == 0
    assert np.abs(p.adj(e, np.zeros(0, complex))).max() == 0.0


def test_clustered_nodes_large_bins(gpu, oracle):
    # many nodes in one grid tile exercise the sub-problem split of the binning
    N = (16, 16, 16)
    rng = np.random.default_rng(14)
    x = np.concatenate([rng.uniform(-0.5, 0.5, (500, 3)), 0.2 + 0.002 * rng.standard_normal((5000, 3))])
    fh = rng.standard_normal(4096) + 1j * rng.standard_normal(4096)
    f = rng.standard_normal(x.shape[0]) + 0j
    for prec, tol in (("fp64", FP64_TOL), ("fp32", FP32_TOL)):
        p = gpu.Plan(N, m=5, precision=prec)
        o = oracle.OraclePlan(N, m=5)
        assert rel(p.trafo(x, fh)[0], o.trafo(x, fh)[0]) < tol
        assert rel(p.adj(x, f), o.adj(x, f)) < tol


def test_zero_copy_device_api_matches_host(gpu):
    torch = pytest.importorskip("torch")
    N = (16, 16, 16)
    x, fh, f, g = case(N, 1000, 15)
    p = gpu.Plan(N, m=6, precision="fp32")
    fa, ga, _ = p.trafo(x, fh, 1 | 2)
    aa = p.adj(x, f, None, 1)
    q = gpu.Plan(N, m=6, precision="fp32")
    xd = torch.tensor(x, device="cuda")
    fhd = torch.tensor(fh, device="cuda")
    fd, gd, _ = q.trafo_device(xd, fhd, 1 | 2)
    ad = q.adj_device(xd, torch.tensor(f, device="cuda"))
    torch.cuda.synchronize()
    assert rel(fd.cpu().numpy(), fa) < 1e-6
    assert rel(gd.cpu().numpy(), ga) < 1e-6
    assert rel(ad.cpu().numpy(), aa) < 1e-6


def test_fixed_nodes_reuse_device_coordinates(gpu, oracle):
    # with fixed nodes the device copy of x and the binning are reused across
    # host-array calls; a new x array (pnfft_set_x with another pointer) or
    # releasing the promise brings the new coordinates in
    N = (16, 16, 16)
    x, fh, f, g = case(N, 800, 17)
    L = gpu.load()
    p = gpu.Plan(N, m=5, precision="fp32")
    o = oracle.OraclePlan(N, m=5)
    nd = p._nodes_for(x.shape[0])
    L.pnfft_gb300_nodes_set_fixed(nd, 1)
    a1 = p.trafo(x, fh)[0].copy()
    a2 = p.trafo(x, fh)[0].copy()
    np.testing.assert_array_equal(a1, a2)
    assert rel(a1, o.trafo(x, fh)[0]) < FP32_TOL
    x2 = np.ascontiguousarray(np.roll(x, 1, axis=0))  # another array: pnfft_set_x sees a new pointer
    b = p.trafo(x2, fh)[0]
    assert rel(b, o.trafo(x2, fh)[0]) < FP32_TOL
    L.pnfft_gb300_nodes_set_fixed(nd, 0)
    assert rel(p.adj(x, f), o.adj(x, f)) < FP32_TOL


@pytest.mark.parametrize("flags", ["interlaced", "diff_ik", "interlaced_ik", "transposed_interlaced"])
def test_c2r_mode_combinations(gpu, oracle, flags):
    fl = {"interlaced": gpu.INTERLACED, "diff_ik": gpu.DIFF_IK, "interlaced_ik": gpu.INTERLACED | gpu.DIFF_IK,
          "transposed_interlaced": gpu.TRANSPOSED_F_HAT | gpu.INTERLACED}[flags]
    N = (12, 8, 16)
    for prec, tol in (("fp64", FP64_TOL), ("fp32", FP32_TOL)):
        p = gpu.Plan(N, m=4, flags=fl, c2r=True, precision=prec)
        o = oracle.OraclePlan(N, m=4, flags=fl, c2r=True)
        x, fh, f, g = case(N, 600, 18, c2r=True, local_N=p.local_N)
        a = p.trafo(x, fh, CF_ALL)
        b = o.trafo(x, fh, CF_ALL)
        for u, v in zip(a, b):
            assert rel(u, v) < tol, (flags, prec)
        assert rel(p.adj(x, f, g, 1 | 2), o.adj(x, f, g, 1 | 2)) < tol, (flags, prec)


@pytest.mark.parametrize("table", ["cub", "quad", "const"])
def test_fp32_tables_fraction_rounding_to_one(gpu, oracle, table):
    # nodes just below a grid point: n x - floor(n x) = 1 - 2^-30 rounds to 1.0
    # in FP32, one past the last sample interval of the PRE_*_PSI tables
    N, n, m = (16, 16, 16), (32, 32, 32), 6
    rng = np.random.default_rng(77)
    k = rng.integers(-16, 16, (64, 3))
    x_edge = (k + 1 - 2.0 ** -30) / 32.0
    x = np.concatenate([x_edge, rng.uniform(-0.5, 0.5, (400, 3))])
    x = np.where(x >= 0.5, x - 1.0, x)
    fh = rng.standard_normal(4096) + 1j * rng.standard_normal(4096)
    f = rng.standard_normal(x.shape[0]) + 1j * rng.standard_normal(x.shape[0])
    flags = {"cub": gpu.PRE_CUB_PSI, "quad": gpu.PRE_QUAD_PSI, "const": gpu.PRE_CONST_PSI}[table]
    p = gpu.Plan(N, n, m=m, flags=flags, precision="fp32")
    o = oracle.OraclePlan(N, n, m=m, flags=flags)
    assert rel(p.adj(x, f), o.adj(x, f)) < FP32_TOL
    assert rel(p.trafo(x, fh)[0], o.trafo(x, fh)[0]) < FP32_TOL


def test_fp64_vs_reference_fixtures(gpu):
    # outputs of the reference's own C code (tests/golden/ref_golden.npz, made
    # by tests/golden/make_ref_golden.py from oracle/_ref): FP64 to 1e-12
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_golden.npz"))
    for case in sorted({k.split("/")[0] for k in d.files}):
        N, n = tuple(int(v) for v in d[case + "/N"]), tuple(int(v) for v in d[case + "/n"])
        m, flags, cf = int(d[case + "/m"]), int(d[case + "/flags"]), int(d[case + "/cflags"])
        p = gpu.Plan(N, n, m=m, flags=flags)
        x, fh, f, g = d[case + "/x"], d[case + "/f_hat"], d[case + "/f"], d[case + "/grad"]
        got = p.trafo(x, fh, cf)
        keys = [k.split("/")[1] for k in d.files if k.startswith(case + "/")]
        for name, a in zip(("trafo_f", "trafo_grad", "trafo_hess"), got):
            if name in keys:
                assert rel(a, d[case + "/" + name]) < FP64_TOL, (case, name)
        assert rel(p.adj(x, f, g, 1 | 2), d[case + "/adj"]) < FP64_TOL, case
        p.close()


def _c_arrays(L, nd, M):
    import ctypes
    dp = ctypes.POINTER(ctypes.c_double)
    x = np.ctypeslib.as_array(ctypes.cast(L.pnfft_get_x(nd), dp), (3 * M,))
    f = np.ctypeslib.as_array(ctypes.cast(L.pnfft_get_f(nd), dp), (2 * M,))
    return x, f


@pytest.mark.parametrize("prec,tol", [("fp64", FP64_TOL), ("fp32", FP32_TOL)])
def test_precompute_psi_through_the_c_abi(gpu, oracle, prec, tol):
    # the reference caller sequence: pnfft_init_nodes, pnfft_precompute_psi
    # (PNFFT_PRE_PSI), pnfft_trafo / pnfft_adj; then the coordinates change in
    # place and pnfft_precompute_psi is called again, as the reference asks
    # (ndft-parallel.c:1144): the results follow the new coordinates
    import ctypes
    L = gpu.load()
    N, n, m, M = (16, 16, 16), (32, 32, 32), 5, 2000
    Nc, nc = (ctypes.c_ssize_t * 3)(*N), (ctypes.c_ssize_t * 3)(*n)
    xm = (ctypes.c_double * 3)(0.5, 0.5, 0.5)
    flags = gpu.MALLOC_F_HAT | (gpu.GB300_FP32 if prec == "fp32" else 0)
    p = L.pnfft_init_guru(3, Nc, nc, xm, m, ctypes.c_uint(flags), gpu.PFFT_ESTIMATE, gpu.MPI_COMM_WORLD)
    nd = L.pnfft_init_nodes(M, gpu.MALLOC_X | gpu.MALLOC_F)
    hx, hf = _c_arrays(L, nd, M)
    hfh = np.ctypeslib.as_array(ctypes.cast(L.pnfft_get_f_hat(p), ctypes.POINTER(ctypes.c_double)), (2 * 4096,))
    o = oracle.OraclePlan(N, n, m=m)
    rng = np.random.default_rng(51)
    fh = rng.standard_normal(4096) + 1j * rng.standard_normal(4096)
    for rep in range(2):
        x = rng.uniform(-0.5, 0.5, (M, 3))
        hx[:] = x.ravel()  # in place: the same array, new coordinates
        L.pnfft_precompute_psi(p, nd, gpu.PRE_PSI)
        for _ in range(2):  # the second call reuses the fixed nodes' binning
            hfh[:] = fh.view(np.float64)
            L.pnfft_trafo(p, nd, gpu.COMPUTE_F)
            assert rel(hf.view(np.complex128), o.trafo(x, fh)[0]) < tol, rep
        f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
        hf[:] = f.view(np.float64)
        L.pnfft_adj(p, nd, gpu.COMPUTE_F)
        assert rel(hfh.view(np.complex128), o.adj(x, f)) < tol, rep
    L.pnfft_free_nodes(nd, gpu.FREE_X | gpu.FREE_F)
    L.pnfft_finalize(p, gpu.FREE_F_HAT)


@pytest.mark.parametrize("prec,tol", [("fp64", FP64_TOL), ("fp32", FP32_TOL)])
def test_x_max_below_half(gpu, oracle, prec, tol):
    # x_max < 0.5: the reference prunes its FFT output to the grid points the
    # nodes reach (api-guru.c:195-218); here the whole grid is kept, which gives
    # the same values for nodes in [-x_max, x_max)
    N, n, m = (16, 16, 16), (32, 32, 32), 4
    xmax = np.array([0.25, 0.5, 0.125])
    rng = np.random.default_rng(52)
    x = rng.uniform(-1, 1, (1500, 3)) * xmax
    fh = rng.standard_normal(4096) + 1j * rng.standard_normal(4096)
    f = rng.standard_normal(1500) + 1j * rng.standard_normal(1500)
    p = gpu.Plan(N, n, m=m, x_max=xmax, precision=prec)
    assert p.lower_border == tuple(-xmax) and p.upper_border == tuple(xmax)
    o = oracle.OraclePlan(N, n, m=m)
    for a, b in zip(p.trafo(x, fh, 1 | 2)[:2], o.trafo(x, fh, 1 | 2)[:2]):
        assert rel(a, b) < tol
    assert rel(p.adj(x, f), o.adj(x, f)) < tol
