"""Parity at the benchmark configurations themselves, through the C ABI.

Configuration 1 (the reference's CPU-runnable case), exactly: N = 32^3,
n = 64^3, M = 32768 nodes i.i.d. uniform in [-0.5, 0.5)^3, f_hat and f complex
standard normal (numpy PCG64, seed 1), Kaiser-Bessel m = 4.  FP64 trafo and
adj agree with the oracle's NFFT to 1e-12 relative l2, and with the oracle's
direct NDFT (kernel/ndft-parallel.c:377-722) exactly as closely as the
oracle's own NFFT does.

Configuration 2 (the workload of the headline number): N = 128^3, n = 256^3,
M = 2^22 uniform nodes, f_hat complex normal scaled by (1 + |k|^2)^-1, f
complex normal (seed 2), Kaiser-Bessel m = 6, trafo with COMPUTE_F |
COMPUTE_GRAD_F.
  * FP64: f and grad_f on the first 4096 nodes against the oracle's NFFT of
    the same f_hat on those nodes (D, F and B at full size), and the adjoint
    over all M nodes against the oracle's adjoint, to 1e-12.
  * FP32-mixed: trafo (f and grad_f) against the FP64 direct NDFT on the
    first 4096 nodes, and adj against the FP64 adjoint NDFT over all M nodes
    at 4096 frequencies (a random 16 x 16 x 16 sub-lattice of the 128^3), to
    1e-6 relative l2, the bar of the FP32-mixed form.  The same for the
    PNFFT_PRE_CUB_PSI tables.
  * Size-independent: <trafo(f_hat), f> = <f_hat, adj(f)> (the adjoint
    identity of B F D) in both precisions, at full size.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-6  # the FP32-mixed bar: relative l2 against the FP64 NDFT
SUB = 4096


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel())


@pytest.fixture(scope="module")
def gpu(lib):
    if lib.device_count() == 0:
        pytest.fail("no CUDA device visible for a -m gpu test")
    return lib


# ---------------------------------------------------------------------------
# configuration 1
# ---------------------------------------------------------------------------
def config1():
    N, M = (32, 32, 32), 32768
    rng = np.random.default_rng(1)
    x = rng.uniform(-0.5, 0.5, (M, 3))
    S = int(np.prod(N))
    fh = rng.standard_normal(S) + 1j * rng.standard_normal(S)
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    return N, (64, 64, 64), x, fh, f


def test_config1_fp64_vs_oracle_nfft_and_ndft(gpu, oracle):
    N, n, x, fh, f = config1()
    p = gpu.Plan(N, n, m=4)
    o = oracle.OraclePlan(N, n, m=4)
    ft = p.trafo(x, fh)[0]
    fo = o.trafo(x, fh)[0]
    assert rel(ft, fo) < FP64_TOL
    fa = p.adj(x, f)
    ao = o.adj(x, f)
    assert rel(fa, ao) < FP64_TOL
    # the direct NDFT: the GPU's window error is the oracle's window error
    fd = o.trafo(x, fh, oracle.COMPUTE_F | oracle.COMPUTE_DIRECT)[0]
    ad = o.adj(x, f, None, oracle.COMPUTE_F | oracle.COMPUTE_DIRECT)
    e_gpu, e_or = rel(ft, fd), rel(fo, fd)
    assert e_gpu < 1e-6 and abs(e_gpu - e_or) <= 1e-9 * e_or
    e_gpu, e_or = rel(fa, ad), rel(ao, ad)
    assert e_gpu < 1e-6 and abs(e_gpu - e_or) <= 1e-9 * e_or
    # the error figure check_trafo.c prints, max |f - f_direct| / sum |f_hat|,
    # is the oracle's (the window's aliasing error at m = 4)
    e_gpu = np.abs(ft - fd).max() / np.abs(fh).sum()
    e_or = np.abs(fo - fd).max() / np.abs(fh).sum()
    assert e_gpu < 1e-8 and abs(e_gpu - e_or) <= 1e-6 * e_or


def test_config1_fp32_mixed_vs_ndft(gpu, oracle):
    N, n, x, fh, f = config1()
    p = gpu.Plan(N, n, m=4, precision="fp32")
    o = oracle.OraclePlan(N, n, m=4)
    fd = o.trafo(x, fh, oracle.COMPUTE_F | oracle.COMPUTE_DIRECT)[0]
    ad = o.adj(x, f, None, oracle.COMPUTE_F | oracle.COMPUTE_DIRECT)
    assert rel(p.trafo(x, fh)[0], fd) < FP32_TOL
    assert rel(p.adj(x, f), ad) < FP32_TOL


# ---------------------------------------------------------------------------
# configuration 2
# ---------------------------------------------------------------------------
CF_FG = 1 | 2  # COMPUTE_F | COMPUTE_GRAD_F


@pytest.fixture(scope="module")
def cfg2(oracle):
    N, n, M = (128, 128, 128), (256, 256, 256), 1 << 22
    rng = np.random.default_rng(2)
    x = rng.uniform(-0.5, 0.5, (M, 3))
    k = [np.arange(-v // 2, v // 2) for v in N]
    K0, K1, K2 = np.meshgrid(*k, indexing="ij")
    w = 1.0 / (1.0 + K0 ** 2 + K1 ** 2 + K2 ** 2)
    fh = ((rng.standard_normal(N) + 1j * rng.standard_normal(N)) * w).ravel()
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    o = oracle.OraclePlan(N, n, m=6)
    xs = x[:SUB].copy()
    fd, gd, _ = o.trafo(xs, fh, CF_FG | oracle.COMPUTE_DIRECT)
    lat = [np.sort(np.random.default_rng(20 + t).choice(np.arange(-64, 64), 16, replace=False)) for t in range(3)]
    ad = oracle.ndft_adj_lattice(x, f, *lat)
    return dict(N=N, n=n, M=M, x=x, fh=fh, f=f, o=o, xs=xs, fd=fd, gd=gd, lat=lat, ad=ad)


def lattice_of(fh_flat, N, lat):
    c = fh_flat.reshape(N)
    return c[np.ix_(*[np.asarray(k) + v // 2 for k, v in zip(lat, N)])]


def test_config2_fp64_trafo_with_gradient_vs_oracle(gpu, cfg2):
    c = cfg2
    p = gpu.Plan(c["N"], c["n"], m=6)
    f, g, _ = p.trafo(c["x"], c["fh"], CF_FG)
    fo, go, _ = c["o"].trafo(c["xs"], c["fh"], CF_FG)
    assert rel(f[:SUB], fo) < FP64_TOL
    assert rel(g[:SUB], go) < FP64_TOL
    # the window's aliasing error against the direct NDFT is the oracle's
    for got, want, nd in ((f[:SUB], fo, c["fd"]), (g[:SUB], go, c["gd"])):
        e_gpu, e_or = rel(got, nd), rel(want, nd)
        assert e_gpu < 1e-8 and abs(e_gpu - e_or) <= 1e-3 * e_or


def test_config2_fp64_adj_vs_oracle(gpu, cfg2):
    c = cfg2
    p = gpu.Plan(c["N"], c["n"], m=6)
    a = p.adj(c["x"], c["f"])
    ao = c["o"].adj(c["x"], c["f"])
    assert rel(a, ao) < FP64_TOL
    assert rel(lattice_of(a, c["N"], c["lat"]), c["ad"]) < 1e-10


@pytest.mark.parametrize("tables", [False, True], ids=["fitted_windows", "pre_cub_psi"])
def test_config2_fp32_mixed_vs_ndft(gpu, cfg2, tables):
    c = cfg2
    flags = gpu.PRE_CUB_PSI if tables else 0
    p = gpu.Plan(c["N"], c["n"], m=6, flags=flags, precision="fp32")
    f, g, _ = p.trafo(c["x"], c["fh"], CF_FG)
    assert rel(f[:SUB], c["fd"]) < FP32_TOL
    assert rel(g[:SUB], c["gd"]) < FP32_TOL
    a = p.adj(c["x"], c["f"])
    assert rel(lattice_of(a, c["N"], c["lat"]), c["ad"]) < FP32_TOL


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-13), ("fp32", 1e-6)])
def test_config2_adjoint_identity(gpu, cfg2, prec, tol):
    # <B F D f_hat, f> = <f_hat, D^T F^H B^T f>: holds for any size, so it is
    # checked on the whole workload
    c = cfg2
    p = gpu.Plan(c["N"], c["n"], m=6, precision=prec)
    ft = p.trafo(c["x"], c["fh"])[0]
    a = p.adj(c["x"], c["f"])
    lhs = np.vdot(c["f"], ft)
    rhs = np.vdot(a, c["fh"])
    scale = np.linalg.norm(ft) * np.linalg.norm(c["f"])
    assert abs(lhs - rhs) / scale < tol
