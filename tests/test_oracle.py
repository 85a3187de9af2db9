"""Pins the CPU oracle (oracle/) to the known answers the reference's own tests
rely on -- no GPU needed.

  * check_vs_pfft.c:167-201: with the nodes on the equispaced grid x = k/N and
    M = N^3, adj(trafo(f_hat)) / N^3 == f_hat for the closed-form f_hat;
  * the direct NDFT (ndft-parallel.c:377-722) of single coefficients is the
    closed form exp(-2 pi i k.x) (trafo) / the adjoint sum (adj);
  * NFFT vs NDFT errors at the window's aliasing level for every window, with
    gradients, Hessians, ik differentiation, interlacing and tables
    (check_trafo.c, check_adj.c with -pnfft_compare_direct 1);
  * c2c vs c2r NDFT agreement on the Hermitian `semirandom` input of
    check_trafo_vs_ndft_c2r.c:202-231;
  * special functions against scipy (GSL I0/I1 and libcerf stand-ins);
  * the stable radix sort of util.c against numpy's stable argsort;
  * glibc rand() input generators against committed golden vectors.
"""
import json
import os

import numpy as np
import pytest
import scipy.special

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
WINDOWS = {
    "kaiser_bessel": 0,
    "gaussian": 1 << 13,
    "bspline": 1 << 14,
    "sinc_power": 1 << 15,
    "bessel_i0": 1 << 16,
    "gaussian_t": (1 << 17) | (1 << 13),
}
# max|f - f_ndft| / sum|f_hat| bounds at m = 6, sigma = 2 (measured on the
# restatement, with ~10x headroom); the reference prints these same ratios
TRAFO_TOL_M6 = {"kaiser_bessel": 1e-11, "gaussian": 1e-6, "bspline": 5e-7, "sinc_power": 5e-7, "bessel_i0": 3e-11,
                "gaussian_t": 1e-6}


def equispaced_case(N):
    k = [np.arange(-n // 2, n // 2) for n in N]
    K0, K1, K2 = np.meshgrid(*k, indexing="ij")
    x = np.stack([K0.ravel() / N[0], K1.ravel() / N[1], K2.ravel() / N[2]], 1)
    g = np.arange(int(np.prod(N)))
    fh = 1000.0 / (2 * g + 1) + 1j * 1000.0 / (2 * g + 2)
    return x, fh


@pytest.mark.parametrize("win", list(WINDOWS))
def test_check_vs_pfft_identity(oracle, win):
    N = (8, 8, 8)
    p = oracle.OraclePlan(N, m=6, flags=WINDOWS[win])
    x, fh = equispaced_case(N)
    f, _, _ = p.trafo(x, fh)
    back = p.adj(x, f) / np.prod(N)
    rel = np.abs(back - fh).max() / np.abs(fh).sum()
    assert rel < {"kaiser_bessel": 1e-10, "bessel_i0": 1e-9}.get(win, 1e-5), rel


def test_ndft_single_coefficient(oracle):
    rng = np.random.default_rng(0)
    N = (4, 6, 8)
    x = rng.uniform(-0.5, 0.5, (7, 3))
    for tr in (0, oracle.TRANSPOSED_F_HAT):
        p = oracle.OraclePlan(N, m=2, flags=tr)
        for k in [(0, 0, 0), (-2, 1, 3), (1, -3, -4)]:
            fh = np.zeros(p.fhat_shape, complex)
            idx = [k[t] + N[t] // 2 for t in range(3)]
            if tr:
                fh[idx[1], idx[2], idx[0]] = 1.0
            else:
                fh[idx[0], idx[1], idx[2]] = 1.0
            f, g, h = p.trafo(x, fh.ravel(), oracle.COMPUTE_F | oracle.COMPUTE_GRAD_F | oracle.COMPUTE_HESSIAN_F |
                              oracle.COMPUTE_DIRECT)
            e = np.exp(-2j * np.pi * (x @ np.array(k, float)))
            np.testing.assert_allclose(f, e, atol=1e-13)
            for t in range(3):
                np.testing.assert_allclose(g[:, t], -2j * np.pi * k[t] * e, atol=1e-11)
            pairs = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
            for c, (a, b) in enumerate(pairs):
                np.testing.assert_allclose(h[:, c], -4 * np.pi ** 2 * k[a] * k[b] * e, atol=1e-9)


def test_ndft_adjoint_closed_form(oracle):
    rng = np.random.default_rng(1)
    N = (4, 4, 6)
    M = 5
    x = rng.uniform(-0.5, 0.5, (M, 3))
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    g = rng.standard_normal((M, 3)) + 1j * rng.standard_normal((M, 3))
    p = oracle.OraclePlan(N, m=2)
    fh = p.adj(x, f, g, oracle.COMPUTE_F | oracle.COMPUTE_GRAD_F | oracle.COMPUTE_DIRECT).reshape(N)
    ks = [np.arange(-n // 2, n // 2) for n in N]
    K = np.stack(np.meshgrid(*ks, indexing="ij"), -1).reshape(-1, 3)
    e = np.exp(2j * np.pi * K @ x.T)
    want = e @ f + 2j * np.pi * ((K @ g.T) * e).sum(1)
    np.testing.assert_allclose(fh.ravel(), want, atol=1e-10)


def _rand_case(N, M, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-0.5, 0.5, (M, 3))
    fh = rng.standard_normal(int(np.prod(N))) + 1j * rng.standard_normal(int(np.prod(N)))
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    g = rng.standard_normal((M, 3)) + 1j * rng.standard_normal((M, 3))
    return x, fh, f, g


@pytest.mark.parametrize("win", list(WINDOWS))
def test_nfft_vs_ndft_accuracy(oracle, win):
    N = (16, 16, 16)
    x, fh, fv, gv = _rand_case(N, 300, 7)
    p = oracle.OraclePlan(N, m=6, flags=WINDOWS[win])
    cf = oracle.COMPUTE_F | oracle.COMPUTE_GRAD_F
    f, g, _ = p.trafo(x, fh, cf)
    f2, g2, _ = p.trafo(x, fh, cf | oracle.COMPUTE_DIRECT)
    s = np.abs(fh).sum()
    assert np.abs(f - f2).max() / s < TRAFO_TOL_M6[win]
    assert np.abs(g - g2).max() / s < 2e3 * TRAFO_TOL_M6[win]
    a1 = p.adj(x, fv, gv, cf)
    a2 = p.adj(x, fv, gv, cf | oracle.COMPUTE_DIRECT)
    assert np.linalg.norm(a1 - a2) / np.linalg.norm(a2) < 1e3 * TRAFO_TOL_M6[win]


@pytest.mark.parametrize("extra", ["interlaced", "diff_ik", "cub", "quad_c2c_real_only", "const", "transposed"])
def test_nfft_modes(oracle, extra):
    N = (8, 12, 16)
    flags = {"interlaced": oracle.INTERLACED, "diff_ik": oracle.DIFF_IK, "cub": oracle.PRE_CUB_PSI,
             "quad_c2c_real_only": oracle.PRE_QUAD_PSI, "const": oracle.PRE_CONST_PSI,
             "transposed": oracle.TRANSPOSED_F_HAT}[extra]
    x, fh, fv, gv = _rand_case(N, 200, 3)
    p = oracle.OraclePlan(N, m=6, flags=flags)
    cf = oracle.COMPUTE_F | oracle.COMPUTE_GRAD_F | oracle.COMPUTE_HESSIAN_F
    f, g, h = p.trafo(x, fh, cf)
    f2, g2, h2 = p.trafo(x, fh, cf | oracle.COMPUTE_DIRECT)
    s = np.abs(fh).sum()
    if extra == "quad_c2c_real_only":
        # PNFFT_PRE_QUAD_PSI shares bit 4 with PNFFT_REAL_F: the c2c trafo reads
        # only Re(g) (ndft-parallel.c:2804-2842), so f is Re-part only
        assert np.abs(f.imag).max() == 0.0
        p0 = oracle.OraclePlan(N, m=6, flags=0)
        fr, _, _ = p0.trafo(x, fh.real.astype(complex))
        fi, _, _ = p0.trafo(x, (1j * fh.imag))
        np.testing.assert_allclose(f.real, (fr + fi).real, atol=5e-4 * s / np.prod(N))
        return
    tol = 5e-3 if extra == "const" else 1e-10
    assert np.abs(f - f2).max() / s < tol
    assert np.abs(g - g2).max() / s < 1e4 * tol
    assert np.abs(h - h2).max() / s < 1e7 * tol
    a1 = p.adj(x, fv, gv, oracle.COMPUTE_F | oracle.COMPUTE_GRAD_F)
    a2 = p.adj(x, fv, gv, oracle.COMPUTE_F | oracle.COMPUTE_GRAD_F | oracle.COMPUTE_DIRECT)
    assert np.linalg.norm(a1 - a2) / np.linalg.norm(a2) < 1e3 * tol


def _semirandom(N, k0, k1, k2):
    """check_trafo_vs_ndft_c2r.c:202-222"""
    def di(i):
        return 1000.0 / (1 if i == 0 else i)
    if k0 == -N[0] // 2 or k1 == -N[1] // 2 or k2 == -N[2] // 2:
        return 0j
    if k0 == (N[0] + 1) // 2:
        return _semirandom(N, -k0, k1, k2)
    if k1 == (N[1] + 1) // 2:
        return _semirandom(N, k0, -k1, k2)
    if k2 == (N[2] + 1) // 2:
        return _semirandom(N, k0, k1, -k2)
    l0 = k0 + N[0] if k0 else 1
    l1 = k1 - 2 * N[1] if k1 else 1
    l2 = k2 + N[2] if k2 else 1
    re = di(l0 + l1 * l2) + 3 * di(l0 * l1 + l2) + di(l2 * l0 + l1)
    im = 3 * di(l0 + l1 * l1) + di(l1 + l2 * l2) - di(l2 + l0 * l0)
    return complex(re, im)


def semirandom_input(N, local_N, start):
    out = np.zeros(local_N, complex)
    for a in range(local_N[0]):
        for b in range(local_N[1]):
            for c in range(local_N[2]):
                k = (start[0] + a, start[1] + b, start[2] + c)
                out[a, b, c] = _semirandom(N, *k) + np.conj(_semirandom(N, -k[0], -k[1], -k[2]))
    return out.ravel()


def test_c2r_vs_c2c_ndft_and_nfft(oracle):
    N = (8, 8, 8)
    rng = np.random.default_rng(5)
    x = rng.uniform(-0.5, 0.5, (64, 3))
    pc = oracle.OraclePlan(N, m=6)
    pr = oracle.OraclePlan(N, m=6, c2r=True)
    fc_in = semirandom_input(N, pc.local_N, pc.local_N_start)
    fr_in = semirandom_input(N, pr.local_N, pr.local_N_start)
    fc, _, _ = pc.trafo(x, fc_in, oracle.COMPUTE_F | oracle.COMPUTE_DIRECT)
    fr, _, _ = pr.trafo(x, fr_in, oracle.COMPUTE_F | oracle.COMPUTE_DIRECT)
    assert np.abs(fc.imag).max() < 1e-9 * np.abs(fc).max()
    np.testing.assert_allclose(fr, fc.real, rtol=0, atol=1e-9 * np.abs(fc).max())
    fn, _, _ = pr.trafo(x, fr_in, oracle.COMPUTE_F)
    assert np.abs(fn - fr).max() / np.abs(fr_in).sum() < 1e-11


def test_special_functions_vs_scipy(oracle):
    xs = np.concatenate([np.linspace(0, 5, 11), np.linspace(5, 80, 16)])
    for v in xs:
        assert abs(oracle.bessel_i0(v) - scipy.special.i0(v)) <= 4e-15 * scipy.special.i0(v)
        assert abs(oracle.bessel_i1(v) - scipy.special.i1(v)) <= 4e-15 * max(scipy.special.i1(v), 1e-300)
    for a in (1.0, 2.5, 3.76):
        for y in (0.0, 0.3, 1.2, 2.5):
            want = scipy.special.erf(complex(a, y)).real
            assert abs(oracle.re_erf_complex(a, y) - want) < 1e-13 * max(1.0, abs(want))
    with open(os.path.join(GOLDEN, "special.json")) as fh:
        gold = json.load(fh)
    for x, v in gold["i0"]:
        assert abs(oracle.bessel_i0(x) - v) <= 4e-15 * v
    for a, y, v in gold["re_erf"]:
        assert abs(oracle.re_erf_complex(a, y) - v) < 1e-13 * max(1, abs(v))


def test_bspline_vs_scipy(oracle):
    from scipy.interpolate import BSpline
    for p in (2, 3, 4, 8, 12, 16):
        b = BSpline.basis_element(np.arange(p + 1), extrapolate=False)
        for t in np.linspace(0.01, p - 0.01, 37):
            assert abs(oracle.bspline(p, t) - b(t)) < 1e-13


def test_sort_nodes_is_stable_radix(oracle):
    rng = np.random.default_rng(11)
    p = oracle.OraclePlan((8, 8, 8), m=3)
    x = rng.uniform(-0.5, 0.5, (5000, 3))
    x[100:200] = x[7]  # many equal keys: order must be the input order
    pairs = p.sort_nodes(x)
    n = np.array(p.n)
    u = (np.floor(n * x - p.m).astype(np.int64) % n)
    key = (u[:, 0] * n[1] + u[:, 1]) * n[2] + u[:, 2]
    order = np.argsort(key, kind="stable")
    np.testing.assert_array_equal(pairs[:, 1], order)
    np.testing.assert_array_equal(pairs[:, 0], key[order])


def test_glibc_rand_generators_golden(oracle):
    with open(os.path.join(GOLDEN, "rand_inputs.json")) as fh:
        gold = json.load(fh)
    oracle.srand(0)
    x = oracle.init_x_3d_adv([-0.5] * 3, [0.5] * 3, [0.5] * 3, 8)
    np.testing.assert_array_equal(x.ravel(), np.array(gold["x_srand0"]))
    oracle.srand(1)
    f = oracle.init_f(4)
    np.testing.assert_array_equal(f.view(np.float64), np.array(gold["f_srand1"]))


def test_flag_promotion_quirk(oracle):
    # api-guru.c:152-155 tests precompute-flag bits on plan flags: PRE_LIN_PSI
    # (bit 3) pulls in bits 2 and 1, so the plan interpolates with order 0
    p = oracle.OraclePlan((8, 8, 8), m=4, flags=oracle.PRE_LIN_PSI)
    assert p.flags & oracle.PRE_CONST_PSI and p.flags & oracle.FAST_GAUSSIAN
    from oracle.pnfft_oracle import lib
    assert lib().or_intpol_order(p._h) == 0
