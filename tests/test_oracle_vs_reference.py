"""The oracle against the reference itself (CPU).

oracle/_ref/libpnfft_ref.so is the reference's own C code (kernel/, api/,
util/, cerf/), compiled unmodified against single-process stand-ins for MPI,
PFFT and GSL (oracle/refbuild/), and driven here through its public API
(pnfft_init_guru, pnfft_init_nodes, pnfft_trafo, pnfft_adj).  The oracle's
restatement agrees with it to 1e-13 relative l2 on every window and mode of a
1x1x1 c2c plan, and on the benchmark's configuration 1 exactly.  Where the
reference tree is absent (no build), these tests are skipped; the committed
fixtures of tests/golden/ref_golden.npz, made by the same library, pin the
oracle there (test_oracle_vs_reference_fixtures).
"""
import os

import numpy as np
import pytest

from oracle import pnfft_oracle as O

TOL = 1e-13
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_golden.npz")


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    nb = np.linalg.norm(b.ravel())
    return np.linalg.norm((a - b).ravel()) / nb if nb > 0 else np.linalg.norm(a.ravel())


@pytest.fixture(scope="module")
def ref():
    from oracle import reference
    if not reference.available():
        pytest.skip("the reference tree was not present when the oracle was built (no oracle/_ref)")
    reference.lib()
    return reference


MODES = {
    "kaiser_bessel": 0,
    "gaussian": O.WINDOW_GAUSSIAN,
    "fast_gaussian": O.WINDOW_GAUSSIAN | O.FAST_GAUSSIAN,
    "gaussian_t": O.WINDOW_GAUSSIAN_T,
    "bspline": O.WINDOW_BSPLINE,
    "sinc_power": O.WINDOW_SINC_POWER,
    "bessel_i0": O.WINDOW_BESSEL_I0,
    "interlaced": O.INTERLACED,
    "diff_ik": O.DIFF_IK,
    "ik_interlaced": O.DIFF_IK | O.INTERLACED,
    "pre_const_psi": O.PRE_CONST_PSI,
    "pre_lin_psi": O.PRE_LIN_PSI,
    "pre_quad_psi": O.PRE_QUAD_PSI,
    "pre_cub_psi": O.PRE_CUB_PSI,
    "pre_phi_hat": O.PRE_PHI_HAT,
    "sort_nodes": O.SORT_NODES,
}


def inputs(N, M, seed):
    rng = np.random.default_rng(seed)
    S = int(np.prod(N))
    x = rng.uniform(-0.5, 0.5, (M, 3))
    fh = rng.standard_normal(S) + 1j * rng.standard_normal(S)
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    g = rng.standard_normal((M, 3)) + 1j * rng.standard_normal((M, 3))
    return x, fh, f, g


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("m", [2, 4, 6])
def test_oracle_matches_reference(ref, mode, m):
    N = (8, 12, 10)
    x, fh, f, g = inputs(N, 400, m)
    r = ref.RefPlan(N, m=m, flags=MODES[mode])
    o = O.OraclePlan(N, m=m, flags=MODES[mode])
    cf = O.COMPUTE_F | O.COMPUTE_GRAD_F | O.COMPUTE_HESSIAN_F
    for a, b in zip(r.trafo(x, fh, cf), o.trafo(x, fh, cf)):
        assert rel(b, a) < TOL, mode
    # the same inputs with the direct NDFT (PNFFT_COMPUTE_DIRECT) on 64 nodes
    d_ref = r.trafo(x[:64], fh, cf | O.COMPUTE_DIRECT)
    d_or = o.trafo(x[:64], fh, cf | O.COMPUTE_DIRECT)
    for a, b in zip(d_ref, d_or):
        assert rel(b, a) < 1e-12, mode
    assert rel(o.adj(x, f, g, O.COMPUTE_F | O.COMPUTE_GRAD_F), r.adj(x, f, g, O.COMPUTE_F | O.COMPUTE_GRAD_F)) < TOL


@pytest.mark.parametrize("N,n,m", [((16, 8, 12), (24, 12, 18), 5), ((8, 8, 8), (10, 9, 13), 3),
                                   ((6, 10, 8), (12, 12, 12), 7)])
def test_oracle_matches_reference_odd_grids(ref, N, n, m):
    # oversampling factors other than 2, odd grids, stencils wider than the
    # grid.  For odd n_t the reference indexes a node with n_t x_t < -(n_t/2)
    # (C division) one plane below its ghost-celled array, so the nodes are
    # drawn above that edge here.  Oversampling as low as 1.2 makes 1/phi_hat
    # large, and the sums cancel: the two FP64 FFTs (scipy, the stand-in's)
    # then differ by a few 1e-12
    x, fh, f, g = inputs(N, 500, 7)
    lo = np.array([-(v // 2) / v for v in n])
    x = lo + (0.5 - lo) * (x + 0.5)
    r = ref.RefPlan(N, n, m=m)
    o = O.OraclePlan(N, n, m=m)
    got = o.trafo(x, fh, 3)
    want = r.trafo(x, fh, 3)
    for a, b in zip(want[:2], got[:2]):
        assert rel(b, a) < 1e-11
    assert rel(o.adj(x, f, g, 3), r.adj(x, f, g, 3)) < 1e-11


def test_oracle_matches_reference_precompute_psi(ref):
    # pnfft_precompute_psi with PNFFT_PRE_PSI: windows stored per node, f only
    N = (8, 8, 8)
    x, fh, f, g = inputs(N, 300, 9)
    r = ref.RefPlan(N, m=4)
    o = O.OraclePlan(N, m=4)
    assert rel(o.trafo(x, fh)[0], r.trafo(x, fh, 1, precompute=1 << 10)[0]) < TOL


def test_oracle_matches_reference_configuration_1(ref):
    # N = 32^3, n = 64^3, M = 32768 uniform nodes, Kaiser-Bessel m = 4, seed 1
    N, M = (32, 32, 32), 32768
    rng = np.random.default_rng(1)
    x = rng.uniform(-0.5, 0.5, (M, 3))
    S = int(np.prod(N))
    fh = rng.standard_normal(S) + 1j * rng.standard_normal(S)
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    r = ref.RefPlan(N, (64, 64, 64), m=4)
    o = O.OraclePlan(N, (64, 64, 64), m=4)
    assert rel(o.trafo(x, fh)[0], r.trafo(x, fh)[0]) < TOL
    assert rel(o.adj(x, f), r.adj(x, f)) < TOL


def test_oracle_vs_reference_fixtures():
    # outputs of the reference build committed in tests/golden (runs without the tree)
    d = np.load(GOLDEN)
    for case in sorted({k.split("/")[0] for k in d.files}):
        N, n, m, flags = (tuple(d[case + "/N"]), tuple(d[case + "/n"]), int(d[case + "/m"]), int(d[case + "/flags"]))
        o = O.OraclePlan(N, n, m=m, flags=flags)
        x, fh, f, g = d[case + "/x"], d[case + "/f_hat"], d[case + "/f"], d[case + "/grad"]
        cf = int(d[case + "/cflags"])
        for name, got in zip(("trafo_f", "trafo_grad", "trafo_hess"), o.trafo(x, fh, cf)):
            if name in [k.split("/")[1] for k in d.files if k.startswith(case + "/")]:
                assert rel(got, d[case + "/" + name]) < TOL, (case, name)
        assert rel(o.adj(x, f, g, O.COMPUTE_F | O.COMPUTE_GRAD_F), d[case + "/adj"]) < TOL, case
