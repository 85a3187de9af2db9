"""pnfft_gb300_sort_nodes_noalloc: the node sort with its scratch in a static
device array instead of device allocations.  Called through the C ABI on
device arrays and compared with the allocating pnfft_gb300_sort_nodes on two
calls in a row (the second finds the first call's contents in the shared
scratch), at the size limit, and for sizes the entry point must refuse.  At
the size limit it is also compared with the oracle's CPU restatement of the
reference sort, so that a fault shared by both device sorts cannot pass.
This file is collected last on purpose: it must pass alone in a fresh process
and after every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(L, plan, dx, dpairs, M):
    return L.pnfft_gb300_sort_nodes_noalloc(plan._p, M, ctypes.c_void_p(dx.data_ptr()),
                                            ctypes.c_void_p(dpairs.data_ptr()), None)


def test_sort_noalloc_matches_allocating_sort(lib, oracle):
    torch = pytest.importorskip("torch")
    if lib.device_count() == 0:
        pytest.fail("no CUDA device visible for a -m gpu test")
    L = lib.load()
    MAX = lib.SORT_NOALLOC_MAX_NODES
    rng = np.random.default_rng(41)
    plan = lib.Plan((32, 48, 64), m=5)  # n = 64 x 96 x 128: three radix passes
    cases = [
        rng.uniform(-0.5, 0.5, (200_000, 3)),
        # clustered, many equal keys, smaller than the previous call
        np.mod(0.1 + 0.003 * rng.standard_normal((5_000, 3)) + 0.5, 1.0) - 0.5,
        rng.uniform(-0.5, 0.5, (MAX, 3)),
    ]
    for x in cases:
        M = x.shape[0]
        dx = torch.tensor(x, dtype=torch.float64, device="cuda")
        dpairs = torch.full((2 * M,), -7, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        L.pnfft_gb300_clear_error()
        assert _noalloc(L, plan, dx, dpairs, M) == 0, lib.last_error()
        torch.cuda.synchronize()
        got = dpairs.cpu().numpy().reshape(-1, 2)
        want = plan.sort_nodes(x)
        np.testing.assert_array_equal(got, want)
        if M == MAX:
            # the same plan on the CPU: sort_nodes_for_better_cache_handle restated
            o = oracle.OraclePlan((32, 48, 64), m=5)
            np.testing.assert_array_equal(got, o.sort_nodes(x))
    # a plan with an odd number of radix passes ends in the scratch buffer
    small = lib.Plan((8, 8, 8), m=2)  # n = 16^3: 12 key bits, two passes
    odd = lib.Plan((64, 64, 64), m=3)  # n = 128^3: 21 key bits, three passes
    for p in (small, odd):
        for _ in range(2):
            x = rng.uniform(-0.5, 0.5, (3000, 3))
            dx = torch.tensor(x, device="cuda")
            dpairs = torch.empty(6000, dtype=torch.int64, device="cuda")
            assert _noalloc(L, p, dx, dpairs, 3000) == 0, lib.last_error()
            torch.cuda.synchronize()
            np.testing.assert_array_equal(dpairs.cpu().numpy().reshape(-1, 2), p.sort_nodes(x))


def test_sort_noalloc_refuses_sizes_beyond_its_scratch(lib):
    torch = pytest.importorskip("torch")
    if lib.device_count() == 0:
        pytest.fail("no CUDA device visible for a -m gpu test")
    L = lib.load()
    plan = lib.Plan((16, 16, 16), m=3)
    dx = torch.zeros(3, dtype=torch.float64, device="cuda")
    dpairs = torch.zeros(2, dtype=torch.int64, device="cuda")
    L.pnfft_gb300_clear_error()
    assert _noalloc(L, plan, dx, dpairs, lib.SORT_NOALLOC_MAX_NODES + 1) == -1
    assert "capacity of the static scratch" in lib.last_error()
    assert _noalloc(L, plan, dx, dpairs, -1) == -1
    L.pnfft_gb300_clear_error()
    assert _noalloc(L, plan, dx, dpairs, 0) == 0
    assert lib.last_error() == ""
