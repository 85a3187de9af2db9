"""Error budget of the FP32-mixed form: how much of its error comes from the
FP32 accumulation of the convolution sums, and how much from rounding the
grid (FP32 FFT) and the window values.

A compensated (Kahan) sum removes only the first part.  This test emulates,
in numpy, the summation order of the FP32-mixed line kernels:
- B (k_interp_line): per grid column two alternating FP32 chains over the z
  window, the column pair weighted by psi_x psi_y, then the 128 thread shares
  of a node summed by four threads, each two Kahan-compensated runs over 16
  shares combined with TwoSum, and two pairwise steps;
- B^T (k_spread_line_f): per line of 4x4 columns, nodes in slab order, each
  grid value accumulated in FP32 over runs of at most 127 nodes (a slab
  change, or a batch start after 64 nodes, ends a run) before it is added
  (the float atomics) into the FP32 grid, without compensation.
Each FP32-mixed result is compared with (a) the same FP32 terms summed in FP64
(exact accumulation) and (b) the all-FP64 computation.  The accumulation
error is the distance to (a), the total error the distance to (b); the
emulation uses a Kaiser-Bessel window, m = 6, sigma = 2, N = 16^3.
Asserted: for B the compensated node sums cut the total error by more than
15 % against plain FP32 runs (1.34e-7 against 1.65e-7 here) and leave the
accumulation error (the z chains and products) at the level of the rounding
error (below 1.5 times it); for B^T on a dense cluster the
total stays below 1e-6 and the accumulation error (the larger part there,
3.5e-7) below 4e-7.  The printout gives the numbers.
"""
import numpy as np

N, n, m = 16, 32, 6
CUT = 2 * m + 1
B = np.pi * (2.0 - 1.0 / 2.0)  # Kaiser-Bessel shape for sigma = 2 (the reference's default)


def kb_psi(d):
    """Kaiser-Bessel window at distance d (grid units / n), FP64."""
    z = m * m - (n * d) ** 2
    out = np.empty_like(z)
    pos, zero, neg = z > 0, z == 0, z < 0
    r = np.sqrt(np.abs(z))
    out[pos] = np.sinh(B * r[pos]) / (np.pi * r[pos])
    out[zero] = B / np.pi
    out[neg] = np.sin(B * r[neg]) / (np.pi * r[neg])
    return out


def kb_phi_hat(k):
    return np.i0(m * np.sqrt(B * B - (2 * np.pi * k / n) ** 2)) / n


def grid_from_fhat(fhat, dtype):
    """D then the FFT: f_hat / phi_hat zero-padded into n^3, FFT in `dtype`."""
    k = np.arange(-N // 2, N // 2)
    ph = kb_phi_hat(k)
    d = fhat / (ph[:, None, None] * ph[None, :, None] * ph[None, None, :])
    g = np.zeros((n, n, n), np.complex128)
    idx = np.mod(k, n)
    g[np.ix_(idx, idx, idx)] = d
    return np.fft.fftn(g.astype(dtype))


def stencil(x):
    """Lowest stencil index u (per axis) and the FP64 window rows (M, 3, CUT)."""
    u = np.floor(n * x).astype(np.int64) - m
    s = np.arange(CUT)
    d = x[:, :, None] - (u[:, :, None] + s) / n
    return u, kb_psi(d)


def plain(v):
    """FP32 sum in order."""
    return np.cumsum(v, dtype=np.complex64)[-1]


def kahan_run(v):
    """One Kahan run in order: (sum, correction)."""
    s = c = np.complex64(0)
    for x in v.astype(np.complex64):
        y = np.complex64(x - c)
        t = np.complex64(s + y)
        c = np.complex64(np.complex64(t - s) - y)
        s = t
    return s, c


def kahan(v):
    """As kahan_quarter_sum (line_f32.cuh): two Kahan runs over alternate
    entries, their sums added with TwoSum and both corrections applied."""
    s, c = kahan_run(v[0::2])
    u, e = kahan_run(v[1::2])
    t = np.complex64(s + u)
    bb = np.complex64(t - s)
    err = np.complex64(np.complex64(s - np.complex64(t - bb)) + np.complex64(u - bb))
    return np.complex64(t + np.complex64(err - np.complex64(c + e)))


def interp_emulated(x, g32, g64, compensated=True):
    """B three ways: kernel-order FP32, FP32 terms summed in FP64, all FP64."""
    M = x.shape[0]
    u, w64 = stencil(x)
    w32 = w64.astype(np.float32)
    out32 = np.empty(M, np.complex64)
    exact = np.empty(M, np.complex128)
    ref = np.empty(M, np.complex128)
    for j in range(M):
        # the 16 x 16 region of the node's line: the stencil sits at offset o
        o = u[j] % 4
        rows = [(u[j, t] - o[t] + np.arange(16)) % n for t in range(3)]
        G32 = g32[np.ix_(rows[0], rows[1], (u[j, 2] + np.arange(CUT)) % n)]
        G64 = g64[np.ix_(rows[0], rows[1], (u[j, 2] + np.arange(CUT)) % n)]
        wx = np.zeros((3, 16), np.float32)
        wx64 = np.zeros((3, 16))
        for t in range(2):
            wx[t, o[t]:o[t] + CUT] = w32[j, t]
            wx64[t, o[t]:o[t] + CUT] = w64[j, t]
        wz = w32[j, 2]
        # z sums: two alternating FP32 chains per column
        ca = np.zeros((16, 16), np.complex64)
        cb = np.zeros((16, 16), np.complex64)
        for p in range(CUT):
            term = (G32[:, :, p] * wz[p]).astype(np.complex64)
            if p % 2 == 0:
                ca = (ca + term).astype(np.complex64)
            else:
                cb = (cb + term).astype(np.complex64)
        col = (ca + cb).astype(np.complex64)
        # shares: thread (a, b) owns columns (a, b) and (a, b + 8)
        sh = (wx[0][:, None] * ((wx[1][None, :8] * col[:, :8]).astype(np.complex64)
                                + (wx[1][None, 8:] * col[:, 8:]).astype(np.complex64))).astype(np.complex64)
        sh = sh.ravel()  # 128 shares; thread r of the node takes shares r, r + 4, ...
        runs = [(kahan if compensated else plain)(sh[r::4]) for r in range(4)]
        out32[j] = np.complex64(np.complex64(runs[0] + runs[1]) + np.complex64(runs[2] + runs[3]))
        # the same FP32 terms (window products rounded as in the kernel) summed in FP64
        t32 = (wx[0][:, None, None] * wx[1][None, :, None]).astype(np.float32)
        exact[j] = np.sum(G32.astype(np.complex128) * (t32.astype(np.float64) * wz.astype(np.float64)))
        ref[j] = np.sum(G64 * (wx64[0][:, None, None] * wx64[1][None, :, None] * w64[j, 2][None, None, :]))
    return out32, exact, ref


def spread_emulated(x, f):
    """B^T three ways on the grid: kernel-order FP32 (64-node runs per line
    committed into an FP32 grid), FP32 terms summed in FP64, all FP64."""
    u, w64 = stencil(x)
    w32 = w64.astype(np.float32)
    f32 = f.astype(np.complex64)
    # nodes in line order (4x4 columns), then slab order
    key = ((u[:, 0] // 4) * 64 + u[:, 1] // 4) * 64 + u[:, 2] // 4
    order = np.argsort(key, kind="stable")
    line = (u[:, 0] // 4) * 64 + u[:, 1] // 4
    g32 = np.zeros(n ** 3, np.complex64)
    gex = np.zeros(n ** 3, np.complex128)
    g64 = np.zeros(n ** 3, np.complex128)
    s = np.arange(CUT)
    run = np.zeros(n ** 3, np.complex64)
    # the kernel's rule: per line (sub-problems of 512 nodes), batches of 64
    # nodes; a slab change commits; at a batch start, 64 or more nodes since
    # the last commit commit everything (runs of at most 127 nodes)
    since, cur, pos, slab = 0, None, 0, None
    for j in order:
        s_j = u[j, 2] // 4
        new_line = cur is None or line[j] != cur or pos == 512
        if new_line:
            pos = 0
        if cur is not None and (new_line or s_j != slab or (pos % 64 == 0 and since >= 64)):
            g32 = (g32 + run).astype(np.complex64)
            run[:] = 0
            since = 0
        cur, slab = line[j], s_j
        pos += 1
        since += 1
        i0, i1, i2 = [(u[j, t] + s) % n for t in range(3)]
        idx = ((i0[:, None, None] * n + i1[None, :, None]) * n + i2[None, None, :]).ravel()
        wxy = (w32[j, 0][:, None] * w32[j, 1][None, :]).astype(np.float32)
        w = (wxy[:, :, None] * w32[j, 2][None, None, :]).astype(np.float32).ravel()
        term = (w * f32[j]).astype(np.complex64)
        np.add.at(run, idx, term)
        gex[idx] += term.astype(np.complex128)
        g64[idx] += (w64[j, 0][:, None, None] * w64[j, 1][None, :, None] * w64[j, 2][None, None, :]).ravel() * f[j]
    g32 = (g32 + run).astype(np.complex64)
    return g32, gex, g64


def fhat_from_grid(g, dtype):
    """F^H then D^T: inverse-direction FFT in `dtype`, crop, divide by phi_hat."""
    G = np.fft.ifftn(g.reshape(n, n, n).astype(dtype)) * n ** 3
    k = np.arange(-N // 2, N // 2)
    idx = np.mod(k, n)
    ph = kb_phi_hat(k)
    return G[np.ix_(idx, idx, idx)].astype(np.complex128) / (ph[:, None, None] * ph[None, :, None] * ph[None, None, :])


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_interp_accumulation_share():
    rng = np.random.default_rng(5)
    fhat = rng.standard_normal((N, N, N)) + 1j * rng.standard_normal((N, N, N))
    g64 = grid_from_fhat(fhat, np.complex128)
    g32 = grid_from_fhat(fhat, np.complex64)
    x = rng.uniform(-0.5, 0.5, (300, 3))
    out32, exact, ref = interp_emulated(x, g32, g64)
    plain32, _, _ = interp_emulated(x, g32, g64, compensated=False)
    e_total, e_acc, e_round = rel(out32, ref), rel(out32, exact), rel(exact, ref)
    e_plain = rel(plain32, ref)
    print(f"B: total {e_total:.2e} (plain FP32 node sums: {e_plain:.2e}), accumulation {e_acc:.2e}, "
          f"grid and window rounding {e_round:.2e}")
    assert e_total < 1e-6
    assert e_total < 0.85 * e_plain  # the compensated node sums remove the largest accumulation term
    assert e_acc < 1.5 * e_round


def test_spread_accumulation_dense_cluster():
    rng = np.random.default_rng(6)
    M = 3000
    x = np.concatenate([rng.uniform(-0.5, 0.5, (M // 3, 3)),
                        0.1 + 0.004 * rng.standard_normal((M - M // 3, 3))])  # 2000 nodes in ~1/8 cell
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    g32, gex, g64 = spread_emulated(x, f)
    fh32 = fhat_from_grid(g32, np.complex64)
    fhex = fhat_from_grid(gex.astype(np.complex64), np.complex64)
    fh64 = fhat_from_grid(g64, np.complex128)
    e_total, e_acc, e_round = rel(fh32, fh64), rel(fh32, fhex), rel(fhex, fh64)
    print(f"B^T (dense cluster): total {e_total:.2e}, accumulation {e_acc:.2e}, "
          f"grid and window rounding {e_round:.2e}; grid: accumulation {rel(g32, gex):.2e}")
    assert e_total < 1e-6
    assert e_acc < 4e-7
