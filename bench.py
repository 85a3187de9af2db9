"""Throughput of PNFFT's trafo+adj on one GB300 (and the CPU oracle beside it).

Workload (the configuration the headline metric is quoted on): c2c 3-D NFFT,
N = 128^3 Fourier coefficients, oversampled grid n = 256^3, M = 2^22 nodes
i.i.d. uniform in [-0.5,0.5)^3, Kaiser-Bessel window m = 6, f_hat complex
normal scaled by (1+|k|^2)^-1, adj input f complex normal (seeded synthetic
data).  One step = pnfft_trafo (D, F, B) + pnfft_adj (B^T, F^H, D^T).

  value   Mpts/s = M / (t_trafo + t_adj), FP32-mixed, inputs resident in HBM
          (zero-copy device entry points), nodes re-binned every call
  e2e     same metric through the C ABI (pnfft_trafo/pnfft_adj) on host
          arrays from pnfft_malloc (page-locked): copies inside the timed step
  fp64    the plain FP64 path, same workload
  roofline  the dominant kernel against the FP32 FFMA2 rate measured in the
          run, its ncu DRAM traffic (profiles/traffic.json), and the whole
          step's roofline (sum of stage roofline times / step time)
  accuracy  FP32-mixed trafo against the FP64 NDFT on 4096 nodes, adjoint
          against the FP64 NDFT at 4096 frequencies over all nodes
  cpu_baseline  the oracle (FP64 restatement of the reference, all host
          cores) on whole steps of the same workload
Further rows (one GPU): with_grad, pre_cub_psi, amortised_fixed_nodes,
batched (65 plans + 8 right-hand sides in one CUDA graph), particles
(clustered c2r charges, autotuned), charge_dipole (one C call against four),
float_api (pnfftf_* on host float arrays).  --impl reference times the oracle
alone on whole steps (the reference arm).
Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
       [--no-cpu] [--no-batch] [--profile]
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CFG = dict(N=(128, 128, 128), n=(256, 256, 256), M=1 << 22, m=6)
WORKLOAD = "c2c NFFT trafo+adj, N=128^3, n=256^3, M=2^22 uniform nodes, Kaiser-Bessel m=6"
METRIC = "trafo+adj Mpts/s, N=128^3 M=2^22"
L2_BYTES = 129 * 1024 * 1024
# the kernels of B and B^T at the workload (FP32-mixed, cutoff 13)
INTERP_KERNEL = "k_interp_line<13>"
SPREAD_KERNEL = "k_spread_line_f<13>"


def make_inputs(seed=2):
    N, M = CFG["N"], CFG["M"]
    rng = np.random.default_rng(seed)
    x = rng.uniform(-0.5, 0.5, (M, 3))
    k = [np.arange(-n // 2, n // 2) for n in N]
    K0, K1, K2 = np.meshgrid(*k, indexing="ij")
    w = 1.0 / (1.0 + K0 ** 2 + K1 ** 2 + K2 ** 2)
    fh = ((rng.standard_normal(N) + 1j * rng.standard_normal(N)) * w).ravel()
    f = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    return x, fh, f


def replica_throughput(local_seconds, units_per_rank, world, dist=None, device=None):
    """Whole-job throughput of N independent replicas: every rank processes
    units_per_rank units; the job time is the slowest rank's (MAX all-reduce),
    so value = world * units_per_rank / max_rank_seconds."""
    import torch
    t = torch.tensor([float(local_seconds)], dtype=torch.float64, device=device)
    if dist is not None and world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return world * units_per_rank / t.item(), t.item()


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            dev = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0] or "0"
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={dev}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            c = [v.strip() for v in line.split(",")]
            if len(c) < 9:
                continue
            try:
                sm.append(float(c[1]))
                smax.append(float(c[2]))
            except ValueError:
                continue
            for nm, v in zip(names, c[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
def cpu_threads():
    """Host threads for the CPU legs: every core this process may use."""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_step(inputs, nthreads):
    """One step of the workload on the oracle, the CPU restatement of the
    reference's FP64 path (OpenMP over nthreads, scipy FFT for PFFT): trafo =
    D, F and B over all M nodes; adj = B^T over all M nodes, F^H and D^T.
    Returns the step's seconds and the seconds of each stage, split like the
    reference's timers (MATRIX_D, MATRIX_F, MATRIX_B of trafo and adj)."""
    from oracle import pnfft_oracle as O
    x, fh, f = inputs
    N, n, M, m = CFG["N"], CFG["n"], CFG["M"], CFG["m"]
    p = O.OraclePlan(N, n, m=m, flags=0, nthreads=nthreads)
    out = np.zeros(M, complex)
    acc = np.zeros(int(np.prod(p.local_N)), complex)
    t = [time.perf_counter()]
    g1 = p.trafo_D(fh, 0)
    t.append(time.perf_counter())
    grid = p.forward_F(g1)
    t.append(time.perf_counter())
    p.trafo_B(x, grid, f=out.view(np.float64), cflags=O.COMPUTE_F)
    t.append(time.perf_counter())
    g = p.adjoint_B(x, f=f.view(np.float64), cflags=O.COMPUTE_F)
    t.append(time.perf_counter())
    gh = p.adjoint_F(g)
    t.append(time.perf_counter())
    p.adjoint_D(gh, 0, acc)
    t.append(time.perf_counter())
    stages = dict(zip(["trafo_D", "trafo_F", "trafo_B", "adj_B", "adj_F", "adj_D"], np.diff(t).tolist()))
    return t[-1] - t[0], stages


def cpu_baseline(steps=1, warmup=0, inputs=None):
    """The oracle timed on the host cores over whole steps of the workload
    (all M nodes, no sampling or scaling)."""
    inputs = inputs if inputs is not None else make_inputs()
    nt = cpu_threads()
    for _ in range(warmup):
        cpu_step(inputs, nt)
    secs, stages = [], []
    for _ in range(steps):
        s, st = cpu_step(inputs, nt)
        secs.append(s)
        stages.append(st)
    M = CFG["M"]
    med = statistics.median(secs)
    stage_med = {k: statistics.median(st[k] for st in stages) for k in stages[0]}
    return {"value": M / med / 1e6, "unit": "Mpts/s", "cores": nt, "kind": "port",
            "sample": f"oracle FP64 (C + OpenMP, scipy FFT): whole trafo+adj steps of the workload, all 2^22 nodes, "
                      f"{steps} step(s), median {med:.2f} s",
            "seconds_per_step": med, "stage_seconds": stage_med}, secs


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    r, secs = cpu_baseline(steps=args.steps, warmup=args.warmup)
    v = CFG["M"] * len(secs) / sum(secs) / 1e6
    line = {"metric": METRIC, "value": v, "unit": "Mpts/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(secs) / len(secs), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "precision": "fp64", "l2": "n/a (CPU)"}, "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "Mpts/s", "cores": r["cores"], "kind": r["kind"],
                             "sample": r["sample"], "stage_seconds": r["stage_seconds"]},
            "e2e": {"value": v, "unit": "Mpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def run_gpu(args):
    import torch
    import pnfft_gb300 as P

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    N, n, M, m = CFG["N"], CFG["n"], CFG["M"], CFG["m"]
    x, fh, f = make_inputs(seed=2 + rank)
    dev = torch.device("cuda", local)
    xd = torch.tensor(x, device=dev)
    fhd = torch.tensor(fh, device=dev)
    fd = torch.tensor(f, device=dev)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)
    work_stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(work_stream)  # all library and torch work on one stream

    def device_steps(plan, K, W, fixed=False, tflags=None):
        tflags = P.COMPUTE_F if tflags is None else tflags
        out_f = torch.empty(M, dtype=torch.complex128, device=dev)
        out_g = torch.empty(M, 3, dtype=torch.complex128, device=dev) if tflags & P.COMPUTE_GRAD_F else None
        out_fh = torch.empty(int(np.prod(N)), dtype=torch.complex128, device=dev)
        s = torch.cuda.current_stream(dev)  # a dedicated stream, see run_gpu
        for _ in range(W):
            plan.trafo_device(xd, fhd, tflags, f=out_f, grad=out_g, fixed_nodes=fixed)
            plan.adj_device(xd, fd, f_hat=out_fh, fixed_nodes=fixed)
        plan.synchronize()  # collect the warm-up's stage timers before the timed steps
        barrier()
        evs = []
        stage_b = [[], []]
        for _ in range(K):
            flush.fill_(1.0)  # L2 flush between timed steps (not timed)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(s)
            plan.trafo_device(xd, fhd, tflags, f=out_f, grad=out_g, fixed_nodes=fixed)
            plan.adj_device(xd, fd, f_hat=out_fh, fixed_nodes=fixed)
            b.record(s)
            evs.append((a, b))
            plan.synchronize()
            stage_b[0].append(plan.stage_ms(False)[P.TIMER_MATRIX_B])
            stage_b[1].append(plan.stage_ms(True)[P.TIMER_MATRIX_B])
        barrier()
        ms = [a.elapsed_time(b) for a, b in evs]
        return ms, stage_b, out_f, out_fh

    # --- FP32-mixed, device resident (headline value) ---------------------
    p32 = P.Plan(N, n, m=m, precision="fp32")
    sampler = ClockSampler()
    sampler.start()
    ms, stage_b, f32_out, fh32_out = device_steps(p32, args.steps, args.warmup)
    clocks = sampler.stop()
    step_ms = sum(ms) / len(ms)
    value, _ = replica_throughput(sum(ms) * 1e-3, M * args.steps, world, dist, dev)
    value /= 1e6

    # amortised: nodes declared fixed (binning reused)
    p32f = P.Plan(N, n, m=m, precision="fp32")
    ms_fixed, _, _, _ = device_steps(p32f, max(3, args.steps // 2), 2, fixed=True)
    p32f.close()
    # the same step with COMPUTE_F | COMPUTE_GRAD_F in the trafo (analytic gradient)
    p32g = P.Plan(N, n, m=m, precision="fp32")
    ms_grad, _, _, _ = device_steps(p32g, max(3, args.steps // 2), 2, tflags=P.COMPUTE_F | P.COMPUTE_GRAD_F)
    p32g.close()
    # windows from PNFFT_PRE_CUB_PSI tables (6144 samples per cell at m=6)
    p32t = P.Plan(N, n, m=m, flags=P.PRE_CUB_PSI, precision="fp32")
    ms_tab, _, ftab, _ = device_steps(p32t, max(3, args.steps // 2), 2)
    p32t.close()

    # --- roofline of the dominant kernel (B or B^T, from the stage timers) --
    # B and B^T do 2197 complex-by-real multiply-adds per node (5 flops with the
    # weight), far above the HBM ridge: their roof is the FP32 FMA rate of the
    # device, measured here with the paired FMA (FFMA2) the kernels use
    L = P.load()
    peak_ffma2, peak_ffma = ctypes.c_double(0), ctypes.c_double(0)
    if L.pnfft_gb300_measure_fp32_fma(1, ctypes.byref(peak_ffma2)) or \
            L.pnfft_gb300_measure_fp32_fma(0, ctypes.byref(peak_ffma)):
        raise RuntimeError("FP32 FMA rate measurement failed: " + P.last_error())
    b_ms = statistics.mean(stage_b[0])
    bt_ms = statistics.mean(stage_b[1])
    kern_ms, kname = (b_ms, "interp") if b_ms >= bt_ms else (bt_ms, "spread")
    alg_bytes = M * (24 + 16) + int(np.prod(n)) * 8  # x (f64 x3) + f (c128) + grid (c64)
    alg_flops = M * (2 * m + 1) ** 3 * 5
    hbm, peak_kind = peaks()
    tflops = lambda ms_: alg_flops / (ms_ * 1e-3) / 1e12  # noqa: E731
    gbs = alg_bytes / (kern_ms * 1e-3) / 1e9
    kernels = {"interp": INTERP_KERNEL, "spread": SPREAD_KERNEL}
    roof = {"bound": "fp32", "achieved": tflops(kern_ms), "peak": peak_ffma2.value, "unit": "TFLOP/s",
            "frac": tflops(kern_ms) / peak_ffma2.value, "traffic": None, "kernel": kernels[kname],
            "kernel_ms": kern_ms,
            "peak_source": "measured in this run: independent FFMA2 chains on every SM "
                           "(pnfft_gb300_measure_fp32_fma), CUDA events",
            "peak_scalar_ffma": peak_ffma.value,
            "alg_flops_per_launch": alg_flops, "alg_bytes_per_launch": alg_bytes,
            "stage_ms": {"B": b_ms, "BT": bt_ms},
            "frac_by_kernel": {kernels["interp"]: tflops(b_ms) / peak_ffma2.value,
                               kernels["spread"]: tflops(bt_ms) / peak_ffma2.value},
            "hbm": {"achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm, "peak_source": peak_kind}}
    # the step's roofline: per stage the larger of its compulsory bytes over
    # the measured HBM bandwidth and its flops over the measured FP32 rate,
    # summed over one trafo + adj, against the measured step time
    nn, NN = int(np.prod(n)), int(np.prod(N))
    peak_f = peak_ffma2.value * 1e12
    t_stage = {
        "binning_x2": 2 * M * (24 + 16 + 4) / (hbm * 1e9),         # x in, records and permutation out
        "D": (NN * 16 + nn * 8) / (hbm * 1e9),                       # f_hat in, padded grid out
        "F_x2": 2 * (2 * 2 * nn * 8) / (hbm * 1e9),                  # two passes over the grid each way
        "B": max(alg_bytes / (hbm * 1e9), alg_flops / peak_f),
        "BT": max(alg_bytes / (hbm * 1e9), alg_flops / peak_f),
        "DT": (nn * 8 + NN * 32) / (hbm * 1e9),                      # grid in, f_hat read and written
    }
    t_roof = sum(t_stage.values())
    roof["step"] = {"t_roof_ms": 1e3 * t_roof, "t_measured_ms": step_ms, "frac": 1e3 * t_roof / step_ms,
                    "stages_roof_ms": {k: 1e3 * v for k, v in t_stage.items()},
                    "rule": "sum over stages of max(bytes / measured HBM, flops / measured FP32 FFMA2)"}
    traffic_file = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(traffic_file):
        try:
            with open(traffic_file) as fh_:
                roof["traffic"] = json.load(fh_).get(roof["kernel"])
        except Exception:
            pass

    # --- accuracy: FP32-mixed vs FP64 NDFT on 4096 nodes; adj vs FP64 path --
    sub = 4096
    pd = P.Plan(N, n, m=m, precision="fp64")
    fd_direct, _, _ = pd.trafo_device(xd[:sub].contiguous(), fhd, P.COMPUTE_F | P.COMPUTE_DIRECT)
    torch.cuda.synchronize()
    err_trafo = (torch.linalg.vector_norm(f32_out[:sub] - fd_direct) / torch.linalg.vector_norm(fd_direct)).item()

    err_tab = (torch.linalg.vector_norm(ftab[:sub] - fd_direct) / torch.linalg.vector_norm(fd_direct)).item()

    # --- FP64 plain path -----------------------------------------------------
    k64 = max(1, min(3, args.steps))
    ms64, _, f64_out, fh64_out = device_steps(pd, k64, 1)
    err_adj = (torch.linalg.vector_norm(fh32_out - fh64_out) / torch.linalg.vector_norm(fh64_out)).item()
    # the adjoint against the FP64 NDFT at 4096 random frequencies over all M
    # nodes, f_hat_k = sum_j f_j exp(+2 pi i k x_j) (torch FP64 on the GPU, a
    # check outside any timed region), beside the FP64 NFFT's own error there
    kidx = torch.tensor(np.random.default_rng(11).choice(int(np.prod(N)), 4096, replace=False), device=dev)
    kvec = torch.stack([kidx // (N[1] * N[2]) - N[0] // 2, (kidx // N[2]) % N[1] - N[1] // 2,
                        kidx % N[2] - N[2] // 2], 1).to(torch.float64)
    ndft = torch.zeros(4096, dtype=torch.complex128, device=dev)
    for c0 in range(0, 4096, 16):
        for j0 in range(0, M, 1 << 20):
            ph = (2 * np.pi) * (xd[j0:j0 + (1 << 20)] @ kvec[c0:c0 + 16].T)
            ndft[c0:c0 + 16] += (fd[j0:j0 + (1 << 20), None] * torch.polar(torch.ones_like(ph), ph)).sum(0)
    nn_ = torch.linalg.vector_norm(ndft)
    err_adj_ndft = (torch.linalg.vector_norm(fh32_out[kidx] - ndft) / nn_).item()
    err_adj_ndft64 = (torch.linalg.vector_norm(fh64_out[kidx] - ndft) / nn_).item()
    err_trafo_64 = (torch.linalg.vector_norm(f64_out[:sub] - fd_direct) / torch.linalg.vector_norm(fd_direct)).item()
    value64 = M / (statistics.mean(ms64) * 1e-3) / 1e6
    pd.close()

    # --- e2e through the C ABI on page-locked host arrays -------------------
    Nc = (ctypes.c_ssize_t * 3)(*N)
    nc = (ctypes.c_ssize_t * 3)(*n)
    xm = (ctypes.c_double * 3)(0.5, 0.5, 0.5)
    plan = L.pnfft_init_guru(3, Nc, nc, xm, m, ctypes.c_uint(P.MALLOC_F_HAT | P.GB300_FP32), P.PFFT_ESTIMATE,
                             P.MPI_COMM_WORLD)
    nodes = L.pnfft_init_nodes(M, P.MALLOC_X | P.MALLOC_F)
    hx = np.ctypeslib.as_array(ctypes.cast(L.pnfft_get_x(nodes), ctypes.POINTER(ctypes.c_double)), (M * 3,))
    hf = np.ctypeslib.as_array(ctypes.cast(L.pnfft_get_f(nodes), ctypes.POINTER(ctypes.c_double)), (2 * M,))
    hfh = np.ctypeslib.as_array(ctypes.cast(L.pnfft_get_f_hat(plan), ctypes.POINTER(ctypes.c_double)),
                                (2 * fh.size,))
    hx[:] = x.ravel()
    fh_in = fh.view(np.float64)
    f_in = f.view(np.float64)
    for _ in range(args.warmup):
        hfh[:] = fh_in
        L.pnfft_trafo(plan, nodes, P.COMPUTE_F)
        hf[:] = f_in
        L.pnfft_adj(plan, nodes, P.COMPUTE_F)
    barrier()
    e2e_s = []
    for _ in range(args.steps):
        hfh[:] = fh_in  # (re)fill inputs outside the timed region
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        L.pnfft_trafo(plan, nodes, P.COMPUTE_F)
        t1 = time.perf_counter()
        hf[:] = f_in
        t2 = time.perf_counter()
        L.pnfft_adj(plan, nodes, P.COMPUTE_F)
        t3 = time.perf_counter()
        e2e_s.append((t1 - t0) + (t3 - t2))
    barrier()
    e2e_value, _ = replica_throughput(sum(e2e_s), M * args.steps, world, dist, dev)
    e2e_value /= 1e6
    # the same calls with the nodes declared fixed (as after pnfft_precompute_psi):
    # the device copy of x and the binning are reused
    L.pnfft_gb300_nodes_set_fixed(nodes, 1)
    hfh[:] = fh_in
    L.pnfft_trafo(plan, nodes, P.COMPUTE_F)
    hf[:] = f_in
    L.pnfft_adj(plan, nodes, P.COMPUTE_F)
    e2e_fixed = []
    for _ in range(args.steps):
        hfh[:] = fh_in
        t0 = time.perf_counter()
        L.pnfft_trafo(plan, nodes, P.COMPUTE_F)
        t1 = time.perf_counter()
        hf[:] = f_in
        t2 = time.perf_counter()
        L.pnfft_adj(plan, nodes, P.COMPUTE_F)
        t3 = time.perf_counter()
        e2e_fixed.append((t1 - t0) + (t3 - t2))
    e2e_fixed_value = M / statistics.mean(e2e_fixed) / 1e6
    nfh = int(np.prod(N))
    h2d = 2 * M * 24 + nfh * 16 + M * 16
    d2h = M * 16 + nfh * 16
    L.pnfft_free_nodes(nodes, P.FREE_X | P.FREE_F)
    L.pnfft_finalize(plan, P.FREE_F_HAT)

    # trafo: binning (keys, 3 scans, scatter, tile sub-problems, line
    # sub-problems) + D + B; adj: the same binning + B^T + D^T (cuFFT not counted)
    launches_per_step = 18
    line = {"metric": METRIC, "value": value, "unit": "Mpts/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "N": list(N), "n": list(n), "M": M, "m": m,
                       "window": "kaiser_bessel", "precision": "fp32-mixed (f64 index math and deconvolution)",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "l2": "flushed between timed steps (258 MB write); inputs > L2"},
            "e2e": {"value": e2e_value, "unit": "Mpts/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "fixed_nodes_value": e2e_fixed_value,
                    "fixed_nodes_h2d_bytes_per_step": nfh * 16 + M * 16},
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clocks, "roofline": roof,
            "fp64": {"value": value64, "unit": "Mpts/s", "ms_per_step": statistics.mean(ms64),
                     "err_trafo_vs_ndft": err_trafo_64},
            "accuracy": {"fp32_trafo_rel_l2_vs_fp64_ndft_4096": err_trafo, "fp32_adj_rel_l2_vs_fp64_path": err_adj,
                         "fp32_adj_rel_l2_vs_fp64_ndft_4096_freqs_all_nodes": err_adj_ndft,
                         "fp64_nfft_adj_rel_l2_vs_fp64_ndft_4096_freqs_all_nodes": err_adj_ndft64},
            "amortised_fixed_nodes": {"value": M / (statistics.mean(ms_fixed) * 1e-3) / 1e6,
                                      "ms_per_step": statistics.mean(ms_fixed)},
            "with_grad": {"value": M / (statistics.mean(ms_grad) * 1e-3) / 1e6,
                          "ms_per_step": statistics.mean(ms_grad), "trafo_flags": "COMPUTE_F|COMPUTE_GRAD_F"},
            "pre_cub_psi": {"value": M / (statistics.mean(ms_tab) * 1e-3) / 1e6,
                            "ms_per_step": statistics.mean(ms_tab), "err_trafo_vs_ndft": err_tab}}
    if rank == 0 and world == 1 and not args.no_batch:
        line["batched"] = run_batched(P, torch, dev)
        line["particles"] = run_particles(P, torch, dev)
        line["charge_dipole"] = run_charge_dipole(P)
        line["float_api"] = run_float_api(P, x, fh, f)
    if rank == 0 and world == 1 and not args.no_cpu:
        line["cpu_baseline"] = {k: v for k, v in cpu_baseline(inputs=(x, fh, f))[0].items()
                                if k != "seconds_per_step"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_batched(P, torch, dev, steps=5):
    """Config 5: 64 FP32-mixed plans of uneven size (N_t from {16..128},
    sigma 2, M log-uniform in [1e3, 2^21], Kaiser-Bessel m = 4..6), each one
    trafo + one adj, plus 8 right-hand sides sharing one node set of 2^20
    nodes at N = 64^3.  One CUDA graph replays the whole batch; the eager loop
    over the same calls is timed beside it.  Error: FP32-mixed trafo against
    the FP64 path on 8 of the plans."""
    from pnfft_gb300.batch import Batch
    rng = np.random.default_rng(5)
    sizes = [16, 32, 48, 64, 96, 128]
    batch = Batch(dev)
    checks = []
    for i in range(64):
        N = tuple(int(v) for v in rng.choice(sizes, 3))
        M = int(round(np.exp(rng.uniform(np.log(1e3), np.log(2 ** 21)))))
        m = int(rng.integers(4, 7))
        p = P.Plan(N, m=m, precision="fp32")
        x = torch.tensor(rng.uniform(-0.5, 0.5, (M, 3)), device=dev)
        S = int(np.prod(N))
        fh = torch.tensor(rng.standard_normal(S) + 1j * rng.standard_normal(S), device=dev)
        fi = torch.tensor(rng.standard_normal(M) + 1j * rng.standard_normal(M), device=dev)
        fo = torch.empty(M, dtype=torch.complex128, device=dev)
        fho = torch.empty(S, dtype=torch.complex128, device=dev)
        batch.add_trafo(p, x, fh, fo)
        batch.add_adj(p, x, fi, fho)
        if i % 8 == 0:
            checks.append((N, m, x, fh, fo))
    Nk, Mk = (64, 64, 64), 2 ** 20
    pk = P.Plan(Nk, m=6, precision="fp32")
    xk = torch.tensor(rng.uniform(-0.5, 0.5, (Mk, 3)), device=dev)
    for _ in range(8):
        fh = torch.tensor(rng.standard_normal(64 ** 3) + 1j * rng.standard_normal(64 ** 3), device=dev)
        fi = torch.tensor(rng.standard_normal(Mk) + 1j * rng.standard_normal(Mk), device=dev)
        batch.add_trafo(pk, xk, fh, torch.empty(Mk, dtype=torch.complex128, device=dev))
        batch.add_adj(pk, xk, fi, torch.empty(64 ** 3, dtype=torch.complex128, device=dev))
    choice = batch.autotune(reps=1)
    batch.capture()

    def timed(fn):
        fn()
        batch.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(batch.stream)
        for _ in range(steps):
            fn()
        b.record(batch.stream)
        b.synchronize()
        return a.elapsed_time(b) / steps

    ms_graph = timed(batch.run)
    ms_eager = timed(batch.run_eager)
    branches = len(batch.side)
    sides = batch.side
    batch.side = sides[:1]  # the same graph with every plan on one stream
    batch.graph = None
    ms_graph_1 = timed(batch.run)
    batch.side = sides
    batch.fused = True  # one batched convolution launch per direction and cutoff
    batch.graph = None
    ms_fused = timed(batch.run)
    fused_calls, fused_launches = batch.fused_stats()
    ms_fused_eager = timed(batch.run_eager)
    nodes = batch.nodes()
    errs = []
    for N, m, x, fh, fo in checks:
        q = P.Plan(N, m=m, precision="fp64")
        ref, _, _ = q.trafo_device(x, fh, P.COMPUTE_F)
        torch.cuda.synchronize()
        errs.append((torch.linalg.vector_norm(fo - ref) / torch.linalg.vector_norm(ref)).item())
        q.close()
    return {"value": nodes / (ms_graph * 1e-3) / 1e6, "unit": "Mpts/s", "ms_per_replay": ms_graph,
            "eager_value": nodes / (ms_eager * 1e-3) / 1e6, "eager_ms": ms_eager, "graph_branches": branches,
            "one_branch_value": nodes / (ms_graph_1 * 1e-3) / 1e6, "one_branch_ms": ms_graph_1,
            "fused_value": nodes / (ms_fused * 1e-3) / 1e6, "fused_ms": ms_fused,
            "fused_eager_value": nodes / (ms_fused_eager * 1e-3) / 1e6,
            "fused_calls": fused_calls, "fused_launches": fused_launches,
            "plans": 65, "rhs_sharing_nodes": 8, "node_transforms_per_replay": nodes,
            "per_node_kernels_chosen": sum(1 for c in choice.values() if c[0] == 1),
            "tunings_chosen": _count_tunings(choice),
            "max_rel_err_fp32_vs_fp64_trafo": max(errs),
            "workload": "64 plans N_t in {16..128}, M log-uniform [1e3, 2^21], KB m 4..6, trafo+adj each; "
                        "8 RHS on one node set M=2^20 at N=64^3; one CUDA graph, plans on 4 concurrent branches"}


def _count_tunings(choice):
    """{"interp method/spread method/line sub-problem nodes": plans} over a batch's choices."""
    out = {}
    for c in choice.values():
        key = "/".join(str(v) for v in c[2])
        out[key] = out.get(key, 0) + 1
    return out


def run_float_api(P, x, fh, f, steps=3):
    """The single-precision API pnfftf_* end to end on the bench workload
    (N=128^3, n=256^3, M=2^22, Kaiser-Bessel m=6): float host arrays
    (page-locked, PNFFT_MALLOC_*), one pnfftf_trafo (COMPUTE_F) + one
    pnfftf_adj per step, each call copying float arrays to the GPU, widening
    and rounding there.  Wall-clock time of the two calls; the float results
    against the double API's FP32-mixed results on the same (float) inputs."""
    import ctypes
    L = P.load()
    Pp, U = ctypes.c_void_p, ctypes.c_uint
    for k, (r, a) in {"pnfftf_init_guru": (Pp, [ctypes.c_int, Pp, Pp, Pp, ctypes.c_int, U, U, ctypes.c_int]),
                      "pnfftf_init_nodes": (Pp, [ctypes.c_ssize_t, U]), "pnfftf_get_x": (Pp, [Pp]),
                      "pnfftf_get_f": (Pp, [Pp]), "pnfftf_get_f_hat": (Pp, [Pp]),
                      "pnfftf_trafo": (None, [Pp, Pp, U]), "pnfftf_adj": (None, [Pp, Pp, U]),
                      "pnfftf_finalize": (None, [Pp, U]), "pnfftf_free_nodes": (None, [Pp, U])}.items():
        getattr(L, k).restype = r
        getattr(L, k).argtypes = a
    N, n, M, m = CFG["N"], CFG["n"], CFG["M"], CFG["m"]
    Nc, nc = (ctypes.c_ssize_t * 3)(*N), (ctypes.c_ssize_t * 3)(*n)
    p = L.pnfftf_init_guru(3, Nc, nc, (ctypes.c_float * 3)(0.5, 0.5, 0.5), m, P.MALLOC_F_HAT, P.PFFT_ESTIMATE,
                           P.MPI_COMM_WORLD)
    nd = L.pnfftf_init_nodes(M, P.MALLOC_X | P.MALLOC_F)
    fv = lambda ptr, k: np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_float)), (k,))  # noqa: E731
    hx, hf, hfh = fv(L.pnfftf_get_x(nd), 3 * M), fv(L.pnfftf_get_f(nd), 2 * M), fv(L.pnfftf_get_f_hat(p), 2 * fh.size)
    x32, fh32, f32 = x.astype(np.float32), fh.astype(np.complex64), f.astype(np.complex64)
    hx[:] = x32.ravel()
    times = []
    for it in range(steps + 1):
        hfh[:] = fh32.view(np.float32)
        t0 = time.perf_counter()
        L.pnfftf_trafo(p, nd, P.COMPUTE_F)
        t1 = time.perf_counter()
        out_f = hf.copy().view(np.complex64)
        hf[:] = f32.view(np.float32)
        t2 = time.perf_counter()
        L.pnfftf_adj(p, nd, P.COMPUTE_F)
        t3 = time.perf_counter()
        if it:
            times.append((t1 - t0) + (t3 - t2))
    out_fh = hfh.copy().view(np.complex64)
    L.pnfftf_free_nodes(nd, P.FREE_X | P.FREE_F)
    L.pnfftf_finalize(p, P.FREE_F_HAT)
    # the double API, FP32-mixed, on the same float-rounded inputs
    q = P.Plan(N, n, m=m, precision="fp32")
    xd = x32.astype(np.float64)
    ref_f = q.trafo(xd, fh32.astype(np.complex128))[0]
    ref_fh = q.adj(xd, f32.astype(np.complex128))
    q.close()
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))  # noqa: E731
    ms = 1e3 * statistics.mean(times)
    return {"value": M / (ms * 1e-3) / 1e6, "unit": "Mpts/s", "ms_per_step": ms,
            "h2d_bytes_per_step": 2 * M * 12 + fh.size * 8 + M * 8, "d2h_bytes_per_step": M * 8 + fh.size * 8,
            "rel_diff_f_vs_double_api": rel(out_f, ref_f), "rel_diff_f_hat_vs_double_api": rel(out_fh, ref_fh),
            "workload": "pnfftf_trafo + pnfftf_adj, float host arrays (page-locked), N=128^3, n=256^3, M=2^22, "
                        "KB m=6; conversions on the GPU"}


def run_particles(P, torch, dev, steps=3):
    """Config 3: clustered real charges, c2r.  M = 2^21 (80% uniform, 20% from
    64 Gaussian clusters of width 0.01, wrapped), weights +-1 with zero sum,
    N = 64^3, n = 128^3, m = 5, Gaussian and B-spline windows, FP32-mixed.
    A step is adj (charges to grid) + trafo with COMPUTE_F | COMPUTE_GRAD_F,
    with the analytic (default) or the ik gradient (PNFFT_DIFF_IK).  Errors:
    f_hat against the FP64 path, and the trafo against the FP64 NDFT on 4096
    nodes for the same f_hat."""
    from pnfft_gb300.particles import charges_c2r
    rng = np.random.default_rng(3)
    N, m, M = (64, 64, 64), 5, 2 ** 21
    mc = M // 5
    x = rng.uniform(-0.5, 0.5, (M, 3))
    centres = rng.uniform(-0.5, 0.5, (64, 3))
    x[:mc] = centres[rng.integers(0, 64, mc)] + 0.01 * rng.standard_normal((mc, 3))
    x = np.mod(x + 0.5, 1.0) - 0.5
    q = np.where(np.arange(M) % 2 == 0, 1.0, -1.0)
    rng.shuffle(q)
    xd, qd = torch.tensor(x, device=dev), torch.tensor(q, device=dev)
    s = torch.cuda.current_stream(dev)
    out = {}
    for win, wflag in (("gaussian", P.WINDOW_GAUSSIAN), ("bspline", P.WINDOW_BSPLINE)):
        for grad, gflag in (("analytic", 0), ("ik", P.DIFF_IK)):
            p = P.Plan(N, m=m, flags=wflag | gflag, c2r=True, precision="fp32")

            def timed():
                charges_c2r(p, xd, qd)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(s)
                for _ in range(steps):
                    res = charges_c2r(p, xd, qd)
                b.record(s)
                b.synchronize()
                return a.elapsed_time(b) / steps, res

            ms_default, _ = timed()
            fh0 = charges_c2r(p, xd, qd)[0]
            tuning = p.autotune_device(xd, fh0, P.COMPUTE_F | P.COMPUTE_GRAD_F, P.COMPUTE_F)
            ms, (fh, phi, gphi) = timed()
            ref = P.Plan(N, m=m, flags=wflag | gflag, c2r=True, precision="fp64")
            fh64 = ref.adj_device(xd, qd)
            sub = 4096
            xs = xd[:sub].contiguous()
            phid, gphid, _ = ref.trafo_device(xs, fh, P.COMPUTE_F | P.COMPUTE_GRAD_F | P.COMPUTE_DIRECT)
            gphid = -gphid  # the reference's c2r NDFT returns minus the gradient (ndft-parallel.c:530-532)
            phi64, gphi64, _ = ref.trafo_device(xs, fh, P.COMPUTE_F | P.COMPUTE_GRAD_F)
            torch.cuda.synchronize()
            rel = lambda u, v: (torch.linalg.vector_norm(u - v) / torch.linalg.vector_norm(v)).item()  # noqa: E731
            out[f"{win}_{grad}"] = {"value": M / (ms * 1e-3) / 1e6, "unit": "Mpts/s", "ms_per_step": ms,
                                    "tuning": list(tuning), "ms_per_step_default_tuning": ms_default,
                                    "err_f_hat_vs_fp64": rel(fh, fh64),
                                    "err_phi_vs_fp64_ndft_4096": rel(phi[:sub], phid),
                                    "err_grad_vs_fp64_ndft_4096": rel(gphi[:sub], gphid),
                                    "window_aliasing_phi_fp64_nfft_vs_ndft": rel(phi64, phid),
                                    "window_aliasing_grad_fp64_nfft_vs_ndft": rel(gphi64, gphid)}
            p.close()
            ref.close()
    out["workload"] = ("c2r, N=64^3, n=128^3, M=2^21 (20% in 64 clusters, sigma 0.01), charges +-1, m=5; "
                       "step = adj + trafo(F|GRAD_F), FP32-mixed; kernels chosen by pnfft_gb300_autotune "
                       "(tuning = interp method, spread method, nodes per line sub-problem)")
    return out


def run_charge_dipole(P, steps=3):
    """The charge/dipole sequence of the reference's particle test
    (tests/check_charge_dipole.c:151-233), c2c, FP32-mixed: N = 64^3,
    n = 128^3, Kaiser-Bessel m = 5, 2^20 charges and 2^18 dipoles uniform in
    [-0.5, 0.5)^3, host node arrays.  One pnfft_gb300_charge_dipole call
    (each node set copied and binned once, f_hat on the GPU throughout)
    against the same four calls through pnfft_adj / pnfft_trafo followed by
    the energies and forces on the host (numpy).  Throughput in particles per
    second; error of the energies against the FP64 call."""
    import ctypes
    from pnfft_gb300.particles import HostNodes, charge_dipole_host
    L = P.load()
    rng = np.random.default_rng(7)
    N, m, Mc, Md = (64, 64, 64), 5, 1 << 20, 1 << 18
    xc, xd = rng.uniform(-0.5, 0.5, (Mc, 3)), rng.uniform(-0.5, 0.5, (Md, 3))
    q = rng.standard_normal(Mc) + 0j
    mu = rng.standard_normal((Md, 3)) + 0j
    out = {}
    for prec in ("fp32", "fp64"):
        p = P.Plan(N, m=m, precision=prec)
        ch, di = HostNodes(Mc), HostNodes(Md)

        def fill():
            ch.x[:] = xc
            ch.f[:] = q
            di.x[:] = xd
            di.grad_f[:] = mu

        fill()
        energy, _, _ = charge_dipole_host(p, ch, di)  # warm-up
        fused = []
        for _ in range(steps if prec == "fp32" else 1):
            fill()
            t0 = time.perf_counter()
            energy, _, _ = charge_dipole_host(p, ch, di)
            fused.append(time.perf_counter() - t0)
        out[prec] = energy.copy()
        if prec == "fp32":
            fh = np.zeros(int(np.prod(N)), np.complex128)
            L.pnfft_set_f_hat(fh.ctypes.data, p._p)
            sep = []
            for _ in range(steps + 1):
                fill()
                t0 = time.perf_counter()
                L.pnfft_adj(p._p, ch.handle, P.COMPUTE_F)
                buf = fh.copy()
                L.pnfft_adj(p._p, di.handle, P.COMPUTE_GRAD_F)
                fh += buf
                L.pnfft_trafo(p._p, ch.handle, P.COMPUTE_F | P.COMPUTE_GRAD_F)
                L.pnfft_trafo(p._p, di.handle, P.COMPUTE_GRAD_F | P.COMPUTE_HESSIAN_F)
                # the energies and forces of the reference's test, on the host
                e_c, f_c = q * ch.f, ch.grad_f * q[:, None]
                e_d = (di.grad_f * mu).sum(1)
                h = di.hessian_f
                f_d = np.stack([h[:, 0] * mu[:, 0] + h[:, 1] * mu[:, 1] + h[:, 2] * mu[:, 2],
                                h[:, 1] * mu[:, 0] + h[:, 3] * mu[:, 1] + h[:, 4] * mu[:, 2],
                                h[:, 2] * mu[:, 0] + h[:, 4] * mu[:, 1] + h[:, 5] * mu[:, 2]], 1)
                sep.append(time.perf_counter() - t0)
            del e_c, f_c, e_d, f_d
            sep = sep[1:]
            t_fused = statistics.median(fused)
            t_sep = statistics.median(sep)
        ch.close()
        di.close()
        p.close()
    err = float(np.linalg.norm(out["fp32"] - out["fp64"]) / np.linalg.norm(out["fp64"]))
    return {"value": (Mc + Md) / t_fused / 1e6, "unit": "Mparticles/s", "ms_per_call": 1e3 * t_fused,
            "four_calls_value": (Mc + Md) / t_sep / 1e6, "four_calls_ms": 1e3 * t_sep,
            "err_energy_fp32_vs_fp64": err,
            "workload": "c2c charge/dipole sequence, N=64^3, n=128^3, KB m=5, 2^20 charges + 2^18 dipoles, "
                        "host arrays, FP32-mixed; energies and forces included"}


def run_profile_case():
    import torch
    import pnfft_gb300 as P
    N, n, M, m = CFG["N"], CFG["n"], CFG["M"], CFG["m"]
    x, fh, f = make_inputs()
    xd, fhd, fd = (torch.tensor(a, device="cuda") for a in (x, fh, f))
    p = P.Plan(N, n, m=m, precision="fp32")
    for _ in range(2):
        out, _, _ = p.trafo_device(xd, fhd, P.COMPUTE_F)
        p.adj_device(xd, fd)
    p.synchronize()
    print("profile case done", float(out.abs().sum()))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-plans (CUDA graph) row")
    ap.add_argument("--profile", action="store_true",
                    help="one warm-up and one FP32-mixed trafo+adj of the workload, for ncu (no timing output)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.profile:
        run_profile_case()
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
