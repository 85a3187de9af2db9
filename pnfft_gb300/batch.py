"""Batches of transforms replayed as one CUDA graph.

A batch is a list of transforms on device-resident torch tensors:
- many plans of uneven sizes N and node counts M;
- several right-hand sides that share one node set (the same plan and the
  same x, different f_hat / f).

``Batch`` runs every item once, eagerly, so that the first call allocates
each plan's grid, FFT plan, window tables and node binning. The node sets
are declared fixed, so the binning is computed once and reused. It can then
pick each plan's convolution kernels by timing them (``autotune``: the line
kernels, the FP32-mixed tile kernels and the one-thread-per-node kernels,
which win for small M on large grids). Finally it captures all items
into a single CUDA graph, the plans spread over a few concurrent branches
(streams) so that small plans do not leave the GPU idle one after another.
``run()`` replays the whole batch with one graph launch, so the per-call host work of the C library (argument
checks, stream and pointer setup, about 50 launches per item) is paid once
at capture.

The captured graph keeps the device pointers of the items: refill the same
tensors in place between replays.
"""
import torch

from . import COMPUTE_F, Plan, _check, _stream_handle, load  # noqa: F401  (Plan for type references in docs)

__all__ = ["Batch"]


class Batch:
    """streams: the number of branches the plans are spread over (all items of
    one plan stay on one branch, in the order they were added); branches run
    concurrently, in eager runs and in the captured graph.  fused: the
    branches run inside a pnfft_gb300 batch, so that the convolutions of the
    small calls that qualify (FP32-mixed, f alone, line kernels) run as one
    launch per direction and cutoff; the items must be independent (no item
    reads what another writes)."""

    def __init__(self, device=None, streams=4, fused=False):
        self.fused = bool(fused)
        self.items = []
        self.device = torch.device(device or "cuda")
        self.stream = torch.cuda.Stream(self.device)
        self.side = [torch.cuda.Stream(self.device) for _ in range(max(1, int(streams)))]
        self.graph = None
        self.choice = {}

    # -- building -------------------------------------------------------------
    def add_trafo(self, plan, x, f_hat, f, compute_flags=COMPUTE_F, grad=None, hess=None):
        """f (and grad / hess) = trafo(f_hat) at nodes x, all CUDA tensors."""
        self.items.append(("trafo", plan, x, f_hat, f, grad, hess, compute_flags))
        self.graph = None

    def add_adj(self, plan, x, f, f_hat, compute_flags=COMPUTE_F, grad=None):
        """f_hat = adj(f) (and grad inputs with COMPUTE_GRAD_F) at nodes x."""
        self.items.append(("adj", plan, x, f_hat, f, grad, None, compute_flags))
        self.graph = None

    def nodes(self):
        """Total node count over the items (one trafo or adj each)."""
        return sum(int(it[2].shape[0]) for it in self.items)

    # -- execution ------------------------------------------------------------
    def _run_item(self, it):
        kind, plan, x, f_hat, f, grad, hess, flags = it
        if kind == "trafo":
            plan.trafo_device(x, f_hat, flags, f=f, grad=grad, hess=hess, fixed_nodes=True)
        else:
            plan.adj_device(x, f, grad, flags, f_hat=f_hat, fixed_nodes=True)

    def _branches(self):
        """The items split into one list per branch: plans by decreasing node
        count, each to the branch with the fewest nodes so far."""
        plans = self._plans()
        load = [sum(int(it[2].shape[0]) for it in self.items if it[1] is p) for p in plans]
        tot = [0] * len(self.side)
        where = {}
        for k in sorted(range(len(plans)), key=lambda k: -load[k]):
            b = min(range(len(tot)), key=tot.__getitem__)
            where[id(plans[k])] = b
            tot[b] += load[k]
        out = [[] for _ in self.side]
        for it in self.items:
            out[where[id(it[1])]].append(it)
        return out

    def _run_branches(self):
        """Fork the branches from the batch stream, run each branch's items on
        its stream, join them back."""
        branches = self._branches()
        for s, items in zip(self.side, branches):
            if not items:
                continue
            s.wait_stream(self.stream)
            with torch.cuda.stream(s):
                for it in items:
                    self._run_item(it)
        for s, items in zip(self.side, branches):
            if items:
                self.stream.wait_stream(s)

    def _run_fused(self):
        """The branches inside pnfft_gb300_batch_begin / _end on the batch
        stream: the FP32-mixed f-only line convolutions of the calls too small
        to fill the GPU run as one launch per direction and cutoff once the
        branches have joined; the larger calls run on their branches."""
        L = load()
        L.pnfft_gb300_clear_error()
        _check(L.pnfft_gb300_batch_begin(_stream_handle(self.stream)), "pnfft_gb300_batch_begin")
        try:
            self._run_branches()
        finally:
            rc = L.pnfft_gb300_batch_end()
        _check(rc, "pnfft_gb300_batch_end")

    def fused_stats(self):
        """(calls deferred, batched convolution launches) of the last fused run."""
        import ctypes
        a, b = ctypes.c_int(0), ctypes.c_int(0)
        _check(load().pnfft_gb300_batch_stats(ctypes.byref(a), ctypes.byref(b)), "pnfft_gb300_batch_stats")
        return a.value, b.value

    def _run_all(self):
        if self.fused:
            self._run_fused()
        else:
            self._run_branches()

    def run_eager(self):
        """Run the items without a graph (branches concurrently, or fused);
        ordered after the work on the batch stream and before what follows on
        it."""
        self._run_all()

    def _time_plan(self, plan, reps):
        items = [it for it in self.items if it[1] is plan]
        with torch.cuda.stream(self.stream):
            for it in items:
                self._run_item(it)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(self.stream)
            for _ in range(reps):
                for it in items:
                    self._run_item(it)
            b.record(self.stream)
        b.synchronize()
        return a.elapsed_time(b) / reps

    def autotune(self, reps=3):
        """Per plan, on the plan's own items: pnfft_gb300_autotune on the nodes
        of the plan's first item (with the flags of its first trafo and first
        adjoint) picks the kernel family of each direction and the
        line sub-problem size ("auto"); that tuning is then timed against the
        one-thread-per-node kernels (method 1) on all of the plan's items and
        the faster kept.  choice[id(plan)] = (winner, {candidate: ms per
        replay of the plan's items}, tuning())."""
        for p in self._plans():
            mine = [it for it in self.items if it[1] is p]
            tr = next((it for it in mine if it[0] == "trafo"), None)
            ad = next((it for it in mine if it[0] == "adj"), None)
            x, f_hat = mine[0][2], mine[0][3]
            auto = p.autotune_device(x, f_hat, tr[7] if tr else 0, ad[7] if ad else 0, reps=1)
            t = {"auto": self._time_plan(p, reps)}
            p.set_conv_method(1)
            t[1] = self._time_plan(p, reps)
            best = min(t, key=t.get)
            if best == "auto":
                p.set_tuning(auto)
            self.choice[id(p)] = (best, t, p.tuning())
        self.graph = None
        return self.choice

    def _plans(self):
        plans = []
        for it in self.items:
            if all(it[1] is not p for p in plans):
                plans.append(it[1])
        return plans

    def capture(self):
        """Warm every item up, then capture all of them into one CUDA graph."""
        self.run_eager()
        for p in self._plans():
            p.synchronize()  # also recycles the stage-timer events of the eager calls
        self.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=self.stream, capture_error_mode="thread_local"):
            self._run_all()
        self.graph = g
        return g

    def run(self):
        """Replay the captured batch (captures it first if needed)."""
        if self.graph is None:
            self.capture()
        with torch.cuda.stream(self.stream):  # replay() launches on the current stream
            self.graph.replay()

    def synchronize(self):
        for s in self.side:
            s.synchronize()
        self.stream.synchronize()
