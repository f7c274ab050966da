"""Batched solves of many independent wave instances of uneven sizes.

The reference solves such families as separate processes farmed out by MPI
(vary_wave.py:7-43).  Here all instances share packed device arrays and one
mixed-precision Newton solve of the whole batch is a fixed sequence of
launches -- per epoch one right-hand-side pass over every cell (FP64 only on
boundary cells) and one persistent FP32 forward-substitution launch that
pulls instances from a work queue, then one FP64 write of the solution --
captured once into a CUDA graph and replayed.
"""
import ctypes

import numpy as np
import torch

from . import _capi, autotune
from ._capi import call, ptr, stream_handle


def _align32(n):
    """Instance starts: 32 elements (128 bytes FP32, 256 bytes FP64), so
    no cache line holds two instances' data and vector accesses stay
    aligned."""
    return (n + 31) // 32 * 32


class WaveBatch:
    """Packed device state of many wave instances.

    ``instances``: list of dicts with nt, nx, dt, dx, c and the boundary
    arrays init_u, init_ut [nx], left_u, right_u [nt] (as WaveOperator).
    """

    def __init__(self, instances, device="cuda"):
        _capi.load()
        self.device = torch.device(device)
        self.n = len(instances)
        if self.n < 1:
            raise ValueError("empty batch")
        descs = (_capi.OdilWaveInstance * self.n)()
        off = offx = offt = 0
        self.offsets, self.shapes = [], []
        bcx_u, bcx_ut, bct_l, bct_r = [], [], [], []
        for d, inst in zip(descs, instances):
            nt, nx = int(inst["nt"]), int(inst["nx"])
            d.nt, d.nx = nt, nx
            d.dt, d.dx, d.c = float(inst["dt"]), float(inst["dx"]), float(inst["c"])
            d.offset, d.offset_x, d.offset_t = off, offx, offt
            self.offsets.append(off)
            self.shapes.append((nt, nx))
            off = _align32(off + nt * nx)
            offx += nx
            offt += nt
            bcx_u.append(np.asarray(inst["init_u"], np.float64))
            bcx_ut.append(np.asarray(inst["init_ut"], np.float64))
            bct_l.append(np.asarray(inst["left_u"], np.float64))
            bct_r.append(np.asarray(inst["right_u"], np.float64))
        self.total = off
        self.max_nx = max(s[1] for s in self.shapes)
        dev = self.device
        raw = bytes(descs)
        self.desc = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(dev)
        self.bc = [torch.as_tensor(np.concatenate(a), device=dev)
                   for a in (bcx_u, bcx_ut, bct_l, bct_r)]
        call("odil_wave_batch_setup", ptr(self.desc), self.n, stream_handle())
        # Largest instances first: the work queue then balances the tail.
        order = np.argsort([-s[0] * s[1] for s in self.shapes], kind="stable")
        self.order = torch.as_tensor(order.astype(np.int32), device=dev)
        b = _capi.OdilWaveBatch()
        b.ninst, b.max_nx, b.total_cells = self.n, self.max_nx, self.total
        b.inst, b.order = self.desc.data_ptr(), self.order.data_ptr()
        b.init_u, b.init_ut, b.left_u, b.right_u = [t.data_ptr() for t in self.bc]
        nts = np.array([sh[0] for sh in self.shapes], np.int64)
        self.row_inst = torch.as_tensor(
            np.repeat(np.arange(self.n, dtype=np.int32), nts), device=dev)
        b.row_inst, b.total_rows = self.row_inst.data_ptr(), int(nts.sum())
        nbnd = np.array([min(nt, 2) * nx + max(nt - 2, 0) * min(nx, 2)
                         for nt, nx in self.shapes], np.int64)
        self.bnd_off = torch.as_tensor(
            np.concatenate([[0], np.cumsum(nbnd)[:-1]]).astype(np.int64),
            device=dev)
        b.bnd_off, b.total_bnd = self.bnd_off.data_ptr(), int(nbnd.sum())
        self.b = b
        kw64 = dict(dtype=torch.float64, device=dev)
        kw32 = dict(dtype=torch.float32, device=dev)
        self.u = torch.zeros(self.total, **kw64)
        self.ub = torch.zeros(self.total, **kw64)
        self.rhs = torch.zeros(self.total, **kw32)
        self.d = torch.zeros(self.total, **kw32)
        self.hi = torch.zeros(self.total, **kw32)
        self.lo = torch.zeros(self.total, **kw32)
        self.ws = torch.zeros(256, dtype=torch.uint8, device=dev)
        # Work queue of the persistent whole-solve kernel (left zeroed by it).
        self.ws_solve = torch.zeros(256, dtype=torch.uint8, device=dev)
        self.march_cfg = None
        self.graph = None
        # Fused loss + gradient of all instances: FP32 boundary data and the
        # work-item tables (the kernel's items per instance, instance by
        # instance).
        self.bc32 = [t.float() for t in self.bc]
        lib = _capi.load()
        tiles = [int(lib.odil_wave_batch_loss_grad_items(nt, nx))
                 for nt, nx in self.shapes]
        self.ntiles = int(sum(tiles))
        self.tile_start = torch.as_tensor(
            np.concatenate([[0], np.cumsum(tiles)]).astype(np.int64),
            device=dev)
        self.tile_inst = torch.as_tensor(
            np.repeat(np.arange(self.n, dtype=np.int32), tiles), device=dev)
        self.lg_partials = torch.zeros(self.ntiles, dtype=torch.float64,
                                       device=dev)
        self.loss_inst = torch.zeros(self.n, dtype=torch.float64, device=dev)
        self.loss_total = torch.zeros(1, dtype=torch.float64, device=dev)

    # -- launches -------------------------------------------------------------
    def update_residual(self, u, d, u_out, rhs):
        call("odil_wave_batch_update_residual_mixed", ctypes.byref(self.b),
             ptr(u), ptr(d), ptr(u_out if d is not None else None), ptr(rhs),
             stream_handle())

    def initial_rhs(self, rhs):
        call("odil_wave_batch_initial_rhs_mixed", ctypes.byref(self.b), ptr(rhs),
             stream_handle())

    def pair_residual(self, hi, lo, rhs):
        call("odil_wave_batch_pair_residual_mixed", ctypes.byref(self.b), ptr(hi),
             ptr(lo), ptr(rhs), stream_handle())

    def march(self, rhs, x, cfg=None):
        cfg = cfg or self.march_cfg or autotune.default_batch_march(self.max_nx)
        call("odil_wave_batch_march_f32", ctypes.byref(self.b), ptr(rhs), ptr(x),
             cfg["threads"], cfg["cpt"], cfg["pf"], cfg["blocks_per_sm"],
             ptr(self.ws), self.ws.numel(), stream_handle())

    def loss_grad(self, u32, grad32):
        """Per-instance losses mean(f_i^2) (self.loss_inst), their sum
        (returned, a device scalar) and the fused adjoint gradients
        (2/N_i) J_i^T f_i into grad32, for the packed FP32 fields u32; one
        launch over all instances plus one small reduction."""
        call("odil_wave_batch_loss_grad_f32", ctypes.byref(self.b),
             ptr(self.tile_start), ptr(self.tile_inst), self.ntiles,
             *[ptr(t) for t in self.bc32],
             ptr(u32), ptr(grad32), ptr(self.lg_partials), ptr(self.loss_inst),
             ptr(self.loss_total), stream_handle())
        return self.loss_total, grad32

    def lbfgs_warm_start(self, iters=20, m=10):
        """The FP32 fused-adjoint L-BFGS stage of the batch: L-BFGS on the
        packed vector for the sum of the instance losses (the instances are
        independent, so its minimisers are each instance's), from u = 0;
        returns the FP32 iterate and the optimizer info."""
        from .optimizer import LbfgsOptimizer
        grad = torch.empty(self.total, dtype=torch.float32, device=self.device)

        def lg(x, epoch):
            loss, g = self.loss_grad(x, grad)
            return loss, g, [loss]

        x0 = torch.zeros(self.total, dtype=torch.float32, device=self.device)
        return LbfgsOptimizer(m=m, graph=True).run_device(x0, lg,
                                                          epochs=iters)

    def refine(self, u0, epochs=2):
        """Mixed-precision Newton epochs from the FP64 iterate u0 (FP64
        residual and update, FP32 forward substitution): self.u holds the
        result."""
        self.u.copy_(u0)
        u, ub = self.u, self.ub
        self.update_residual(u, None, None, self.rhs)
        for _ in range(epochs):
            self.march(self.rhs, self.d)
            self.update_residual(u, self.d, ub, self.rhs)
            u, ub = ub, u
        if u is not self.u:
            self.u.copy_(u)
        return self.u

    def tune(self, cache=True):
        """Chooses the persistent march's launch shape by timing candidates
        on this batch (cached per device and batch size class)."""
        self.initial_rhs(self.rhs)
        self.march_cfg = autotune.tune_batch_march(self, cache=cache)
        return self.march_cfg

    def solve_mixed(self, epochs=2):
        """u <- mixed-precision Newton solution from u = 0 (all instances).

        The iterate is kept as FP32 corrections hi + lo: the first
        right-hand side needs FP64 work on boundary cells only, later ones
        come from the float-pair residual, and one pass writes u in FP64."""
        if epochs < 1:
            self.u.zero_()
            return self.u
        self.initial_rhs(self.rhs)
        self.march(self.rhs, self.hi)
        have_lo = False
        for _ in range(1, epochs):
            self.pair_residual(self.hi, self.lo if have_lo else None, self.rhs)
            if have_lo:
                self.march(self.rhs, self.d)
                call("odil_axpby_f32", ptr(self.lo), ptr(self.lo), ptr(self.d),
                     self.total, 1.0, 1.0, stream_handle())
            else:
                self.march(self.rhs, self.lo)
                have_lo = True
        call("odil_pair_to_f64", ptr(self.hi), ptr(self.lo if have_lo else None),
             ptr(self.u), self.total, stream_handle())
        return self.u

    def tune_persistent(self, epochs=2, per_sm=(1, 2, 3, 4), reps=3):
        """Chooses the launch shape of the persistent whole-solve launch
        (columns per thread, ring depth, blocks per SM) by timing every
        candidate that fits (CUDA events); keeps the fastest in
        self.persistent_cfg and returns {"cpt<c>_pf<p>_bps<b>": ms}."""
        times, cfgs = {}, {}
        for cpt in (1, 2, 4):
            threads = max(32, ((self.max_nx + cpt - 1) // cpt + 31) // 32 * 32)
            if threads > (1024 if cpt == 1 else 512):
                continue
            for pf in ((8, 16) if cpt == 1 else (8,)):
                for b in per_sm:
                    if b * threads > 2048:
                        continue
                    cfg = {"threads": threads, "cpt": cpt, "pf": pf,
                           "blocks_per_sm": int(b)}
                    try:
                        self.solve_persistent(epochs, cfg=cfg)
                    except _capi.OdilError:
                        continue
                    torch.cuda.synchronize(self.device)
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record()
                    for _ in range(reps):
                        self.solve_persistent(epochs, cfg=cfg)
                    e1.record()
                    e1.synchronize()
                    key = "cpt%d_pf%d_bps%d" % (cpt, pf, b)
                    times[key] = e0.elapsed_time(e1) / reps
                    cfgs[key] = cfg
        if not times:
            raise _capi.OdilError("no launch shape of the persistent solve "
                                  "fits max_nx %d" % self.max_nx)
        self.persistent_cfg = cfgs[min(times, key=times.get)]
        return times

    def solve_persistent(self, epochs=2, cfg=None):
        """u <- the same mixed Newton as solve_mixed (bitwise), in ONE
        persistent launch: each block solves whole instances from the work
        queue, forming each march's right-hand side inside the march (see
        odil_wave_batch_solve_mixed)."""
        if epochs < 1:
            self.u.zero_()
            return self.u
        cfg = (cfg or getattr(self, "persistent_cfg", None) or
               autotune.default_batch_solve(self.max_nx))
        call("odil_wave_batch_solve_mixed", ctypes.byref(self.b), int(epochs),
             ptr(self.rhs), ptr(self.hi), ptr(self.lo), ptr(self.u),
             cfg["threads"], cfg["cpt"], cfg["pf"], cfg["blocks_per_sm"],
             ptr(self.ws_solve), self.ws_solve.numel(), stream_handle())
        return self.u

    def capture(self, epochs=2):
        """Captures solve_mixed into a CUDA graph (replay with .replay())."""
        if self.march_cfg is None:
            self.march_cfg = autotune.default_batch_march(self.max_nx)
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.solve_mixed(epochs)  # warm-up outside the graph
        torch.cuda.current_stream(self.device).wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            self.solve_mixed(epochs)
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()
        return self.u

    def unpack(self, u=None):
        u = self.u if u is None else u
        host = u.cpu().numpy()
        return [host[o:o + s[0] * s[1]].reshape(s)
                for o, s in zip(self.offsets, self.shapes)]


def shard_instances(costs, rank, world):
    """Indices of the instances rank `rank` of `world` solves.

    Instances are independent (no exchange between them), so the batch
    shards with no collective on the data path: longest-processing-time
    first, each instance to the currently lightest rank (deterministic, every
    rank computes the same assignment)."""
    if not 0 <= rank < world:
        raise ValueError("rank %d outside world of %d" % (rank, world))
    load = [0.0] * world
    owner = []
    for i in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        r = min(range(world), key=lambda q: (load[q], q))
        load[r] += costs[i]
        owner.append((i, r))
    return sorted(i for i, r in owner if r == rank)
