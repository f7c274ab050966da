"""Solver loops with the reference's entry points (util.py:109-370):

    optimize(args, optname, problem, state, callback)

dispatches to ``optimize_newton`` (Newton with ``linsolver.solve``) or to
``optimize_opt`` (generic optimizers over ``loss_grad``).  The callback
protocol is the reference's: ``callback(packed, epoch, dhistory=None,
opt=None)``.  States and packed vectors stay on the GPU.
"""
import inspect
import os
import re
import sys
import time
from collections import defaultdict

import numpy as np
import torch

from . import linsolver
from . import optimizer as optimizer_mod


_log_file = sys.stderr
_log_echo = False
_time_prev = None


def set_log_file(f, echo=False):
    """util.py:46-49: where printlog writes (and whether it echoes to
    stderr)."""
    global _log_file, _log_echo
    _log_file, _log_echo = f, echo


def printlog(*msg):
    """util.py:52-58: one line to the log file."""
    m = " ".join(map(str, msg)) + "\n"
    if _log_echo and _log_file is not sys.stderr:
        sys.stderr.write(m)
        sys.stderr.flush()
    _log_file.write(m)
    _log_file.flush()


def TIMECLEAR():
    """util.py:61-63: restarts the TIME stopwatch."""
    global _time_prev
    _time_prev = time.time()


def TIME(pattern="{file}:{line}"):
    """util.py:66-75: logs the caller's file:line and the seconds since the
    previous TIME/TIMECLEAR."""
    global _time_prev
    now = time.time()
    if _time_prev is None:
        _time_prev = now
    caller = inspect.stack()[1]
    d = {"file": os.path.basename(caller[1]), "line": caller[2]}
    printlog((pattern + " {:.3f}s".format(now - _time_prev)).format(**d))
    _time_prev = time.time()


def get_error(u, v):
    """util.py:102-106: mean absolute, root-mean-square and maximum
    difference (numpy arrays or tensors)."""
    if isinstance(u, torch.Tensor) or isinstance(v, torch.Tensor):
        d = (torch.as_tensor(u) - torch.as_tensor(v)).abs()
        return (d.mean().item(), (d**2).mean().sqrt().item(),
                d.max().item())
    d = np.abs(np.asarray(u) - np.asarray(v))
    return np.mean(d), np.mean(d**2)**0.5, np.max(d)


def get_memory_usage_kb():
    """util.py:373-379: resident set size of this process in KiB."""
    with open("/proc/self/status") as f:
        return int(re.findall(r"VmRSS:[^0-9]*([0-9]*)", f.read())[0])


class Timer:
    """util.py:78-99: named wall-clock counters (push/pop)."""

    def __init__(self):
        self._starts = []
        self.counters = dict()

    def push(self, key=None):
        self._starts.append((key, time.time()))

    def pop(self, key=None):
        start = self._starts.pop()
        assert start[0] is None or key is None or start[0] == key
        key = start[0] if key is None else key
        self.counters[key] = self.counters.get(key, 0.) + time.time() - start[1]

    def append(self, timer):
        for k, v in timer.counters.items():
            self.counters[k] = self.counters.get(k, 0.) + v


def optimize_newton(args, problem, state, callback=None):
    """util.py:242-268: epochs of linearize -> linsolver.solve -> update.

    With ``args.precision == "mixed"`` (and the default linsolver) the solve
    runs in FP32 on the FP64 residual: every epoch is one step of
    mixed-precision iterative refinement."""
    opt = optimizer_mod.Optimizer(name='newton', displayname='Newton')
    problem.init_missing(state)
    packed = problem.pack_state(state)
    dhistory = defaultdict(list)
    name = getattr(args, "linsolver", "direct")
    if getattr(args, "precision", "fp64") == "mixed" and name == "direct":
        name = "mixed"
    for epoch in range(getattr(args, "epoch_start", 0), args.epochs + 1):
        s = problem.unpack_state(packed)
        problem.domain.assign_active_state(state, s)
        const, m = problem.linearize(state, epoch=epoch)
        opt.last_loss = sum(torch.mean(c**2) for c in const)
        opt.last_residual = [torch.mean(c**2)**0.5 for c in const]
        if callback:
            callback(packed, epoch, dhistory=dhistory, opt=opt)
        if epoch == args.epochs:
            break
        opt.evals += 1
        rhs = -torch.cat([c.reshape(-1) for c in const])
        timer = Timer()
        timer.push('linsolver')
        dpacked = linsolver.solve(m, rhs, args, dhistory, name)
        timer.pop()
        packed += dpacked
    s = problem.unpack_state(packed)
    problem.domain.assign_active_state(state, s)
    return packed


def optimize_opt(args, optname, problem, state, callback=None, **kwargs):
    """util.py:271-317: run a generic optimizer over the packed state."""
    problem.init_missing(state)

    def loss_grad(packed, epoch):
        fields = problem.unpack_fields(packed)
        s = type(state)(fields=fields)
        loss, grads, _, loss_split = problem.eval_loss_grad(s, epoch=epoch)
        g = problem.pack_fields(grads)
        last_residual = [v**0.5 if v >= 0 else v for v in loss_split]
        return loss, g, last_residual

    packed = problem.pack_state(state)
    if getattr(args, "bfgs_m", None) is not None:
        kwargs['m'] = args.bfgs_m
    for key, attr in (('epsilon', 'adam_epsilon'), ('beta_1', 'adam_beta_1'),
                      ('beta_2', 'adam_beta_2')):
        if getattr(args, attr, None) is not None:
            kwargs[key] = getattr(args, attr)
    opt = optimizer_mod.make_optimizer(optname, dtype=problem.domain.dtype,
                                       **kwargs)
    epoch_start = getattr(args, "epoch_start", 0)
    loss, _, residual = loss_grad(packed, epoch_start)
    opt.last_loss = loss
    opt.last_residual = residual
    if callback:
        callback(packed, epoch=epoch_start, opt=opt)
    packed, info = opt.run(packed, loss_grad=loss_grad,
                           epochs=args.epochs - epoch_start,
                           callback=callback, epoch_start=epoch_start,
                           lr=getattr(args, "lr", 1e-3), **kwargs)
    s = problem.unpack_state(packed)
    problem.domain.assign_active_state(state, s)
    return packed, info


def optimize_jacobi(args, problem, state, callback=None):
    """util.py:320-362: gradient steps preconditioned by a running estimate
    of diag(sum_k J_k^T J_k / N_k) (Problem.eval_diag): nsmp0 samples
    before the first epoch, nsmp1 more per epoch with weight jac_factor;
    step -lr/2 g / (diag + jac_epsilon)."""
    opt = optimizer_mod.Optimizer(name='jacobi', displayname='Jacobi')
    problem.init_missing(state)
    packed = problem.pack_state(state)
    dhistory = defaultdict(list)
    nsmp0 = getattr(args, "jac_nsmp0", 50)
    nsmp1 = getattr(args, "jac_nsmp1", 1)
    factor = getattr(args, "jac_factor", 1.0)
    epsilon = getattr(args, "jac_epsilon", 1e-8)
    lr = getattr(args, "lr", 1e-3)
    epoch_start = getattr(args, "epoch_start", 0)
    diag = problem.eval_diag(state, epoch=epoch_start, nsmp=nsmp0)
    ntotal = nsmp0
    for epoch in range(epoch_start, args.epochs + 1):
        s = problem.unpack_state(packed)
        problem.domain.assign_active_state(state, s)
        loss, grads, _, loss_split = problem.eval_loss_grad(state, epoch=epoch)
        diag1 = problem.eval_diag(state, epoch=epoch, nsmp=nsmp1)
        diag = (diag * ntotal + diag1 * nsmp1 * factor) / \
            (ntotal + nsmp1 * factor)
        ntotal += nsmp1
        g = problem.pack_fields(grads)
        dpacked = -(g / (diag + epsilon)) * (lr * 0.5)
        opt.last_loss = loss
        opt.last_residual = [v**0.5 if v >= 0 else v for v in loss_split]
        if callback:
            callback(packed, epoch, dhistory=dhistory, opt=opt)
        if epoch == args.epochs:
            break
        opt.evals += 1
        packed += dpacked
    s = problem.unpack_state(packed)
    problem.domain.assign_active_state(state, s)
    return packed


def optimize_multigrid(args, problem, state, callback=None, datalevels=None):
    """util.py:382-495: Newton epochs whose normal equations
    J^T J d = -J^T r, assembled as sparse CSR matrices on the fields' device,
    are solved by `linsolver_maxiter` (default 50) V-cycles of the CSR
    multigrid (multigrid.Multigrid: R A T coarsening, damped Jacobi on the
    diagonal blocks with `omega`, `smooth_pre` / `smooth_post` sweeps on the
    finest level, direct solve below `ndirect` nodes per axis).  The
    Jacobian must provide `to_csr` (compiled generic operators and families
    with coefficient fields do).

    With `datalevels` (one object per multigrid level with `.problem` and
    `.state`, level 0 the given problem), the matrix of every level is the
    J^T J of that level's own problem, linearised at the previous level's
    fields restricted by the level's single-field restriction
    (util.py:414-441), instead of R A T.  `opt.last_residual` is the finest
    level's (the reference keeps the coarsest level's)."""
    from .multigrid import Multigrid
    opt = optimizer_mod.Optimizer(name='multigrid', displayname='Multigrid')
    problem.init_missing(state)
    packed = problem.pack_state(state)
    dhistory = defaultdict(list)
    dom = problem.domain
    mg = Multigrid(tuple(dom.shape), nvar=len(dom.fieldnames),
                   nlevels=getattr(args, "nlvl", None),
                   restriction=getattr(args, "restriction", "full"),
                   dtype=packed.dtype, device=packed.device)
    omega = getattr(args, "omega", 0.6)
    iters = getattr(args, "linsolver_maxiter", None) or 50

    def smoother(level, u, f):
        return mg.smoother_jacobi(level, u, f, omega=omega, full=False)

    for epoch in range(getattr(args, "epoch_start", 0), args.epochs + 1):
        s = problem.unpack_state(packed)
        dom.assign_active_state(state, s)
        const, J = problem.linearize(state, epoch=epoch)
        opt.last_loss = sum(torch.mean(c**2) for c in const)
        opt.last_residual = [torch.mean(c**2)**0.5 for c in const]
        if callback:
            callback(packed, epoch, dhistory=dhistory, opt=opt)
        if epoch == args.epochs:
            break
        opt.evals += 1
        timer = Timer()
        timer.push('linsolver')
        m = J.to_csr()
        rhs = -(m.t() @ torch.cat([c.reshape(-1) for c in const]))
        if datalevels is None:
            mg.update_A(m.t().to_sparse_csr() @ m)
        else:
            AA = [m.t().to_sparse_csr() @ m]
            for level in range(1, mg.nlevels):
                lproblem = datalevels[level].problem
                lstate = datalevels[level].state
                fine = datalevels[level - 1].state
                R = mg.RRsingle[level - 1]
                for k in dom.fieldnames:
                    f = fine.fields[k]
                    lstate.fields[k] = (R @ f.reshape(-1).to(R.dtype)).reshape(
                        tuple(lproblem.domain.shape))
                lconst, lJ = lproblem.linearize(lstate, epoch=epoch)
                lm = lJ.to_csr()
                AA.append(lm.t().to_sparse_csr() @ lm)
            mg.update_A(AA)
        sol = torch.zeros_like(rhs)
        for _ in range(iters):
            sol = mg.step(sol, rhs, smoother,
                          ndirect=getattr(args, "ndirect", 5),
                          pre=getattr(args, "smooth_pre", 2),
                          post=getattr(args, "smooth_post", 2))
        timer.pop()
        packed += sol
    s = problem.unpack_state(packed)
    dom.assign_active_state(state, s)
    return packed


def optimize_multigridop(args, problem, state, callback=None):
    """util.py:509-617: Newton epochs whose normal equations
    J^T J d = -J^T r are solved by `linsolver_maxiter` (default 50) V-cycles
    of the multigrid on the GPU (stencil.MultigridOp: Galerkin coarsening of
    the J^T J stencils, damped Jacobi with `omega`, `smooth_pre` /
    `smooth_post` sweeps, direct solve below `ndirect` cells per axis).
    The Jacobian must provide its stencils (compiled generic operators and
    families with coefficient fields do)."""
    from .stencil import MultigridOp
    opt = optimizer_mod.Optimizer(name='multigridop',
                                  displayname='MultigridOp')
    problem.init_missing(state)
    packed = problem.pack_state(state)
    dhistory = defaultdict(list)
    dom = problem.domain
    names = list(dom.fieldnames)
    nvar = len(names)
    shape = tuple(dom.shape)
    n = int(np.prod(shape))
    mg = None
    omega = getattr(args, "omega", 0.6)
    iters = getattr(args, "linsolver_maxiter", None) or 50

    def smoother(level, u, f):
        return mg.smoother_jacobi(level, u, f, omega=omega)

    for epoch in range(getattr(args, "epoch_start", 0), args.epochs + 1):
        s = problem.unpack_state(packed)
        dom.assign_active_state(state, s)
        const, J = problem.linearize(state, epoch=epoch)
        opt.last_loss = sum(torch.mean(c**2) for c in const)
        opt.last_residual = [torch.mean(c**2)**0.5 for c in const]
        if callback:
            callback(packed, epoch, dhistory=dhistory, opt=opt)
        if epoch == args.epochs:
            break
        opt.evals += 1
        blocks = J.stencil_blocks()
        if mg is None:
            # The transfer operators wrap where the stencils do; a periodic
            # axis halves exactly, so the depth stops where a size turns odd.
            per = next(iter(blocks.values())).periodic
            nl = getattr(args, "nlvl", None)
            while per and any(p for p in per) and (nl is None or nl > 1):
                lv = nl if nl is not None else 64
                if all(not p or sz % (1 << (lv - 1)) == 0
                       for sz, p in zip(shape, per)):
                    break
                nl = lv - 1
            mg = MultigridOp(shape, nvar=nvar, nlevels=nl,
                             restriction=getattr(args, "restriction", "full"),
                             periodic=per, dtype=packed.dtype,
                             device=packed.device)
        A = [[None] * nvar for _ in range(nvar)]
        for (k, i), Bi in blocks.items():
            for (k2, j), Bj in blocks.items():
                if k2 != k:
                    continue
                C = Bi.mul_transpose_op(Bj)
                A[i][j] = C if A[i][j] is None else A[i][j].add(C)
        mg.update_A(A)
        rhs = -J.rmatvec(torch.cat([c.reshape(-1) for c in const]))
        f = [rhs[q * n:(q + 1) * n].reshape(shape).contiguous()
             for q in range(nvar)]
        sol = [torch.zeros_like(x) for x in f]
        timer = Timer()
        timer.push('linsolver')
        for _ in range(iters):
            sol = mg.step(sol, f, smoother,
                          ndirect=getattr(args, "ndirect", 3),
                          pre=getattr(args, "smooth_pre", 2),
                          post=getattr(args, "smooth_post", 2))
        timer.pop()
        packed += torch.cat([x.reshape(-1) for x in sol])
    s = problem.unpack_state(packed)
    dom.assign_active_state(state, s)
    return packed


# The reference's CuPy variants (util.py:498-506, 619-629); both forms
# above already run on the fields' device.
optimize_multigridcp = optimize_multigrid
optimize_multigridopcp = optimize_multigridop


def optimize(args, optname, problem, state, callback=None, **kwargs):
    """util.py:365-370."""
    if optname == 'newton':
        return optimize_newton(args, problem, state, callback)
    if optname == 'jacobi':
        return optimize_jacobi(args, problem, state, callback)
    return optimize_opt(args, optname, problem, state, callback, **kwargs)


def add_arguments(parser):
    """The flags of util.py:109-239 (solver flags, then driver flags)."""
    parser.add_argument('--epochs', type=int, default=None,
                        help="Maximum epochs")
    parser.add_argument('--epoch_start', type=int, default=0,
                        help="Index of the first epoch")
    parser.add_argument('--optimizer', type=str, default='newton',
                        help="Optimizer: newton, lbfgsb, lbfgs, adam, adamn, gd")
    parser.add_argument('--seed', type=int, default=0,
                        help="Seed for the drivers' random generators")
    parser.add_argument('--double', type=int, default=0,
                        help="Double precision")
    parser.add_argument('--bfgs_m', type=int, default=50,
                        help="L-BFGS history size")
    parser.add_argument('--adam_epsilon', type=float, default=None)
    parser.add_argument('--adam_beta_1', type=float, default=None)
    parser.add_argument('--adam_beta_2', type=float, default=None)
    parser.add_argument('--outdir', type=str, default='.',
                        help="Output directory")
    parser.add_argument('--jac_nsmp0', type=int, default=50,
                        help="Jacobi: samples for the initial diagonal")
    parser.add_argument('--jac_nsmp1', type=int, default=1,
                        help="Jacobi: samples per epoch")
    parser.add_argument('--jac_factor', type=float, default=1,
                        help="Jacobi: weight of the new samples")
    parser.add_argument('--jac_epsilon', type=float, default=1e-8,
                        help="Jacobi: added to the diagonal")
    # Driver flags of util.py:109-239, same names, types and defaults, so
    # that a driver's command line parses unchanged.  Their consumers
    # (plots, frames, reports, checkpoint files) are the driver's own;
    # --multigrid and --nn_initializer select unknowns this engine does not
    # hold (Domain raises for them).
    parser.add_argument('--every_factor', type=int, default=1,
                        help="Multiplier for all *_every options")
    parser.add_argument('--plot_every', type=int, default=5,
                        help="Epochs between plots")
    parser.add_argument('--report_every', type=int, default=10,
                        help="Epochs between reports to stdout")
    parser.add_argument('--history_every', type=int, default=1,
                        help="Epochs between entries of training history")
    parser.add_argument('--checkpoint_every', type=int, default=5,
                        help="Epochs between checkpoints")
    parser.add_argument('--frames', type=int, default=10,
                        help="Frames to plot. Zero disables first frame.")
    parser.add_argument('--plot_title', type=int, default=0,
                        help="Enable title in plots")
    parser.add_argument('--plotext', type=str, default='pdf',
                        help="Extension of plots")
    parser.add_argument('--history_full', type=int, default=0,
                        help="Number of epochs to write history at every "
                        "point")
    parser.add_argument('--montage', type=int, default=1,
                        help="Run montage after plotting")
    parser.add_argument('--frame_start', type=int, default=0,
                        help="Initial value of frame")
    parser.add_argument('--checkpoint', type=str,
                        help="Continue from checkpoint in state_*.pickle")
    parser.add_argument('--checkpoint_train', type=str,
                        help="Continue from history in state_*_train.pickle")
    parser.add_argument('--multigrid', type=int, default=0,
                        help="Use multigrid decomposition")
    parser.add_argument('--mg_interp', type=str, default='conv',
                        choices=['roll', 'conv', 'manual'],
                        help="Multigrid interpolation method")
    parser.add_argument('--dump_data', type=int, default=1,
                        help="Dump data_*.pickle with every plot")
    parser.add_argument('--nn_initializer', type=str, default='legacy',
                        choices=['legacy', 'glorot', 'lecun', 'he'],
                        help="Initializer for weights of neural networks")
