"""Newton solves of registered operator families on the GPU.

The reference's plain method (util.py:242-268 with linsolver.py:28-45) is
Newton: linearize, solve the normal equations of J d = -F(u) directly,
u += d, for a fixed number of epochs.  For an affine operator every epoch
after the first is an iterative-refinement step.  Here the direct solve of
the wave family is forward substitution (J is lower triangular in C order;
same solution as the normal equations).

precision="fp64"   plain method: FP64 residual, FP64 solve, FP64 update.
precision="mixed"  FP64 residual and update, FP32 solve (one fused kernel:
                   r -> -r in FP32 -> forward substitution -> u += d in FP64).
"""
import torch


def solve(problem, state, precision="mixed", epochs=None):
    """Runs ``epochs`` Newton epochs in place on ``state``; returns the field.

    Defaults: 3 epochs for "mixed" (each epoch gains ~5 digits against the
    FP64 discrete solution), 2 for "fp64" (as the reference runs it).
    """
    k = problem.kernels
    if k is None:
        raise NotImplementedError("Newton needs a registered operator family")
    problem.init_missing(state)
    name = problem.domain.fieldnames[0]
    u = state.fields[name]
    if u.dtype != torch.float64:
        raise TypeError("Newton runs on an FP64 state")
    if precision == "mixed":
        epochs = 3 if epochs is None else epochs
        for _ in range(epochs):
            k.refine_mixed(k.residual(u), u)
    elif precision == "fp64":
        epochs = 2 if epochs is None else epochs
        for _ in range(epochs):
            r = k.residual(u)
            r.neg_()
            u.add_(k.march(r))
    else:
        raise ValueError("Unknown precision=" + precision)
    return u
