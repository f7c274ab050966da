"""Oracle: reverse-mode autodiff gradient of the restated operators on the CPU.

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).

Stands in for the reference's TensorFlow tape (util_op.py:627-654:
``tape.gradient(sum_k reduce_mean(square(f_k)), args)``), which cannot run
here (no TensorFlow).  The operator is re-written op by op in torch (FP64,
CPU), mirroring wave.py:67-122 with tf.roll -> torch.roll and tf.where ->
torch.where, and differentiated by torch.autograd.
"""
import numpy as np
import torch


def _quadh(u0, u1, u1p):
    return (u0 - 6 * u1 + 8 * u1p) / 3


def wave_residual_torch(s, u):
    """wave.py:67-122 on a CPU FP64 torch tensor ``u`` of shape (nt, nx)."""
    nt, nx = s.shape
    dt, dx = s.dt, s.dx
    it = torch.arange(nt)[:, None]
    ix = torch.arange(nx)[None, :]
    utm = torch.roll(u, 1, 0)
    utmm = torch.roll(u, 2, 0)
    uxm = torch.roll(utm, 1, 1)
    uxp = torch.roll(utm, -1, 1)
    left_utm = torch.roll(torch.as_tensor(s.left_u), 1, 0)
    right_utm = torch.roll(torch.as_tensor(s.right_u), 1, 0)
    uxm = torch.where(ix == 0, _quadh(uxp, utm, left_utm[:, None]), uxm)
    uxp = torch.where(ix == nx - 1, _quadh(uxm, utm, right_utm[:, None]), uxp)
    u_t_tm = (u - utm) / dt
    u_t_tmm = (utm - utmm) / dt
    u_t_tmm = torch.where(it == 1, torch.as_tensor(s.init_ut)[None, :], u_t_tmm)
    u_tt = (u_t_tm - u_t_tmm) / dt
    u_xx = (uxm - 2 * utm + uxp) / dx**2
    fu = u_tt - s.c**2 * u_xx
    u0 = torch.as_tensor(s.init_u + 0.5 * dt * s.init_ut)
    return torch.where(it == 0, u - u0[None, :], fu)


def wave_loss_grad_autodiff(s, u):
    """(loss, grad) by reverse-mode autodiff, FP64 on the CPU."""
    ut = torch.tensor(np.asarray(u, np.float64), requires_grad=True)
    f = wave_residual_torch(s, ut)
    loss = torch.mean(torch.square(f))
    g, = torch.autograd.grad(loss, [ut])
    return float(loss.detach()), g.numpy()
