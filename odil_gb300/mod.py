"""The ``mod`` namespace handed to user operators: TensorFlow-style names over
torch, so operators written for the reference (``operator(mod, ctx)`` with
mod = tf, util_op.py:569-577) run unchanged on CUDA tensors.

Only the generic (unregistered) operator path uses it; registered operator
families run fused CUDA kernels instead.
"""
import numpy as np
import torch


def _t(x, like=None):
    if isinstance(x, torch.Tensor):
        return x
    if like is not None:
        return torch.as_tensor(np.asarray(x), dtype=like.dtype,
                               device=like.device)
    return torch.as_tensor(np.asarray(x))


class TorchMod:
    """tf-like functions used by ODIL operators."""

    def __init__(self, device="cuda", dtype=torch.float64):
        self.device = device
        self.dtype = dtype
        self.float32 = torch.float32
        self.float64 = torch.float64
        self.pi = np.pi

    def constant(self, x, dtype=None):
        return torch.as_tensor(np.asarray(x), dtype=dtype or self.dtype,
                               device=self.device)

    def cast(self, x, dtype=None):
        return self.constant(x, dtype) if not isinstance(
            x, torch.Tensor) else x.to(dtype or self.dtype)

    def _dev(self, x):
        if isinstance(x, torch.Tensor):
            return x
        a = np.asarray(x)
        if not a.flags.writeable:  # e.g. a broadcast view of the grid
            a = a.copy()
        if a.dtype == bool:
            return torch.as_tensor(a, device=self.device)
        if np.issubdtype(a.dtype, np.integer):
            return torch.as_tensor(a, device=self.device)
        return torch.as_tensor(a, dtype=self.dtype, device=self.device)

    def where(self, cond, a, b):
        cond = self._dev(cond)
        a, b = self._dev(a), self._dev(b)
        return torch.where(cond, a, b)

    def roll(self, x, shift, axis):
        x = self._dev(x)
        if isinstance(axis, range):
            axis = tuple(axis)
        if isinstance(shift, np.ndarray):
            shift = tuple(int(s) for s in shift)
        return torch.roll(x, shift, axis)

    def zeros(self, shape, dtype=None):
        return torch.zeros(shape, dtype=dtype or self.dtype,
                           device=self.device)

    def ones(self, shape, dtype=None):
        return torch.ones(shape, dtype=dtype or self.dtype,
                          device=self.device)

    def zeros_like(self, x):
        return torch.zeros_like(self._dev(x))

    def ones_like(self, x):
        return torch.ones_like(self._dev(x))

    def square(self, x):
        return self._dev(x)**2

    def sqrt(self, x):
        return torch.sqrt(self._dev(x))

    def exp(self, x):
        return torch.exp(self._dev(x))

    def sin(self, x):
        return torch.sin(self._dev(x))

    def cos(self, x):
        return torch.cos(self._dev(x))

    def tanh(self, x):
        return torch.tanh(self._dev(x))

    def abs(self, x):
        return torch.abs(self._dev(x))

    def maximum(self, a, b):
        return torch.maximum(self._dev(a), self._dev(b))

    def minimum(self, a, b):
        return torch.minimum(self._dev(a), self._dev(b))

    def reduce_mean(self, x):
        return torch.mean(self._dev(x))

    def reduce_sum(self, x):
        return torch.sum(self._dev(x))

    def stack(self, xs, axis=0):
        return torch.stack([self._dev(x) for x in xs], axis)

    def reshape(self, x, shape):
        return torch.reshape(self._dev(x), tuple(shape))

    def stop_gradient(self, x):
        return self._dev(x).detach()
