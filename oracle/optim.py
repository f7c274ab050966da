"""Oracle: the reference's optimizers on the CPU (FP64).

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).

  * adam_native: optimizer.py:276-322 (AdamNativeOptimizer.run), the update
    m += (g - m)(1 - b1); v += (g^2 - v)(1 - b2); x -= a m / (sqrt(v) + eps),
    a = lr sqrt(1 - b2^t) / (1 - b1^t), t = 1, 2, ...
  * lbfgsb: optimizer.py:61-99 (LbfgsbOptimizer.run) -- scipy's
    fmin_l_bfgs_b with m=50, pgtol=1e-16, factr=0, maxls=50, maxfun=inf.
"""
import math

import numpy as np
import scipy.optimize


def adam_native(x0, loss_grad, epochs, lr=1e-3, beta_1=0.9, beta_2=0.999,
                epsilon=1e-7):
    x = np.array(x0, np.float64)
    m = np.zeros_like(x)
    v = np.zeros_like(x)
    for t in range(1, epochs + 1):
        _, g = loss_grad(x)
        alpha = lr * math.sqrt(1 - beta_2**t) / (1 - beta_1**t)
        m += (g - m) * (1 - beta_1)
        v += (g * g - v) * (1 - beta_2)
        x -= (m * alpha) / (np.sqrt(v) + epsilon)
    return x


def lbfgsb(x0, loss_grad, epochs, m=50, pgtol=1e-16, factr=0, maxls=50):
    x, f, info = scipy.optimize.fmin_l_bfgs_b(
        func=lambda x: loss_grad(x), x0=np.array(x0, np.float64),
        maxiter=epochs, pgtol=pgtol, m=m, maxls=maxls, factr=factr,
        maxfun=math.inf)
    return x, f, info
