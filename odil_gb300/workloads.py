"""Seeded synthetic problem instances (the benchmark workloads).

No dataset is involved: every input is generated from a seed.

Wave (wave.py:380-483 of the reference, plus a wave speed and a seeded
profile): u_tt = c^2 u_xx on t in [0, 1], x in [-1, 1].
  * profile "cos": the reference's fixed 5-mode cosine profile
    (wave.py:27-39), u_t(x, 0) != 0, c = 1;
  * profile "sine": f(x) = sum_k a_k sin(k pi (x + 1) / 2), a_k ~ N(0,1)/k from
    numpy default_rng(seed); exact solution u = (f(x - ct) + f(x + ct)) / 2
    (odd-periodic extension, zero Dirichlet values, u_t(x, 0) = 0).
"""
import numpy as np

from .domain import Domain
from .wave import WaveOperator


def cell_centers(lower, upper, n):
    x = np.linspace(lower, upper, n, endpoint=False, dtype=np.float64)
    h = (x[1] - x[0]) if n > 1 else (upper - lower)
    return x + h * 0.5


def wave_exact_cos(t, x):
    """u and u_t of the reference profile (u_t analytically)."""
    u = np.zeros(np.broadcast(t, x).shape)
    ut = np.zeros_like(u)
    for i in (1, 2, 3, 4, 5):
        k = i * np.pi
        u = u + np.cos((x - t + 0.5) * k) + np.cos((x + t - 0.5) * k)
        ut = ut + k * np.sin((x - t + 0.5) * k) - k * np.sin((x + t - 0.5) * k)
    return u / 10.0, ut / 10.0


def sine_amplitudes(seed, nmodes):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(nmodes) / np.arange(1, nmodes + 1)


def wave_exact_sine(t, x, amps, c=1.0):
    t = np.asarray(t, np.float64)
    x = np.asarray(x, np.float64)
    u = np.zeros(np.broadcast(t, x).shape)
    ut = np.zeros_like(u)
    for k, a in enumerate(amps, start=1):
        w = k * np.pi / 2
        u = u + a * (np.sin(w * (x - c * t + 1)) + np.sin(w * (x + c * t + 1)))
        ut = ut + a * c * w * (-np.cos(w * (x - c * t + 1)) +
                               np.cos(w * (x + c * t + 1)))
    return 0.5 * u, 0.5 * ut


class WaveInstance:
    """Domain, operator and exact solution of one wave problem."""

    def __init__(self, nt, nx, profile="sine", seed=0, nmodes=5, c=1.0,
                 dtype=np.float64, device="cuda"):
        self.nt, self.nx = int(nt), int(nx)
        self.profile, self.seed, self.nmodes, self.c = profile, seed, nmodes, c
        self.domain = Domain(ndim=2, shape=(nt, nx), lower=(0, -1),
                             upper=(1, 1), varnames=('t', 'x'),
                             fieldnames=('u', ), dtype=dtype, device=device)
        t1 = cell_centers(0.0, 1.0, nt)
        x1 = cell_centers(-1.0, 1.0, nx)
        if profile == "cos":
            if c != 1.0:
                raise ValueError("the reference cosine profile has c = 1")
            ex = wave_exact_cos
        elif profile == "sine":
            amps = sine_amplitudes(seed, nmodes)
            ex = lambda t, x: wave_exact_sine(t, x, amps, c)
        else:
            raise ValueError("Unknown profile=" + profile)
        left_u, _ = ex(t1, t1 * 0 - 1.0)
        right_u, _ = ex(t1, t1 * 0 + 1.0)
        init_u, init_ut = ex(x1 * 0, x1)
        tt, xx = np.meshgrid(t1, x1, indexing="ij")
        self.exact_u, _ = ex(tt, xx)
        self.operator = WaveOperator(init_u, init_ut, left_u, right_u, c=c)


# -- 2D advection (advection_2d.py of the reference) -------------------------
def advect_blob_params(seed, nblobs=8):
    """Velocity |a| <= 1 (direction uniform, magnitude in [0.2, 1]) and 8
    Gaussian blobs: centres in [0,1)^2, widths in [0.05, 0.15], amplitudes in
    [0.5, 1], from numpy default_rng(seed)."""
    rng = np.random.default_rng(seed)
    ang = rng.uniform(0, 2 * np.pi)
    mag = rng.uniform(0.2, 1.0)
    a = (mag * np.cos(ang), mag * np.sin(ang))
    centres = rng.uniform(0, 1, (nblobs, 2))
    widths = rng.uniform(0.05, 0.15, nblobs)
    amps = rng.uniform(0.5, 1.0, nblobs)
    return a, centres, widths, amps


def periodic_blobs(x, y, centres, widths, amps):
    p = np.zeros(np.broadcast(x, y).shape)
    for (cx, cy), w, A in zip(centres, widths, amps):
        dx = (x - cx + 0.5) % 1.0 - 0.5
        dy = (y - cy + 0.5) % 1.0 - 0.5
        p = p + A * np.exp(-(dx * dx + dy * dy) / (2 * w * w))
    return p


class AdvectInstance:
    """(nt, n, n) grid on t in [0, 1], x, y in [0, 1) periodic; the row-0
    previous value is the exact field at the first time cell centre
    (advection_2d.py:196-202); exact solution p0(x - ax t, y - ay t)."""

    def __init__(self, n, seed=0, nt=None, dtype=np.float64, device="cuda"):
        from .advection import AdvectionOperator
        nt = n if nt is None else nt
        (ax, ay), c, w, A = advect_blob_params(seed)
        self.a = (ax, ay)
        self.domain = Domain(ndim=3, shape=(nt, n, n), lower=(0, 0, 0),
                             upper=(1, 1, 1), varnames=('t', 'x', 'y'),
                             fieldnames=('p', ), dtype=dtype, device=device)
        t1 = cell_centers(0.0, 1.0, nt)
        x1 = cell_centers(0.0, 1.0, n)
        xx, yy = np.meshgrid(x1, x1, indexing="ij")
        p_init = periodic_blobs(xx - ax * t1[0], yy - ay * t1[0], c, w, A)
        self.operator = AdvectionOperator(ax, ay, p_init)
        self._exact = lambda: np.stack(
            [periodic_blobs(xx - ax * t, yy - ay * t, c, w, A) for t in t1])

    def exact(self):
        return self._exact()


# -- batched wave instances ---------------------------------------------------
# Largest Courant number c dt / dx of a batch instance.  The wave operator's
# boundary closure (quadratic extrapolation at x = -1, 1) makes forward
# substitution unstable above about 0.93: a perturbation grows by 1e26 over
# 256 rows at 0.94 and stays bounded at 0.92, in FP64 as in FP32, so no direct
# method recovers the discrete solution there.
BATCH_MAX_CFL = 0.9


def wave_batch_instances(count=512, seed=4, nmin=64, nmax=512, cmin=0.5,
                         cmax=2.0, nmodes=5, max_cfl=BATCH_MAX_CFL):
    """Seeded uneven batch: side n ~ U{nmin..nmax}, wave speed
    c ~ U[cmin, cmax], 5-mode sine profile with per-instance seed.  The grid
    is n x n (x in [-1, 1], t in [0, 1], Courant number c / 2) unless that
    exceeds max_cfl; then the time grid is refined to nt = ceil(c n /
    (2 max_cfl)) rows.  Returns the instance dicts of WaveBatch plus each
    one's exact solution."""
    rng = np.random.default_rng(seed)
    sides = rng.integers(nmin, nmax + 1, count)
    speeds = rng.uniform(cmin, cmax, count)
    out = []
    for i, (n, c) in enumerate(zip(sides, speeds)):
        n = int(n)
        nt = n if c / 2 <= max_cfl else int(np.ceil(c * n / (2 * max_cfl)))
        inst = WaveInstance(nt, n, profile="sine",
                            seed=seed * 100003 + i, nmodes=nmodes,
                            c=float(c), device="cpu")
        op = inst.operator
        out.append({"nt": nt, "nx": n, "dt": 1.0 / nt, "dx": 2.0 / n,
                    "c": float(c), "init_u": op.init_u, "init_ut": op.init_ut,
                    "left_u": op.left_u, "right_u": op.right_u,
                    "exact_u": inst.exact_u, "seed": seed * 100003 + i})
    return out
