"""Oracle: the reference's 2D advection problem on the (t, x, y) grid, FP64.

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).

Follows advection_2d.py:103-223 (``operator``, direct problem, defaults
--periodic 1 --central 0 --implicit 0):
    fp = (p - ptm)/dt + uf p_x + vf p_y,
    p_x = where(uf > 0, (p - p[x-1])/dx, (p[x+1] - p)/dx)   (first-order upwind
    on the frozen velocity, advection_2d.py:129-138), same in y,
    ptm = p[i-1] (tf.roll, periodic) except row 0: ptm = exact_pp[0]
    (advection_2d.py:196-202);
    fu = u - exact_uu, fv = v - exact_vv (advection_2d.py:219-223).
Domain: shape (Nt, Nx, Ny), t in [0, tmax], x, y in [0, 1) (advection_2d.py:
335-340), cell centres as util_op.py:130-137.

Pinned: ``residual_uvp`` and ``residual_p`` equal, to rounding, the
residuals of the reference's own ``operator`` function run on NumPy stand-ins
for TensorFlow (tests/golden/advection_ref.npz, made by
tests/golden/make_golden.py; tests/test_advection_oracle.py), on small grids
with velocity fields of both signs and exact zeros.

The benchmark instance has a constant velocity a = (ax, ay), so u and v are
known: after one Newton step fu = fv = 0 and the unknown is p alone
(``residual_p``).  ``residual_uvp`` keeps the reference's three fields.

Solvers:
  * ``newton_direct``: linearize (per-shift Jacobian -> CSR, util_op.py:
    859-937) + normal equations + spsolve(MMD_ATA) (linsolver.py:35-45), for
    small grids;
  * ``solve_fft``: the same discrete solution by an exact direct method for
    large grids: J is block lower-bidiagonal in t with one periodic circulant
    block D per slice, so each 2D Fourier mode obeys a scalar recurrence in t;
  * ``vcycle`` / ``bicgstab``: the matrix-free multigrid preconditioned Krylov
    solve that the GPU path implements (rediscretised coarse operators,
    damped Jacobi, full weighting, trilinear prolongation), for checking it.
"""
import numpy as np
import scipy.sparse
import scipy.sparse.linalg

from .wave import cell_center_1d


class AdvectSetup:

    def __init__(self, nt, nx, ny, ax, ay, p_init, tmax=1.0):
        self.nt, self.nx, self.ny = int(nt), int(nx), int(ny)
        self.dt = tmax / nt
        self.dx = 1.0 / nx
        self.dy = 1.0 / ny
        self.ax, self.ay = float(ax), float(ay)
        self.p_init = np.asarray(p_init, np.float64).reshape(nx, ny)

    @property
    def shape(self):
        return (self.nt, self.nx, self.ny)


def blob_params(seed, nblobs=8):
    """Seeded benchmark instance: velocity |a| <= 1 and 8 Gaussian blobs with
    centres in [0,1)^2, widths in [0.05, 0.15], amplitudes in [0.5, 1]."""
    rng = np.random.default_rng(seed)
    ang = rng.uniform(0, 2 * np.pi)
    mag = rng.uniform(0.2, 1.0)
    a = (mag * np.cos(ang), mag * np.sin(ang))
    centres = rng.uniform(0, 1, (nblobs, 2))
    widths = rng.uniform(0.05, 0.15, nblobs)
    amps = rng.uniform(0.5, 1.0, nblobs)
    return a, centres, widths, amps


def blobs(x, y, centres, widths, amps):
    """Sum of periodic Gaussians (minimum-image distance on the unit torus)."""
    p = np.zeros(np.broadcast(x, y).shape)
    for (cx, cy), w, A in zip(centres, widths, amps):
        dx = (x - cx + 0.5) % 1.0 - 0.5
        dy = (y - cy + 0.5) % 1.0 - 0.5
        p = p + A * np.exp(-(dx * dx + dy * dy) / (2 * w * w))
    return p


def make_setup(n, seed=0, nt=None):
    """Benchmark instance on an (nt, n, n) grid; exact solution
    p(t, x, y) = p0(x - ax t, y - ay t)."""
    nt = n if nt is None else nt
    (ax, ay), c, w, A = blob_params(seed)
    t1 = cell_center_1d(0.0, 1.0, nt)
    x1 = cell_center_1d(0.0, 1.0, n)
    xx, yy = np.meshgrid(x1, x1, indexing="ij")
    # advection_2d.py:196-202: the row-0 previous value is the exact field at
    # the first time cell centre.
    p_init = blobs(xx - ax * t1[0], yy - ay * t1[0], c, w, A)
    s = AdvectSetup(nt, n, n, ax, ay, p_init)
    s.exact = lambda: np.stack([blobs(xx - ax * t, yy - ay * t, c, w, A)
                                for t in t1])
    return s


def _upwind(p, a, h, axis):
    if a > 0:
        return (p - np.roll(p, 1, axis)) / h
    return (np.roll(p, -1, axis) - p) / h


def residual_p(s, p):
    """fp of advection_2d.py:217-220 with constant (frozen) velocity."""
    p = np.asarray(p, np.float64).reshape(s.shape)
    ptm = np.roll(p, 1, 0)
    ptm[0] = s.p_init
    p_t = (p - ptm) / s.dt
    return p_t + s.ax * _upwind(p, s.ax, s.dx, 1) + s.ay * _upwind(p, s.ay, s.dy, 2)


def residual_uvp(s, u, v, p, exact_uu, exact_vv):
    """The reference's three residual terms (fp, fu, fv) with per-cell frozen
    velocity fields u, v (advection_2d.py:179-223)."""
    p = np.asarray(p, np.float64).reshape(s.shape)
    ptm = np.roll(p, 1, 0)
    ptm[0] = s.p_init
    pxm, pxp = np.roll(p, 1, 1), np.roll(p, -1, 1)
    pym, pyp = np.roll(p, 1, 2), np.roll(p, -1, 2)
    p_x = np.where(u > 0, (p - pxm) / s.dx, (pxp - p) / s.dx)
    p_y = np.where(v > 0, (p - pym) / s.dy, (pyp - p) / s.dy)
    fp = (p - ptm) / s.dt + u * p_x + v * p_y
    return [fp, u - exact_uu, v - exact_vv]


def jacobian(s):
    """CSR of d fp / d p (util_op.py:859-937 with periodic roll columns)."""
    nt, nx, ny = s.shape
    N = nt * nx * ny
    idx = np.arange(N).reshape(s.shape)
    it = np.arange(nt)[:, None, None] + 0 * idx
    rows, cols, vals = [], [], []

    def add(col, val):
        rows.append(idx.ravel())
        cols.append(col.ravel())
        vals.append(np.broadcast_to(val, idx.shape).ravel())

    D = 1 / s.dt + abs(s.ax) / s.dx + abs(s.ay) / s.dy
    add(idx, np.full(idx.shape, D))
    add(np.roll(idx, 1, 0), np.where(it >= 1, -1 / s.dt, 0.0))
    if s.ax > 0:
        add(np.roll(idx, 1, 1), -s.ax / s.dx)
    else:
        add(np.roll(idx, -1, 1), s.ax / s.dx)
    if s.ay > 0:
        add(np.roll(idx, 1, 2), -s.ay / s.dy)
    else:
        add(np.roll(idx, -1, 2), s.ay / s.dy)
    J = scipy.sparse.csr_matrix((np.concatenate(vals), (np.concatenate(rows),
                                                        np.concatenate(cols))),
                                shape=(N, N))
    J.eliminate_zeros()
    return J


def newton_direct(s, epochs=2):
    """util.py:242-268 + linsolver.py:35-45 (normal equations, SuperLU)."""
    J = jacobian(s)
    A = (J.T @ J).tocsr()
    p = np.zeros(s.shape)
    for _ in range(epochs):
        r = residual_p(s, p).ravel()
        d = scipy.sparse.linalg.spsolve(A, J.T @ (-r), permc_spec="MMD_ATA")
        p = p + d.reshape(s.shape)
    return p


def jv(s, v):
    """J v (the linear part of residual_p)."""
    return _jv(s, v)


def _jv(s, v):
    v = np.asarray(v, np.float64).reshape(s.shape)
    vtm = np.roll(v, 1, 0)
    vtm[0] = 0.0
    return (v - vtm) / s.dt + s.ax * _upwind(v, s.ax, s.dx, 1) + \
        s.ay * _upwind(v, s.ay, s.dy, 2)


def jtv(s, w):
    return (jacobian(s).T @ np.asarray(w, np.float64).ravel()).reshape(s.shape)


def loss_grad(s, p):
    f = residual_p(s, p)
    return float(np.mean(f**2)), (2.0 / f.size) * jtv(s, f)


def solve_fft(s, b):
    """Exact solve of J x = b: 2D FFT per time slice, per-mode recurrence
    x_i = (b_i + x_{i-1}/dt) / D(k) along t, inverse FFT."""
    nt, nx, ny = s.shape
    kx = np.exp(-2j * np.pi * np.fft.fftfreq(nx))[:, None]  # shift by -1 in x
    ky = np.exp(-2j * np.pi * np.fft.fftfreq(ny))[None, :]
    # symbol of the spatial upwind operator a_x D_x + a_y D_y
    if s.ax > 0:
        sx = s.ax / s.dx * (1 - kx)
    else:
        sx = s.ax / s.dx * (np.conj(kx) - 1)
    if s.ay > 0:
        sy = s.ay / s.dy * (1 - ky)
    else:
        sy = s.ay / s.dy * (np.conj(ky) - 1)
    Dk = 1 / s.dt + sx + sy
    bh = np.fft.fft2(np.asarray(b, np.float64).reshape(s.shape), axes=(1, 2))
    xh = np.zeros_like(bh)
    prev = np.zeros((nx, ny), complex)
    for i in range(nt):
        prev = (bh[i] + (prev / s.dt if i else 0)) / Dk
        xh[i] = prev
    return np.real(np.fft.ifft2(xh, axes=(1, 2)))


def solve(s):
    """FP64 discrete solution (the oracle for large grids)."""
    return solve_fft(s, -residual_p(s, np.zeros(s.shape)))


# -- multigrid pieces of the GPU solver (matrix-free, rediscretised) ---------
def level_setup(s, nmin=4):
    levels = [s]
    while True:
        c = levels[-1]
        if min(c.shape) < 2 * nmin or any(n % 2 for n in c.shape):
            break
        levels.append(AdvectSetup(c.nt // 2, c.nx // 2, c.ny // 2, c.ax, c.ay,
                                  np.zeros((c.nx // 2, c.ny // 2)),
                                  c.dt * c.nt))
    return levels


def _p1(a, axis, periodic):
    """Cell-centred linear interpolation to twice the size along `axis`."""
    am = np.roll(a, 1, axis)
    ap = np.roll(a, -1, axis)
    if not periodic:
        n = a.shape[axis]
        first = [slice(None)] * a.ndim
        first[axis] = 0
        last = [slice(None)] * a.ndim
        last[axis] = n - 1
        am[tuple(first)] = a[tuple(first)]
        ap[tuple(last)] = a[tuple(last)]
    shp = list(a.shape)
    shp[axis] *= 2
    out = np.zeros(shp)
    ev = [slice(None)] * a.ndim
    ev[axis] = slice(0, None, 2)
    od = [slice(None)] * a.ndim
    od[axis] = slice(1, None, 2)
    out[tuple(ev)] = 0.75 * a + 0.25 * am
    out[tuple(od)] = 0.75 * a + 0.25 * ap
    return out


def prolong(e):
    """Trilinear cell-centred prolongation (t clamped, x and y periodic)."""
    return _p1(_p1(_p1(e, 0, False), 1, True), 2, True)


def _r1(a, axis, periodic):
    """Transpose of _p1 along `axis`, divided by 2 (weights (1,3,3,1)/8)."""
    n = a.shape[axis] // 2
    ev = [slice(None)] * a.ndim
    ev[axis] = slice(0, None, 2)
    od = [slice(None)] * a.ndim
    od[axis] = slice(1, None, 2)
    e, o = a[tuple(ev)], a[tuple(od)]
    out = 0.75 * (e + o)
    # e at coarse c feeds coarse c-1 with 0.25 (odd of c-1 uses ap -> c); the
    # transpose: coarse c gets 0.25 * even[c+1] and 0.25 * odd[c-1].
    ep = np.roll(e, -1, axis)
    om = np.roll(o, 1, axis)
    if not periodic:
        first = [slice(None)] * a.ndim
        first[axis] = 0
        last = [slice(None)] * a.ndim
        last[axis] = n - 1
        # clamped ends: even[0] and odd[n-1] put their 0.25 on themselves
        ep = ep.copy()
        om = om.copy()
        ep[tuple(last)] = 0.0
        om[tuple(first)] = 0.0
        out[tuple(first)] += 0.25 * e[tuple(first)]
        out[tuple(last)] += 0.25 * o[tuple(last)]
    out = out + 0.25 * (ep + om)
    return 0.5 * out


def restrict(r):
    """Full weighting: (1/8) P^T, the transpose of `prolong`."""
    return _r1(_r1(_r1(r, 0, False), 1, True), 2, True)


def diag(s):
    return 1 / s.dt + abs(s.ax) / s.dx + abs(s.ay) / s.dy


def coarse_matrix(s):
    return jacobian(s).toarray()


def vcycle(levels, b, lvl=0, omega=0.8, pre=2, post=2):
    s = levels[lvl]
    if lvl == len(levels) - 1:
        return np.linalg.solve(coarse_matrix(s), b.ravel()).reshape(b.shape)
    D = diag(s)
    x = np.zeros_like(b)
    for _ in range(pre):
        x = x + omega * (b - _jv(s, x)) / D
    rc = restrict(b - _jv(s, x))
    x = x + prolong(vcycle(levels, rc, lvl + 1, omega, pre, post))
    for _ in range(post):
        x = x + omega * (b - _jv(s, x)) / D
    return x


def bicgstab(s, b, levels=None, tol=1e-6, maxit=200):
    """Right-preconditioned BiCGStab (van der Vorst 1992) with one V-cycle
    per preconditioner application; returns (x, iterations)."""
    levels = level_setup(s) if levels is None else levels
    M = lambda r: vcycle(levels, r)
    A = lambda v: _jv(s, v)
    x = np.zeros_like(b)
    r = b - A(x)
    rh = r.copy()
    rho = alpha = w = 1.0
    v = np.zeros_like(b)
    p = np.zeros_like(b)
    nb = np.linalg.norm(b)
    for it in range(maxit):
        rho1 = np.vdot(rh, r)
        beta = (rho1 / rho) * (alpha / w)
        rho = rho1
        p = r + beta * (p - w * v)
        ph = M(p)
        v = A(ph)
        alpha = rho / np.vdot(rh, v)
        s_ = r - alpha * v
        if np.linalg.norm(s_) <= tol * nb:
            return x + alpha * ph, it + 1
        sh = M(s_)
        t = A(sh)
        w = np.vdot(t, s_) / np.vdot(t, t)
        x = x + alpha * ph + w * sh
        r = s_ - w * t
        if np.linalg.norm(r) <= tol * nb:
            return x, it + 1
    return x, maxit


def rel_err(u, ref):
    return float(np.linalg.norm(np.asarray(u) - ref) / np.linalg.norm(ref))
