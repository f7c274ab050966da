"""Oracle: the reference's FD wave problem, restated in NumPy (FP64).

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).

Follows
  * wave.py:27-39   ``get_exact``  (reference cosine profile, u_t by autodiff;
                    here by the analytic derivative),
  * wave.py:67-122  ``operator_fd`` (residual with quadratic-half Dirichlet
                    extrapolation in x and the initial-row terms),
  * wave.py:433-464 domain and boundary data,
  * util_op.py:127-137 cell centres, util_op.py:508-563 roll semantics of
    ``Context.field`` (``field(k, -1, 0)[i, j] == u[i-1, j]``, periodic wrap),
  * util_op.py:585-614 + 859-937 per-shift Jacobian -> CSR,
  * util_op.py:627-654 loss = sum_k mean(f_k^2) and its gradient,
  * linsolver.py:28-45 normal equations + ``spsolve(permc_spec='MMD_ATA')``,
  * util.py:242-268 Newton loop.

The wave speed ``c`` (residual ``u_tt - c^2 u_xx``) and the seeded sine
profile are the options added for the benchmark workloads; ``c=1`` and the
cosine profile reproduce the reference exactly.
"""
import numpy as np
import scipy.sparse
import scipy.sparse.linalg

# Shifts requested by operator_fd's stencil_var (wave.py:80-88), in that order.
WAVE_SHIFTS = ((0, 0), (-1, 0), (-2, 0), (-1, -1), (-1, 1))


def cell_center_1d(lower, upper, n):
    """util_op.py:130-137."""
    x = np.linspace(lower, upper, n, endpoint=False, dtype=np.float64)
    h = (x[1] - x[0]) if n > 1 else (upper - lower)
    return x + h * 0.5


class WaveSetup:
    """Grid and boundary data of one wave instance (wave.py:433-464)."""

    def __init__(self, nt, nx, init_u, init_ut, left_u, right_u, c=1.0,
                 lower=(0.0, -1.0), upper=(1.0, 1.0)):
        self.nt, self.nx = int(nt), int(nx)
        self.lower, self.upper = lower, upper
        self.dt = (upper[0] - lower[0]) / nt
        self.dx = (upper[1] - lower[1]) / nx
        self.c = float(c)
        self.init_u = np.asarray(init_u, np.float64)
        self.init_ut = np.asarray(init_ut, np.float64)
        self.left_u = np.asarray(left_u, np.float64)
        self.right_u = np.asarray(right_u, np.float64)

    @property
    def shape(self):
        return (self.nt, self.nx)


def exact_cos(t, x):
    """wave.py:27-39: u and u_t of the reference's 5-mode cosine profile."""
    u = np.zeros(np.broadcast(t, x).shape)
    ut = np.zeros_like(u)
    for i in (1, 2, 3, 4, 5):
        k = i * np.pi
        u = u + np.cos((x - t + 0.5) * k) + np.cos((x + t - 0.5) * k)
        ut = ut + k * np.sin((x - t + 0.5) * k) - k * np.sin((x + t - 0.5) * k)
    return u / 10.0, ut / 10.0


def sine_amplitudes(seed, nmodes):
    """Seeded amplitudes a_k ~ N(0,1)/k, k=1..nmodes (benchmark profile)."""
    rng = np.random.default_rng(seed)
    return rng.standard_normal(nmodes) / np.arange(1, nmodes + 1)


def exact_sine(t, x, amps, c=1.0):
    """d'Alembert solution u = (f(x-ct) + f(x+ct))/2 with
    f(x) = sum_k a_k sin(k pi (x+1)/2); odd about x=-1 and x=1, so the
    Dirichlet values at x=+-1 vanish and u_t(x, 0) = 0."""
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


def make_setup(nt, nx, profile="cos", seed=0, nmodes=5, c=1.0):
    """Boundary data as wave.py:457-464 computes it from the exact solution."""
    lower, upper = (0.0, -1.0), (1.0, 1.0)
    t1 = cell_center_1d(lower[0], upper[0], nt)
    x1 = cell_center_1d(lower[1], upper[1], nx)
    if profile == "cos":
        assert c == 1.0, "the reference cosine profile has unit wave speed"
        ex = exact_cos
    elif profile == "sine":
        amps = sine_amplitudes(seed, nmodes)
        ex = lambda t, x: exact_sine(t, x, amps, c)
    else:
        raise ValueError("Unknown profile=" + profile)
    left_u, _ = ex(t1, t1 * 0 + lower[1])
    right_u, _ = ex(t1, t1 * 0 + upper[1])
    init_u, init_ut = ex(x1 * 0 + lower[0], x1)
    tt, xx = np.meshgrid(t1, x1, indexing="ij")
    exact_u, _ = ex(tt, xx)
    s = WaveSetup(nt, nx, init_u, init_ut, left_u, right_u, c=c)
    s.exact_u = exact_u
    return s


def extrap_quadh(u0, u1, u1p):
    """util_op.py:1017-1023."""
    return (u0 - 6 * u1 + 8 * u1p) / 3


def residual(s, u):
    """wave.py:67-122 with ``Context.field`` = np.roll (util_op.py:545-554)."""
    u = np.asarray(u, np.float64).reshape(s.shape)
    nt, nx = s.shape
    dt, dx = s.dt, s.dx
    it = np.arange(nt)[:, None]
    ix = np.arange(nx)[None, :]
    utm = np.roll(u, 1, axis=0)          # field('u', -1, 0)
    utmm = np.roll(u, 2, axis=0)         # field('u', -2, 0)
    uxm = np.roll(utm, 1, axis=1)        # field('u', -1, -1)
    uxp = np.roll(utm, -1, axis=1)       # field('u', -1, 1)
    left_utm = np.roll(s.left_u, 1)
    right_utm = np.roll(s.right_u, 1)
    uxm = np.where(ix == 0, extrap_quadh(uxp, utm, left_utm[:, None]), uxm)
    uxp = np.where(ix == nx - 1, extrap_quadh(uxm, utm, right_utm[:, None]),
                   uxp)
    u_t_tm = (u - utm) / dt
    u_t_tmm = (utm - utmm) / dt
    u_t_tmm = np.where(it == 1, s.init_ut[None, :], u_t_tmm)
    u_tt = (u_t_tm - u_t_tmm) / dt
    u_xx = (uxm - 2 * utm + uxp) / (dx**2)
    fu = u_tt - s.c**2 * u_xx
    u0 = s.init_u + 0.5 * dt * s.init_ut
    fu = np.where(it == 0, u - u0[None, :], fu)
    return fu


def slot_coefficients(s):
    """Per-shift coefficient fields C[shift][i, j] = d f[i, j] / d u[(i,j)+shift].

    This is what ``Problem._eval_grad0`` (util_op.py:585-614) returns with
    ``split_shifts=True``: one gradient per rolled argument, with zero
    gradient through the branch ``tf.where`` did not select.
    """
    nt, nx = s.shape
    A = 1.0 / s.dt**2
    B = s.c**2 / s.dx**2
    it = np.arange(nt)[:, None] + np.zeros((1, nx), int)
    ix = np.zeros((nt, 1), int) + np.arange(nx)[None, :]
    z = np.zeros((nt, nx))
    cu, ctm, ctmm, cxm, cxp = z + A, z - A, z.copy(), z.copy(), z.copy()
    ctm = np.where(it >= 2, ctm - A, ctm)
    ctmm = np.where(it >= 2, A, 0.0)
    # u_xx_raw = uxm' - 2 utm + uxp'  with the x-halo replacements.
    m_xm = np.where(ix == 0, 0.0, 1.0)
    m_xp = np.where(ix == 0, 1.0 / 3, 0.0)
    m_tm = np.where(ix == 0, -2.0, 0.0)
    last = ix == nx - 1
    p_xm = np.where(last, m_xm / 3, 0.0)
    p_xp = np.where(last, m_xp / 3, 1.0)
    p_tm = np.where(last, m_tm / 3 - 2.0, 0.0)
    cxm = -B * (m_xm + p_xm)
    cxp = -B * (m_xp + p_xp)
    ctm = ctm - B * (m_tm + p_tm - 2.0)
    row0 = it == 0
    res = {
        (0, 0): np.where(row0, 1.0, cu),
        (-1, 0): np.where(row0, 0.0, ctm),
        (-2, 0): np.where(row0, 0.0, ctmm),
        (-1, -1): np.where(row0, 0.0, cxm),
        (-1, 1): np.where(row0, 0.0, cxp),
    }
    return res


def linearize(s, u):
    """util_op.py:859-937 for the single-field wave operator.

    Returns ``(const, J)``: the residual fields and the CSR Jacobian with
    ``J[c, (c + shift) mod shape] += C_shift[c]`` (the ``mod.roll`` of
    util_op.py:885-887)."""
    nt, nx = s.shape
    N = nt * nx
    f = residual(s, u)
    coefs = slot_coefficients(s)
    row = np.arange(N)
    col_diag = row.reshape(s.shape)
    J = scipy.sparse.csr_matrix((N, N), dtype=np.float64)
    for shift in WAVE_SHIFTS:
        col = np.roll(col_diag, np.negative(shift), axis=(0, 1)).flatten()
        g = coefs[shift].flatten()
        J = J + scipy.sparse.csr_matrix((g, (row, col)), shape=(N, N))
    return [f], J.tocsr()


def solve_direct(J, rhs, beta=0.0):
    """linsolver.py:35-45: (J^T J + beta^2 I) x = J^T rhs by SuperLU (MMD_ATA)."""
    A = J.T.dot(J).tocsr()
    if beta:
        A = A + beta**2 * scipy.sparse.identity(A.shape[0], format="csr")
    b = J.T.dot(rhs)
    return scipy.sparse.linalg.spsolve(A, b, permc_spec="MMD_ATA")


def newton(s, u0=None, epochs=2):
    """util.py:242-268: ``epochs`` Newton steps from ``u0`` (zeros by default,
    util_op.py:818-821)."""
    u = np.zeros(s.shape) if u0 is None else np.array(u0, np.float64)
    for _ in range(epochs):
        const, J = linearize(s, u)
        du = solve_direct(J, -const[0].flatten())
        u = u + du.reshape(s.shape)
    return u


def loss_grad(s, u):
    """util_op.py:627-654: loss = mean(f^2), grad = (2/N) J^T f."""
    f = residual(s, u)
    N = f.size
    _, J = linearize(s, u)
    g = (2.0 / N) * J.T.dot(f.flatten())
    return float(np.mean(f**2)), g.reshape(s.shape)


def jv(s, v):
    """J v for the affine wave operator: f(v) - f(0)."""
    return residual(s, v) - residual(s, np.zeros(s.shape))


def jtv(s, w):
    _, J = linearize(s, np.zeros(s.shape))
    return J.T.dot(np.asarray(w).flatten()).reshape(s.shape)


def march(s, b):
    """Forward substitution for J x = b.  J is lower triangular in C order
    (row (i, j) only couples to rows i-1, i-2), so this is the direct solve of
    the same system whose normal equations linsolver.py:35-45 factorizes."""
    nt, nx = s.shape
    C = slot_coefficients(s)
    b = np.asarray(b, np.float64).reshape(s.shape)
    x = np.zeros(s.shape)
    for i in range(nt):
        acc = b[i].copy()
        if i >= 1:
            p = x[i - 1]
            acc -= C[(-1, 0)][i] * p
            acc -= C[(-1, -1)][i] * np.roll(p, 1)
            acc -= C[(-1, 1)][i] * np.roll(p, -1)
        if i >= 2:
            acc -= C[(-2, 0)][i] * x[i - 2]
        x[i] = acc / C[(0, 0)][i]
    return x


def solve_march(s, u0=None, rounds=1):
    """Newton with the forward-substitution direct solve (FP64)."""
    u = np.zeros(s.shape) if u0 is None else np.array(u0, np.float64)
    for _ in range(rounds):
        u = u + march(s, -residual(s, u))
    return u


def rel_err(u, ref):
    u = np.asarray(u, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.linalg.norm(u - ref) / np.linalg.norm(ref))


def l2_error(u, ref):
    """``ref_du_l2`` of wave.py:345: sqrt(mean((exact - u)^2))."""
    return float(np.mean((np.asarray(ref) - np.asarray(u))**2)**0.5)
