"""Oracle: the reference's steady Navier-Stokes cavity operator, FP64.

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).

Restates ns_steady.py:142-433 (``operator``) with its defaults --bc 0 (no
slip, lid u = 1 at y = 1 by quadratic extrapolation), --rhiechow 1,
--fit_mu 0, --plot_stream 0, anneal off, on an (N, N) cell-centred grid of
[0, 1]^2 (ns_steady.py:899-906), mu = 1/Re (ns_steady.py:867):
  fu = uf u_x + vf u_y - mu lap(u) + p_x^c,
  fv = uf v_x + vf v_y - mu lap(v) + p_y^c,
  fp = Rhie-Chow continuity (ns_steady.py:339-386),
  [+ imposed-point terms mask (u - u_imp) alpha N / n_imp (396-404),
   + Laplacian penalty kreg {u_xx, u_yy, v_xx, v_yy} (406-411),
   + optional pressure pin w (p[pin] - 0) (benchmark extension)].
u_x = upwind2(frozen) + upwind1(live) - upwind1(frozen) (deferred
correction, 171-204, 282-283, 320-323).

Written in torch (CPU, FP64) so that the same code evaluates the residual
and, by autograd over the 15 rolled live arguments (u, v, p at the shifts of
stencil_var), the per-shift coefficient fields that Problem._eval_grad0
(util_op.py:585-614) returns -- the reference's Jacobian, assembled to CSR as
util_op.py:877-896 does.
"""
import numpy as np
import scipy.sparse
import scipy.sparse.linalg
import torch

SHIFTS = ((0, 0), (-1, 0), (1, 0), (0, -1), (0, 1))  # stencil_var order
FIELDS = ("u", "v", "p")


def _roll(a, shift):
    # ctx.field(key, *shift) == roll(a, -shift)
    return torch.roll(a, (-shift[0], -shift[1]), (0, 1))


def _quadh(u0, u1, u1p):
    return (u0 - 6 * u1 + 8 * u1p) / 3


def _linear(u0, u1):
    return 2 * u1 - u0


class NsSetup:

    def __init__(self, n, Re, mask=None, u_imp=None, v_imp=None, alpha=1.0,
                 kreg=0.0, pin=None, pin_weight=0.0):
        self.n = int(n)
        self.shape = (self.n, self.n)
        self.dx = self.dy = 1.0 / n
        self.mu = 1.0 / Re
        self.mask = mask
        self.u_imp, self.v_imp = u_imp, v_imp
        self.alpha = alpha
        self.kreg = kreg
        self.pin = pin
        self.pin_weight = pin_weight


def operator(s, live, frozen):
    """Residual terms.  live: dict (field, shift) -> tensor (the rolled live
    arguments); frozen: dict field -> tensor (the state, no gradient)."""
    n = s.n
    dx, dy, mu = s.dx, s.dy, s.mu
    ix = torch.arange(n)[:, None] + torch.zeros((1, n), dtype=torch.long)
    iy = torch.zeros((n, 1), dtype=torch.long) + torch.arange(n)[None, :]
    nx = ny = n
    zero = torch.zeros((n, n), dtype=torch.float64)

    def st_live(key):
        return [live[(key, sh)] for sh in SHIFTS]

    def st_frozen(key):
        a = frozen[key]
        return [_roll(a, sh) for sh in SHIFTS]

    def bc_u(st):
        st[1] = torch.where(ix == 0, _quadh(st[2], st[0], 0), st[1])
        st[2] = torch.where(ix == nx - 1, _quadh(st[1], st[0], 0), st[2])
        st[3] = torch.where(iy == 0, _quadh(st[4], st[0], 0), st[3])
        st[4] = torch.where(iy == ny - 1, _quadh(st[3], st[0], 1), st[4])
        return st

    def bc_v(st):
        st[1] = torch.where(ix == 0, _quadh(st[2], st[0], 0), st[1])
        st[2] = torch.where(ix == nx - 1, _quadh(st[1], st[0], 0), st[2])
        st[3] = torch.where(iy == 0, _quadh(st[4], st[0], 0), st[3])
        st[4] = torch.where(iy == ny - 1, _quadh(st[3], st[0], 0), st[4])
        return st

    def bc_extrap(st):
        st[1] = torch.where(ix == 0, _linear(st[2], st[0]), st[1])
        st[2] = torch.where(ix == nx - 1, _linear(st[1], st[0]), st[2])
        st[3] = torch.where(iy == 0, _linear(st[4], st[0]), st[3])
        st[4] = torch.where(iy == ny - 1, _linear(st[3], st[0]), st[4])
        return st

    def stencil5(st):
        st5 = [torch.roll(st[1], 1, 0), torch.roll(st[2], -1, 0),
               torch.roll(st[3], 1, 1), torch.roll(st[4], -1, 1)]
        st5[0] = torch.where(ix == 0, st[1], st5[0])
        st5[1] = torch.where(ix == nx - 1, st[2], st5[1])
        st5[2] = torch.where(iy == 0, st[3], st5[2])
        st5[3] = torch.where(iy == ny - 1, st[4], st5[3])
        return st5

    def upwind_second(st, st5, u, v):
        q, qxm, qxp, qym, qyp = st
        qxmm, qxpp, qymm, qypp = st5
        q_xm = (qxmm - 4 * qxm + 3 * q) / (2 * dx)
        q_xp = (-3 * q + 4 * qxp - qxpp) / (2 * dx)
        q_ym = (qymm - 4 * qym + 3 * q) / (2 * dy)
        q_yp = (-3 * q + 4 * qyp - qypp) / (2 * dy)
        q_xm = torch.where(ix == 0, (q - qxm) / dx, q_xm)
        q_xp = torch.where(ix == nx - 1, (qxp - q) / dx, q_xp)
        q_ym = torch.where(iy == 0, (q - qym) / dy, q_ym)
        q_yp = torch.where(iy == ny - 1, (qyp - q) / dy, q_yp)
        return torch.where(u > 0, q_xm, q_xp), torch.where(v > 0, q_ym, q_yp)

    def upwind_low(st, u, v):
        q, qxm, qxp, qym, qyp = st
        q_x = torch.where(u > 0, (q - qxm) / dx, (qxp - q) / dx)
        q_y = torch.where(v > 0, (q - qym) / dy, (qyp - q) / dy)
        return q_x, q_y

    def central(st):
        q, qxm, qxp, qym, qyp = st
        return (qxp - qxm) / (2 * dx), (qyp - qym) / (2 * dy)

    def laplace_split(st):
        q, qxm, qxp, qym, qyp = st
        return (qxp - 2 * q + qxm) / dx**2, (qyp - 2 * q + qym) / dy**2

    u_st = bc_u(st_live("u"))
    uf_st = bc_u(st_frozen("u"))
    uf_st5 = stencil5(uf_st)
    uf = uf_st[0]
    v_st = bc_v(st_live("v"))
    vf_st = bc_v(st_frozen("v"))
    vf_st5 = stencil5(vf_st)
    vf = vf_st[0]
    p_st = bc_extrap(st_live("p"))

    def mix(hf, l, lf):
        return [a + b - c for a, b, c in zip(hf, l, lf)]

    u_x, u_y = mix(upwind_second(uf_st, uf_st5, uf, vf),
                   upwind_low(u_st, uf, vf), upwind_low(uf_st, uf, vf))
    v_x, v_y = mix(upwind_second(vf_st, vf_st5, uf, vf),
                   upwind_low(v_st, uf, vf), upwind_low(vf_st, uf, vf))
    p_xc, p_yc = central(p_st)
    u_xx, u_yy = laplace_split(u_st)
    v_xx, v_yy = laplace_split(v_st)
    u_lap = u_xx + u_yy
    v_lap = v_xx + v_yy
    fu = uf * u_x + vf * u_y - mu * u_lap + p_xc
    fv = uf * v_x + vf * v_y - mu * v_lap + p_yc

    # Rhie-Chow (ns_steady.py:339-386), bc = 0.
    g = torch.abs(uf) / dx + torch.abs(vf) / dy + mu * (2 / dx**2 + 2 / dy**2)
    u, uxm, uxp = u_st[0], u_st[1], u_st[2]
    v, vym, vyp = v_st[0], v_st[3], v_st[4]
    pf_st = bc_extrap(st_frozen("p"))
    pf, pfxm, pfxp, pfym, pfyp = pf_st
    pfxmm, pfxpp, pfymm, pfypp = stencil5(pf_st)
    p, pxm, pxp, pym, pyp = p_st
    gxm, gxp = torch.roll(g, 1, 0), torch.roll(g, -1, 0)
    gym, gyp = torch.roll(g, 1, 1), torch.roll(g, -1, 1)
    qxm = (u + uxm) * 0.5 + (1 / gxm * (pf - pfxmm) / (2 * dx)) * 0.5 + \
        (1 / g * (pfxp - pfxm) / (2 * dx)) * 0.5 - \
        (1 / gxm + 1 / g) * 0.5 * (p - pxm) / dx
    qxp = (u + uxp) * 0.5 + (1 / gxp * (pfxpp - pf) / (2 * dx)) * 0.5 + \
        (1 / g * (pfxp - pfxm) / (2 * dx)) * 0.5 - \
        (1 / gxp + 1 / g) * 0.5 * (pxp - p) / dx
    qym = (v + vym) * 0.5 + (1 / gym * (pf - pfymm) / (2 * dy)) * 0.5 + \
        (1 / g * (pfyp - pfym) / (2 * dy)) * 0.5 - \
        (1 / gym + 1 / g) * 0.5 * (p - pym) / dy
    qyp = (v + vyp) * 0.5 + (1 / gyp * (pfypp - pf) / (2 * dy)) * 0.5 + \
        (1 / g * (pfyp - pfym) / (2 * dy)) * 0.5 - \
        (1 / gyp + 1 / g) * 0.5 * (pyp - p) / dy
    qxm = torch.where(ix == 0, zero, qxm)
    qxp = torch.where(ix == nx - 1, zero, qxp)
    qym = torch.where(iy == 0, zero, qym)
    qyp = torch.where(iy == ny - 1, zero, qyp)
    fp = (qxp - qxm) / dx + (qyp - qym) / dy
    res = [fu, fv, fp]
    if s.mask is not None:
        n_imp = float(np.sum(s.mask))
        coeff = s.alpha * n * n / n_imp
        m = torch.as_tensor(s.mask)
        res += [m * (u - torch.as_tensor(s.u_imp)) * coeff,
                m * (v - torch.as_tensor(s.v_imp)) * coeff]
    if s.kreg:
        k = s.kreg
        res += [u_xx * k, u_yy * k, v_xx * k, v_yy * k]
    if s.pin is not None:
        pin = torch.zeros((n, n), dtype=torch.float64)
        pin[s.pin] = 1.0
        res += [pin * p * s.pin_weight]
    return res


def _live_from(state, requires_grad=False):
    live = {}
    for key in FIELDS:
        a = torch.as_tensor(np.asarray(state[key], np.float64))
        for sh in SHIFTS:
            t = _roll(a, sh).clone()
            t.requires_grad_(requires_grad)
            live[(key, sh)] = t
    return live


def residual(s, state):
    """List of residual fields at ``state`` = {'u','v','p'} (numpy)."""
    frozen = {k: torch.as_tensor(np.asarray(state[k], np.float64))
              for k in FIELDS}
    with torch.no_grad():
        return [f.numpy() for f in operator(s, _live_from(state), frozen)]


def coefficients(s, state):
    """Per-equation, per-(field, shift) coefficient fields at ``state``
    (util_op.py:585-614): coefs[e][(field, shift)] = d f_e / d arg."""
    frozen = {k: torch.as_tensor(np.asarray(state[k], np.float64))
              for k in FIELDS}
    live = _live_from(state, requires_grad=True)
    ff = operator(s, live, frozen)
    args = list(live.keys())
    coefs = []
    for f in ff:
        gs = torch.autograd.grad(f.sum(), [live[k] for k in args],
                                 retain_graph=True, allow_unused=True)
        coefs.append({k: (g.numpy() if g is not None else np.zeros(s.shape))
                      for k, g in zip(args, gs)})
    return [f.detach().numpy() for f in ff], coefs


def linearize(s, state):
    """util_op.py:859-937: (const, CSR J) with J columns rolled by -shift."""
    n = s.n
    N = n * n
    const, coefs = coefficients(s, state)
    row = np.arange(N)
    col_diag = row.reshape(s.shape)
    J = scipy.sparse.csr_matrix((len(const) * N, 3 * N))
    for i, c in enumerate(coefs):
        for (key, sh), g in c.items():
            if not np.any(g):
                continue
            col = np.roll(col_diag, np.negative(sh), axis=(0, 1)).ravel()
            j = FIELDS.index(key)
            J = J + scipy.sparse.csr_matrix(
                (g.ravel(), (row + i * N, col + j * N)),
                shape=(len(const) * N, 3 * N))
    return const, J.tocsr()


def newton(s, state, epochs=1):
    """util.py:242-268 with linsolver.py:35-45."""
    st = {k: np.array(state[k], np.float64) for k in FIELDS}
    n = s.n
    for _ in range(epochs):
        const, J = linearize(s, st)
        rhs = -np.concatenate([c.ravel() for c in const])
        A = (J.T @ J).tocsr()
        d = scipy.sparse.linalg.spsolve(A, J.T @ rhs, permc_spec="MMD_ATA")
        for i, k in enumerate(FIELDS):
            st[k] = st[k] + d[i * n * n:(i + 1) * n * n].reshape(s.shape)
    return st


def newton_pinned(s, state, epochs=1, pin=(0, 0)):
    """Newton on the square system with the continuity row of cell `pin`
    replaced by p[pin] = 0 (the forward problem's constant-pressure null
    space removed), each step solved directly (scipy spsolve).  Same fixed
    point as newton() up to the pressure constant."""
    st = {k: np.array(state[k], np.float64) for k in FIELDS}
    n = s.n
    N = n * n
    pidx = pin[0] * n + pin[1]
    for _ in range(epochs):
        const, J = linearize(s, st)
        if len(const) != 3:
            raise ValueError("forward problem only")
        r = np.concatenate([c.ravel() for c in const])
        J = J.tolil()
        row = 2 * N + pidx
        J.rows[row] = [2 * N + pidx]
        J.data[row] = [1.0]
        r[row] = st["p"].ravel()[pidx]
        d = scipy.sparse.linalg.spsolve(J.tocsc(), -r)
        for i, k in enumerate(FIELDS):
            st[k] = st[k] + d[i * N:(i + 1) * N].reshape(s.shape)
    return st


def loss_grad_live(s, state):
    """loss = sum_e mean(f_e^2) and its gradient through the live (rolled)
    arguments only, the reference's tape gradient (util_op.py:627-654), by
    one reverse pass: returns (list of residual rms, loss, {field: grad})."""
    frozen = {k: torch.as_tensor(np.asarray(state[k], np.float64))
              for k in FIELDS}
    live = _live_from(state, requires_grad=True)
    ff = operator(s, live, frozen)
    loss = sum((f**2).mean() for f in ff)
    keys = list(live)
    gs = torch.autograd.grad(loss, [live[k] for k in keys], allow_unused=True)
    g = {k: torch.zeros(s.shape, dtype=torch.float64) for k in FIELDS}
    for (k, sh), ga in zip(keys, gs):
        if ga is not None:
            g[k] += torch.roll(ga, (sh[0], sh[1]), (0, 1))  # undo _roll
    rms = [float(f.detach().pow(2).mean().sqrt()) for f in ff]
    return rms, float(loss.detach()), {k: v.numpy() for k, v in g.items()}
