"""Newton linear solves, the interface of linsolver.py:28-167.

``solve(J, rhs, args, dhistory, linsolver)`` returns d with J d ~= rhs (the
reference solves the normal equations J^T J d = J^T rhs, which has the same
solution for the square, nonsingular Jacobians of the registered families).

linsolver="direct"    exact direct solve on the GPU (FP64: forward
                      substitution for the wave family);
linsolver="mixed"     the same direct solve in FP32 on an FP64 right-hand
                      side (one step of mixed-precision iterative refinement
                      per Newton epoch);
linsolver="multigrid" matrix-free Krylov solve preconditioned by the
                      geometric multigrid V-cycle (families that provide it);
                      other Jacobians with `to_csr`: flexible CG on the
                      normal equations preconditioned by a V-cycle of the
                      CSR multigrid (the reference's pyamg SA + CG,
                      linsolver.py:77-89; pyamg is not used);
linsolver="bicgstab"  BiCGStab on the (relaxed) normal equations, stopped at
                      |r| <= linsolver_tol or linsolver_maxiter (scipy's
                      bicgstab with tol=0, linsolver.py:90-103);
linsolver="lsqr"      LSQR of Paige and Saunders on J d = rhs with damping
                      beta (scipy's lsqr, linsolver.py:57-69).
The other reference choices (direct_cu, sparseqr, lsqr_cu) map to "direct".
With --beta or --betadiag set, "direct" and "mixed" solve the relaxed normal
equations of linsolver.py:35-41 (solve_regularized).  The iterative choices
record linsolver_residual and linsolver_niter (lsqr also linsolver_anorm and
linsolver_acond) in `dhistory`, as the reference does.
"""
import numpy as np
import torch

ALIASES = {"direct_cu": "direct", "sparseqr": "direct", "lsqr_cu": "direct"}


DENSE_MAX = 16384  # unknowns up to which the regularised solve is dense


def solve_regularized(matr, rhs, beta=0.0, betadiag=0.0, tol=1e-12,
                      maxiter=None):
    """d of (J^T J + beta^2 I + betadiag^2 diag(J^T J + beta^2 I)) d = J^T rhs,
    the relaxed normal equations of linsolver.py:35-41: dense (cuSOLVER
    through torch) up to DENSE_MAX unknowns, else conjugate gradients with
    J and J^T matrix-free."""
    n = matr.shape[1]
    rhs = rhs.to(torch.float64)
    if n <= DENSE_MAX and hasattr(matr, "to_csr"):
        J = matr.to_csr().to_dense().to(torch.float64)
        A = J.T @ J
        if beta:
            A += beta**2 * torch.eye(n, dtype=A.dtype, device=A.device)
        if betadiag:
            A += betadiag**2 * torch.diag(torch.diagonal(A))
        return torch.linalg.solve(A, J.T @ rhs)
    A, b = _normal_equations(matr, rhs, beta, betadiag)
    x = torch.zeros_like(b)
    r = b.clone()
    p = r.clone()
    rr = torch.dot(r, r)
    r0 = rr.sqrt().item()
    for _ in range(maxiter or 10 * n):
        if rr.sqrt().item() <= tol * max(r0, 1e-300):
            break
        Ap = A(p)
        alpha = rr / torch.dot(p, Ap)
        x += alpha * p
        r -= alpha * Ap
        rn = torch.dot(r, r)
        p = r + (rn / rr) * p
        rr = rn
    return x


def _normal_equations(matr, rhs, beta=0.0, betadiag=0.0):
    """x -> (J^T J + beta^2 I + betadiag^2 diag(J^T J + beta^2 I)) x
    matrix-free, and J^T rhs (linsolver.py:35-41)."""
    n = matr.shape[1]
    rhs = rhs.to(torch.float64)
    diag = None
    if betadiag:
        if hasattr(matr, "jtj_diag"):
            diag = matr.jtj_diag().to(torch.float64)
        elif hasattr(matr, "to_csr"):
            J = matr.to_csr().to_sparse_coo().coalesce()
            diag = torch.zeros(n, dtype=torch.float64, device=rhs.device)
            diag.index_add_(0, J.indices()[1],
                            J.values().to(torch.float64)**2)
        else:
            raise ValueError("betadiag needs diag(J^T J) or to_csr()")
        diag = betadiag**2 * (diag + beta**2)
    jtj = getattr(matr, "jtj_v", None)

    def A(x):
        y = jtj(x) if jtj is not None else matr.rmatvec(matr.matvec(x))
        if beta:
            y = y + beta**2 * x
        if diag is not None:
            y = y + diag * x
        return y

    return A, matr.rmatvec(rhs).to(torch.float64)


def bicgstab(matr, rhs, atol=1e-6, maxiter=50, beta=0.0, betadiag=0.0,
             dhistory=None):
    """linsolver.py:90-103: BiCGStab (van der Vorst) on the relaxed normal
    equations from zero, shadow residual r0, stopped when |r| <= atol after
    a half or a full step or after `maxiter` iterations, as scipy's
    bicgstab(tol=0, atol=atol).  dhistory gets the RMS of A x - b and the
    iteration count."""
    A, b = _normal_equations(matr, rhs, beta, betadiag)
    x = torch.zeros_like(b)
    r = b.clone()
    rt = r.clone()
    p = v = None
    rho_prev = alpha = omega = None
    tiny = np.finfo(np.float64).eps**2
    niter = 0  # completed full iterations (scipy's callback count)
    for it in range(maxiter):
        if torch.linalg.norm(r).item() < atol:
            break
        rho = torch.dot(rt, r)
        if abs(rho.item()) < tiny:
            break  # breakdown
        if it == 0:
            p = r.clone()
        else:
            p = r + (rho / rho_prev) * (alpha / omega) * (p - omega * v)
        v = A(p)
        alpha = rho / torch.dot(rt, v)
        s = r - alpha * v
        if torch.linalg.norm(s).item() < atol:
            x += alpha * p
            break
        t = A(s)
        omega = torch.dot(t, s) / torch.dot(t, t)
        x += alpha * p + omega * s
        r = s - omega * t
        rho_prev = rho
        niter += 1
    if dhistory is not None:
        dhistory['linsolver_residual'] = torch.sqrt(
            torch.mean((A(x) - b)**2)).item()
        dhistory['linsolver_niter'] = niter
    return x


def lsqr(matr, rhs, damp=0.0, atol=1e-6, btol=1e-6, conlim=1e8,
         iter_lim=None, dhistory=None):
    """linsolver.py:57-69: LSQR (Paige and Saunders, ACM TOMS 8, 1982) for
    min |J x - rhs|^2 + damp^2 |x|^2 from zero, with its estimates of |A|,
    cond(A), |r| and |A^T r| and its stopping rules (atol, btol, conlim,
    iter_lim; default iter_lim 2 n).  Vectors stay on the device; the
    scalar recurrences run on the host.  Returns x; dhistory gets
    linsolver_residual (|A^T r| estimate), linsolver_anorm,
    linsolver_acond and linsolver_niter."""
    m, n = matr.shape
    iter_lim = 2 * n if iter_lim is None else iter_lim
    eps = np.finfo(np.float64).eps
    ctol = 1.0 / conlim if conlim > 0 else 0.0
    u = rhs.to(torch.float64).clone()
    bnorm = beta = torch.linalg.norm(u).item()
    x = None
    anorm = acond = ddnorm = res2 = xnorm = xxnorm = z = 0.0
    cs2, sn2 = -1.0, 0.0
    arnorm = 0.0
    itn = 0
    if beta > 0:
        u = (1.0 / beta) * u
        v = matr.rmatvec(u).to(torch.float64)
        alpha = torch.linalg.norm(v).item()
    else:
        v = torch.zeros(n, dtype=torch.float64, device=u.device)
        alpha = 0.0
    x = torch.zeros(n, dtype=torch.float64, device=u.device)
    if alpha > 0:
        v = (1.0 / alpha) * v
    w = v.clone()
    rhobar, phibar = alpha, beta
    arnorm = alpha * beta
    if arnorm == 0:
        iter_lim = 0
    while itn < iter_lim:
        itn += 1
        u = matr.matvec(v).to(torch.float64) - alpha * u
        beta = torch.linalg.norm(u).item()
        if beta > 0:
            u = (1.0 / beta) * u
            anorm = (anorm**2 + alpha**2 + beta**2 + damp**2)**0.5
            v = matr.rmatvec(u).to(torch.float64) - beta * v
            alpha = torch.linalg.norm(v).item()
            if alpha > 0:
                v = (1.0 / alpha) * v
        if damp > 0:
            rhobar1 = (rhobar**2 + damp**2)**0.5
            cs1, sn1 = rhobar / rhobar1, damp / rhobar1
            psi = sn1 * phibar
            phibar = cs1 * phibar
        else:
            rhobar1, psi = rhobar, 0.0
        rho = (rhobar1**2 + beta**2)**0.5
        cs, sn = rhobar1 / rho, beta / rho
        theta = sn * alpha
        rhobar = -cs * alpha
        phi = cs * phibar
        phibar = sn * phibar
        tau = sn * phi
        t1, t2 = phi / rho, -theta / rho
        dk = (1.0 / rho) * w
        x += t1 * w
        w = v + t2 * w
        ddnorm += torch.dot(dk, dk).item()
        delta = sn2 * rho
        gambar = -cs2 * rho
        rhs_ = phi - delta * z
        zbar = rhs_ / gambar
        xnorm = (xxnorm + zbar**2)**0.5
        gamma = (gambar**2 + theta**2)**0.5
        cs2, sn2 = gambar / gamma, theta / gamma
        z = rhs_ / gamma
        xxnorm += z**2
        acond = anorm * ddnorm**0.5
        res2 += psi**2
        rnorm = (phibar**2 + res2)**0.5
        arnorm = alpha * abs(tau)
        test1 = rnorm / bnorm
        test2 = arnorm / (anorm * rnorm + eps)
        test3 = 1.0 / (acond + eps)
        t1 = test1 / (1 + anorm * xnorm / bnorm)
        rtol = btol + atol * anorm * xnorm / bnorm
        if (itn >= iter_lim or 1 + test3 <= 1 or 1 + test2 <= 1 or
                1 + t1 <= 1 or test3 <= ctol or test2 <= atol or
                test1 <= rtol):
            break
    if dhistory is not None:
        dhistory['linsolver_residual'] = arnorm
        dhistory['linsolver_anorm'] = anorm
        dhistory['linsolver_acond'] = acond
        dhistory['linsolver_niter'] = itn
    return x


def _grid(matr):
    """(grid shape, fields) of a Jacobian's unknowns."""
    if hasattr(matr, "grid") and hasattr(matr, "nfields"):
        return tuple(matr.grid), int(matr.nfields)
    if hasattr(matr, "kernels"):
        return tuple(matr.kernels.shape), 1
    raise ValueError("linsolver=multigrid needs the grid of the unknowns")


def multigrid_cg(matr, rhs, args=None, dhistory=None):
    """linsolver.py:77-89 with a geometric preconditioner: CG on the relaxed
    normal equations (assembled as a sparse matrix on the device),
    preconditioned by one V-cycle of the CSR multigrid (damped Jacobi with
    `omega`, `smooth_pre` / `smooth_post` sweeps, `nlvl` levels, direct
    solve below `ndirect` nodes).  The V-cycle is not exactly symmetric
    (injection at boundary coarse nodes), so the flexible (Polak-Ribiere)
    form of CG is used.  Stops at |r| < linsolver_tol |b| or after
    linsolver_maxiter iterations, as pyamg's solve(tol, accel='cg')."""
    from .multigrid import Multigrid
    shape, nvar = _grid(matr)
    tol = float(getattr(args, "linsolver_tol", 1e-6) or 1e-6)
    maxiter = getattr(args, "linsolver_maxiter", None) or 50
    beta = float(getattr(args, "beta", 0) or 0)
    betadiag = float(getattr(args, "betadiag", 0) or 0)
    J = matr.to_csr().to(torch.float64)
    A = (J.t().to_sparse_csr() @ J).to_sparse_coo().coalesce()
    idx, val = A.indices(), A.values()
    on = idx[0] == idx[1]
    d = torch.zeros(A.shape[0], dtype=val.dtype, device=val.device)
    d.index_add_(0, idx[0][on], val[on])
    # J^T J + beta^2 I, then + betadiag^2 times its diagonal
    add = beta**2 + betadiag**2 * (d + beta**2)
    ii = torch.arange(A.shape[0], device=val.device)
    A = torch.sparse_coo_tensor(torch.cat([idx, torch.stack([ii, ii])], 1),
                                torch.cat([val, add]),
                                A.shape).coalesce().to_sparse_csr()
    b = J.t().to_sparse_csr() @ rhs.to(torch.float64)
    mg = Multigrid(shape, nvar=nvar, nlevels=getattr(args, "nlvl", None),
                   restriction=getattr(args, "restriction", "full"),
                   dtype=torch.float64, device=b.device)
    mg.update_A(A)
    omega = getattr(args, "omega", 0.6)

    def smoother(level, u, f):
        return mg.smoother_jacobi(level, u, f, omega=omega)

    def M(r):
        return mg.step(torch.zeros_like(r), r, smoother,
                       ndirect=getattr(args, "ndirect", 3),
                       pre=getattr(args, "smooth_pre", 2),
                       post=getattr(args, "smooth_post", 2))

    x = torch.zeros_like(b)
    r = b.clone()
    bnorm = torch.linalg.norm(b).item()
    residuals = [bnorm]
    z = M(r)
    p = z.clone()
    rz = torch.dot(r, z)
    for _ in range(maxiter):
        if residuals[-1] < tol * bnorm:
            break
        Ap = A @ p
        alpha = rz / torch.dot(p, Ap)
        x += alpha * p
        r_new = r - alpha * Ap
        residuals.append(torch.linalg.norm(r_new).item())
        z_new = M(r_new)
        rz_new = torch.dot(r_new, z_new)
        p = z_new + (torch.dot(r_new, z_new - z) / rz) * p
        r, z, rz = r_new, z_new, rz_new
    if dhistory is not None:
        dhistory['linsolver_residual'] = residuals[-1]
        dhistory['linsolver_niter'] = len(residuals)
    return x


def solve(matr, rhs, args=None, dhistory=None, linsolver="direct"):
    beta = float(getattr(args, "beta", 0) or 0)
    betadiag = float(getattr(args, "betadiag", 0) or 0)
    name = ALIASES.get(linsolver, linsolver)
    tol = float(getattr(args, "linsolver_tol", 1e-6) or 1e-6)
    maxiter = getattr(args, "linsolver_maxiter", None)
    if name == "bicgstab":
        return bicgstab(matr, rhs, tol, maxiter or 50, beta, betadiag,
                        dhistory).to(rhs.dtype)
    if name == "lsqr":
        return lsqr(matr, rhs, beta, tol, tol, iter_lim=maxiter or 1000,
                    dhistory=dhistory).to(rhs.dtype)
    if name == "multigrid" and not hasattr(matr, "solve_mg"):
        if not hasattr(matr, "to_csr"):
            raise ValueError("linsolver=multigrid needs a family with a "
                             "multigrid preconditioner or an assembled "
                             "Jacobian (to_csr)")
        return multigrid_cg(matr, rhs, args, dhistory).to(rhs.dtype)
    if beta or betadiag:
        out = solve_regularized(matr, rhs, beta, betadiag)
        return out.to(rhs.dtype)
    if name == "direct":
        return matr.solve(rhs)
    if name == "mixed":
        return matr.solve(rhs.float()).double()
    if name == "multigrid":
        return matr.solve_mg(rhs, args)
    raise ValueError("Unknown linsolver=" + linsolver)


def add_arguments(parser):
    """linsolver.py:110-167 (same names and defaults)."""
    parser.add_argument('--linsolver', type=str,
                        choices=["multigrid", "direct", "mixed", "direct_cu",
                                 "sparseqr", "lsqr", "lsqr_cu", "bicgstab"],
                        default="direct", help="Linear solver to use")
    parser.add_argument('--linsolver_maxiter', type=int, default=None,
                        help="Maximum number of iterations of linear solver")
    parser.add_argument('--linsolver_tol', type=float, default=1e-6,
                        help="Tolerance for linear solver")
    parser.add_argument('--beta', type=float, default=0,
                        help="Relaxation factor (0: no relaxation)")
    parser.add_argument('--betadiag', type=float, default=0,
                        help="Multiplier for diagonal (0: no relaxation)")
    parser.add_argument('--linsolver_verbose', type=int, default=0,
                        help="Verbosity level for linsolver messages")
    parser.add_argument('--lr', type=float, default=1e-3, help="Learning rate")
    parser.add_argument('--nlvl', type=int, default=5, help="Multigrid levels")
    parser.add_argument('--smooth_pre', type=int, default=2,
                        help="Pre-smoothing steps")
    parser.add_argument('--smooth_post', type=int, default=2,
                        help="Post-smoothing steps")
    parser.add_argument('--omega', type=float, default=0.6,
                        help="Jacobi smoother relaxation factor")
    parser.add_argument('--ndirect', type=int, default=3,
                        help="Systems on smaller grids are solved with "
                        "direct solver")
    parser.add_argument('--restriction', type=str,
                        choices=('full', 'half', 'injection'), default='full',
                        help="Multigrid restriction type")
    parser.add_argument('--precision', type=str, choices=('fp64', 'mixed'),
                        default='fp64',
                        help="Newton: FP64 solve, or FP32 solve with FP64 "
                        "residual and update")
