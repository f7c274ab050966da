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
                      geometric multigrid V-cycle (families that provide it).
Other reference choices (direct_cu, sparseqr, lsqr, lsqr_cu, bicgstab) map
to "direct".  With --beta or --betadiag set, every choice solves the relaxed
normal equations of linsolver.py:35-41 (solve_regularized).
"""
import torch

ALIASES = {"direct_cu": "direct", "sparseqr": "direct", "lsqr": "direct",
           "lsqr_cu": "direct", "bicgstab": "direct"}


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

    b = matr.rmatvec(rhs)
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


def solve(matr, rhs, args=None, dhistory=None, linsolver="direct"):
    beta = float(getattr(args, "beta", 0) or 0)
    betadiag = float(getattr(args, "betadiag", 0) or 0)
    if beta or betadiag:
        out = solve_regularized(matr, rhs, beta, betadiag)
        return out.to(rhs.dtype)
    name = ALIASES.get(linsolver, linsolver)
    if name == "direct":
        return matr.solve(rhs)
    if name == "mixed":
        return matr.solve(rhs.float()).double()
    if name == "multigrid":
        if not hasattr(matr, "solve_mg"):
            raise ValueError("linsolver=multigrid needs a family with a "
                             "multigrid preconditioner")
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
