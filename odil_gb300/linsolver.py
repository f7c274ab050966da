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
to "direct".
"""
import torch

ALIASES = {"direct_cu": "direct", "sparseqr": "direct", "lsqr": "direct",
           "lsqr_cu": "direct", "bicgstab": "direct"}


def solve(matr, rhs, args=None, dhistory=None, linsolver="direct"):
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
