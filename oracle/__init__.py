"""CPU oracle for the ODIL hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, in plain NumPy/SciPy (FP64), the reference algorithm of
odil22/odil for the residual -> loss/gradient -> Newton/L-BFGS/Adam/multigrid
path.  Every function cites the reference file:line it follows (paths relative
to the reference's ``code/`` directory).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline and
``--impl reference`` legs may import it, and only as the checker or as the
timed CPU baseline.  The product package ``odil_gb300`` never imports it: the
GPU path has no CPU fallback.

Parity pins (see tests/test_oracle_pins.py):
  * wave FD + Newton: error against the exact solution reproduces the
    reference's shipped ``cases/wave_cost/precomputed/fd_newton/lines.pickle``
    for every grid it lists (fixture ``tests/golden/wave_fd_newton.json``);
  * multigrid restriction / interpolation / Galerkin / SparseOperator pieces
    reproduce the reference's own ``multigrid.py`` outputs (fixtures generated
    by ``tests/golden/make_golden.py``);
  * NS cavity operator: the reference's shipped FP64 Newton solutions
    ``cases/cavity_stream/cavity_N128_Re*.pickle`` are roots of the restated
    operator.
"""
