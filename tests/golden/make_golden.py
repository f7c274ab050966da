#!/usr/bin/env python3
"""Regenerates the golden fixtures in this folder from the reference checkout.

Run from the repository root, on a machine that has a checkout of the
reference (odil22/odil); give its root with --ref or in the environment
variable ODIL_REFERENCE.  The GPU machines do not have it: they only read the
committed JSON/NPZ files.

    python tests/golden/make_golden.py --ref <reference checkout>

Fixtures
  advection_ref.npz     residuals (fp, fu, fv) of the reference's own
                        `operator` of advection_2d.py:103-223 (its function
                        body, taken from the source with `ast` and run with
                        NumPy stand-ins for TensorFlow's `mod` and the
                        Context of util_op.py:457-563) on small (t, x, y)
                        grids with seeded fields, velocities of both signs
                        and exact zeros (see make_advection).
  wave_fd_newton.json   N and ref_du_l2 after 2 Newton epochs, read from the
                        reference's cases/wave_cost/precomputed/fd_newton/
                        lines.pickle (fields N, error).
  wave_fd_lbfgsb.json   same for the L-BFGS-B runs (fd_lbfgsb/lines.pickle).
  multigrid_ref.npz     outputs of the reference's multigrid.py (NumPy
                        backend) on small odd grids: restriction and
                        interpolation operators, stencil products, Galerkin
                        coarsening, transposed products (see make_multigrid).
  multigrid_csr_ref.npz outputs of the reference's CSR Multigrid class on SPD
                        matrices: coarse matrices, block diagonals, V-cycle
                        iterates, one Gauss-Seidel sweep (make_multigrid_csr).
  mgdecomp_ref.npz      outputs of the reference's MultigridDecomp (node and
                        cell interpolation, weights to fields) with every
                        interpolation method, run on NumPy statements of
                        the TensorFlow primitives it calls (make_mgdecomp).
  cavity_N128.npz       u, v, p fields of the reference's FP64 Newton cavity
                        solutions cases/cavity_stream/cavity_N128_Re{100,400}.
"""
import argparse
import json
import os
import pickle
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_lines(ref, name):
    path = os.path.join(ref, "code/cases/wave_cost/precomputed", name,
                        "lines.pickle")
    with open(path, "rb") as f:
        d = pickle.load(f)
    return {
        "source": "code/cases/wave_cost/precomputed/%s/lines.pickle" % name,
        "N": [int(n) for n in d.N],
        "error": [float(e) for e in d.error],
        "time_epoch": [float(t) for t in d.time_epoch],
        "epochs": [float(e) for e in d.epochs],
    }


def make_multigrid(ref):
    """Evaluates the reference's multigrid.py on deterministic inputs."""
    sys.path.insert(0, os.path.join(ref, "code"))
    import types
    sys.modules.setdefault("multigrid_plot", types.ModuleType("multigrid_plot"))
    import scipy.sparse as sp
    import multigrid as mg

    mod = mg.ModNumpy(np, sp)
    out = {}
    dtype = np.float64

    def field(nw, seed):
        n = int(np.prod(nw))
        return np.sin(seed * 0.123 + np.linspace(0, 3, n)).reshape(nw)

    for nw in [(9,), (17,), (9, 9), (5, 9), (17, 17), (5, 5, 9)]:
        key = "x".join(map(str, nw))
        nw_a = np.array(nw)
        R = mg.MultigridOp.get_R(nw_a, mod=mod, dtype=dtype)
        TT = mg.MultigridOp.get_TT(nw_a, mod=mod, dtype=dtype)
        u = field(nw, 1)
        uh = field(R.nwh, 2)
        out["R_%s" % key] = R.mul_field(u)
        out["T_%s" % key] = TT.mul_transpose_field(uh)
        out["Rcsr_%s" % key] = R.tocsr().toarray() if np.prod(nw) <= 81 \
            else np.zeros(1)
        # A generic stencil operator with random coefficient fields.
        dim = len(nw)
        shifts = [tuple(s) for s in np.array(np.meshgrid(
            *[[-1, 0, 1]] * dim, indexing="ij")).reshape(dim, -1).T]
        stf = {}
        for i, s in enumerate(shifts):
            stf[s] = field(nw, 10 + i)
        A = mg.SparseOperator(stf, nw_a, mod=mod, dtype=dtype)
        out["A_shifts_%s" % key] = np.array(shifts)
        out["A_coefs_%s" % key] = np.stack([stf[s] for s in shifts])
        out["Au_%s" % key] = A.mul_field(u)
        out["ATu_%s" % key] = A.mul_transpose_field(u)
        AtA = A.mul_transpose_op(A)
        out["AtA_shifts_%s" % key] = np.array(
            [list(k) for k in AtA.shift_to_field.keys()])
        out["AtA_coefs_%s" % key] = np.stack(
            [np.asarray(c).reshape(nw) for c in AtA.shift_to_field.values()])
        # Galerkin coarsening as the reference defines it for CSR matrices
        # (Multigrid.update_A, multigrid.py:125-131: A_{l+1} = R A_l T with
        # R, T from Multigrid.get_R / get_T).  The reference's stencil path
        # (coarsen_sparse_operator) agrees with it only for the zero-padded
        # constant Laplacian of its test_coarsen, stored separately below.
        Rc = mg.Multigrid.get_R(nw_a, mod=mod, dtype=dtype)
        Tc = mg.Multigrid.get_T(nw_a, mod=mod, dtype=dtype)
        out["AhCSR_%s" % key] = (Rc @ A.tocsr() @ Tc).toarray()
    # test_multigrid.py:197-249: the 11x11 padded Laplacian through the
    # stencil coarsening.
    nw = np.array((11, 11))
    pad = [[1, 1]] * 2
    Aop = mg.SparseOperator(
        {
            (0, 0): 4 * np.ones(nw),
            (-1, 0): -np.pad(np.ones(nw - 2), pad),
            (1, 0): -np.pad(np.ones(nw - 2), pad),
            (0, -1): -np.pad(np.ones(nw - 2), pad),
            (0, 1): -np.pad(np.ones(nw - 2), pad),
        }, nw, mod=mod, dtype=dtype)
    Rop = mg.MultigridOp.get_R(nw, mod=mod, dtype=dtype)
    TTop = mg.MultigridOp.get_TT(nw, mod=mod, dtype=dtype)
    Ahop = mg.MultigridOp.coarsen_sparse_operator(Aop, Rop, TTop, mod=mod,
                                                  dtype=dtype)
    out["lap11_Ah"] = Ahop.tocsr().toarray()
    return out


def make_multigrid_csr(ref):
    """Evaluates the reference's CSR Multigrid (multigrid.py:70-339) with its
    default transfer operators (g_reuse_multigridop = True) on SPD matrices
    M^T M of random stencils: the coarse matrices of every level, the
    block diagonals, and the iterates of a few V-cycles."""
    sys.path.insert(0, os.path.join(ref, "code"))
    import types
    from functools import partial
    sys.modules.setdefault("multigrid_plot", types.ModuleType("multigrid_plot"))
    import scipy.sparse as sp
    import multigrid as mg

    mod = mg.ModNumpy(np, sp)
    out = {}
    rng = np.random.default_rng(7)

    def stencil_csr(nw):
        dim = len(nw)
        shifts = [tuple(s) for s in np.array(np.meshgrid(
            *[[-1, 0, 1]] * dim, indexing="ij")).reshape(dim, -1).T]
        stf = {s: rng.uniform(-0.3, 0.3, nw) for s in shifts}
        stf[(0, ) * dim] = stf[(0, ) * dim] + 2.0
        return mg.SparseOperator(stf, np.array(nw), mod=mod,
                                 dtype=np.float64).tocsr()

    cases = [
        # name, nw, nvar, restriction, ndirect, pre, post, cycles
        ("p17", (17, 17), 1, "full", 5, 2, 2, 3),
        ("h17", (17, 17), 1, "half", 5, 2, 2, 3),
        ("i33", (33, ), 1, "injection", 5, 2, 2, 3),
        ("v9", (9, 9), 2, "full", 3, 2, 2, 2),
        ("d3", (5, 5, 9), 1, "full", 2, 1, 3, 2),
    ]
    for name, nw, nvar, restr, ndirect, pre, post, cycles in cases:
        n = int(np.prod(nw))
        B = sp.bmat([[stencil_csr(nw) for _ in range(nvar)]
                     for _ in range(nvar)]).tocsr()
        A = (B.T @ B).tocsr()
        f = rng.standard_normal(n * nvar)
        m = mg.Multigrid(np.array(nw), nvar=nvar, restriction=restr, mod=mod,
                         dtype=np.float64)
        m.update_A(A)
        out["%s_nnw" % name] = np.array([list(v) for v in m.nnw])
        out["%s_A0" % name] = A.toarray()
        out["%s_f" % name] = f
        for level in range(1, m.nlevels):
            out["%s_A%d" % (name, level)] = m.AA[level].toarray()
        for level in range(m.nlevels):
            out["%s_D%d" % (name, level)] = np.array(
                [[np.asarray(d) for d in row] for row in m.DD[level]])
        u = np.zeros_like(f)
        for it in range(cycles):
            u = m.step(u.copy(), f, ndirect=ndirect, pre=pre, post=post,
                       smoother=partial(m.smoother_jacobi, omega=0.7))
            out["%s_u%d" % (name, it)] = u.copy()
        if nvar == 1:
            # update_A(compute_lower=True) raises NameError in the reference
            # (multigrid.py:149 names an undefined `mod`); its intended
            # lower-triangular parts are set directly.
            m.LL = [sp.tril(a).tocsr() for a in m.AA]
            v = m.smoother_gauss_seidel(0, f * 0.1, f, omega=0.9)
            out["%s_gs" % name] = v.copy()
    # The variant the reference's unit tests use (test_multigrid.py:4):
    # transfer operators from node multi-indices, first axis fastest.
    mg.g_reuse_multigridop = False
    out["fortran_R_9x5"] = mg.Multigrid.get_R(np.array((9, 5)), mod=mod,
                                              dtype=np.float64).toarray()
    out["fortran_T_9x5"] = mg.Multigrid.get_T(np.array((9, 5)), mod=mod,
                                              dtype=np.float64).toarray()
    mg.g_reuse_multigridop = True
    return out


class _TfPrimitives:
    """NumPy statements of the TensorFlow primitives MultigridDecomp calls
    (the reference's NumPy `mod` lacks them), from their documented
    semantics: batch_to_space (the batch index is the C-order index of the
    block offset, then crops), nn.conv_transpose with VALID padding and
    stride s (out[s i + t] += w[t] x[i], no kernel flip), pad with REFLECT /
    SYMMETRIC modes, concat."""

    def __init__(self, base):
        self._base = base
        self.nn = self

    def __getattr__(self, k):
        return getattr(self._base, k)

    @staticmethod
    def batch_to_space(uu, block_shape, crops):
        uu = np.asarray(uu)
        dim = len(block_shape)
        shape = uu.shape[1:1 + dim]
        out = np.zeros(tuple(n * b for n, b in zip(shape, block_shape)))
        for k, off in enumerate(np.ndindex(*block_shape)):
            sel = tuple(slice(o, None, b) for o, b in zip(off, block_shape))
            out[sel] = uu[k]
        sel = tuple(slice(c0, out.shape[d] - c1)
                    for d, (c0, c1) in enumerate(crops))
        return out[sel][None]

    @staticmethod
    def conv_transpose(u, filters, output_shape, strides, padding):
        assert padding == "VALID"
        x = np.asarray(u)[0, ..., 0]
        w = np.asarray(filters)[..., 0, 0]
        out = np.zeros(tuple(output_shape[1:-1]))
        for t in np.ndindex(*w.shape):
            sel = tuple(slice(td, td + strides * (n - 1) + 1, strides)
                        for td, n in zip(t, x.shape))
            out[sel] += w[t] * x
        return out[None, ..., None]

    @staticmethod
    def pad(u, paddings, mode="CONSTANT", constant_values=0):
        if mode == "CONSTANT":
            return np.pad(u, paddings, constant_values=constant_values)
        return np.pad(u, paddings, mode={"REFLECT": "reflect",
                                         "SYMMETRIC": "symmetric"}[mode])

    @staticmethod
    def concat(xs, axis):
        return np.concatenate(xs, axis)


def make_mgdecomp(ref):
    """Evaluates the reference's MultigridDecomp (multigrid.py:1217-1426)
    with every interpolation method it defines, on the NumPy statements of
    the TensorFlow primitives above; the methods must agree."""
    sys.path.insert(0, os.path.join(ref, "code"))
    import types
    sys.modules.setdefault("multigrid_plot", types.ModuleType("multigrid_plot"))
    import scipy.sparse as sp
    import multigrid as mg
    D = mg.MultigridDecomp
    mod = _TfPrimitives(mg.ModNumpy(np, sp))
    rng = np.random.default_rng(17)
    out = {}
    for cell, shapes in ((False, [(5, ), (9, ), (5, 9), (3, 5, 5)]),
                         (True, [(4, ), (6, ), (3, 5), (2, 3, 4)])):
        kind = "cell" if cell else "node"
        for shape in shapes:
            u = rng.standard_normal(shape)
            key = "%s_%s" % (kind, "x".join(map(str, shape)))
            out[key + "_u"] = u
            for depth in (1, 2):
                methods = ["conv", "roll"]
                if len(shape) <= (2 if cell else 3):
                    methods.append("manual")
                res = [D.interp_field(u, depth=depth, mod=mod, method=m,
                                      cell=cell) for m in methods]
                for m, r in zip(methods[1:], res[1:]):
                    assert np.allclose(r, res[0], rtol=0, atol=1e-13), (key, m)
                out["%s_d%d" % (key, depth)] = res[0]
    # Weights on levels (finest first) to one field and to per-level fields.
    for cell, nnw in ((False, [(9, 17), (5, 9), (3, 5)]),
                      (True, [(8, 12), (4, 6), (2, 3)])):
        kind = "cell" if cell else "node"
        n = sum(int(np.prod(nw)) for nw in nnw)
        uw = rng.standard_normal(n)
        factors = [1.0, 0.5, 2.0]
        out["w2f_%s_uw" % kind] = uw
        out["w2f_%s_nnw" % kind] = np.array(nnw)
        out["w2f_%s_field" % kind] = D.weights_to_field(
            uw, nnw, mod, factors=factors, cell=cell)
        for i, f in enumerate(D.weights_to_fields(uw, nnw, mod, factors=factors,
                                                  cell=cell)):
            out["w2f_%s_fields%d" % (kind, i)] = f
        out["w2f_%s_ones" % kind] = D.get_weights_coarse_ones(
            nnw, np.float64, mod)
    return out


def make_cavity(ref):
    res = {}
    for re_ in (100, 400):
        path = os.path.join(ref, "code/cases/cavity_stream",
                            "cavity_N128_Re%d.pickle" % re_)
        with open(path, "rb") as f:
            s = pickle.load(f)
        for k in ("u", "v", "p"):
            res["Re%d_%s" % (re_, k)] = np.asarray(s["fields"][k], np.float64)
    return res


class _NpContext:
    """The parts of util_op.py's Context (lines 457-563) that the advection
    operator uses, on NumPy arrays: ``field(name, *shift)`` is the state
    field rolled by -shift on every axis (periodic, util_op.py:548-551;
    freeze changes nothing in a forward evaluation), ``zeros``/``ones`` are
    the custom fields of util_op.py:229-234, ``cell_index`` the index grid
    of util_op.py:185-187, ``step`` the cell size of util_op.py:127-128."""

    def __init__(self, fields, shape, upper, varnames=("t", "x", "y")):
        self.fields = fields
        self.shape = shape
        self.upper = upper
        self.varnames = varnames
        self.epoch = 0

    def _dim(self, i):
        return self.varnames.index(i) if isinstance(i, str) else i

    def step(self, i):
        i = self._dim(i)
        return self.upper[i] / self.shape[i]

    def size(self, i):
        return self.shape[self._dim(i)]

    def cell_index(self, i):
        return np.meshgrid(*[np.arange(n) for n in self.shape],
                           indexing="ij")[self._dim(i)]

    def field(self, name, *shift, freeze=False):
        if name == "zeros":
            return np.zeros(self.shape)
        if name == "ones":
            return np.ones(self.shape)
        shift = tuple(shift) + (0,) * (len(self.shape) - len(shift))
        return np.roll(self.fields[name], np.negative(shift),
                       tuple(range(len(self.shape))))


def _reference_function(path, name):
    """Compiles the top-level function `name` of the reference source file
    `path` on its own (the module's imports need TensorFlow)."""
    import ast
    tree = ast.parse(open(path).read(), filename=path)
    for node in tree.body:
        if isinstance(node, ast.FunctionDef) and node.name == name:
            return compile(ast.Module(body=[node], type_ignores=[]), path,
                           "exec")
    raise KeyError(name)


def make_advection(ref):
    """Residuals of advection_2d.py's `operator` (direct problem, the
    driver's defaults --periodic 1 --central 0 --implicit 0) on small grids.
    Velocity fields: per-cell random values of both signs with some exact
    zeros (the where(u > 0, ...) branch), and constant velocities of each
    sign pair (the benchmark's form)."""
    from types import SimpleNamespace
    code = os.path.join(ref, "code")
    op_code = _reference_function(os.path.join(code, "advection_2d.py"),
                                  "operator")
    ex_code = _reference_function(os.path.join(code, "util_op.py"),
                                  "extrap_linear")
    rng = np.random.default_rng(20)
    res = {}
    cases = [("mixed_a", (3, 4, 5), None), ("mixed_b", (4, 3, 6), None),
             ("mixed_c", (2, 5, 4), None)]
    for sx in (1, -1):
        for sy in (1, -1):
            cases.append(("const_%s%s" % ("p" if sx > 0 else "m",
                                          "p" if sy > 0 else "m"),
                          (3, 4, 5), (0.7 * sx, 0.4 * sy)))
    for name, shape, vel in cases:
        tmax = 0.8
        if vel is None:
            u = rng.standard_normal(shape)
            v = rng.standard_normal(shape)
            u[rng.random(shape) < 0.15] = 0.0
            v[rng.random(shape) < 0.15] = 0.0
        else:
            u = np.full(shape, vel[0])
            v = np.full(shape, vel[1])
        p = rng.standard_normal(shape)
        exact_uu = rng.standard_normal(shape)
        exact_vv = rng.standard_normal(shape)
        exact_pp = rng.standard_normal(shape)
        ns = {"np": np}
        exec(ex_code, ns)
        ns.update(args=SimpleNamespace(periodic=1, central=0, implicit=0,
                                       problem="direct"),
                  exact_uu=exact_uu, exact_vv=exact_vv, exact_pp=exact_pp)
        exec(op_code, ns)
        mod = SimpleNamespace(where=np.where, roll=np.roll)
        ctx = _NpContext({"u": u, "v": v, "p": p}, shape, (tmax, 1.0, 1.0))
        fp, fu, fv = ns["operator"](mod, ctx)
        for key, val in (("u", u), ("v", v), ("p", p), ("exact_uu", exact_uu),
                         ("exact_vv", exact_vv), ("exact_pp", exact_pp),
                         ("fp", fp), ("fu", fu), ("fv", fv)):
            res["%s_%s" % (name, key)] = np.asarray(val, np.float64)
        res[name + "_tmax"] = np.float64(tmax)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("ODIL_REFERENCE"),
                    help="root of the reference checkout (default: "
                    "$ODIL_REFERENCE)")
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    if not a.ref:
        ap.error("give the reference checkout with --ref or ODIL_REFERENCE")
    todo = a.only.split(",") if a.only else ["wave", "multigrid", "multigrid_csr",
                                                  "mgdecomp", "cavity",
                                                  "advection"]
    if "wave" in todo:
        for name in ("fd_newton", "fd_lbfgsb"):
            with open(os.path.join(HERE, "wave_%s.json" % name), "w") as f:
                json.dump(load_lines(a.ref, name), f, indent=1)
    if "multigrid" in todo:
        np.savez_compressed(os.path.join(HERE, "multigrid_ref.npz"),
                            **make_multigrid(a.ref))
    if "multigrid_csr" in todo:
        np.savez_compressed(os.path.join(HERE, "multigrid_csr_ref.npz"),
                            **make_multigrid_csr(a.ref))
    if "mgdecomp" in todo:
        np.savez_compressed(os.path.join(HERE, "mgdecomp_ref.npz"),
                            **make_mgdecomp(a.ref))
    if "cavity" in todo:
        np.savez_compressed(os.path.join(HERE, "cavity_N128.npz"),
                            **make_cavity(a.ref))
    if "advection" in todo:
        np.savez_compressed(os.path.join(HERE, "advection_ref.npz"),
                            **make_advection(a.ref))


if __name__ == "__main__":
    main()
