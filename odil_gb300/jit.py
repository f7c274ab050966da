"""Stencil compiler for generic ODIL operators.

A user operator ``operator(mod, ctx)`` (util_op.py:569-577) that is not a
registered family is traced once with symbolic ``mod`` and ``ctx`` objects:
every ``ctx.field(name, *shift)`` becomes a leaf read at a fixed offset, cell
indices and coordinates become index leaves, and numpy arrays that broadcast
against the grid (boundary data, masks) become array leaves.  The residual
terms are then expression graphs over these leaves (hash-consed, so common
subexpressions are shared).  From them this module writes one CUDA source
with

  * a residual kernel: f_k at every cell, one thread per cell;
  * loss + gradient in two passes: loss = sum_k mean(f_k^2) and
    grad_u[c] = sum_k (2/N_k) sum_s f_k(c - s) * df_k/du[. + s](c - s) (what
    util_op.py:627-654 gets from the TF tape).  Pass 1 evaluates every term
    and its symbolic derivatives once per cell and stores the products
    (2/N_k) f_k df_k/du(. + s), one grid per read, plus the per-block loss
    partials; pass 2 gathers them at the shifted cells.  Storing the products
    costs a few bytes per read and cell; re-evaluating each term at every
    read offset instead costs FP64 arithmetic, the scarce resource on GB300;

compiles it with nvcc for sm_103a into an in-tree shared library (cached by a
hash of the source) and launches it through ctypes.  Shifts wrap
periodically, as ``ctx.field`` does with ``roll`` (util_op.py:508-563).

Operators that use anything the tracer does not model (neural networks,
``Problem.Raw`` terms, reductions, reshapes) raise ``JitUnsupported`` while
tracing; ``Problem`` then runs them op by op on CUDA tensors instead.
"""
import ctypes
import hashlib
import math
import os
import platform
import subprocess
import threading

import numpy as np
import torch

from . import _build
from ._capi import ODIL_OK


class JitUnsupported(Exception):
    """The operator uses a construct the stencil compiler does not trace."""


# ---------------------------------------------------------------------------
# Expression graph

_FLOAT, _INT, _BOOL = "f", "i", "b"


class Node:
    """A hash-consed expression node.  ``op`` names the operation, ``args``
    its operands (nodes or Python constants), ``kind`` its value type."""

    __array_ufunc__ = None  # numpy defers to the reflected operators
    __slots__ = ("g", "op", "args", "kind", "id")

    def __init__(self, g, op, args, kind, nid):
        self.g, self.op, self.args, self.kind, self.id = g, op, args, kind, nid

    __hash__ = object.__hash__

    def _bin(self, op, other, rev=False):
        o = self.g.lift(other)
        return self.g.binop(op, o, self) if rev else self.g.binop(op, self, o)

    def __add__(self, o):
        return self._bin("add", o)

    def __radd__(self, o):
        return self._bin("add", o, True)

    def __sub__(self, o):
        return self._bin("sub", o)

    def __rsub__(self, o):
        return self._bin("sub", o, True)

    def __mul__(self, o):
        return self._bin("mul", o)

    def __rmul__(self, o):
        return self._bin("mul", o, True)

    def __truediv__(self, o):
        return self._bin("div", o)

    def __rtruediv__(self, o):
        return self._bin("div", o, True)

    def __neg__(self):
        return self.g.binop("sub", self.g.const(0), self)

    def __pos__(self):
        return self

    def __pow__(self, p):
        if isinstance(p, Node) or not np.isscalar(p):
            raise JitUnsupported("only constant exponents are traced")
        return self.g.pow(self, float(p))

    def __abs__(self):
        return self.g.fn("abs", self)

    def __eq__(self, o):
        return self._bin("eq", o)

    def __ne__(self, o):
        return self._bin("ne", o)

    def __lt__(self, o):
        return self._bin("lt", o)

    def __le__(self, o):
        return self._bin("le", o)

    def __gt__(self, o):
        return self._bin("gt", o)

    def __ge__(self, o):
        return self._bin("ge", o)

    def __and__(self, o):
        return self._bin("and", o)

    def __rand__(self, o):
        return self._bin("and", o, True)

    def __or__(self, o):
        return self._bin("or", o)

    def __ror__(self, o):
        return self._bin("or", o, True)

    def __invert__(self):
        return self.g.unop("not", self)

    def __bool__(self):
        raise JitUnsupported("a traced value was used as a Python bool")

    def __getitem__(self, idx):
        raise JitUnsupported("indexing of traced fields is not traced")

    def __getattr__(self, name):
        if name in ("shape", "dtype"):
            raise JitUnsupported("traced values have no concrete " + name)
        raise AttributeError(name)


_CMP = ("eq", "ne", "lt", "le", "gt", "ge")
_LOGIC = ("and", "or")


class Graph:
    """Node factory with constant folding and hash-consing."""

    def __init__(self, shape):
        self.shape = tuple(int(s) for s in shape)
        self.table = {}
        self.nodes = []
        self.ext = []  # broadcast-shaped float64 arrays

    def _mk(self, op, args, kind):
        key = (op, ) + tuple(a.id if isinstance(a, Node) else
                             ("c", type(a).__name__, a) for a in args)
        n = self.table.get(key)
        if n is None:
            n = Node(self, op, tuple(args), kind, len(self.nodes))
            self.table[key] = n
            self.nodes.append(n)
        return n

    # leaves
    def const(self, v):
        if isinstance(v, (bool, np.bool_)):
            return self._mk("const", (bool(v), ), _BOOL)
        if isinstance(v, (int, np.integer)):
            return self._mk("const", (int(v), ), _INT)
        return self._mk("const", (float(v), ), _FLOAT)

    def field(self, name, shift, frozen=False):
        return self._mk("ffield" if frozen else "field",
                        (name, tuple(int(s) for s in shift)), _FLOAT)

    def index(self, axis):
        return self._mk("idx", (int(axis), ), _INT)

    def param(self, name):
        """A scalar set per launch (the epoch)."""
        return self._mk("param", (name, ), _INT)

    def shifted(self, node, off, memo=None):
        """`node` evaluated at cell c - off (numpy.roll by `off`, periodic):
        field reads move their offset, index and array leaves read the
        wrapped cell."""
        off = tuple(int(o) for o in off)
        if not any(off):
            return node
        memo = {} if memo is None else memo
        if node.id in memo:
            return memo[node.id]
        op, a = node.op, node.args
        if op in ("const", "param"):
            r = node
        elif op in ("field", "ffield"):
            r = self._mk(op, (a[0], tuple(s - o for s, o in zip(a[1], off))),
                         node.kind)
        elif op == "idx":
            o = off[a[0]]
            r = node if o == 0 else self._mk("idxs", (a[0], o), _INT)
        elif op == "idxs":
            o = a[1] + off[a[0]]
            r = self._mk("idx", (a[0], ), _INT) if o == 0 else \
                self._mk("idxs", (a[0], o), _INT)
        elif op in ("ext", "exts"):
            arr = self.ext[a[0]][0]
            base = a[1] if op == "exts" else (0, ) * len(off)
            o = tuple(b + (d if arr.shape[ax] != 1 else 0)
                      for ax, (b, d) in enumerate(zip(base, off)))
            r = self._mk("ext", (a[0], ), node.kind) if not any(o) else \
                self._mk("exts", (a[0], o), node.kind)
        else:
            args = tuple(self.shifted(x, off, memo) if isinstance(x, Node)
                         else x for x in a)
            r = self._mk(op, args, node.kind)
        memo[node.id] = r
        return r

    def array(self, a):
        a = np.asarray(a)
        if a.size == 1:
            return self.const(a.reshape(()).item())
        # Axes a broadcast view repeats (stride 0) are kept at length 1.
        if a.ndim and 0 in a.strides:
            a = a[tuple(slice(0, 1) if st == 0 else slice(None)
                        for st in a.strides)]
        nd = len(self.shape)
        if a.ndim > nd:
            raise JitUnsupported("array of rank %d on a rank-%d grid" %
                                 (a.ndim, nd))
        b = a.reshape((1, ) * (nd - a.ndim) + a.shape)
        for s, n in zip(b.shape, self.shape):
            if s not in (1, n):
                raise JitUnsupported("array of shape %s does not broadcast "
                                     "to the grid %s" % (a.shape, self.shape))
        kind = _BOOL if a.dtype == bool else _FLOAT
        data = np.ascontiguousarray(b, dtype=np.float64)
        for i, (arr, k) in enumerate(self.ext):
            if k == kind and arr.shape == data.shape and np.array_equal(
                    arr, data):
                return self._mk("ext", (i, ), kind)
        self.ext.append((data, kind))
        return self._mk("ext", (len(self.ext) - 1, ), kind)

    def lift(self, v):
        if isinstance(v, Node):
            return v
        if isinstance(v, torch.Tensor):
            v = v.detach().cpu().numpy()
        if isinstance(v, np.ndarray):
            return self.array(v)
        if np.isscalar(v):
            return self.const(v.item() if hasattr(v, "item") else v)
        raise JitUnsupported("cannot trace a value of type %s" % type(v))

    # operations
    def binop(self, op, a, b):
        a, b = self.lift(a), self.lift(b)
        if op in _CMP:
            if a.op == "const" and b.op == "const":
                x, y = a.args[0], b.args[0]
                return self.const({"eq": x == y, "ne": x != y, "lt": x < y,
                                   "le": x <= y, "gt": x > y,
                                   "ge": x >= y}[op])
            return self._mk(op, (a, b), _BOOL)
        if op in _LOGIC:
            if a.kind != _BOOL or b.kind != _BOOL:
                raise JitUnsupported("logic on non-boolean values")
            return self._mk(op, (a, b), _BOOL)
        kind = _INT if (a.kind == _INT and b.kind == _INT and
                        op != "div") else _FLOAT
        ca = a.args[0] if a.op == "const" else None
        cb = b.args[0] if b.op == "const" else None
        if ca is not None and cb is not None:
            v = {"add": ca + cb, "sub": ca - cb, "mul": ca * cb,
                 "div": (ca / cb) if cb != 0 else None}[op]
            if v is not None:
                return self.const(float(v) if kind == _FLOAT else v)
        if op == "add":
            if ca == 0:
                return b if b.kind == kind else self._mk(op, (a, b), kind)
            if cb == 0:
                return a if a.kind == kind else self._mk(op, (a, b), kind)
        elif op == "sub":
            if cb == 0:
                return a if a.kind == kind else self._mk(op, (a, b), kind)
        elif op == "mul":
            if ca == 0 or cb == 0:
                return self.const(0.0 if kind == _FLOAT else 0)
            if ca == 1 and b.kind == kind:
                return b
            if cb == 1 and a.kind == kind:
                return a
        elif op == "div":
            if ca == 0:
                return self.const(0.0)
            if cb == 1 and a.kind == _FLOAT:
                return a
        return self._mk(op, (a, b), kind)

    def unop(self, op, a):
        a = self.lift(a)
        if op == "not":
            if a.kind != _BOOL:
                raise JitUnsupported("logical not of a non-boolean")
            return self._mk("not", (a, ), _BOOL)
        raise JitUnsupported(op)

    def pow(self, a, p):
        a = self.lift(a)
        if p == 1.0:
            return a
        if p == 0.0:
            return self.const(1.0)
        if p == 2.0:
            return self.binop("mul", a, a)
        if a.op == "const":
            return self.const(float(a.args[0])**p)
        return self._mk("pow", (a, p), _FLOAT)

    def fn(self, name, a):
        a = self.lift(a)
        if a.op == "const" and a.kind != _BOOL:
            v = float(a.args[0])
            f = {"sqrt": math.sqrt, "exp": math.exp, "log": math.log,
                 "sin": math.sin, "cos": math.cos, "tanh": math.tanh,
                 "abs": abs}[name]
            return self.const(f(v))
        return self._mk("fn", (name, a), _FLOAT)

    def maxmin(self, op, a, b):
        return self._mk(op, (self.lift(a), self.lift(b)), _FLOAT)

    def where(self, c, a, b):
        c, a, b = self.lift(c), self.lift(a), self.lift(b)
        if c.kind != _BOOL:
            c = self.binop("ne", c, self.const(0))
        if c.op == "const":
            return a if c.args[0] else b
        if a is b:
            return a
        kind = _FLOAT if _FLOAT in (a.kind, b.kind) else a.kind
        return self._mk("where", (c, a, b), kind)

    # differentiation
    def diff(self, node, wrt, memo):
        """d node / d (field, shift) as a node."""
        key = node.id
        if key in memo:
            return memo[key]
        op, args = node.op, node.args
        zero = self.const(0.0)
        if op == "field":
            r = self.const(1.0) if (args[0], args[1]) == wrt else zero
        elif op in ("const", "ffield", "idx", "idxs", "ext", "exts") or \
                node.kind != _FLOAT:
            r = zero
        elif op in ("add", "sub"):
            da = self.diff(args[0], wrt, memo)
            db = self.diff(args[1], wrt, memo)
            r = self.binop(op, da, db)
        elif op == "mul":
            a, b = args
            r = self.binop("add", self.binop("mul", self.diff(a, wrt, memo), b),
                           self.binop("mul", a, self.diff(b, wrt, memo)))
        elif op == "div":
            a, b = args
            da, db = self.diff(a, wrt, memo), self.diff(b, wrt, memo)
            r = self.binop("sub", self.binop("div", da, b),
                           self.binop("div", self.binop("mul", node, db), b))
        elif op == "pow":
            a, p = args
            r = self.binop("mul", self.binop("mul", self.const(p),
                                             self.pow(a, p - 1.0)),
                           self.diff(a, wrt, memo))
        elif op == "fn":
            name, a = args
            da = self.diff(a, wrt, memo)
            if name == "sqrt":
                r = self.binop("div", da, self.binop("mul", self.const(2.0),
                                                     node))
            elif name == "exp":
                r = self.binop("mul", node, da)
            elif name == "log":
                r = self.binop("div", da, a)
            elif name == "sin":
                r = self.binop("mul", self.fn("cos", a), da)
            elif name == "cos":
                r = self.binop("sub", zero, self.binop("mul", self.fn("sin", a),
                                                       da))
            elif name == "tanh":
                r = self.binop("mul", self.binop("sub", self.const(1.0),
                                                 self.binop("mul", node, node)),
                               da)
            elif name == "abs":
                r = self.where(self.binop("ge", a, self.const(0.0)), da,
                               self.binop("sub", zero, da))
            else:
                raise JitUnsupported(name)
        elif op in ("max", "min"):
            a, b = args
            c = self.binop("ge" if op == "max" else "le", a, b)
            r = self.where(c, self.diff(a, wrt, memo), self.diff(b, wrt, memo))
        elif op == "where":
            c, a, b = args
            r = self.where(c, self.diff(a, wrt, memo), self.diff(b, wrt, memo))
        else:
            raise JitUnsupported("no derivative for " + op)
        memo[key] = r
        return r


def reads(node):
    """(field, shift) pairs a term reads, differentiable ones only."""
    out, seen, stack = set(), set(), [node]
    while stack:
        n = stack.pop()
        if n.id in seen:
            continue
        seen.add(n.id)
        if n.op == "field":
            out.add((n.args[0], n.args[1]))
        for a in n.args:
            if isinstance(a, Node):
                stack.append(a)
    return sorted(out)


# ---------------------------------------------------------------------------
# Tracing objects


class SymMod:
    """The ``mod`` namespace during tracing (tf-style names)."""

    float32 = np.float32
    float64 = np.float64
    pi = np.pi

    def __init__(self, g):
        self.g = g

    def _np(self, *xs):
        return all(not isinstance(x, Node) for x in xs)

    def constant(self, x, dtype=None):
        return x

    def cast(self, x, dtype=None):
        if isinstance(x, Node):
            if x.kind == _BOOL:
                return self.g.where(x, 1.0, 0.0)
            return self.g.binop("mul", x, self.g.const(1.0))
        return x

    def where(self, c, a, b):
        if self._np(c, a, b):
            return np.where(c, a, b)
        return self.g.where(c, a, b)

    def roll(self, x, shift, axis):
        if not isinstance(x, Node):
            return np.roll(np.asarray(x), shift, axis)
        shifts = np.atleast_1d(shift)
        axes = np.atleast_1d(list(axis) if isinstance(axis, range) else axis)
        off = [0] * len(self.g.shape)
        for s_, ax in zip(np.broadcast_to(shifts, axes.shape), axes):
            off[int(ax)] += int(s_)
        return self.g.shifted(x, off)

    def zeros(self, shape, dtype=None):
        return np.zeros(shape)

    def ones(self, shape, dtype=None):
        return np.ones(shape)

    def zeros_like(self, x):
        return self.g.const(0.0) if isinstance(x, Node) else np.zeros_like(x)

    def ones_like(self, x):
        return self.g.const(1.0) if isinstance(x, Node) else np.ones_like(x)

    def square(self, x):
        return x * x

    def _f(self, name, npf, x):
        if self._np(x):
            return npf(x)
        return self.g.fn(name, x)

    def sqrt(self, x):
        return self._f("sqrt", np.sqrt, x)

    def exp(self, x):
        return self._f("exp", np.exp, x)

    def log(self, x):
        return self._f("log", np.log, x)

    def sin(self, x):
        return self._f("sin", np.sin, x)

    def cos(self, x):
        return self._f("cos", np.cos, x)

    def tanh(self, x):
        return self._f("tanh", np.tanh, x)

    def abs(self, x):
        return self._f("abs", np.abs, x)

    def maximum(self, a, b):
        if self._np(a, b):
            return np.maximum(a, b)
        return self.g.maxmin("max", a, b)

    def minimum(self, a, b):
        if self._np(a, b):
            return np.minimum(a, b)
        return self.g.maxmin("min", a, b)

    def stop_gradient(self, x):
        if isinstance(x, Node):
            raise JitUnsupported("stop_gradient of a traced expression")
        return x

    def __getattr__(self, name):
        raise JitUnsupported("mod.%s is not traced" % name)


class SymContext:
    """The ``ctx`` of util_op.py:432-563 during tracing."""

    def __init__(self, domain, g, extra=None):
        self.domain = domain
        self.g = g
        self.extra = extra

    @property
    def epoch(self):
        """A kernel argument: the compiled operator follows the epoch it is
        evaluated at (Python branches on it are not traced)."""
        return self.g.param("epoch")

    def cast(self, value, dtype=None):
        return value

    def size(self, i):
        return self.domain.size(i)

    def step(self, i):
        return self.domain.step(i)

    def cell_index(self, i):
        return self.g.index(self.domain._axis(i))

    def node_index(self, i):
        raise JitUnsupported("node_index is not traced")

    def cell_center(self, i):
        return self.g.array(np.asarray(self.domain.cell_center(i)))

    def neural_net(self, name, *inputs, **kw):
        raise JitUnsupported("neural networks are not traced")

    def field(self, name, *shift, freeze=False):
        d = self.domain
        assert len(shift) <= d.ndim, "Shift is too long {:}".format(shift)
        shift = tuple(shift) + (0, ) * (d.ndim - len(shift))
        if name == "zeros":
            return self.g.const(0.0)
        if name == "ones":
            return self.g.const(1.0)
        if name not in d.fieldnames:
            raise ValueError("Unknown field name '" + name + "'")
        # ctx.field(k, *s)[i] == u[i + s] with a periodic wrap.
        return self.g.field(name, shift, frozen=freeze)


def trace(operator, domain, extra=None):
    """Traces ``operator`` on ``domain``; returns (graph, term nodes).
    ``extra`` and the numpy arrays the operator reads are captured as they
    are now; the epoch stays a kernel argument."""
    from .problem import Problem
    g = Graph(domain.shape)
    terms = operator(SymMod(g), SymContext(domain, g, extra))
    if not isinstance(terms, (list, tuple)):
        terms = [terms]
    out = []
    for t in terms:
        if isinstance(t, Problem.Raw):
            raise JitUnsupported("Problem.Raw terms are not traced")
        n = g.lift(t)
        if n.kind == _BOOL:
            raise JitUnsupported("boolean residual")
        out.append(n)
    return g, out


# ---------------------------------------------------------------------------
# Code generation


def _lit(v, kind):
    if kind == _BOOL:
        return "true" if v else "false"
    if kind == _INT:
        return "%d" % v
    if math.isnan(v) or math.isinf(v):
        raise JitUnsupported("non-finite constant")
    return "T(%r)" % float(v)


_FN = {"sqrt": "sqrt", "exp": "exp", "log": "log", "sin": "sin",
       "cos": "cos", "tanh": "tanh", "abs": "fabs"}
_BINC = {"add": "+", "sub": "-", "mul": "*", "div": "/", "eq": "==",
         "ne": "!=", "lt": "<", "le": "<=", "gt": ">", "ge": ">=",
         "and": "&&", "or": "||"}


class _Emitter:
    """Writes the nodes a set of roots needs, in dependency order, as local
    variables of a device function."""

    def __init__(self, fields, ndim):
        self.fields = fields
        self.ndim = ndim
        self.lines = []
        self.names = {}

    def _ctype(self, kind):
        return {"f": "T", "i": "int", "b": "bool"}[kind]

    def emit(self, root):
        order, seen, stack = [], set(), [(root, False)]
        while stack:
            n, done = stack.pop()
            if n.id in self.names or (n.id in seen and not done):
                continue
            if done:
                order.append(n)
                seen.add(n.id)
                continue
            stack.append((n, True))
            for a in n.args:
                if isinstance(a, Node) and a.id not in self.names:
                    stack.append((a, False))
        for n in order:
            if n.id in self.names:
                continue
            self.names[n.id] = self._expr(n)
        return self.names[root.id]

    def _expr(self, n):
        op, a = n.op, n.args
        if op == "const":
            return _lit(a[0], n.kind)
        name = "v%d" % n.id
        if op in ("field", "ffield"):
            fi = self.fields.index(a[0])
            idx = ", ".join("wrap(i%d + (%d), a.n[%d])" % (d, a[1][d], d)
                            for d in range(self.ndim))
            rhs = "a.f[%d][lin(a, %s)]" % (fi, idx)
        elif op == "idx":
            rhs = "i%d" % a[0]
        elif op == "param":
            rhs = "a.%s" % a[0]
        elif op == "idxs":
            rhs = "wrap(i%d - (%d), a.n[%d])" % (a[0], a[1], a[0])
        elif op == "exts":
            idx = " + ".join(
                "(long long)wrap(i%d - (%d), a.n[%d]) * a.es[%d][%d]"
                % (d, a[1][d], d, a[0], d) for d in range(self.ndim))
            rhs = "a.e[%d][%s]" % (a[0], idx)
            if n.kind == _BOOL:
                rhs = "(%s != T(0))" % rhs
        elif op == "ext":
            idx = " + ".join("(long long)i%d * a.es[%d][%d]" % (d, a[0], d)
                             for d in range(self.ndim))
            rhs = "a.e[%d][%s]" % (a[0], idx)
            if n.kind == _BOOL:
                rhs = "(%s != T(0))" % rhs
        elif op in _BINC:
            x, y = self.names[a[0].id], self.names[a[1].id]
            if n.kind == _FLOAT and op in ("add", "sub", "mul", "div"):
                x, y = "T(%s)" % x, "T(%s)" % y
            rhs = "(%s %s %s)" % (x, _BINC[op], y)
        elif op == "not":
            rhs = "(!%s)" % self.names[a[0].id]
        elif op == "pow":
            x, p = self.names[a[0].id], a[1]
            if p == int(p) and abs(p) <= 4:
                k = int(abs(p))
                prod = " * ".join(["T(%s)" % x] * k) if k else "T(1)"
                rhs = "(%s)" % prod if p > 0 else "(T(1) / (%s))" % prod
            else:
                rhs = "pow(T(%s), T(%r))" % (x, p)
        elif op == "fn":
            rhs = "%s(T(%s))" % (_FN[a[0]], self.names[a[1].id])
        elif op in ("max", "min"):
            rhs = "%s(T(%s), T(%s))" % ("fmax" if op == "max" else "fmin",
                                        self.names[a[0].id],
                                        self.names[a[1].id])
        elif op == "where":
            c, x, y = (self.names[v.id] for v in a)
            cast = "T" if n.kind == _FLOAT else ""
            rhs = "(%s ? %s(%s) : %s(%s))" % (c, cast, x, cast, y)
        else:
            raise JitUnsupported(op)
        self.lines.append("    const %s %s = %s;" % (self._ctype(n.kind), name,
                                                     rhs))
        return name


_PRELUDE = r"""
#include <cstdint>
#include <cuda_runtime.h>
typedef @T@ T;
#define NF @NF@
#define NE @NE@
#define NK @NK@
#define NC @NC@
struct Args {
    const T* f[NF > 0 ? NF : 1];
    const T* e[NE > 0 ? NE : 1];
    T* out[NK];
    T* grad[NF > 0 ? NF : 1];
    T* contrib[NC > 0 ? NC : 1];
    double* partial;
    int n[3];
    int epoch;
    long long es[NE > 0 ? NE : 1][3];
    double scale[NK];
};
__device__ __forceinline__ int wrap(int i, int n) {
    if (i >= 0 && i < n) return i;
    const int r = i % n;
    return r < 0 ? r + n : r;
}
__device__ __forceinline__ long long lin(const Args& a, int i0, int i1 = 0, int i2 = 0) {
    return ((long long)i0 * a.n[1] + i1) * a.n[2] + i2;
}
"""


def _cell_decode(ndim):
    s = ["    const long long c = (long long)blockIdx.x * blockDim.x + "
         "threadIdx.x;",
         "    const long long ncell = (long long)a.n[0] * a.n[1] * a.n[2];",
         "    const bool live = c < ncell;",
         "    const long long cc = live ? c : 0;",
         "    const int i2 = (int)(cc % a.n[2]);",
         "    const int i1 = (int)((cc / a.n[2]) % a.n[1]);",
         "    const int i0 = (int)(cc / ((long long)a.n[1] * a.n[2]));"]
    return "\n".join(s)


def generate(g, terms, fields, dtype):
    """CUDA source of the residual and loss + gradient kernels, and for each
    term the (field, shift) reads its gradient gathers."""
    ndim = len(g.shape)
    T = "double" if dtype == torch.float64 else "float"
    nk = len(terms)
    if nk < 1:
        raise JitUnsupported("the operator returns no residual")
    src = [_PRELUDE.replace("@T@", T).replace("@NF@", str(len(fields)))
           .replace("@NE@", str(len(g.ext))).replace("@NK@", str(nk))]
    params = ", ".join("int i%d" % d for d in range(ndim))
    term_reads = []
    for k, t in enumerate(terms):
        rd = reads(t)
        term_reads.append(rd)
        # value only
        em = _Emitter(fields, ndim)
        v = em.emit(t)
        src.append("__device__ __forceinline__ T term%d(const Args& a, %s) {"
                   % (k, params))
        src += em.lines
        src.append("    return T(%s);\n}" % v)
        # value and derivatives along every read
        em = _Emitter(fields, ndim)
        v = em.emit(t)
        ds = []
        for wrt in rd:
            ds.append(em.emit(g.diff(t, wrt, {})))
        src.append("__device__ __forceinline__ T term%d_d(const Args& a, %s, "
                   "T* d) {" % (k, params))
        src += em.lines
        for m, dn in enumerate(ds):
            src.append("    d[%d] = T(%s);" % (m, dn))
        src.append("    return T(%s);\n}" % v)
    idx = ", ".join("i%d" % d for d in range(ndim))
    # residual kernel
    src.append("__global__ void __launch_bounds__(256) residual_kernel(Args a) {")
    src.append(_cell_decode(ndim))
    src.append("    if (!live) return;")
    for k in range(nk):
        src.append("    a.out[%d][c] = term%d(a, %s);" % (k, k, idx))
    src.append("}")
    # loss + gradient in two passes.  Pass 1 (contrib_kernel): every term
    # and its derivatives once per cell; contribution q of read (field j,
    # offset s) is C_q[c] = (2/N) f_k(c) df_k/du_j(c + s)(c), and the loss
    # partials.  Pass 2 (gather_kernel): grad_j[c] = sum_q C_q[c - s_q].
    reads_flat = []  # (term, m, field index, shift)
    for k, rd in enumerate(term_reads):
        for m, (name, sh) in enumerate(rd):
            reads_flat.append((k, m, fields.index(name), sh))
    src.append("__global__ void __launch_bounds__(256) contrib_kernel(Args a) {")
    src.append(_cell_decode(ndim))
    src.append("    double lk[NK];")
    q = 0
    for k, rd in enumerate(term_reads):
        src.append("    {")
        src.append("        T d[%d];" % max(1, len(rd)))
        src.append("        const T f = term%d_d(a, %s, d);" % (k, idx))
        src.append("        lk[%d] = live ? (double)f * (double)f : 0.0;" % k)
        src.append("        const T sf = T(a.scale[%d]) * f;" % k)
        src.append("        if (live) {")
        for m in range(len(rd)):
            src.append("            a.contrib[%d][c] = sf * d[%d];" % (q, m))
            q += 1
        src.append("        }")
        src.append("    }")
    src[0] = src[0].replace("@NC@", str(len(reads_flat)))
    src.append(r"""    __shared__ double red[NK][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k = 0; k < NK; ++k) {
        double v = lk[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[k][w] = v;
    }
    __syncthreads();
    if (threadIdx.x < NK) {
        double s = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[threadIdx.x][q];
        a.partial[(long long)blockIdx.x * NK + threadIdx.x] = s;
    }
}
""")
    src.append("__global__ void __launch_bounds__(256) gather_kernel(Args a) {")
    src.append(_cell_decode(ndim))
    src.append("    if (!live) return;")
    for fi in range(len(fields)):
        terms_j = [(qq, sh) for qq, (_, _, fj, sh) in enumerate(reads_flat)
                   if fj == fi]
        src.append("    {")
        src.append("        T gsum = T(0);")
        for qq, sh in terms_j:
            cell = ", ".join("wrap(i%d - (%d), a.n[%d])" % (d, sh[d], d)
                             for d in range(ndim))
            src.append("        gsum += a.contrib[%d][lin(a, %s)];" % (qq, cell))
        src.append("        a.grad[%d][c] = gsum;" % fi)
        src.append("    }")
    src.append("}")
    # Jacobian coefficient fields: coef_q[c] = df_k(c)/du_j(c + s_q), the
    # per-shift form of util_op.py:585-614.
    src.append("__global__ void __launch_bounds__(256) jacobian_kernel(Args a) {")
    src.append(_cell_decode(ndim))
    src.append("    if (!live) return;")
    q = 0
    for k, rd in enumerate(term_reads):
        src.append("    {")
        src.append("        T d[%d];" % max(1, len(rd)))
        src.append("        (void)term%d_d(a, %s, d);" % (k, idx))
        for m in range(len(rd)):
            src.append("        a.contrib[%d][c] = d[%d];" % (q, m))
            q += 1
        src.append("    }")
    src.append("}")
    src.append(r"""static int launch_status() { return cudaGetLastError() == cudaSuccess ? 0 : -4; }
extern "C" __attribute__((visibility("default"))) int odil_jit_jacobian(const Args* a, long long ncell, void* stream) {
    jacobian_kernel<<<(unsigned)((ncell + 255) / 256), 256, 0, (cudaStream_t)stream>>>(*a);
    return launch_status();
}
extern "C" __attribute__((visibility("default"))) int odil_jit_residual(const Args* a, long long ncell, void* stream) {
    residual_kernel<<<(unsigned)((ncell + 255) / 256), 256, 0, (cudaStream_t)stream>>>(*a);
    return launch_status();
}
extern "C" __attribute__((visibility("default"))) int odil_jit_loss_grad(const Args* a, long long ncell, void* stream) {
    const unsigned nb = (unsigned)((ncell + 255) / 256);
    contrib_kernel<<<nb, 256, 0, (cudaStream_t)stream>>>(*a);
    gather_kernel<<<nb, 256, 0, (cudaStream_t)stream>>>(*a);
    return launch_status();
}
""")
    return "\n".join(src), term_reads


# ---------------------------------------------------------------------------
# Build and run

_LOCK = threading.Lock()


def _jit_dir():
    d = os.environ.get("ODIL_GB300_JIT_DIR",
                       os.path.join(_build.LIBDIR, "jit"))
    os.makedirs(d, exist_ok=True)
    return d


def compile_source(code):
    """Compiles `code` to a shared library (cached by content); returns its
    path."""
    h = hashlib.sha1((code + repr(_build.ARCH) + platform.machine())
                     .encode()).hexdigest()[:20]
    d = _jit_dir()
    so = os.path.join(d, "odil_jit_%s.so" % h)
    with _LOCK:
        if os.path.exists(so):
            return so
        cu = os.path.join(d, "odil_jit_%s.cu" % h)
        with open(cu, "w") as f:
            f.write(code)
        tmp = so + ".%d.tmp" % os.getpid()
        cmd = [_build.nvcc_path(), *_build.ARCH, "-O3", "-lineinfo",
               "-std=c++17", "-shared", "-Xcompiler", "-fPIC", cu, "-o", tmp]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on the generated operator:\n" +
                               r.stderr[-4000:])
        os.replace(tmp, so)
    return so


class JitOperator:
    """A traced operator compiled to CUDA (see the module docstring)."""

    def __init__(self, operator, domain, extra=None):
        self.domain = domain
        self.dtype = (torch.float32 if np.dtype(domain.dtype) == np.float32
                      else torch.float64)
        self.fields = list(domain.fieldnames)
        self.graph, self.terms = trace(operator, domain, extra)
        if len(self.graph.shape) > 3:
            raise JitUnsupported("grids of rank > 3")
        self.code, self.term_reads = generate(self.graph, self.terms,
                                              self.fields, self.dtype)
        self._lib = None
        self._ext = None
        nf, ne, nk = len(self.fields), len(self.graph.ext), len(self.terms)
        self.ncontrib = sum(len(rd) for rd in self.term_reads)
        nc = self.ncontrib

        class Args(ctypes.Structure):
            _fields_ = [("f", ctypes.c_void_p * max(1, nf)),
                        ("e", ctypes.c_void_p * max(1, ne)),
                        ("out", ctypes.c_void_p * nk),
                        ("grad", ctypes.c_void_p * max(1, nf)),
                        ("contrib", ctypes.c_void_p * max(1, nc)),
                        ("partial", ctypes.c_void_p),
                        ("n", ctypes.c_int * 3),
                        ("epoch", ctypes.c_int),
                        ("es", (ctypes.c_longlong * 3) * max(1, ne)),
                        ("scale", ctypes.c_double * nk)]

        self._Args = Args

    def lib(self):
        if self._lib is None:
            lib = ctypes.CDLL(compile_source(self.code))
            for name in ("odil_jit_residual", "odil_jit_loss_grad",
                         "odil_jit_jacobian"):
                fn = getattr(lib, name)
                fn.restype = ctypes.c_int
                fn.argtypes = [ctypes.c_void_p, ctypes.c_longlong,
                               ctypes.c_void_p]
            self._lib = lib
        return self._lib

    def _args(self, fields, device, epoch=0):
        g = self.graph
        if self._ext is None or self._ext[0] != device:
            ext = [torch.tensor(a, dtype=self.dtype, device=device)
                   for a, _ in g.ext]
            self._ext = (device, ext)
        a = self._Args()
        for i, name in enumerate(self.fields):
            t = fields[name]
            if not t.is_cuda or t.dtype != self.dtype or not t.is_contiguous():
                raise ValueError("field '%s' must be a contiguous CUDA %s "
                                 "tensor" % (name, self.dtype))
            a.f[i] = t.data_ptr()
        shp = list(g.shape) + [1] * (3 - len(g.shape))
        for d in range(3):
            a.n[d] = shp[d]
        for i, t in enumerate(self._ext[1]):
            a.e[i] = t.data_ptr()
            st = [0, 0, 0]
            stride = 1
            for d in reversed(range(len(g.shape))):
                if t.shape[d] != 1:
                    st[d] = stride
                stride *= t.shape[d]
            for d in range(3):
                a.es[i][d] = st[d]
        n = int(np.prod(g.shape))
        for k in range(len(self.terms)):
            a.scale[k] = 2.0 / n
        a.epoch = int(epoch)
        return a, n

    def residual(self, fields, epoch=0):
        """The residual fields f_k (list of tensors)."""
        from ._capi import stream_handle
        u0 = fields[self.fields[0]]
        a, n = self._args(fields, u0.device, epoch)
        outs = [torch.empty(self.graph.shape, dtype=self.dtype,
                            device=u0.device) for _ in self.terms]
        for k, o in enumerate(outs):
            a.out[k] = o.data_ptr()
        st = self.lib().odil_jit_residual(ctypes.byref(a), n, stream_handle())
        if st != ODIL_OK:
            raise RuntimeError("odil_jit_residual failed (%d)" % st)
        return outs

    def jacobian(self, fields, epoch=0):
        """Coefficient fields of the Jacobian: a tensor [reads, *grid] and,
        per (term, field), the read indices and shifts (row q holds
        df_k(c)/du_j(c + s_q))."""
        from ._capi import stream_handle
        u0 = fields[self.fields[0]]
        a, n = self._args(fields, u0.device, epoch)
        dummy = torch.empty(1, dtype=self.dtype, device=u0.device)
        for k in range(len(self.terms)):
            a.out[k] = dummy.data_ptr()
        coef = torch.empty((max(1, self.ncontrib), ) + self.graph.shape,
                           dtype=self.dtype, device=u0.device)
        for q in range(self.ncontrib):
            a.contrib[q] = coef[q].data_ptr()
        st = self.lib().odil_jit_jacobian(ctypes.byref(a), n, stream_handle())
        if st != ODIL_OK:
            raise RuntimeError("odil_jit_jacobian failed (%d)" % st)
        blocks = {}
        q = 0
        for k, rd in enumerate(self.term_reads):
            for name, sh in rd:
                blocks.setdefault((k, self.fields.index(name)), []).append(
                    (q, sh))
                q += 1
        return coef, blocks

    def loss_grad(self, fields, epoch=0):
        """(loss, {field: grad}, [mean(f_k^2)]) with the FP64 loss summed in
        a fixed order."""
        from ._capi import stream_handle
        u0 = fields[self.fields[0]]
        dev = u0.device
        a, n = self._args(fields, dev, epoch)
        nk = len(self.terms)
        nb = (n + 255) // 256
        partial = torch.empty((nb, nk), dtype=torch.float64, device=dev)
        grads = {name: torch.empty(self.graph.shape, dtype=self.dtype,
                                   device=dev) for name in self.fields}
        dummy = torch.empty(1, dtype=self.dtype, device=dev)
        for k in range(nk):
            a.out[k] = dummy.data_ptr()
        for i, name in enumerate(self.fields):
            a.grad[i] = grads[name].data_ptr()
        # Pass-1 contributions, one grid per (term, read): scratch.
        contrib = torch.empty((max(1, self.ncontrib), ) + self.graph.shape,
                              dtype=self.dtype, device=dev)
        for q in range(self.ncontrib):
            a.contrib[q] = contrib[q].data_ptr()
        a.partial = partial.data_ptr()
        st = self.lib().odil_jit_loss_grad(ctypes.byref(a), n, stream_handle())
        if st != ODIL_OK:
            raise RuntimeError("odil_jit_loss_grad failed (%d)" % st)
        split = partial.sum(0) / n
        return split.sum(), grads, list(split)
