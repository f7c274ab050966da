"""Uniform space-time grid and solver state (the API of util_op.py:15-337).

Geometry is host-side NumPy (setup only); fields live on the GPU as torch
tensors.  Cell centres follow util_op.py:130-137: x_i = lower + (i + 1/2) h
with h = (upper - lower) / n, fields are C-order arrays of ``shape``.
"""
import numpy as np


class Domain:
    """Cell-centred grid; same constructor arguments as util_op.py:17-35.

    ``device`` (default "cuda") is where fields are created.  Unknowns held
    as a multigrid decomposition (``multigrid=True``) and neural-network
    weights raise NotImplementedError.
    """

    def __init__(self,
                 ndim=None,
                 lower=0.,
                 upper=1.,
                 shape=None,
                 varnames=('x', 'y', 'z'),
                 fieldnames=(),
                 neuralnets=None,
                 frozen_weights=(),
                 frozen_fields=(),
                 dtype=np.float64,
                 multigrid=False,
                 device="cuda",
                 **kwargs):
        if ndim is None:
            ndim = len(varnames)
        self.ndim = ndim
        if shape is not None:
            assert len(shape) == ndim, "len(shape) must equal ndim"
            shape = tuple(int(s) for s in shape)
        if multigrid:
            raise NotImplementedError(
                "multigrid decomposition of unknowns (util_op.py:61-95) needs "
                "MultigridDecomp.check_nnw and field_to_weights, which the "
                "reference does not define; the decomposition itself is "
                "odil_gb300.multigrid.MultigridDecomp")
        if neuralnets:
            raise NotImplementedError(
                "neural-network unknowns (util_op.py:354-429) are not on the "
                "GPU hot path")
        self.lower = np.ones(ndim, dtype=np.float64) * lower
        self.upper = np.ones(ndim, dtype=np.float64) * upper
        self.varnames = tuple(varnames[:ndim])
        self.dtype = np.dtype(dtype).type
        self.shape = shape
        self.fieldnames = tuple(fieldnames)
        self.frozen_fields = tuple(frozen_fields)
        self.frozen_weights = tuple(frozen_weights)
        self.neuralnets = {}
        self.aweights = []
        self.mg_fieldnames = []
        self.multigrid = False
        self.device = device

    # -- sizes -------------------------------------------------------------
    def fields_size(self):
        return len(self.fieldnames) * int(np.prod(self.shape))

    def aweights_size(self):
        return 0

    def weights_size(self):
        return 0

    def cells(self):
        return int(np.prod(self.shape))

    # -- geometry (util_op.py:127-227) ---------------------------------------
    def _axis(self, i):
        if isinstance(i, str):
            return self.varnames.index(i)
        return i

    def step_by_dim(self, i):
        return (self.upper[i] - self.lower[i]) / self.shape[i]

    def cell_center_1d(self, i):
        n = self.shape[i]
        x = np.linspace(self.lower[i], self.upper[i], n, endpoint=False,
                        dtype=np.float64)
        h = (x[1] - x[0]) if n > 1 else (self.upper[i] - self.lower[i])
        return x + h * 0.5

    def cell_center_all(self):
        xx = [self.cell_center_1d(i) for i in range(self.ndim)]
        return np.meshgrid(*xx, indexing='ij')

    def cell_center_by_dim(self, i):
        xx = [self.cell_center_1d(i)]
        shp = [1] * self.ndim
        shp[i] = self.shape[i]
        return np.broadcast_to(xx[0].reshape(shp), self.shape)

    def cell_center_by_name(self, name):
        if name in self.varnames:
            return self.cell_center_by_dim(self.varnames.index(name))
        return None

    def cell_node_1d(self, i):
        return np.linspace(self.lower[i], self.upper[i], self.shape[i] + 1,
                           dtype=np.float64)

    def cell_node_all(self):
        xx = [self.cell_node_1d(i) for i in range(self.ndim)]
        return np.meshgrid(*xx, indexing='ij')

    def cell_node_by_dim(self, i):
        return self.cell_node_all()[i]

    def cell_index_all(self):
        return np.meshgrid(*[np.arange(s) for s in self.shape], indexing='ij')

    def cell_index_by_dim(self, i):
        shp = [1] * self.ndim
        shp[i] = self.shape[i]
        return np.broadcast_to(np.arange(self.shape[i]).reshape(shp),
                               self.shape)

    def cell_index_by_name(self, name):
        names = ['i' + n for n in self.varnames]
        if name in names:
            return self.cell_index_by_dim(names.index(name))
        return None

    def node_index_all(self):
        return np.meshgrid(*[np.arange(s + 1) for s in self.shape],
                           indexing='ij')

    def node_index_by_dim(self, i):
        return self.node_index_all()[i]

    def step(self, i):
        return self.step_by_dim(self._axis(i))

    def cell_index(self, i):
        return self.cell_index_by_dim(self._axis(i))

    def node_index(self, i):
        return self.node_index_by_dim(self._axis(i))

    def cell_center(self, i):
        return self.cell_center_by_dim(self._axis(i))

    def size(self, i):
        return self.shape[self._axis(i)]

    def get_minimal(self):
        """util_op.py:112-113: a picklable copy of the geometry
        (util_min.py:5-28): ndim, lower, upper, varnames, fieldnames,
        dtype, shape, and the step and cell-centre helpers."""
        return MinimalDomain(self)

    def cell_node_by_name(self, name):
        """util_op.py:173-180: cell nodes along axis `name`, or None."""
        if name in self.varnames:
            return self.cell_node_by_dim(self.varnames.index(name))
        return None

    def custom_by_name(self, name):
        """util_op.py:229-234: the named constant fields."""
        import torch
        dt = torch.float32 if np.dtype(self.dtype) == np.float32 \
            else torch.float64
        if name == "zeros":
            return torch.zeros(self.shape, dtype=dt, device=self.device)
        if name == "ones":
            return torch.ones(self.shape, dtype=dt, device=self.device)
        return None

    def random_inner(self, size, rng=None):
        """util_op.py:236-241: `size` Latin-hypercube points inside the
        domain, as a list of coordinate arrays (one per axis)."""
        from .problem import latin_hypercube
        res = latin_hypercube(self.ndim, size, rng).T
        for i in range(self.ndim):
            res[i] = self.lower[i] + (self.upper[i] - self.lower[i]) * res[i]
        return [p for p in res]

    def random_boundary(self, normal, side, size, rng=None):
        """util_op.py:243-263: `size` Latin-hypercube points on the face
        normal to axis `normal` at side 0 (lower) or 1 (upper)."""
        from .problem import latin_hypercube
        assert normal < self.ndim
        assert side in (0, 1)
        res = latin_hypercube(self.ndim - 1, size, rng).T
        res = np.vstack((res[:normal], np.full(size, float(side)),
                         res[normal:]))
        for i in range(self.ndim):
            res[i] = self.lower[i] + (self.upper[i] - self.lower[i]) * res[i]
        return [p for p in res]

    def state_to_field(self, key, state, mod=None):
        """util_op.py:309-315 (fields only: multigrid weights are not
        supported)."""
        return state.fields[key]

    def add_field_to_state(self, u, key, state, mod=None):
        """util_op.py:317-330 (fields only): state.fields[key] += u."""
        state.fields[key] += u

    def assign_active_state(self, dst, src):
        """util_op.py:263-268."""
        for name in self.fieldnames:
            dst.fields[name].copy_(src.fields[name])


class MinimalDomain:
    """util_min.py:5-28: the geometry of a Domain without device state."""

    def __init__(self, domain):
        self.ndim = int(domain.ndim)
        self.lower = np.array(domain.lower, np.float64)
        self.upper = np.array(domain.upper, np.float64)
        self.varnames = np.array(domain.varnames)
        self.fieldnames = np.array(domain.fieldnames)
        self.dtype = domain.dtype
        self.shape = tuple(domain.shape)

    def step_by_dim(self, i):
        return (self.upper[i] - self.lower[i]) / self.shape[i]

    def cell_center_1d(self, i):
        s = self.shape[i]
        return np.asarray(self.lower[i] + (np.arange(s) + 0.5) / s *
                          (self.upper[i] - self.lower[i]), dtype=self.dtype)

    def cell_center_all(self):
        return np.meshgrid(*[self.cell_center_1d(i) for i in range(self.ndim)],
                           indexing='ij')


class State:
    """util_op.py:333-337: named fields (and weights, unused here)."""

    def __init__(self, fields=None, weights=None):
        self.fields = dict(fields or {})
        self.weights = dict(weights or {})
