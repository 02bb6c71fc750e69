"""
Equivalent sources on a GB300: the Jacobian and the prediction of point
sources with the Green's function 1 / distance, and estimators around them.

Mirrors harmonica ``src/harmonica/_equivalent_sources``: ``EquivalentSources``
(cartesian.py:33-415: depth "default" = 4.5 x the mean nearest-neighbour
distance, the checks of ``depth``, ``estimate_required_memory``, ``fit``,
``predict``, ``jacobian``) and ``EquivalentSourcesSph`` (spherical.py:33-330:
sources ``relative_depth`` below the data).  The Jacobian
(``hg_eqs_jacobian``, the loop of utils.py:54-74) and the prediction
(``hg_eqs_predict``, utils.py:77-96) run in CUDA kernels.

``fit`` solves the damped least-squares problem on the GPU (torch): the
Jacobian's columns are scaled by their standard deviations, the (weighted)
least-squares or ridge problem with damping ``damping`` is solved, and the
solution is unscaled -- the algorithm of the reference's least-squares step
(verde's ``least_squares``: scikit-learn's standard scaler without centring,
then ordinary least squares or ridge regression without intercept, with the
sample weights; the coefficients divided by the scales).
``block_size`` (block-averaging with verde's ``BlockReduce``), ``grid``,
``scatter`` and ``profile`` (verde gridding) are outside the GPU path and
raise ``NotImplementedError``.
"""

import numpy as np

from . import _native

__all__ = ["EquivalentSources", "EquivalentSourcesSph", "greens_jacobian", "greens_predict"]


def _device(device):
    from .gravity import _device as dev  # noqa: PLC0415

    return dev(device)


def _tensors(arrays, dev):
    import torch  # noqa: PLC0415

    return [torch.from_numpy(np.array(np.ravel(a), dtype=np.float64)).to(dev) for a in arrays]


def _same_sizes(arrays, what):
    """The three coordinates of the data or of the sources have one value per
    point each (the kernels read all three at every index)."""
    sizes = [np.size(a) for a in arrays[:3]]
    if len(sizes) != 3 or len(set(sizes)) != 1:
        raise ValueError(f"The coordinates of the {what} must be three arrays of the same "
                         f"number of elements (got sizes {sizes})")
    return sizes[0]


def greens_jacobian(coordinates, points, spherical=False, device=None, as_tensor=False):
    """(n_data, n_points) matrix of 1 / distance between data points and
    sources (``jacobian`` of the reference) computed on the GPU."""
    import torch  # noqa: PLC0415

    from .gravity import _ptr  # noqa: PLC0415

    _same_sizes(coordinates, "data points")
    _same_sizes(points, "sources")
    dev = _device(device)
    with torch.cuda.device(dev):
        c = _tensors(coordinates[:3], dev)
        p = _tensors(points[:3], dev)
        jac = torch.empty((c[0].numel(), p[0].numel()), dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        _native.check(_native.lib().hg_eqs_jacobian(
            _ptr(c[0]), _ptr(c[1]), _ptr(c[2]), c[0].numel(), _ptr(p[0]), _ptr(p[1]),
            _ptr(p[2]), p[0].numel(), int(bool(spherical)), _ptr(jac), stream))
        return jac if as_tensor else jac.cpu().numpy()


def greens_predict(coordinates, points, coefs, spherical=False, device=None):
    """sum_j coefs[j] / distance(i, j) at every data point (``predict`` of the
    reference) on the GPU; returns an array of the coordinates' shape."""
    import torch  # noqa: PLC0415

    from .gravity import _ptr  # noqa: PLC0415

    n_points = _same_sizes(points, "sources")
    if np.size(coefs) != n_points:
        raise ValueError(f"Number of coefficients ({np.size(coefs)}) mismatch the number of "
                         f"sources ({n_points})")
    dev = _device(device)
    shape = np.broadcast(*coordinates[:3]).shape
    coords = [np.broadcast_to(np.asarray(c, dtype=np.float64), shape) for c in coordinates[:3]]
    lib = _native.lib()
    with torch.cuda.device(dev):
        c = _tensors(coords, dev)
        p = _tensors(points[:3], dev)
        (q,) = _tensors([coefs], dev)
        n_obs, n_pts = c[0].numel(), p[0].numel()
        out = torch.empty(max(n_obs, 1), dtype=torch.float64, device=dev)
        ws = _native.ctypes.c_size_t(0)
        _native.check(lib.hg_point_forward_workspace(n_obs, n_pts, _native.ctypes.byref(ws)))
        work = torch.empty(max(1, (ws.value + 7) // 8), dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        _native.check(lib.hg_eqs_predict(
            _ptr(c[0]), _ptr(c[1]), _ptr(c[2]), n_obs, _ptr(p[0]), _ptr(p[1]), _ptr(p[2]),
            _ptr(q), n_pts, int(bool(spherical)), _ptr(out), _ptr(work) if ws.value else None,
            ws.value, stream))
        return out[:n_obs].cpu().numpy().reshape(shape)


def _least_squares(jac, data, weights, damping):
    """Column-scaled (weighted) least squares or ridge regression on the
    device; jac is a (n_data, n_params) float64 tensor."""
    import torch  # noqa: PLC0415

    scale = jac.std(dim=0, unbiased=False)
    scale = torch.where(scale > 0, scale, torch.ones_like(scale))
    a = jac / scale
    y = data
    if weights is not None:
        sw = torch.sqrt(weights)
        a = a * sw[:, None]
        y = y * sw
    if damping is None:
        params = torch.linalg.lstsq(a, y[:, None]).solution[:, 0]
    else:
        normal = a.T @ a
        normal.diagonal().add_(float(damping))
        params = torch.linalg.solve(normal, a.T @ y)
    return params / scale


def _mean_nearest_neighbour_distance(easting, northing):
    """Mean over the points of the horizontal distance to the nearest other
    point (the reference's 4.5 x ... default depth rule)."""
    from scipy.spatial import cKDTree  # noqa: PLC0415

    xy = np.column_stack([np.ravel(easting), np.ravel(northing)])
    dist, _ = cKDTree(xy).query(xy, k=2)
    return np.mean(dist[:, 1])


class EquivalentSources:
    """Cartesian equivalent sources (cartesian.py:33-415) with the Jacobian,
    the fit and the prediction on the GPU."""

    def __init__(self, damping=None, points=None, depth="default", block_size=None,
                 parallel=True, dtype="float64", device=None):
        if isinstance(depth, str) and depth != "default":
            msg = (
                f"Found invalid 'depth' value equal to '{depth}'. "
                "It should be 'default' or a numeric value."
            )
            raise ValueError(msg)
        if depth == 0:
            msg = "Depth value cannot be zero. It should be a non-zero numeric value."
            raise ValueError(msg)
        self.damping = damping
        self.points = points
        self.depth = depth
        self.block_size = block_size
        self.parallel = parallel
        self.dtype = dtype
        self.device = device

    _spherical = False

    def _build_points(self, coordinates):
        if self.block_size is not None:
            raise NotImplementedError(
                "block_size (block-averaging with verde's BlockReduce) is not supported"
            )
        if self.depth == "default":
            self.depth_ = 4.5 * _mean_nearest_neighbour_distance(coordinates[0], coordinates[1])
        else:
            self.depth_ = self.depth
        return (coordinates[0], coordinates[1], coordinates[2] - self.depth_)

    def _points_for(self, coordinates):
        if self.points is None:
            return tuple(np.asarray(p, dtype=self.dtype) for p in self._build_points(coordinates))
        self.depth_ = None
        return tuple(np.ravel(np.asarray(p, dtype=self.dtype)) for p in self.points[:3])

    def estimate_required_memory(self, coordinates):
        """Bytes of the (n_data, n_points) Jacobian."""
        coordinates = tuple(np.ravel(np.asarray(c)) for c in coordinates[:3])
        points = self._build_points(coordinates) if self.points is None else self.points
        return coordinates[0].size * np.ravel(points[0]).size * np.dtype(self.dtype).itemsize

    def jacobian(self, coordinates, points):
        """(n_data, n_points) matrix of the Green's function (numpy)."""
        return greens_jacobian(coordinates, points, spherical=self._spherical,
                               device=self.device).astype(self.dtype, copy=False)

    def fit(self, coordinates, data, weights=None):
        """Fit the source coefficients to ``data`` at ``coordinates``."""
        import torch  # noqa: PLC0415

        coordinates = tuple(np.ravel(np.asarray(c, dtype=self.dtype)) for c in coordinates[:3])
        data = np.ravel(np.asarray(data, dtype=self.dtype))
        if data.size != coordinates[0].size:
            raise ValueError("Data and coordinates must have the same number of elements.")
        if weights is not None:
            weights = np.ravel(np.asarray(weights, dtype=self.dtype))
        self.region_ = (float(coordinates[0].min()), float(coordinates[0].max()),
                        float(coordinates[1].min()), float(coordinates[1].max()))
        self.points_ = self._points_for(coordinates)
        dev = _device(self.device)
        jac = greens_jacobian(coordinates, self.points_, spherical=self._spherical, device=dev,
                              as_tensor=True)
        with torch.cuda.device(dev):
            d = torch.from_numpy(np.ascontiguousarray(data, dtype=np.float64)).to(dev)
            w = (torch.from_numpy(np.ascontiguousarray(weights, dtype=np.float64)).to(dev)
                 if weights is not None else None)
            self.coefs_ = _least_squares(jac, d, w, self.damping).cpu().numpy().astype(self.dtype)
        return self

    def predict(self, coordinates):
        """The field of the fitted sources at ``coordinates``."""
        if not hasattr(self, "coefs_"):
            msg = (f"This {type(self).__name__} instance is not fitted yet. Call 'fit' with "
                   "appropriate arguments before using this estimator.")
            raise ValueError(msg)
        out = greens_predict(coordinates, self.points_, self.coefs_, spherical=self._spherical,
                             device=self.device)
        return out.astype(self.dtype, copy=False)

    def grid(self, *args, **kwargs):
        raise NotImplementedError("grid (verde gridding) is not supported; use predict")

    def scatter(self, *args, **kwargs):
        raise NotImplementedError

    def profile(self, *args, **kwargs):
        raise NotImplementedError("profile (verde gridding) is not supported; use predict")


class EquivalentSourcesSph(EquivalentSources):
    """Spherical equivalent sources (spherical.py:33-330): longitude, latitude
    (degrees) and radius (m); sources ``relative_depth`` below the data."""

    _spherical = True

    def __init__(self, damping=None, points=None, relative_depth=500, parallel=True,
                 device=None):
        self.damping = damping
        self.points = points
        self.relative_depth = relative_depth
        self.parallel = parallel
        self.dtype = "float64"
        self.device = device
        self.block_size = None

    def _build_points(self, coordinates):
        return (coordinates[0], coordinates[1], coordinates[2] - self.relative_depth)

    def _points_for(self, coordinates):
        if self.points is None:
            return tuple(np.asarray(p, dtype=np.float64) for p in self._build_points(coordinates))
        return tuple(np.ravel(np.asarray(p, dtype=np.float64)) for p in self.points[:3])
