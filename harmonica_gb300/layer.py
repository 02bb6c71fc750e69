"""
Layer of prisms on a regular horizontal grid and its ``prism_layer`` accessor.

Mirrors harmonica ``src/harmonica/_forward/prisms/layer.py``:
``prism_layer`` (:23-138), ``_check_regular_grid`` (:141-155) and
``DatasetAccessorPrismLayer`` (:157-519, without ``to_pyvista``, which is
visualization).  The forward sum of ``gravity`` (:314-433) runs on the GPU
through the C ABI ``hg_layer_forward``, which builds the prism boundaries
from the grid on the fly and applies the same skips (:596-607).

When :mod:`xarray` is importable, ``prism_layer`` returns an
``xarray.Dataset`` and the accessor is registered as ``.prism_layer``, like
the reference.  Without xarray it returns a :class:`PrismLayer`, a small
numpy container with the same attribute surface (``easting``, ``northing``,
``top``, ``bottom``, data variables, ``coords``, ``attrs``, ``.prism_layer``).
"""

import warnings

import numpy as np

from . import _native
from ._trace import stage
from .fields import FIELD_CODES, field_mask

try:  # optional, as in the reference environment
    import xarray as xr
except ImportError:  # pragma: no cover - depends on the environment
    xr = None

DIMS = ("northing", "easting")


def _check_regular_grid(easting, northing):
    """Same check and messages as layer.py:141-155."""
    if not np.allclose(easting[1] - easting[0], easting[1:] - easting[:-1]):
        msg = "Passed easting coordinates are not evenly spaced."
        raise ValueError(msg)
    if not np.allclose(northing[1] - northing[0], northing[1:] - northing[:-1]):
        msg = "Passed northing coordinates are not evenly spaced."
        raise ValueError(msg)


class _Var(np.ndarray):
    """ndarray with a ``.values`` view, standing in for an xarray.DataArray."""

    @property
    def values(self):
        return self.view(np.ndarray)


def _var(a):
    return np.array(a, dtype=np.float64 if np.asarray(a).dtype.kind in "iu" else None).view(_Var)


class _Coords(dict):
    def __setitem__(self, key, value):
        if isinstance(value, tuple) and len(value) == 2:
            value = value[1]
        super().__setitem__(key, _var(value))


class PrismLayer:
    """
    Numpy stand-in for the xarray Dataset that ``prism_layer`` builds.

    Coordinates ``easting`` (n_e,), ``northing`` (n_n,), ``top`` and
    ``bottom`` (n_n, n_e), data variables (n_n, n_e), ``attrs``.
    """

    def __init__(self, easting, northing, data=None, attrs=None):
        object.__setattr__(self, "coords", _Coords())
        object.__setattr__(self, "data_vars", {})
        object.__setattr__(self, "attrs", dict(attrs or {}))
        self.coords["easting"] = np.asarray(easting, dtype=np.float64)
        self.coords["northing"] = np.asarray(northing, dtype=np.float64)
        for name, value in (data or {}).items():
            self.data_vars[name] = _var(np.asarray(value))

    def __getattr__(self, name):
        coords = object.__getattribute__(self, "coords")
        if name in coords:
            return coords[name]
        data_vars = object.__getattribute__(self, "data_vars")
        if name in data_vars:
            return data_vars[name]
        if name == "prism_layer":
            return DatasetAccessorPrismLayer(self)
        raise AttributeError(name)

    def __getitem__(self, name):
        if name in self.data_vars:
            return self.data_vars[name]
        return self.coords[name]

    def __contains__(self, name):
        return name in self.data_vars or name in self.coords

    @property
    def dims(self):
        return {"northing": self.northing.size, "easting": self.easting.size}

    def __repr__(self):
        return (
            f"<PrismLayer northing: {self.northing.size}, easting: {self.easting.size}; "
            f"coords: {list(self.coords)}; data_vars: {list(self.data_vars)}>"
        )


def _grid_axes(coordinates):
    easting, northing = (np.asarray(c, dtype=np.float64) for c in coordinates[:2])
    if easting.ndim == 2:
        easting = easting[0, :]
    if northing.ndim == 2:
        northing = northing[:, 0]
    return easting, northing


def prism_layer(coordinates, surface, reference, properties=None):
    """
    Create a layer of prisms of equal horizontal size (layer.py:23-138).

    Parameters
    ----------
    coordinates : tuple
        ``easting`` and ``northing`` of the prism centres: 1d arrays per axis
        or 2d arrays from :func:`numpy.meshgrid`.  Must define a regular grid.
    surface : 2d-array
        Upper boundary where it is above ``reference`` (lower otherwise).
    reference : float or 2d-array
        Lower boundary where ``surface`` is above it.
    properties : dict or None
        Physical properties as (northing, easting) 2d-arrays, in SI units.

    Returns
    -------
    dataset : xarray.Dataset or PrismLayer
        Layer with ``easting``, ``northing``, ``top``, ``bottom`` coordinates
        and the properties as data variables.
    """
    easting, northing = _grid_axes(coordinates)
    data = None
    if properties:
        data = {name: np.asarray(value) for name, value in properties.items()}
        for name, value in data.items():
            # xarray refuses these too (its dimensions would conflict)
            if value.shape != (northing.size, easting.size):
                raise ValueError(
                    f"Invalid property '{name}' with shape '{value.shape}'. "
                    "Its shape should be (northing, easting) = "
                    + f"'{(northing.size, easting.size)}'."
                )
    if xr is not None:
        data_vars = {k: (DIMS, v) for k, v in (data or {}).items()}
        prisms = xr.Dataset(data_vars, coords={"easting": easting, "northing": northing})
    else:
        prisms = PrismLayer(easting, northing, data)
    _check_regular_grid(prisms.easting.values, prisms.northing.values)
    prisms.attrs = {"coords_units": "meters", "properties_units": "SI"}
    DatasetAccessorPrismLayer(prisms).update_top_bottom(surface, reference)
    return prisms


class DatasetAccessorPrismLayer:
    """
    Accessor for a layer of prisms (layer.py:157-519).

    Use it through the ``prism_layer`` attribute of the layer returned by
    :func:`prism_layer`.
    """

    def __init__(self, xarray_obj):
        self._obj = xarray_obj

    @property
    def dims(self):
        """The dims tuple of the layer: ``("northing", "easting")``."""
        return DIMS

    @property
    def spacing(self):
        """Spacing between prism centres: ``(s_north, s_east)``."""
        easting, northing = self._obj.easting.values, self._obj.northing.values
        _check_regular_grid(easting, northing)
        s_north, s_east = northing[1] - northing[0], easting[1] - easting[0]
        return s_north, s_east

    @property
    def boundaries(self):
        """Boundaries of the layer: ``(west, east, south, north)``."""
        s_north, s_east = self.spacing
        west = self._obj.easting.values.min() - s_east / 2
        east = self._obj.easting.values.max() + s_east / 2
        south = self._obj.northing.values.min() - s_north / 2
        north = self._obj.northing.values.max() + s_north / 2
        return west, east, south, north

    @property
    def size(self):
        """Total number of prisms in the layer."""
        return self._obj.northing.size * self._obj.easting.size

    @property
    def shape(self):
        """Number of prisms per direction: ``(n_north, n_east)``."""
        return (self._obj.northing.size, self._obj.easting.size)

    def _get_prism_horizontal_boundaries(self, easting, northing):
        spacing = self.spacing
        west = easting - spacing[1] / 2
        east = easting + spacing[1] / 2
        south = northing - spacing[0] / 2
        north = northing + spacing[0] / 2
        return west, east, south, north

    def update_top_bottom(self, surface, reference):
        """
        Set ``top``/``bottom`` from ``surface`` and ``reference``
        (layer.py:264-312): the top is the higher of the two on every cell.
        """
        surface, reference = np.asarray(surface), np.asarray(reference)
        if surface.shape != self.shape:
            raise ValueError(
                f"Invalid surface array with shape '{surface.shape}'. "
                + "Its shape should be compatible with the coordinates "
                + "of the layer of prisms."
            )
        if reference.ndim != 0:
            if reference.shape != self.shape:
                raise ValueError(
                    f"Invalid reference array with shape '{reference.shape}'. "
                    + "Its shape should be compatible with the coordinates "
                    + "of the layer of prisms."
                )
        else:
            reference = reference * np.ones(self.shape)
        top = surface.copy()
        bottom = reference.copy()
        reverse = surface < reference
        top[reverse] = reference[reverse]
        bottom[reverse] = surface[reverse]
        self._obj.coords["top"] = (self.dims, top)
        self._obj.coords["bottom"] = (self.dims, bottom)

    def gravity(
        self,
        coordinates,
        field,
        *,
        density_name="density",
        thickness_threshold=None,
        parallel=True,
        progressbar=False,
        device=None,
    ):
        """
        Gravity field of the layer on the observation points (layer.py:314-433).

        Prisms with zero or NaN density, NaN top or bottom, or thinner than
        ``thickness_threshold`` are ignored.  Returns float64 in harmonica's
        units (potential J/kg, accelerations mGal, tensor Eotvos).
        ``parallel`` and ``progressbar`` are accepted for compatibility.
        """
        if field not in FIELD_CODES:
            msg = f"Gravitational field '{field}' not recognized."
            raise ValueError(msg)
        _check_regular_grid(self._obj.easting.values, self._obj.northing.values)
        cast = np.broadcast(*coordinates[:3])
        coords = tuple(
            np.array(np.broadcast_to(np.asarray(c, dtype=np.float64), cast.shape)).ravel()
            for c in coordinates[:3]
        )
        thickness_threshold = 0.0 if thickness_threshold is None else thickness_threshold
        density = np.asarray(self._obj[density_name].values, dtype=np.float64)
        if np.isnan(density).any():
            msg = (
                "Found NaN values in 'density' property of the prisms layer. "
                "Their respective prisms will be ignored."
            )
            warnings.warn(msg, stacklevel=2)
        result = layer_forward(
            coords,
            self._obj.easting.values,
            self._obj.northing.values,
            self._obj.bottom.values,
            self._obj.top.values,
            density,
            field_mask([field]),
            float(thickness_threshold),
            device=device,
        )
        return result[0].reshape(cast.shape)

    def _to_prisms(self):
        """Boundaries of every prism, one row each, in (northing, easting) order."""
        easting, northing = np.meshgrid(self._obj.easting.values, self._obj.northing.values)
        west, east, south, north = self._get_prism_horizontal_boundaries(
            easting.ravel(), northing.ravel()
        )
        bottom = np.asarray(self._obj.bottom.values).ravel()
        top = np.asarray(self._obj.top.values).ravel()
        return np.vstack((west, east, south, north, bottom, top)).T

    def get_prism(self, indices):
        """Boundaries of the prism at ``(index_northing, index_easting)``."""
        center_easting = self._obj.easting.values[indices[1]]
        center_northing = self._obj.northing.values[indices[0]]
        west, east, south, north = self._get_prism_horizontal_boundaries(
            center_easting, center_northing
        )
        bottom = self._obj.bottom.values[indices]
        top = self._obj.top.values[indices]
        return west, east, south, north, bottom, top


def layer_forward(coords, easting, northing, bottom, top, density, mask, threshold, device=None):
    """Run ``hg_layer_forward`` on host arrays; returns (n_fields, N) float64."""
    import torch  # noqa: PLC0415

    from .gravity import _device, _ptr  # noqa: PLC0415

    lib = _native.lib()
    dev = _device(device)
    n_obs = coords[0].size
    n_rows = bin(mask).count("1")
    with torch.cuda.device(dev):
        with stage("upload layer and points"):
            e, n, u = (torch.from_numpy(np.ascontiguousarray(c)).to(dev) for c in coords)
            ce = torch.from_numpy(np.ascontiguousarray(easting, dtype=np.float64)).to(dev)
            cn = torch.from_numpy(np.ascontiguousarray(northing, dtype=np.float64)).to(dev)
            bt = torch.from_numpy(np.ascontiguousarray(bottom, dtype=np.float64)).to(dev)
            tp = torch.from_numpy(np.ascontiguousarray(top, dtype=np.float64)).to(dev)
            rho = torch.from_numpy(np.ascontiguousarray(density, dtype=np.float64)).to(dev)
        with stage("layer forward"):
            out = layer_forward_device(e, n, u, ce, cn, bt, tp, rho, mask, threshold)
        with stage("download"):
            return out.cpu().numpy()


def layer_forward_device(e, n, u, ce, cn, bottom, top, density, mask, threshold):
    """``hg_layer_forward`` on device tensors (current stream); returns (n_fields, N)."""
    import torch  # noqa: PLC0415

    from .gravity import _ptr  # noqa: PLC0415

    # the kernel reads one value of each grid per prism and three coordinates
    # per point: a short array would be read past its end on the device
    n_prisms = ce.numel() * cn.numel()
    for name, grid in (("bottom", bottom), ("top", top), ("density", density)):
        if grid.numel() != n_prisms:
            raise ValueError(
                f"Invalid '{name}' with {grid.numel()} values: the layer has "
                f"{cn.numel()} x {ce.numel()} prisms (northing x easting)."
            )
    if not e.numel() == n.numel() == u.numel():
        raise ValueError("The coordinates of the observation points must have the same "
                         "number of elements.")
    lib = _native.lib()
    n_obs = e.numel()
    n_rows = bin(mask).count("1")
    out = torch.empty((n_rows, n_obs), dtype=torch.float64, device=e.device)
    ws_bytes = _native.ctypes.c_size_t(0)
    _native.check(
        lib.hg_layer_forward_workspace(
            n_obs, ce.numel(), cn.numel(), mask, _native.ctypes.byref(ws_bytes)
        )
    )
    ws = None
    if ws_bytes.value:
        ws = torch.empty((ws_bytes.value + 7) // 8, dtype=torch.float64, device=e.device)
    stream = torch.cuda.current_stream(e.device).cuda_stream
    _native.check(
        lib.hg_layer_forward(
            _ptr(e), _ptr(n), _ptr(u), n_obs, _ptr(ce), ce.numel(), _ptr(cn), cn.numel(),
            _ptr(bottom), _ptr(top), _ptr(density), threshold, mask, _ptr(out), _ptr(ws),
            ws_bytes.value, stream,
        )
    )
    return out
