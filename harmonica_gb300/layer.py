"""
Layer of prisms on a regular horizontal grid and its ``prism_layer`` accessor.

Mirrors harmonica ``src/harmonica/_forward/prisms/layer.py``:
``prism_layer`` (:23-138), ``_check_regular_grid`` (:141-155) and
``DatasetAccessorPrismLayer`` (:157-519, without ``to_pyvista``, which is
visualization).  The members the prism and tesseroid layers share live in
:mod:`harmonica_gb300._grid_layer`.  The forward sum of ``gravity``
(:314-433) runs on the GPU through the C ABI ``hg_layer_forward``, which
builds the prism boundaries from the grid on the fly and applies the same
skips (:596-607).

When :mod:`xarray` is importable, ``prism_layer`` returns an
``xarray.Dataset`` and the accessor is registered on it as ``.prism_layer``
when this module is imported, like the reference.  Without xarray it returns
a :class:`PrismLayer`, a numpy container with the same attribute surface
(``easting``, ``northing``, ``top``, ``bottom``, data variables, ``coords``,
``attrs``, ``.prism_layer``).
"""

import warnings

import numpy as np

from . import _native
from ._grid_layer import (
    GridDataset,
    GridLayerAccessor,
    check_even_spacing,
    check_property_shapes,
    grid_axes,
    new_layer_dataset,
    register_layer_accessor,
)
from ._trace import stage
from .fields import FIELD_CODES, field_mask

DIMS = ("northing", "easting")


def _check_regular_grid(easting, northing):
    """ValueError unless both axes are evenly spaced (layer.py:141-155)."""
    check_even_spacing(easting, "easting")
    check_even_spacing(northing, "northing")


class PrismLayer(GridDataset):
    """
    Numpy stand-in for the xarray Dataset that ``prism_layer`` builds.

    Coordinates ``easting`` (n_e,), ``northing`` (n_n,), ``top`` and
    ``bottom`` (n_n, n_e), data variables (n_n, n_e), ``attrs``.
    """

    def __init__(self, easting, northing, data=None):
        super().__init__(DIMS, {"easting": easting, "northing": northing}, data)


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
    easting, northing = grid_axes(coordinates)
    data = check_property_shapes(properties, *DIMS, (northing.size, easting.size))
    layer = new_layer_dataset(DIMS, {"easting": easting, "northing": northing}, data,
                              lambda dims, axes, d: PrismLayer(axes["easting"],
                                                               axes["northing"], d))
    _check_regular_grid(easting, northing)
    layer.attrs = {"coords_units": "meters", "properties_units": "SI"}
    DatasetAccessorPrismLayer(layer).update_top_bottom(surface, reference)
    return layer


@register_layer_accessor("prism_layer")
class DatasetAccessorPrismLayer(GridLayerAccessor):
    """
    Accessor for a layer of prisms (layer.py:157-519).

    Use it through the ``prism_layer`` attribute of the layer returned by
    :func:`prism_layer`: ``spacing`` is ``(s_north, s_east)``, ``shape``
    ``(n_north, n_east)``, ``boundaries`` ``(west, east, south, north)``.
    """

    _dims = DIMS
    _bodies = "prisms"

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
        return self._cells()

    def get_prism(self, indices):
        """Boundaries of the prism at ``(index_northing, index_easting)``."""
        return self._cell(indices)


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
