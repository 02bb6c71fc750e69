"""
Layer of tesseroids on a regular longitude/latitude grid and its
``tesseroid_layer`` accessor.

Mirrors harmonica ``src/harmonica/_forward/tesseroid_layer.py``:
``tesseroid_layer`` (:20-150), ``_check_regular_grid`` (:153-167),
``_check_overlap`` (:170-180), ``DatasetAccessorTesseroidLayer`` (:183-520)
and ``_discard_thin_tesseroids`` (:523-560).  The members the prism and
tesseroid layers share live in :mod:`harmonica_gb300._grid_layer`.
``gravity`` keeps the cells with valid top, bottom and density (with the
reference's warning for a missing density), drops the thin ones and runs
:func:`harmonica_gb300.tesseroid_gravity` on the GPU.

When :mod:`xarray` is importable ``tesseroid_layer`` returns an
``xarray.Dataset`` and the accessor is registered on it as
``.tesseroid_layer`` when this module is imported, like the reference;
otherwise a :class:`TesseroidLayer`, a numpy container with the same
attribute surface (``longitude``, ``latitude``, ``top``, ``bottom``, data
variables, ``coords``, ``attrs``, ``.tesseroid_layer``).
"""

import warnings

import numpy as np

from ._grid_layer import (
    GridDataset,
    GridLayerAccessor,
    check_even_spacing,
    check_property_shapes,
    grid_axes,
    new_layer_dataset,
    register_layer_accessor,
)
from .tesseroid import tesseroid_gravity

DIMS = ("latitude", "longitude")

__all__ = ["DatasetAccessorTesseroidLayer", "TesseroidLayer", "tesseroid_layer"]


def _check_regular_grid(longitude, latitude):
    """ValueError unless both axes are evenly spaced (tesseroid_layer.py:153-167)."""
    check_even_spacing(longitude, "longitude")
    check_even_spacing(latitude, "latitude")


def _check_overlap(longitude):
    """ValueError when the cells would wrap around the globe onto each other:
    the longitude span plus one cell reaches 360 degrees (tesseroid_layer.py:170-180)."""
    step = longitude[1] - longitude[0]
    if np.ptp(longitude) >= 360 - step:
        raise ValueError(
            "Found invalid longitude coordinates that would create overlapping "
            "tesseroids around the globe."
        )


def _discard_thin_tesseroids(tesseroids, density, thickness_threshold):
    """The tesseroids (and densities) whose radial thickness is not below the
    threshold (tesseroid_layer.py:523-560)."""
    thin = (tesseroids[:, 5] - tesseroids[:, 4]) < thickness_threshold
    return tesseroids[~thin], density[~thin]


class TesseroidLayer(GridDataset):
    """
    Numpy stand-in for the xarray Dataset that ``tesseroid_layer`` builds.

    Coordinates ``longitude`` (n_lon,), ``latitude`` (n_lat,), ``top`` and
    ``bottom`` (n_lat, n_lon), data variables (n_lat, n_lon), ``attrs``.
    """

    def __init__(self, longitude, latitude, data=None):
        super().__init__(DIMS, {"longitude": longitude, "latitude": latitude}, data)


def tesseroid_layer(coordinates, surface, reference, properties=None):
    """
    Create a layer of tesseroids of equal size (tesseroid_layer.py:20-150).

    Parameters
    ----------
    coordinates : tuple
        ``longitude`` and ``latitude`` of the tesseroid centres in degrees:
        1d arrays per axis or 2d arrays from :func:`numpy.meshgrid`.  Must
        define a regular grid that does not overlap itself around the globe.
    surface : 2d-array
        Upper radius (m) where it is above ``reference`` (lower otherwise).
    reference : float or 2d-array
        Lower radius (m) where ``surface`` is above it.
    properties : dict or None
        Physical properties as (latitude, longitude) 2d-arrays, in SI units.

    Returns
    -------
    dataset : xarray.Dataset or TesseroidLayer
    """
    longitude, latitude = grid_axes(coordinates)
    data = check_property_shapes(properties, *DIMS, (latitude.size, longitude.size))
    layer = new_layer_dataset(DIMS, {"longitude": longitude, "latitude": latitude}, data,
                              lambda dims, axes, d: TesseroidLayer(axes["longitude"],
                                                                   axes["latitude"], d))
    _check_regular_grid(longitude, latitude)
    _check_overlap(longitude)
    layer.attrs = {
        "longitude_units": "degrees",
        "latitude_units": "degrees",
        "radius_units": "meters",
        "properties_units": "SI",
    }
    DatasetAccessorTesseroidLayer(layer).update_top_bottom(surface, reference)
    return layer


@register_layer_accessor("tesseroid_layer")
class DatasetAccessorTesseroidLayer(GridLayerAccessor):
    """
    Accessor for a layer of tesseroids (tesseroid_layer.py:183-520): use it
    through the ``tesseroid_layer`` attribute of the layer.  ``spacing`` is
    ``(s_latitude, s_longitude)``, ``shape`` ``(n_latitude, n_longitude)``,
    ``boundaries`` ``(longitude_w, longitude_e, latitude_s, latitude_n)``.
    """

    _dims = DIMS
    _bodies = "tesseroids"

    def gravity(self, coordinates, field, progressbar=False, density_name="density",
                thickness_threshold=None, **kwargs):
        """
        Gravity field of the layer (tesseroid_layer.py:322-404): tesseroids
        with NaN top, bottom or density are ignored (with a warning for the
        density), as are those thinner than ``thickness_threshold``; the rest
        go to :func:`harmonica_gb300.tesseroid_gravity` with ``kwargs``.
        """
        keep = self._get_nonans_mask(property_name=density_name).reshape(-1)
        cells = self._to_tesseroids()[keep]
        density = np.asarray(self._obj[density_name].values).reshape(-1)[keep]
        if thickness_threshold is not None:
            cells, density = _discard_thin_tesseroids(cells, density, thickness_threshold)
        return tesseroid_gravity(coordinates, tesseroids=cells, density=density, field=field,
                                 progressbar=progressbar, **kwargs)

    def _get_nonans_mask(self, property_name=None):
        """Cells whose top, bottom (and property, if named) are not NaN
        (tesseroid_layer.py:406-441); warns when a property is NaN on a cell
        whose top and bottom are valid."""
        valid = ~(np.isnan(np.asarray(self._obj.top.values))
                  | np.isnan(np.asarray(self._obj.bottom.values)))
        if property_name is None:
            return valid
        has_value = ~np.isnan(np.asarray(self._obj[property_name].values))
        if not np.all(has_value[valid]):
            warnings.warn(
                f"Found missing values in '{property_name}' property "
                + "of the tesseroid layer. The tesseroids with nan as "
                + f"'{property_name}' will be ignored.",
                stacklevel=1,
            )
        return valid & has_value

    def _to_tesseroids(self):
        """Boundaries of every tesseroid, one row each, (latitude, longitude) order."""
        return self._cells()

    def get_tesseroid(self, indices):
        """Boundaries of the tesseroid at ``(index_latitude, index_longitude)``."""
        return self._cell(indices)
