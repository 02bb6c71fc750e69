"""
Layer of tesseroids on a regular longitude/latitude grid and its
``tesseroid_layer`` accessor.

Mirrors harmonica ``src/harmonica/_forward/tesseroid_layer.py``:
``tesseroid_layer`` (:20-150), ``_check_regular_grid`` (:153-167),
``_check_overlap`` (:170-180), ``DatasetAccessorTesseroidLayer`` (:183-520)
and ``_discard_thin_tesseroids`` (:523-560).  ``gravity`` masks the
tesseroids with NaN top, bottom or density (with the reference's warning),
drops the thin ones and runs :func:`harmonica_gb300.tesseroid_gravity` on
the GPU.

When :mod:`xarray` is importable ``tesseroid_layer`` returns an
``xarray.Dataset`` (use ``DatasetAccessorTesseroidLayer(ds)`` or register
it); otherwise a :class:`TesseroidLayer`, a small numpy container with the
same attribute surface (``longitude``, ``latitude``, ``top``, ``bottom``,
data variables, ``coords``, ``attrs``, ``.tesseroid_layer``).
"""

import warnings

import numpy as np

from .layer import _Coords, _var
from .tesseroid import tesseroid_gravity

try:  # optional, as in the reference environment
    import xarray as xr
except ImportError:  # pragma: no cover - depends on the environment
    xr = None

DIMS = ("latitude", "longitude")

__all__ = ["DatasetAccessorTesseroidLayer", "TesseroidLayer", "tesseroid_layer"]


def _check_regular_grid(longitude, latitude):
    """Same check and messages as tesseroid_layer.py:153-167."""
    if not np.allclose(longitude[1] - longitude[0], longitude[1:] - longitude[:-1]):
        msg = "Passed longitude coordinates are not evenly spaced."
        raise ValueError(msg)
    if not np.allclose(latitude[1] - latitude[0], latitude[1:] - latitude[:-1]):
        msg = "Passed latitude coordinates are not evenly spaced."
        raise ValueError(msg)


def _check_overlap(longitude):
    """Same check and message as tesseroid_layer.py:170-180."""
    spacing = longitude[1] - longitude[0]
    if longitude.max() - longitude.min() >= 360 - spacing:
        msg = (
            "Found invalid longitude coordinates that would create overlapping "
            "tesseroids around the globe."
        )
        raise ValueError(msg)


def _discard_thin_tesseroids(tesseroids, density, thickness_threshold):
    """Drop tesseroids thinner than the threshold (tesseroid_layer.py:523-560)."""
    thickness = tesseroids[:, -1] - tesseroids[:, -2]
    keep = np.logical_not(thickness < thickness_threshold)
    return tesseroids[keep, :], density[keep]


class TesseroidLayer:
    """
    Numpy stand-in for the xarray Dataset that ``tesseroid_layer`` builds.

    Coordinates ``longitude`` (n_lon,), ``latitude`` (n_lat,), ``top`` and
    ``bottom`` (n_lat, n_lon), data variables (n_lat, n_lon), ``attrs``.
    """

    def __init__(self, longitude, latitude, data=None, attrs=None):
        object.__setattr__(self, "coords", _Coords())
        object.__setattr__(self, "data_vars", {})
        object.__setattr__(self, "attrs", dict(attrs or {}))
        self.coords["longitude"] = np.asarray(longitude, dtype=np.float64)
        self.coords["latitude"] = np.asarray(latitude, dtype=np.float64)
        for name, value in (data or {}).items():
            self.data_vars[name] = _var(np.asarray(value))

    def __getattr__(self, name):
        coords = object.__getattribute__(self, "coords")
        if name in coords:
            return coords[name]
        data_vars = object.__getattribute__(self, "data_vars")
        if name in data_vars:
            return data_vars[name]
        if name == "tesseroid_layer":
            return DatasetAccessorTesseroidLayer(self)
        raise AttributeError(name)

    def __getitem__(self, name):
        if name in self.data_vars:
            return self.data_vars[name]
        return self.coords[name]

    def __contains__(self, name):
        return name in self.data_vars or name in self.coords

    @property
    def dims(self):
        return {"latitude": self.latitude.size, "longitude": self.longitude.size}

    def __repr__(self):
        return (
            f"<TesseroidLayer latitude: {self.latitude.size}, longitude: "
            f"{self.longitude.size}; coords: {list(self.coords)}; "
            f"data_vars: {list(self.data_vars)}>"
        )


def _grid_axes(coordinates):
    longitude, latitude = (np.asarray(c, dtype=np.float64) for c in coordinates[:2])
    if longitude.ndim == 2:
        longitude = longitude[0, :]
    if latitude.ndim == 2:
        latitude = latitude[:, 0]
    return longitude, latitude


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
    longitude, latitude = _grid_axes(coordinates)
    data = None
    if properties:
        data = {name: np.asarray(value) for name, value in properties.items()}
        for name, value in data.items():
            # xarray refuses these too (its dimensions would conflict)
            if value.shape != (latitude.size, longitude.size):
                raise ValueError(
                    f"Invalid property '{name}' with shape '{value.shape}'. "
                    "Its shape should be (latitude, longitude) = "
                    + f"'{(latitude.size, longitude.size)}'."
                )
    if xr is not None:
        data_vars = {k: (DIMS, v) for k, v in (data or {}).items()}
        layer = xr.Dataset(data_vars, coords={"longitude": longitude, "latitude": latitude})
    else:
        layer = TesseroidLayer(longitude, latitude, data)
    _check_regular_grid(layer.longitude.values, layer.latitude.values)
    _check_overlap(layer.longitude.values)
    layer.attrs = {
        "longitude_units": "degrees",
        "latitude_units": "degrees",
        "radius_units": "meters",
        "properties_units": "SI",
    }
    DatasetAccessorTesseroidLayer(layer).update_top_bottom(surface, reference)
    return layer


class DatasetAccessorTesseroidLayer:
    """Accessor for a layer of tesseroids (tesseroid_layer.py:183-520)."""

    def __init__(self, xarray_obj):
        self._obj = xarray_obj

    @property
    def dims(self):
        """The dims tuple of the layer: ``("latitude", "longitude")``."""
        return DIMS

    @property
    def spacing(self):
        """Spacing between tesseroid centres: ``(s_latitude, s_longitude)``."""
        longitude, latitude = self._obj.longitude.values, self._obj.latitude.values
        _check_regular_grid(longitude, latitude)
        return latitude[1] - latitude[0], longitude[1] - longitude[0]

    @property
    def size(self):
        """Total number of tesseroids in the layer."""
        return self._obj.latitude.size * self._obj.longitude.size

    @property
    def shape(self):
        """Number of tesseroids per direction: ``(n_latitude, n_longitude)``."""
        return (self._obj.latitude.size, self._obj.longitude.size)

    @property
    def boundaries(self):
        """Boundaries of the layer: ``(longitude_w, longitude_e, latitude_s, latitude_n)``."""
        s_lat, s_lon = self.spacing
        west = self._obj.longitude.values.min() - s_lon / 2
        east = self._obj.longitude.values.max() + s_lon / 2
        south = self._obj.latitude.values.min() - s_lat / 2
        north = self._obj.latitude.values.max() + s_lat / 2
        return west, east, south, north

    def update_top_bottom(self, surface, reference):
        """Set ``top``/``bottom`` from ``surface`` and ``reference``
        (tesseroid_layer.py:273-320): the top is the higher of the two."""
        surface, reference = np.asarray(surface), np.asarray(reference)
        if surface.shape != self.shape:
            raise ValueError(
                f"Invalid surface array with shape '{surface.shape}'. "
                + "Its shape should be compatible with the coordinates "
                + "of the layer of tesseroids."
            )
        if reference.ndim != 0:
            if reference.shape != self.shape:
                raise ValueError(
                    f"Invalid reference array with shape '{reference.shape}'. "
                    + "Its shape should be compatible with the coordinates "
                    + "of the layer of tesseroids."
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

    def gravity(self, coordinates, field, progressbar=False, density_name="density",
                thickness_threshold=None, **kwargs):
        """
        Gravity field of the layer (tesseroid_layer.py:322-404): tesseroids
        with NaN top, bottom or density are ignored (with a warning for the
        density), as are those thinner than ``thickness_threshold``; the rest
        go to :func:`harmonica_gb300.tesseroid_gravity` with ``kwargs``.
        """
        boundaries = self._to_tesseroids()
        density = np.asarray(self._obj[density_name].values)
        mask = self._get_nonans_mask(property_name=density_name)
        boundaries = boundaries[mask.ravel()]
        density = density[mask]
        if thickness_threshold is not None:
            boundaries, density = _discard_thin_tesseroids(boundaries, density,
                                                           thickness_threshold)
        return tesseroid_gravity(coordinates, tesseroids=boundaries, density=density,
                                 field=field, progressbar=progressbar, **kwargs)

    def _get_nonans_mask(self, property_name=None):
        """Tesseroids with no NaN top, bottom or property (:406-441)."""
        mask = np.logical_and(
            np.logical_not(np.isnan(np.asarray(self._obj.top.values))),
            np.logical_not(np.isnan(np.asarray(self._obj.bottom.values))),
        )
        if property_name is not None:
            mask_property = np.logical_not(np.isnan(np.asarray(self._obj[property_name].values)))
            if not mask_property[mask].all():
                warnings.warn(
                    f"Found missing values in '{property_name}' property "
                    + "of the tesseroid layer. The tesseroids with nan as "
                    + f"'{property_name}' will be ignored.",
                    stacklevel=1,
                )
            mask = np.logical_and(mask, mask_property)
        return mask

    def _get_tesseroid_horizontal_boundaries(self, longitude, latitude):
        s_lat, s_lon = self.spacing
        return (longitude - s_lon / 2, longitude + s_lon / 2,
                latitude - s_lat / 2, latitude + s_lat / 2)

    def _to_tesseroids(self):
        """Boundaries of every tesseroid, one row each, (latitude, longitude) order."""
        longitude, latitude = np.meshgrid(self._obj.longitude.values, self._obj.latitude.values)
        west, east, south, north = self._get_tesseroid_horizontal_boundaries(
            longitude.ravel(), latitude.ravel()
        )
        bottom = np.asarray(self._obj.bottom.values).ravel()
        top = np.asarray(self._obj.top.values).ravel()
        return np.vstack((west, east, south, north, bottom, top)).T

    def get_tesseroid(self, indices):
        """Boundaries of the tesseroid at ``(index_latitude, index_longitude)``."""
        center_longitude = self._obj.longitude.values[indices[1]]
        center_latitude = self._obj.latitude.values[indices[0]]
        west, east, south, north = self._get_tesseroid_horizontal_boundaries(
            center_longitude, center_latitude
        )
        bottom = self._obj.bottom.values[indices]
        top = self._obj.top.values[indices]
        return west, east, south, north, bottom, top
