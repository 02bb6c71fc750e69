"""
What the prism layer and the tesseroid layer have in common: a layer is a
regular 2-D grid of cell centres with a ``top`` and a ``bottom`` per cell and
physical properties per cell, kept in an ``xarray.Dataset`` (dims
``(row axis, column axis)``) and queried through an accessor registered on
the dataset.

* :func:`register_layer_accessor` registers an accessor class under a name
  on ``xarray.Dataset`` (when xarray is importable, as harmonica does with
  ``xr.register_dataset_accessor``, prisms/layer.py:157 and
  tesseroid_layer.py:183) and on :class:`GridDataset`, the numpy stand-in
  used without xarray.
* :class:`GridLayerAccessor` holds the members both accessors share (dims,
  spacing, size, shape, boundaries, update_top_bottom, cell boundaries),
  written once for both grids.  The numbers and error texts are the
  reference's (prisms/layer.py:141-312, 435-483; tesseroid_layer.py:153-320,
  406-520).
"""

import numpy as np

try:  # optional, as in the reference environment
    import xarray as xr
except ImportError:  # pragma: no cover - depends on the environment
    xr = None


def check_even_spacing(centres, axis_name):
    """Raise the reference's ValueError when the steps between consecutive
    ``centres`` are not all close to the first step."""
    steps = np.diff(centres)
    if not np.allclose(steps[0], steps):
        raise ValueError(f"Passed {axis_name} coordinates are not evenly spaced.")


def grid_axes(coordinates):
    """1-d column and row centres from 1-d axes or from 2-d meshgrid arrays."""
    cols, rows = (np.asarray(c, dtype=np.float64) for c in coordinates[:2])
    return (cols[0, :] if cols.ndim == 2 else cols), (rows[:, 0] if rows.ndim == 2 else rows)


def check_property_shapes(properties, row_axis, col_axis, shape):
    """The properties as arrays; ValueError for one whose shape is not the
    grid's (xarray would refuse it: its dims would conflict)."""
    data = {name: np.asarray(value) for name, value in (properties or {}).items()}
    for name, value in data.items():
        if value.shape != shape:
            raise ValueError(
                f"Invalid property '{name}' with shape '{value.shape}'. "
                f"Its shape should be ({row_axis}, {col_axis}) = '{shape}'."
            )
    return data


class _Values(np.ndarray):
    """ndarray with a ``.values`` view, standing in for an xarray.DataArray."""

    @property
    def values(self):
        return self.view(np.ndarray)


def as_values(a):
    a = np.asarray(a)
    return np.array(a, dtype=np.float64 if a.dtype.kind in "iu" else None).view(_Values)


class _Coords(dict):
    """Coordinates of a :class:`GridDataset`; accepts xarray's ``(dims, values)``."""

    def __setitem__(self, key, value):
        if isinstance(value, tuple) and len(value) == 2:
            value = value[1]
        super().__setitem__(key, as_values(value))


class GridDataset:
    """
    Numpy stand-in for the ``xarray.Dataset`` of a layer, used when xarray is
    not importable: coordinates (the two 1-d axes, then ``top`` and
    ``bottom`` on the grid), data variables on the grid, ``attrs``, and the
    accessors registered with :func:`register_layer_accessor` as attributes.
    """

    _accessors = {}

    def __init__(self, dims, axes, data=None):
        object.__setattr__(self, "coords", _Coords())
        object.__setattr__(self, "data_vars", {})
        object.__setattr__(self, "attrs", {})
        object.__setattr__(self, "_dims", tuple(dims))
        for name in dims:
            self.coords[name] = np.asarray(axes[name], dtype=np.float64)
        for name, value in (data or {}).items():
            self.data_vars[name] = as_values(value)

    def __getattr__(self, name):
        for table in ("coords", "data_vars"):
            entries = object.__getattribute__(self, table)
            if name in entries:
                return entries[name]
        accessor = GridDataset._accessors.get(name)
        if accessor is not None:
            return accessor(self)
        raise AttributeError(name)

    def __getitem__(self, name):
        return self.data_vars[name] if name in self.data_vars else self.coords[name]

    def __contains__(self, name):
        return name in self.data_vars or name in self.coords

    @property
    def dims(self):
        return {name: self.coords[name].size for name in self._dims}

    def __repr__(self):
        sizes = ", ".join(f"{k}: {v}" for k, v in self.dims.items())
        return (f"<{type(self).__name__} {sizes}; coords: {list(self.coords)}; "
                f"data_vars: {list(self.data_vars)}>")


def register_layer_accessor(name):
    """Class decorator: make ``cls(dataset)`` available as ``dataset.<name>``
    on xarray Datasets (when xarray is importable) and on GridDatasets."""

    def register(cls):
        if xr is not None:
            xr.register_dataset_accessor(name)(cls)
        GridDataset._accessors[name] = cls
        return cls

    return register


def new_layer_dataset(dims, axes, data, container):
    """An xarray.Dataset when xarray is importable, else ``container``."""
    if xr is not None:
        data_vars = {k: (tuple(dims), v) for k, v in (data or {}).items()}
        return xr.Dataset(data_vars, coords={name: axes[name] for name in dims})
    return container(dims, axes, data)


class GridLayerAccessor:
    """
    Accessor members shared by the prism and tesseroid layers.  Subclasses
    set ``_dims`` (row axis, column axis) and ``_bodies`` (the plural noun
    of the error messages).
    """

    _dims = ("northing", "easting")
    _bodies = "prisms"

    def __init__(self, xarray_obj):
        self._obj = xarray_obj

    def _axis(self, name):
        return np.asarray(self._obj[name].values)

    @property
    def dims(self):
        """The dims tuple of the layer (xarray order: rows, then columns)."""
        return self._dims

    @property
    def spacing(self):
        """Spacing between cell centres: ``(row spacing, column spacing)``."""
        rows, cols = (self._axis(a) for a in self._dims)
        check_even_spacing(cols, self._dims[1])
        check_even_spacing(rows, self._dims[0])
        return rows[1] - rows[0], cols[1] - cols[0]

    @property
    def size(self):
        """Total number of cells in the layer."""
        n_rows, n_cols = self.shape
        return n_rows * n_cols

    @property
    def shape(self):
        """Number of cells per direction: ``(n_rows, n_cols)``."""
        return tuple(self._axis(a).size for a in self._dims)

    @property
    def boundaries(self):
        """Horizontal extent of the layer: ``(west, east, south, north)``
        (the outer edges of the outermost cells)."""
        half_row, half_col = (s / 2 for s in self.spacing)
        rows, cols = (self._axis(a) for a in self._dims)
        return cols.min() - half_col, cols.max() + half_col, rows.min() - half_row, \
            rows.max() + half_row

    def _cell_edges(self, col_centre, row_centre):
        """(west, east, south, north) of cells with these centres."""
        half_row, half_col = (s / 2 for s in self.spacing)
        return (col_centre - half_col, col_centre + half_col,
                row_centre - half_row, row_centre + half_row)

    def update_top_bottom(self, surface, reference):
        """
        Set the ``top`` and ``bottom`` coordinates: on each cell the higher of
        ``surface`` and ``reference`` is the top and the lower the bottom (a
        NaN surface stays the top, with the reference as bottom).
        ``reference`` is a scalar or a grid.
        """
        surface = np.asarray(surface)
        reference = np.asarray(reference)
        for label, grid in (("surface", surface), ("reference", reference)):
            if (label == "surface" or grid.ndim != 0) and grid.shape != self.shape:
                raise ValueError(
                    f"Invalid {label} array with shape '{grid.shape}'. "
                    "Its shape should be compatible with the coordinates "
                    f"of the layer of {self._bodies}."
                )
        if reference.ndim == 0:
            reference = np.full(self.shape, reference * 1.0)
        below = surface < reference
        # each grid keeps the dtype of the array it starts from
        top = np.where(below, reference, surface).astype(surface.dtype, copy=False)
        bottom = np.where(below, surface, reference).astype(reference.dtype, copy=False)
        self._obj.coords["top"] = (self.dims, top)
        self._obj.coords["bottom"] = (self.dims, bottom)

    def _cells(self):
        """Boundaries of every cell, one row each (w, e, s, n, bottom, top),
        rows of the grid first (row-major over (row axis, column axis))."""
        rows, cols = (self._axis(a) for a in self._dims)
        col_centre = np.tile(cols, rows.size)
        row_centre = np.repeat(rows, cols.size)
        west, east, south, north = self._cell_edges(col_centre, row_centre)
        bottom = np.asarray(self._obj.bottom.values).reshape(-1)
        top = np.asarray(self._obj.top.values).reshape(-1)
        return np.column_stack((west, east, south, north, bottom, top))

    def _cell(self, indices):
        """Boundaries of the cell at ``(row index, column index)``."""
        i_row, i_col = indices
        west, east, south, north = self._cell_edges(
            self._axis(self._dims[1])[i_col], self._axis(self._dims[0])[i_row])
        return (west, east, south, north, self._obj.bottom.values[indices],
                self._obj.top.values[indices])
