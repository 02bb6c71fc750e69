"""
A layer of prisms held on the GPU (harmonica's ``prism_layer`` and its
``prism_layer`` accessor, src/harmonica/_forward/prisms/layer.py:23-138 and
157-519, with the grids as device tensors).

``prism_layer_device`` builds the layer from numpy arrays or torch tensors;
``update_top_bottom`` runs ``hg_layer_top_bottom`` on the device and
``gravity`` runs ``hg_layer_forward`` on device tensors, returning a device
tensor: a loop that updates the layer and recomputes its field (an
inversion) never copies the grids to the host.  ``to_host`` gives the
numpy/xarray layer of :func:`harmonica_gb300.prism_layer` for everything
else.
"""

import warnings

import numpy as np

from . import _native
from .fields import FIELD_CODES, field_mask
from .layer import DIMS, _check_regular_grid, prism_layer

__all__ = ["DevicePrismLayer", "prism_layer_device"]


def _tensor(a, dev, torch):
    if isinstance(a, torch.Tensor):
        return a.to(device=dev, dtype=torch.float64).contiguous()
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=dev)


def _axis(a, along, torch):
    """1d centre coordinates from a 1d or meshgrid 2d array/tensor."""
    if a.dim() == 2:
        a = a[0, :] if along == "easting" else a[:, 0]
    return a.contiguous()


class DevicePrismLayer:
    """
    Layer of prisms of equal horizontal size with its grids on one GPU.

    Attributes ``easting``, ``northing`` (1d), ``top``, ``bottom`` and the
    properties (2d, ``(northing, easting)``) are float64 device tensors.
    """

    def __init__(self, easting, northing, properties, device):
        self.device = device
        self.easting = easting
        self.northing = northing
        self.properties = properties
        self.top = None
        self.bottom = None
        _check_regular_grid(easting.cpu().numpy(), northing.cpu().numpy())
        for name, value in properties.items():
            if tuple(value.shape) != self.shape:
                raise ValueError(
                    f"Invalid property '{name}' with shape '{tuple(value.shape)}'. "
                    "Its shape should be (northing, easting) = " + f"'{self.shape}'."
                )
        self._spacing = (
            float(northing[1] - northing[0]) if northing.numel() > 1 else 0.0,
            float(easting[1] - easting[0]) if easting.numel() > 1 else 0.0,
        )

    # ---------------------------------------------------------- geometry
    @property
    def dims(self):
        return DIMS

    @property
    def shape(self):
        """Number of prisms per direction: ``(n_north, n_east)``."""
        return (self.northing.numel(), self.easting.numel())

    @property
    def size(self):
        return self.northing.numel() * self.easting.numel()

    @property
    def spacing(self):
        """Spacing between prism centres: ``(s_north, s_east)``."""
        return self._spacing

    @property
    def boundaries(self):
        """``(west, east, south, north)`` of the layer."""
        s_north, s_east = self._spacing
        return (
            float(self.easting.min()) - s_east / 2,
            float(self.easting.max()) + s_east / 2,
            float(self.northing.min()) - s_north / 2,
            float(self.northing.max()) + s_north / 2,
        )

    def __getitem__(self, name):
        return self.properties[name]

    # ---------------------------------------------------------- top/bottom
    def update_top_bottom(self, surface, reference):
        """
        Set ``top``/``bottom`` from ``surface`` and ``reference`` on the device
        (layer.py:264-312): the top is the higher of the two on every cell.
        """
        import torch  # noqa: PLC0415

        surface = _tensor(surface, self.device, torch)
        if tuple(surface.shape) != self.shape:
            raise ValueError(
                f"Invalid surface array with shape '{tuple(surface.shape)}'. "
                + "Its shape should be compatible with the coordinates "
                + "of the layer of prisms."
            )
        ref_value = 0.0
        ref = None
        if isinstance(reference, torch.Tensor) or np.ndim(reference) != 0:
            ref = _tensor(reference, self.device, torch)
            if ref.dim() == 0:
                ref_value, ref = float(ref), None
            elif tuple(ref.shape) != self.shape:
                raise ValueError(
                    f"Invalid reference array with shape '{tuple(ref.shape)}'. "
                    + "Its shape should be compatible with the coordinates "
                    + "of the layer of prisms."
                )
        else:
            ref_value = float(reference)
        top = torch.empty(self.shape, dtype=torch.float64, device=self.device)
        bottom = torch.empty_like(top)
        lib = _native.lib()
        with torch.cuda.device(self.device):
            stream = torch.cuda.current_stream(self.device).cuda_stream
            _native.check(
                lib.hg_layer_top_bottom(
                    surface.data_ptr(), ref.data_ptr() if ref is not None else None, ref_value,
                    surface.numel(), top.data_ptr(), bottom.data_ptr(), stream,
                )
            )
        self.top, self.bottom = top, bottom

    # ---------------------------------------------------------- forward
    def gravity(self, coordinates, field, *, density_name="density", thickness_threshold=None,
                check_nan=True):
        """
        Gravity field of the layer on the observation points, as a float64
        device tensor in harmonica's units (layer.py:314-433 semantics:
        prisms with zero or NaN density, NaN top or bottom, or thinner than
        ``thickness_threshold`` are ignored).  ``coordinates`` are arrays or
        tensors of equal shape; the result has that shape.  ``check_nan``
        keeps the reference's warning on NaN densities (one device-to-host
        read of a flag); pass False inside a loop that must not synchronise.
        """
        import torch  # noqa: PLC0415

        from .layer import layer_forward_device  # noqa: PLC0415

        if field not in FIELD_CODES:
            msg = f"Gravitational field '{field}' not recognized."
            raise ValueError(msg)
        if self.top is None:
            raise ValueError("The layer has no top and bottom: call update_top_bottom first.")
        density = self.properties[density_name]
        if check_nan and bool(torch.isnan(density).any()):
            warnings.warn(
                "Found NaN values in 'density' property of the prisms layer. "
                "Their respective prisms will be ignored.",
                stacklevel=2,
            )
        coords = [_tensor(c, self.device, torch) for c in coordinates[:3]]
        shape = torch.broadcast_shapes(*(c.shape for c in coords))
        e, n, u = (c.expand(shape).reshape(-1).contiguous() for c in coords)
        threshold = 0.0 if thickness_threshold is None else float(thickness_threshold)
        with torch.cuda.device(self.device):
            out = layer_forward_device(
                e, n, u, self.easting, self.northing, self.bottom.reshape(-1),
                self.top.reshape(-1), density.reshape(-1).contiguous(), field_mask([field]),
                threshold,
            )
        return out[0].reshape(shape)

    # ---------------------------------------------------------- interop
    def to_prisms(self):
        """Boundaries of every prism as an ``(n_prisms, 6)`` device tensor,
        rows in ``(northing, easting)`` order (layer.py _to_prisms)."""
        import torch  # noqa: PLC0415

        s_north, s_east = self._spacing
        n_grid, e_grid = torch.meshgrid(self.northing, self.easting, indexing="ij")
        e_c, n_c = e_grid.reshape(-1), n_grid.reshape(-1)
        return torch.stack(
            (e_c - s_east / 2, e_c + s_east / 2, n_c - s_north / 2, n_c + s_north / 2,
             self.bottom.reshape(-1), self.top.reshape(-1)), dim=1,
        )

    def to_host(self):
        """The layer as :func:`harmonica_gb300.prism_layer` returns it (numpy
        arrays; an xarray Dataset when xarray is importable)."""
        props = {k: v.cpu().numpy() for k, v in self.properties.items()}
        layer = prism_layer(
            (self.easting.cpu().numpy(), self.northing.cpu().numpy()),
            self.top.cpu().numpy(), self.bottom.cpu().numpy(), properties=props or None,
        )
        return layer


def prism_layer_device(coordinates, surface, reference, properties=None, device=None):
    """
    Create a layer of prisms on the GPU (layer.py:23-138 semantics).

    ``coordinates``: easting and northing of the prism centres (1d, or 2d
    meshgrid arrays/tensors; a regular grid); ``surface``: 2d; ``reference``:
    a number or 2d; ``properties``: dict of 2d arrays/tensors.  Returns a
    :class:`DevicePrismLayer` with ``top``/``bottom`` set on the device.
    """
    import torch  # noqa: PLC0415

    from .gravity import _device  # noqa: PLC0415

    dev = _device(device)
    easting = _axis(_tensor(coordinates[0], dev, torch), "easting", torch)
    northing = _axis(_tensor(coordinates[1], dev, torch), "northing", torch)
    props = {k: _tensor(v, dev, torch) for k, v in (properties or {}).items()}
    layer = DevicePrismLayer(easting, northing, props, dev)
    layer.update_top_bottom(surface, reference)
    return layer
