"""
Drop-in replacement for ``harmonica.point_gravity`` running on a GB300.

Mirrors ``src/harmonica/_forward/point.py:30-268`` (harmonica): same
signature, coordinate systems (``cartesian`` with the ten fields plus the
``g_ne``, ``g_ze``, ``g_zn`` aliases; ``spherical`` with ``potential`` and
``g_z``, ``g_n``/``g_e`` raising ``NotImplementedError``), same errors and
units.  The all-pairs sum runs in the CUDA library through ``hg_point_forward``.
"""

import numpy as np

from . import _native

_CART = {"potential": 0, "g_e": 1, "g_n": 2, "g_z": 3, "g_ee": 4, "g_nn": 5, "g_zz": 6,
         "g_en": 7, "g_ez": 8, "g_nz": 9, "g_ne": 7, "g_ze": 8, "g_zn": 9}
_SPH = {"potential": 0, "g_z": 3, "g_n": None, "g_e": None}


def check_coordinate_system(coordinate_system, valid_coord_systems=("cartesian", "spherical")):
    """Same check and message as harmonica _forward/utils.py:71-87."""
    if coordinate_system not in valid_coord_systems:
        msg = f"Coordinate system {coordinate_system} not recognized."
        raise ValueError(msg)


def _kernel_code(coordinate_system, field):
    table = _CART if coordinate_system == "cartesian" else _SPH
    if field not in table:
        msg = f"Gravitational field '{field}' not recognized"
        raise ValueError(msg)
    if table[field] is None:
        raise NotImplementedError
    return table[field]


def point_gravity(coordinates, points, masses, field, coordinate_system="cartesian",
                  parallel=True, dtype="float64", device=None):
    """
    Gravitational fields of point masses (``harmonica.point_gravity``).

    Parameters as in harmonica: ``coordinates`` and ``points`` are
    (easting, northing, upward) in meters, or (longitude, latitude, radius) in
    degrees/meters for ``coordinate_system="spherical"``; ``masses`` in kg.
    ``parallel`` is accepted for compatibility.  Returns potential in J/kg,
    accelerations in mGal (g_z downward), tensor components in Eotvos, with
    the broadcast shape of the coordinates.
    """
    import torch

    from .gravity import _device, _ptr

    check_coordinate_system(coordinate_system, valid_coord_systems=("cartesian", "spherical"))
    cast = np.broadcast(*coordinates[:3])
    coords = tuple(np.array(np.broadcast_to(np.asarray(c, dtype=np.float64), cast.shape)).ravel()
                   for c in coordinates[:3])
    pts = tuple(np.ascontiguousarray(np.atleast_1d(np.asarray(p, dtype=np.float64)).ravel())
                for p in points[:3])
    masses = np.ascontiguousarray(np.atleast_1d(np.asarray(masses, dtype=np.float64)).ravel())
    # the kernels read three coordinates and one mass per point
    if not pts[0].size == pts[1].size == pts[2].size:
        raise ValueError(
            "The coordinates of the point masses must have the same number of elements "
            f"({pts[0].size}, {pts[1].size}, {pts[2].size})"
        )
    if masses.size != pts[0].size:
        raise ValueError(
            f"Number of elements in masses ({masses.size}) "
            + f"mismatch the number of points ({pts[0].size})"
        )
    code = _kernel_code(coordinate_system, field)
    lib = _native.lib()
    dev = _device(device)
    n_obs = coords[0].size
    with torch.cuda.device(dev):
        c = [torch.from_numpy(x).to(dev) for x in coords]
        p = [torch.from_numpy(x).to(dev) for x in pts]
        m = torch.from_numpy(masses).to(dev)
        out = torch.empty(max(n_obs, 1), dtype=torch.float64, device=dev)
        ws = _native.ctypes.c_size_t(0)
        _native.check(lib.hg_point_forward_workspace(n_obs, masses.size,
                                                     _native.ctypes.byref(ws)))
        work = None
        if ws.value:
            work = torch.empty((ws.value + 7) // 8, dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        _native.check(lib.hg_point_forward(
            _ptr(c[0]), _ptr(c[1]), _ptr(c[2]), n_obs, _ptr(p[0]), _ptr(p[1]), _ptr(p[2]),
            _ptr(m), masses.size, int(coordinate_system == "spherical"), code, _ptr(out),
            _ptr(work), ws.value, stream))
        result = out[:n_obs].cpu().numpy()
    return result.astype(dtype).reshape(cast.shape)
