"""
Drop-in replacement for ``harmonica.dipole_magnetic`` running on a GB300.

Mirrors ``src/harmonica/_forward/dipole.py:23-290`` (harmonica): fields
``b`` (the three components), ``b_e``, ``b_n``, ``b_u`` in nT, the checks
and messages of the field name and of the dipoles and magnetic moments.
The all-pairs sum runs in the CUDA library (``hg_dipole_magnetic``).
``parallel`` and ``progressbar`` are accepted for compatibility.
"""

import numpy as np

from . import _native

VALID_FIELDS = ("b", "b_e", "b_n", "b_u")
_COMPONENT = {"b_e": 0, "b_n": 1, "b_u": 2, "b": 3}

__all__ = ["dipole_magnetic"]


def _check_dipoles_and_magnetic_moments(dipoles, magnetic_moments):
    """Same checks and messages as dipole.py:274-289."""
    if (size := len(magnetic_moments)) != 3:
        msg = (
            f"Invalid magnetic moments with '{size}' elements."
            " Magnetic moments vectors should have 3 components."
        )
        raise ValueError(msg)
    if magnetic_moments[0].size != dipoles[0].size:
        msg = (
            f"Number of elements in magnetic_moments ({magnetic_moments[0].size})"
            f" mismatch the number of dipoles ({dipoles[0].size})."
        )
        raise ValueError(msg)


def dipole_magnetic(coordinates, dipoles, magnetic_moments, field, parallel=True,
                    dtype="float64", progressbar=False, disable_checks=False, device=None):
    """
    Magnetic field of dipoles (``harmonica.dipole_magnetic``): ``coordinates``
    and ``dipoles`` are (easting, northing, upward) in m, ``magnetic_moments``
    the (m_e, m_n, m_u) moments in A m^2.  Returns nT: one array of the
    coordinates' shape, or a tuple of three for ``field="b"``.
    """
    import torch  # noqa: PLC0415

    from .gravity import _device, _ptr  # noqa: PLC0415

    if field not in VALID_FIELDS:
        msg = (
            f"Invalid field '{field}'. "
            f"Please choose one of '{', '.join(VALID_FIELDS)}'."
        )
        raise ValueError(msg)
    cast = np.broadcast(*coordinates[:3])
    coords = tuple(np.array(np.broadcast_to(np.asarray(c, dtype=np.float64), cast.shape)).ravel()
                   for c in coordinates[:3])
    dipoles = tuple(np.atleast_1d(np.asarray(d, dtype=np.float64)).ravel() for d in dipoles[:3])
    magnetic_moments = tuple(np.atleast_1d(np.asarray(m, dtype=np.float64)).ravel()
                             for m in magnetic_moments)
    if not disable_checks:
        _check_dipoles_and_magnetic_moments(dipoles, magnetic_moments)
    # the kernels read three moment components per dipole whatever the checks
    if len(magnetic_moments) != 3 or any(m.size != dipoles[0].size for m in magnetic_moments):
        raise ValueError("magnetic_moments must hold 3 components of one value per dipole")
    if not dipoles[0].size == dipoles[1].size == dipoles[2].size:
        raise ValueError(
            "The coordinates of the dipoles must have the same number of elements "
            f"({dipoles[0].size}, {dipoles[1].size}, {dipoles[2].size})"
        )
    comp = _COMPONENT[field]
    rows = 3 if comp == 3 else 1
    n_obs, n_dip = coords[0].size, dipoles[0].size
    lib = _native.lib()
    dev = _device(device)
    with torch.cuda.device(dev):
        T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
        c = [T(x) for x in coords]
        d = [T(x) for x in dipoles]
        m = [T(x) for x in magnetic_moments]
        out = torch.empty((rows, max(n_obs, 1)), dtype=torch.float64, device=dev)
        ws = _native.ctypes.c_size_t(0)
        _native.check(lib.hg_dipole_workspace(n_obs, n_dip, comp, _native.ctypes.byref(ws)))
        work = torch.empty(max(1, (ws.value + 7) // 8), dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        _native.check(lib.hg_dipole_magnetic(
            _ptr(c[0]), _ptr(c[1]), _ptr(c[2]), n_obs, _ptr(d[0]), _ptr(d[1]), _ptr(d[2]),
            _ptr(m[0]), _ptr(m[1]), _ptr(m[2]), n_dip, comp, _ptr(out),
            _ptr(work) if ws.value else None, ws.value, stream))
        result = out[:, :n_obs].cpu().numpy().astype(dtype)
    if comp == 3:
        return tuple(result[k].reshape(cast.shape) for k in range(3))
    return result[0].reshape(cast.shape)
