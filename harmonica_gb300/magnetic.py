"""
Drop-in replacement for ``harmonica.prism_magnetic`` running on a GB300.

Mirrors ``src/harmonica/_forward/prisms/magnetic.py:28-136`` (harmonica):
same signature, field names (``b``, ``b_e``, ``b_n``, ``b_u``), errors and
units (nT); ``field="b"`` returns the tuple ``(b_e, b_n, b_u)``.  The sum runs
in ``hg_prism_magnetic`` (b = mu0/(4 pi) T M with the gradient-tensor kernel
of the prism gravity formulation).
"""

import numpy as np

from . import _native
from .gravity import check_prisms, check_sizes

VALID_FIELDS = ("b", "b_e", "b_n", "b_u")
_COMPONENT = {"b_e": 0, "b_n": 1, "b_u": 2, "b": 3}


def prism_magnetic(coordinates, prisms, magnetization, field, parallel=True, dtype=np.float64,
                   progressbar=False, disable_checks=False, device=None):
    """
    Magnetic field of right-rectangular prisms in Cartesian coordinates (nT).

    ``magnetization`` is a tuple ``(m_e, m_n, m_u)`` of arrays (A/m), one
    value per prism.  ``parallel`` and ``progressbar`` are accepted for
    compatibility.
    """
    import torch

    from .gravity import _device, _ptr

    if field not in VALID_FIELDS:
        msg = f"Invalid field '{field}'. Please choose one of '{','.join(VALID_FIELDS)}'."
        raise ValueError(msg)
    cast = np.broadcast(*coordinates[:3])
    coords = tuple(np.array(np.broadcast_to(np.asarray(c, dtype=np.float64), cast.shape)).ravel()
                   for c in coordinates[:3])
    prisms = np.atleast_2d(np.asarray(prisms, dtype=np.float64))
    mag = tuple(np.atleast_1d(np.asarray(m, dtype=np.float64)).ravel() for m in magnetization)
    # the sizes are checked even with disable_checks: the kernels read six
    # boundaries and three magnetization components per prism, and a short
    # array would be read past its end on the device
    if (size := len(mag)) != 3:
        raise ValueError(
            f"Invalid magnetization vectors with '{size}' elements. "
            + "Magnetization vectors should have only 3 elements."
        )
    for component in mag:
        if component.size != prisms.shape[0]:
            raise ValueError(
                f"Number of magnetization vectors ({component.size}) "
                + f"mismatch the number of prisms ({prisms.shape[0]})"
            )
    check_sizes(prisms, mag[0], name="magnetization")
    if not disable_checks:
        check_prisms(prisms)
    comp = _COMPONENT[field]
    rows = 3 if comp == 3 else 1
    lib = _native.lib()
    dev = _device(device)
    n_obs = coords[0].size
    m = prisms.shape[0]
    with torch.cuda.device(dev):
        c = [torch.from_numpy(x).to(dev) for x in coords]
        aos = torch.from_numpy(np.ascontiguousarray(prisms)).to(dev)
        mt = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in mag[:3]]
        soa = torch.empty((9, max(m, 1)), dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        if m:
            _native.check(lib.hg_pack_prisms_magnetic(_ptr(aos), _ptr(mt[0]), _ptr(mt[1]),
                                                      _ptr(mt[2]), m, _ptr(soa), soa.shape[1],
                                                      stream))
        out = torch.empty((rows, max(n_obs, 1)), dtype=torch.float64, device=dev)
        ws = _native.ctypes.c_size_t(0)
        _native.check(lib.hg_prism_magnetic_workspace(n_obs, m, comp, _native.ctypes.byref(ws)))
        work = None
        if ws.value:
            work = torch.empty((ws.value + 7) // 8, dtype=torch.float64, device=dev)
        _native.check(lib.hg_prism_magnetic(_ptr(c[0]), _ptr(c[1]), _ptr(c[2]), n_obs, _ptr(soa),
                                            soa.shape[1], m, comp, _ptr(out), _ptr(work),
                                            ws.value, stream))
        result = out[:, :n_obs].cpu().numpy()
    if comp == 3:
        return tuple(result[r].astype(dtype).reshape(cast.shape) for r in range(3))
    return result[0].astype(dtype).reshape(cast.shape)
