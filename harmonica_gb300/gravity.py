"""
Drop-in replacement for ``harmonica.prism_gravity`` running on a GB300.

Mirrors ``src/harmonica/_forward/prisms/gravity.py:51-236`` (harmonica):
same signature, same ``ValueError`` messages, same ``UserWarning`` for
observation points on singular points, same units (potential J/kg,
accelerations mGal, tensor Eotvos) and signs (``g_z`` downward).  The
all-pairs sum runs in the CUDA library through the C ABI
``hg_prism_forward``; PyTorch only provides device memory and the stream.

Differences that do not change results:

* ``parallel`` is accepted and ignored: the sum always runs on the GPU.
* ``progressbar=True`` prints a plain progress line on stderr (per chunk of
  observation points) instead of requiring ``numba_progress``.
* Sums are accumulated in float64 and cast to ``dtype`` at the end, where the
  reference accumulates in ``dtype``.
* Null prisms (``gravity.py:452-486``) are skipped inside the kernel and the
  singular-point scan (``gravity.py:239-269``) is fused into the same launch.
"""

import sys
import warnings

import numpy as np

from . import _native
from ._trace import stage
from .fields import FIELD_CODES, FIELDS, TENSOR_FIELDS, field_mask


def check_prisms(prisms):
    """
    Check that prism boundaries are well defined (west <= east, south <= north,
    bottom <= top).  Same checks and messages as harmonica
    ``src/harmonica/_forward/prisms/utils.py:12-43``.
    """
    west, east, south, north, bottom, top = tuple(prisms[:, i] for i in range(6))
    err_msg = "Invalid prism or prisms. "
    bad_we = west > east
    bad_sn = south > north
    bad_bt = bottom > top
    if bad_we.any():
        err_msg += "The west boundary can't be greater than the east one.\n"
        for prism in prisms[bad_we]:
            err_msg += f"\tInvalid prism: {prism}\n"
        raise ValueError(err_msg)
    if bad_sn.any():
        err_msg += "The south boundary can't be greater than the north one.\n"
        for prism in prisms[bad_sn]:
            err_msg += f"\tInvalid prism: {prism}\n"
        raise ValueError(err_msg)
    if bad_bt.any():
        err_msg += "The bottom boundary can't be greater than the top one.\n"
        for prism in prisms[bad_bt]:
            # the reference's message says "tesseroid" here (utils.py:42)
            err_msg += f"\tInvalid tesseroid: {prism}\n"
        raise ValueError(err_msg)


def _torch():
    import torch  # noqa: PLC0415

    return torch


def _device(device):
    torch = _torch()
    if device is None:
        if not torch.cuda.is_available():
            raise RuntimeError(
                "harmonica_gb300 needs a CUDA GPU (sm_103a); none is available"
            )
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device(device)


def _ptr(t):
    return t.data_ptr() if t is not None else None


def forward_on_device(easting, northing, upward, prisms_soa, n_prisms, mask, check_singular=True):
    """
    Run the all-pairs forward on device tensors (current stream).

    ``easting``, ``northing``, ``upward``: contiguous float64 CUDA tensors of
    one length N; ``prisms_soa``: float64 (7, stride) CUDA tensor as written
    by :func:`pack_prisms`.  Returns ``(out, flag)`` with ``out`` of shape
    (n_fields, N) and ``flag`` a one-element int32 tensor (1 if a singular
    point was met for a requested tensor field).
    """
    torch = _torch()
    _check_device_arrays(easting=easting, northing=northing, upward=upward)
    if not easting.numel() == northing.numel() == upward.numel():
        raise ValueError("The coordinates of the observation points must have the same "
                         "number of elements.")
    if n_prisms and (prisms_soa is None or prisms_soa.dim() != 2 or prisms_soa.shape[0] != 7
                     or prisms_soa.shape[1] < n_prisms):
        raise ValueError(f"prisms_soa must be a (7, >= {n_prisms}) tensor from pack_prisms")
    lib = _native.lib()
    n_obs = easting.numel()
    n_rows = bin(mask).count("1")
    dev = easting.device
    out = torch.empty((n_rows, n_obs), dtype=torch.float64, device=dev)
    flag = torch.zeros(1, dtype=torch.int32, device=dev)
    ws_bytes = _native.ctypes.c_size_t(0)
    _native.check(
        lib.hg_prism_forward_workspace(n_obs, n_prisms, mask, _native.ctypes.byref(ws_bytes))
    )
    ws = None
    if ws_bytes.value:
        ws = torch.empty((ws_bytes.value + 7) // 8, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    _native.check(
        lib.hg_prism_forward(
            _ptr(easting), _ptr(northing), _ptr(upward), n_obs, _ptr(prisms_soa),
            prisms_soa.shape[1] if prisms_soa is not None else 0, n_prisms, mask, _ptr(out),
            _ptr(flag) if check_singular else None, _ptr(ws), ws_bytes.value, stream,
        )
    )
    return out, flag


def _check_device_arrays(**tensors):
    """Float64 and contiguous: the kernels read the raw buffers as packed
    doubles."""
    torch = _torch()
    for name, t in tensors.items():
        if t.dtype != torch.float64 or not t.is_contiguous():
            raise ValueError(f"'{name}' must be a contiguous float64 tensor "
                             f"(got {t.dtype}, contiguous={t.is_contiguous()})")


def pack_prisms(prisms, density):
    """Pack (M, 6) prisms and (M,) densities (CUDA float64) into a (7, M) SoA tensor."""
    torch = _torch()
    _check_device_arrays(prisms=prisms, density=density)
    if prisms.dim() != 2 or prisms.shape[1] != 6 or density.numel() != prisms.shape[0]:
        raise ValueError(
            f"pack_prisms needs (M, 6) prisms and M densities, got {tuple(prisms.shape)} "
            f"and {density.numel()}"
        )
    lib = _native.lib()
    m = prisms.shape[0]
    soa = torch.empty((7, max(m, 1)), dtype=torch.float64, device=prisms.device)
    if m:
        stream = torch.cuda.current_stream(prisms.device).cuda_stream
        _native.check(
            lib.hg_pack_prisms(_ptr(prisms), _ptr(density), m, _ptr(soa), soa.shape[1], stream)
        )
    return soa


def _prepare(coordinates, prisms, density, disable_checks):
    cast = np.broadcast(*coordinates[:3])
    coords = tuple(
        np.array(np.broadcast_to(np.asarray(c, dtype=np.float64), cast.shape)).ravel()
        for c in coordinates[:3]
    )
    prisms = np.atleast_2d(np.asarray(prisms, dtype=np.float64))
    density = np.atleast_1d(np.asarray(density, dtype=np.float64)).ravel()
    # the array sizes are checked even with disable_checks: the kernels read
    # six boundaries and one density per prism, and a short array would be
    # read past its end on the device
    check_sizes(prisms, density)
    if not disable_checks:
        check_prisms(prisms)
    return cast, coords, prisms, density


def check_sizes(prisms, density, name="density"):
    """Six boundaries per prism and one ``name`` value per prism
    (``ValueError`` otherwise, with the reference's message for the count)."""
    if prisms.ndim != 2 or prisms.shape[1] != 6:
        raise ValueError(
            f"Invalid prisms array with shape {prisms.shape}: each prism needs its six "
            "boundaries [west, east, south, north, bottom, top]."
        )
    if density.size != prisms.shape[0]:
        raise ValueError(
            f"Number of elements in {name} ({density.size}) "
            + f"mismatch the number of prisms ({prisms.shape[0]})"
        )


class _Progress:
    """Plain stderr progress line, updated per chunk of observation points."""

    def __init__(self, total, enabled):
        self.total = total
        self.done = 0
        self.enabled = enabled

    def update(self, n):
        self.done += n
        if self.enabled:
            pct = 100.0 * self.done / max(self.total, 1)
            sys.stderr.write(f"\rprism_gravity: {self.done}/{self.total} points ({pct:5.1f}%)")
            if self.done >= self.total:
                sys.stderr.write("\n")
            sys.stderr.flush()


def _run_host(coords, prisms, density, mask, check_singular, device, progressbar):
    torch = _torch()
    dev = _device(device)
    n_obs = coords[0].size
    with torch.cuda.device(dev):
        with stage("upload prisms"):
            pr = torch.from_numpy(np.ascontiguousarray(prisms)).to(dev)
            rho = torch.from_numpy(np.ascontiguousarray(density)).to(dev)
            soa = pack_prisms(pr, rho)
        n_rows = bin(mask).count("1")
        result = np.empty((n_rows, n_obs), dtype=np.float64)
        flagged = False
        n_chunks = 20 if (progressbar and n_obs >= 20) else 1
        bounds = np.linspace(0, n_obs, n_chunks + 1).astype(np.int64)
        progress = _Progress(n_obs, progressbar)
        for c in range(n_chunks):
            lo, hi = int(bounds[c]), int(bounds[c + 1])
            with stage("upload points"):
                e, n, u = (torch.from_numpy(x[lo:hi]).to(dev) for x in coords)
            with stage("forward"):
                out, flag = forward_on_device(e, n, u, soa, prisms.shape[0], mask,
                                              check_singular)
            with stage("download"):
                result[:, lo:hi] = out.cpu().numpy()
                flagged |= bool(flag.item())
            progress.update(hi - lo)
    return result, flagged


def prism_gravity(
    coordinates,
    prisms,
    density,
    field,
    parallel=True,
    dtype="float64",
    progressbar=False,
    disable_checks=False,
    device=None,
):
    """
    Gravitational fields of right-rectangular prisms in Cartesian coordinates.

    Drop-in for harmonica's ``prism_gravity``
    (``src/harmonica/_forward/prisms/gravity.py:51-236``).

    Parameters
    ----------
    coordinates : list of arrays
        ``easting``, ``northing`` and ``upward`` of the observation points in
        meters (broadcastable; extra coordinates are ignored).
    prisms : list, 1d-array, or 2d-array
        Prism boundaries ``west, east, south, north, bottom, top`` in meters,
        one prism per row.
    density : list or array
        Density of each prism in kg/m^3.
    field : str
        One of ``potential``, ``g_e``, ``g_n``, ``g_z``, ``g_ee``, ``g_nn``,
        ``g_zz``, ``g_en``, ``g_ez``, ``g_nz``.
    parallel : bool
        Accepted for compatibility; the sum always runs in parallel on the GPU.
    dtype : data-type
        Data type of the returned array (sums are accumulated in float64).
    progressbar : bool
        Print progress on stderr while the points are processed in chunks.
    disable_checks : bool
        Skip the density/prism count check, the boundary check and the
        singular-point warning.
    device : torch device or None
        CUDA device to run on (default: the current one).

    Returns
    -------
    result : array
        Potential in J/kg, accelerations in mGal, tensor components in Eotvos,
        with the broadcast shape of the coordinates.
    """
    if field not in FIELD_CODES:
        raise ValueError(f"Gravitational field {field} not recognized")
    with stage("prism_gravity checks"):
        cast, coords, prisms, density = _prepare(coordinates, prisms, density, disable_checks)
    check_singular = (not disable_checks) and field in TENSOR_FIELDS
    result, flagged = _run_host(
        coords, prisms, density, field_mask([field]), check_singular, device, progressbar
    )
    if flagged:
        warnings.warn(
            "Found observation point on singular point of a prism.",
            UserWarning,
            stacklevel=2,
        )
    return result[0].astype(dtype).reshape(cast.shape)


def prism_gravity_fields(
    coordinates, prisms, density, fields=FIELDS, dtype="float64", disable_checks=False,
    device=None,
):
    """
    Several fields of the same prisms and points in one fused forward.

    Returns a dict ``{field: array}``; every array equals what
    :func:`prism_gravity` returns for that field.  The edge logarithms and
    face angles of each (point, prism) pair are computed once and shared by
    all requested fields: the logarithms in one launch, the angles in a
    second that adds its terms to the first's sums.
    """
    for f in fields:
        if f not in FIELD_CODES:
            raise ValueError(f"Gravitational field {f} not recognized")
    cast, coords, prisms, density = _prepare(coordinates, prisms, density, disable_checks)
    mask = field_mask(fields)
    check_singular = (not disable_checks) and any(f in TENSOR_FIELDS for f in fields)
    result, flagged = _run_host(coords, prisms, density, mask, check_singular, device, False)
    if flagged:
        warnings.warn(
            "Found observation point on singular point of a prism.",
            UserWarning,
            stacklevel=2,
        )
    ordered = [f for f in FIELDS if (mask >> FIELD_CODES[f]) & 1]
    return {f: result[r].astype(dtype).reshape(cast.shape) for r, f in enumerate(ordered)}
