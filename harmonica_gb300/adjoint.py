"""
Differentiable prism forward: ``torch.autograd.Function`` wrappers whose
backward pass runs the hand-written adjoint kernels (``hg_layer_adjoint``,
``hg_prism_adjoint``).

* :func:`layer_gravity_torch` -- field of a regular prism layer, differentiable
  with respect to the density grid (any field) and the bottom/top grids
  (g_z), e.g. for a basement inversion step.
* :func:`prism_gravity_torch` -- field of a prism list, differentiable with
  respect to the densities (any field) and the bottoms/tops (g_z).

The forward is the same launch as :mod:`harmonica_gb300.gravity` /
:mod:`harmonica_gb300.layer` (harmonica units); the backward computes the
transpose sums ``sum_i w_i dd_i/dtheta_j`` with one thread per prism.  The
reference (harmonica) has no derivatives; its gradients would be assembled
from repeated ``prism_gravity`` calls (src/harmonica/_forward/prisms/gravity.py:51-236).
"""

import ctypes

import torch

from . import _native
from .fields import FIELD_CODES
from .gravity import _ptr, pack_prisms
from .layer import layer_forward_device


def _f64(t, dev):
    return t.to(device=dev, dtype=torch.float64).contiguous()


class _LayerGravity(torch.autograd.Function):
    @staticmethod
    def forward(ctx, density, bottom, top, e, n, u, ce, cn, field, threshold):
        out = layer_forward_device(e, n, u, ce, cn, bottom, top, density, 1 << field,
                                   threshold)[0]
        ctx.save_for_backward(density, bottom, top, e, n, u, ce, cn)
        ctx.field = field
        ctx.threshold = threshold
        return out

    @staticmethod
    def backward(ctx, grad_out):
        density, bottom, top, e, n, u, ce, cn = ctx.saved_tensors
        lib = _native.lib()
        w = grad_out.to(torch.float64).contiguous()
        need_rho, need_b, need_t = ctx.needs_input_grad[:3]
        geom = need_b or need_t
        if geom and ctx.field != FIELD_CODES["g_z"]:
            raise NotImplementedError("bottom/top gradients are available for g_z only")
        g_rho = torch.empty_like(density) if need_rho else None
        g_b = torch.empty_like(bottom) if need_b else None
        g_t = torch.empty_like(top) if need_t else None
        ws = ctypes.c_size_t(0)
        _native.check(lib.hg_layer_adjoint_workspace(e.numel(), ce.numel(), cn.numel(),
                                                     ctypes.byref(ws)))
        work = torch.empty(max(1, (ws.value + 7) // 8), dtype=torch.float64, device=e.device)
        stream = torch.cuda.current_stream(e.device).cuda_stream
        _native.check(lib.hg_layer_adjoint(
            _ptr(e), _ptr(n), _ptr(u), _ptr(w), e.numel(), _ptr(ce), ce.numel(), _ptr(cn),
            cn.numel(), _ptr(bottom), _ptr(top), _ptr(density), ctx.threshold, ctx.field,
            _ptr(g_rho), _ptr(g_b), _ptr(g_t), _ptr(work), ws.value, stream))
        return g_rho, g_b, g_t, None, None, None, None, None, None, None


def layer_gravity_torch(coordinates, easting, northing, bottom, top, density, field="g_z",
                        thickness_threshold=None):
    """
    Field of a prism layer as a differentiable torch function.

    ``coordinates``: 3 CUDA tensors (N,) of observation points; ``easting``
    (n_e,), ``northing`` (n_n,): prism centres; ``bottom``, ``top``,
    ``density``: (n_n, n_e) tensors (may require grad).  Returns an (N,)
    float64 tensor in harmonica units, the same values as
    ``layer.prism_layer.gravity``.
    """
    if field not in FIELD_CODES:
        raise ValueError(f"Gravitational field '{field}' not recognized.")
    dev = coordinates[0].device
    e, n, u = (_f64(c, dev).ravel() for c in coordinates[:3])
    ce, cn = _f64(easting, dev), _f64(northing, dev)
    threshold = 0.0 if thickness_threshold is None else float(thickness_threshold)
    return _LayerGravity.apply(_f64(density, dev), _f64(bottom, dev), _f64(top, dev), e, n, u,
                               ce, cn, FIELD_CODES[field], threshold)


class _PrismGravity(torch.autograd.Function):
    @staticmethod
    def forward(ctx, density, bottom, top, horizontal, e, n, u, field):
        from .gravity import forward_on_device

        prisms = torch.cat([horizontal, bottom[:, None], top[:, None]], dim=1).contiguous()
        soa = pack_prisms(prisms, density)
        out, _ = forward_on_device(e, n, u, soa, prisms.shape[0], 1 << field, False)
        ctx.save_for_backward(soa, e, n, u)
        ctx.field = field
        ctx.m = prisms.shape[0]
        return out[0]

    @staticmethod
    def backward(ctx, grad_out):
        soa, e, n, u = ctx.saved_tensors
        lib = _native.lib()
        w = grad_out.to(torch.float64).contiguous()
        need_rho, need_b, need_t = ctx.needs_input_grad[:3]
        if (need_b or need_t) and ctx.field != FIELD_CODES["g_z"]:
            raise NotImplementedError("bottom/top gradients are available for g_z only")
        m = ctx.m
        mk = lambda flag: torch.empty(m, dtype=torch.float64, device=e.device) if flag else None  # noqa: E731
        g_rho, g_b, g_t = mk(need_rho), mk(need_b), mk(need_t)
        ws = ctypes.c_size_t(0)
        _native.check(lib.hg_prism_adjoint_workspace(e.numel(), m, ctypes.byref(ws)))
        work = torch.empty(max(1, (ws.value + 7) // 8), dtype=torch.float64, device=e.device)
        stream = torch.cuda.current_stream(e.device).cuda_stream
        _native.check(lib.hg_prism_adjoint(
            _ptr(e), _ptr(n), _ptr(u), _ptr(w), e.numel(), _ptr(soa), soa.shape[1], m,
            ctx.field, _ptr(g_rho), _ptr(g_b), _ptr(g_t), _ptr(work), ws.value, stream))
        return g_rho, g_b, g_t, None, None, None, None, None


def prism_gravity_torch(coordinates, horizontal, bottom, top, density, field="g_z"):
    """
    Field of a prism list as a differentiable torch function.

    ``horizontal``: (M, 4) tensor of ``west, east, south, north``;
    ``bottom``, ``top``, ``density``: (M,) tensors (may require grad).
    Returns an (N,) float64 tensor equal to ``prism_gravity`` (harmonica
    units).  No boundary checks or singular-point warnings are done here.
    """
    if field not in FIELD_CODES:
        raise ValueError(f"Gravitational field {field} not recognized")
    dev = coordinates[0].device
    e, n, u = (_f64(c, dev).ravel() for c in coordinates[:3])
    return _PrismGravity.apply(_f64(density, dev), _f64(bottom, dev), _f64(top, dev),
                               _f64(horizontal, dev), e, n, u, FIELD_CODES[field])
