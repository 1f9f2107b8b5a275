"""Differentiable 2D conservative regridding (``torch.autograd``).

``regrid_conservative_2d(values, grid_input, grid_output)`` builds the
conservative weights of the two vertex grids on the GPU and applies them;
its backward pass gives

* the gradient with respect to ``values``: the transposed weights applied to
  the output gradient (``rg_apply_transpose``; equal to
  ``transpose_weights_conservative()`` applied to ``grad * vol_out`` and
  divided by ``vol_in``),
* the gradient with respect to the output-grid vertex coordinates: the
  adjoint of the overlap areas (``rg_conservative_2d_grad_output``), which
  needs convex input cells.

The input grid and ``weights_input`` are constants.  Float64 values give the
upstream float64 result bit for bit in the forward pass; float32 values use
the float32 fast apply.  The upstream has no differentiable path; the
forward pass is ``regrid(method="conservative", perturb=False)`` of
regridding/_regrid/_regrid.py:12-149 for 2D grids.
"""

from __future__ import annotations

import ctypes

from . import _device, _lib

__all__ = ["regrid_conservative_2d"]


def _function():
    torch = _device.torch()

    class ConservativeRegrid2d(torch.autograd.Function):
        @staticmethod
        def forward(ctx, values, xo, yo, xi, yi, w_in):
            dw = _device.build_conservative_2d((xi, yi), (xo.detach(), yo.detach()), w_in)
            exact = values.dtype == torch.float64
            out = dw.apply(values, accumulate="exact" if exact else "fast")
            ctx.dw = dw
            ctx.exact = exact
            ctx.save_for_backward(values, xo.detach(), yo.detach(), xi, yi, w_in)
            return out

        @staticmethod
        def backward(ctx, grad):
            values, xo, yo, xi, yi, w_in = ctx.saved_tensors
            dw = ctx.dw
            grad = grad.contiguous().to(values.dtype)
            g_values = g_xo = g_yo = None
            if ctx.needs_input_grad[0]:
                g_values = dw.apply(grad, transpose=True, accumulate="exact" if ctx.exact else "fast")
            if ctx.needs_input_grad[1] or ctx.needs_input_grad[2]:
                g_xo = torch.empty_like(xo)
                g_yo = torch.empty_like(yo)
                dtype = _lib.RG_F64 if values.dtype == torch.float64 else _lib.RG_F32
                _lib.call("rg_conservative_2d_grad_output", dw.handle, _device.ptr(xi), _device.ptr(yi),
                          xi.shape[0], xi.shape[1], _device.ptr(xo), _device.ptr(yo), xo.shape[0], xo.shape[1],
                          _device.ptr(w_in), _device.ptr(values), _device.ptr(grad), dtype, values.shape[0],
                          _device.ptr(g_xo), _device.ptr(g_yo), None, _device.stream())
            return g_values, g_xo, g_yo, None, None, None

    return ConservativeRegrid2d


_FN = None


def regrid_conservative_2d(values, grid_input, grid_output, weights_input=None):
    """Conservative regrid of ``values`` (``(..., nxi - 1, nyi - 1)``, CUDA,
    float32 or float64) from the vertex grid ``grid_input = (xi, yi)``
    (``(nxi, nyi)`` each) to ``grid_output = (xo, yo)`` (``(nxo, nyo)``),
    differentiable with respect to ``values`` and the output coordinates.
    Returns ``(..., nxo - 1, nyo - 1)`` in the dtype of ``values``."""
    global _FN
    torch = _device.torch()
    if _FN is None:
        _FN = _function()
    xi, yi = (torch.as_tensor(a, device="cuda").detach().to(torch.float64).contiguous() for a in grid_input)
    xo, yo = (torch.as_tensor(a, device="cuda").to(torch.float64).contiguous() for a in grid_output)
    if xi.dim() != 2 or xo.dim() != 2 or xi.shape != yi.shape or xo.shape != yo.shape:
        raise ValueError("grid_input and grid_output must each be two 2D vertex arrays of one shape")
    nci = (xi.shape[0] - 1) * (xi.shape[1] - 1)
    v = torch.as_tensor(values, device="cuda")
    if v.dtype not in (torch.float32, torch.float64):
        v = v.to(torch.float64)
    if tuple(v.shape[-2:]) != (xi.shape[0] - 1, xi.shape[1] - 1):
        raise ValueError(f"values end in {tuple(v.shape[-2:])}, the input grid has "
                         f"{(xi.shape[0] - 1, xi.shape[1] - 1)} cells")
    lead = v.shape[:-2]
    w_in = None
    if weights_input is not None:
        w_in = torch.as_tensor(weights_input, device="cuda").detach().to(torch.float64)
        w_in = torch.broadcast_to(w_in, (xi.shape[0] - 1, xi.shape[1] - 1)).contiguous()
    out = _FN.apply(v.reshape(-1, nci).contiguous(), xo, yo, xi, yi, w_in)
    return out.reshape(*lead, xo.shape[0] - 1, xo.shape[1] - 1)


def grad_output_check(dw, grid_input, grid_output, weights_input=None):
    """The weights of every stored entry of ``dw`` (CSR order) recomputed
    from the overlap polygons the adjoint uses; for tests of its geometry."""
    torch = _device.torch()
    xi, yi = (torch.as_tensor(a, device="cuda").to(torch.float64).contiguous() for a in grid_input)
    xo, yo = (torch.as_tensor(a, device="cuda").to(torch.float64).contiguous() for a in grid_output)
    w_in = None if weights_input is None else torch.as_tensor(weights_input, device="cuda").to(
        torch.float64).contiguous()
    gx, gy = torch.empty_like(xo), torch.empty_like(yo)
    check = torch.empty(dw.nnz, dtype=torch.float64, device="cuda")
    z_in = torch.zeros((1, dw.n_in), dtype=torch.float64, device="cuda")
    z_out = torch.zeros((1, dw.n_out), dtype=torch.float64, device="cuda")
    _lib.call("rg_conservative_2d_grad_output", dw.handle, _device.ptr(xi), _device.ptr(yi), xi.shape[0],
              xi.shape[1], _device.ptr(xo), _device.ptr(yo), xo.shape[0], xo.shape[1], _device.ptr(w_in),
              _device.ptr(z_in), _device.ptr(z_out), _lib.RG_F64, 1, _device.ptr(gx), _device.ptr(gy),
              ctypes.c_void_p(check.data_ptr()), _device.stream())
    return check
