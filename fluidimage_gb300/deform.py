"""Image deformation and the differentiable deform-and-correlate chain.

The reference measures each pass after the first with integer window shifts and
leaves the deformation of im1 as a to-do (works/piv/singlepass.py:736-738).  This
module provides, on device:

* ``warp(nodes, xn, yn, im, scale)``: an image deformed by a displacement field
  given on nodes (bilinear in the field and in the image):
  ``imw(x) = im(x + scale d(x))``;
* ``DeformCorrelate``: a ``torch.autograd.Function`` mapping the node field to the
  residual displacement ``r`` of every non-overlapping 32 x 32 window, read out by a
  soft-argmax (temperature ``T``) from the normalised correlation plane of the
  deformed windows (the plane of CorrelFFTNumpy.__call__, calcul/correl.py:671-685,
  over its norm).  Central scheme (default): im0 deformed by -d/2 and im1 by +d/2,
  so that a window's displacement belongs to its centre; ``symmetric=False``
  deforms im1 by d only (the measured displacement then belongs to the point half
  a displacement downstream).  Its backward pass is hand-written
  (``fi_dc_windows_backward``, ``fi_dc_warp_backward``): it recomputes the planes
  instead of storing them and returns the gradients with respect to the nodes and
  to the pixels of im1;
* ``refine``: Adam steps on the node field minimising the mean squared soft-argmax
  residual ``mean |r|^2`` (zero when every window's correlation peak sits at lag 0).

Field convention: ``nodes`` is [batch, 2, ny, nx] (u then v) at coordinates ``xn``
(nx), ``yn`` (ny), both increasing; outside the outer nodes the field is constant.
"""

from __future__ import annotations

import numpy as np

from . import _lib as L

WINDOW = 32


def _dtype_code(t):
    import torch

    return {torch.uint8: L.FI_U8, torch.int16: L.FI_U16, torch.float32: L.FI_F32}[t.dtype]


def _check_nodes(nodes, xn, yn, im):
    import torch

    if nodes.dim() != 4 or nodes.shape[1] != 2:
        raise ValueError("nodes must be [batch, 2, ny, nx]")
    if nodes.dtype != torch.float32 or not nodes.is_contiguous():
        raise TypeError("nodes must be contiguous float32")
    if xn.numel() != nodes.shape[3] or yn.numel() != nodes.shape[2]:
        raise ValueError("node coordinates do not match the node grid")
    if im.dim() != 3 or im.shape[0] != nodes.shape[0]:
        raise ValueError("images must be [batch, height, width] with the field's batch")


def warp(nodes, xn, yn, im, scale=1.0, stream=None):
    """im [batch, H, W] (uint8, uint16 as int16, float32) deformed by ``scale`` times
    the node field: float32 [batch, H, W]."""
    import torch

    _check_nodes(nodes, xn, yn, im)
    im = im.contiguous()
    out = torch.empty(im.shape, dtype=torch.float32, device=im.device)
    B, H, W = im.shape
    L.check(L.load().fi_dc_warp(L.ptr(nodes), L.ptr(xn), xn.numel(), L.ptr(yn), yn.numel(),
                                float(scale), L.ptr(im), _dtype_code(im), B, H, W, L.ptr(out),
                                L.stream_handle(stream)), "fi_dc_warp")
    return out


def windows(im0, im1w, temperature, stream=None):
    """Soft-argmax residual r [batch, H/32, W/32, 2] (x, y) of every 32 x 32 window,
    with the normalised correlation at lag 0 and its maximum."""
    import torch

    B, H, W = im0.shape
    nwy, nwx = H // WINDOW, W // WINDOW
    r = torch.empty((B, nwy, nwx, 2), dtype=torch.float32, device=im0.device)
    cz = torch.empty((B, nwy, nwx), dtype=torch.float32, device=im0.device)
    cpk = torch.empty_like(cz)
    L.check(L.load().fi_dc_windows(L.ptr(im0), L.ptr(im1w), B, H, W, float(temperature),
                                   L.ptr(r), L.ptr(cz), L.ptr(cpk), L.stream_handle(stream)),
            "fi_dc_windows")
    return r, cz, cpk


class DeformCorrelate:
    """``apply(nodes, im0, im1, xn, yn, temperature, symmetric) -> r`` (see the module
    doc); differentiable with respect to ``nodes`` and ``im1`` (float32)."""

    _fn = None

    @classmethod
    def function(cls):
        if cls._fn is None:
            import torch

            class _F(torch.autograd.Function):
                @staticmethod
                def forward(ctx, nodes, im0, im1, xn, yn, temperature, symmetric):
                    im0c = im0.contiguous()
                    im1c = im1.contiguous()
                    s1 = 0.5 if symmetric else 1.0
                    im0w = warp(nodes, xn, yn, im0c, -0.5) if symmetric else im0c.float()
                    im1w = warp(nodes, xn, yn, im1c, s1)
                    r, _, _ = windows(im0w, im1w, temperature)
                    ctx.save_for_backward(nodes, im0c, im1c, xn, yn, im0w, im1w)
                    ctx.temperature = float(temperature)
                    ctx.symmetric = bool(symmetric)
                    return r

                @staticmethod
                def backward(ctx, grad_r):
                    nodes, im0, im1, xn, yn, im0w, im1w = ctx.saved_tensors
                    lib = L.load()
                    B, H, W = im0.shape
                    s = L.stream_handle()
                    grad_r = grad_r.contiguous().float()
                    g_w1 = torch.zeros_like(im1w)
                    g_w0 = torch.zeros_like(im0w) if ctx.symmetric else None
                    L.check(lib.fi_dc_windows_backward(L.ptr(im0w), L.ptr(im1w), B, H, W,
                                                       ctx.temperature, L.ptr(grad_r),
                                                       L.ptr(g_w1), L.ptr(g_w0), s),
                            "fi_dc_windows_backward")
                    g_nodes = torch.zeros_like(nodes)
                    want_im1 = ctx.needs_input_grad[2]
                    if want_im1 and im1.dtype != torch.float32:
                        raise TypeError("the gradient with respect to im1 needs a float32 im1")
                    g_im1 = torch.zeros_like(im1) if want_im1 else None
                    s1 = 0.5 if ctx.symmetric else 1.0
                    L.check(lib.fi_dc_warp_backward(L.ptr(nodes), L.ptr(xn), xn.numel(),
                                                    L.ptr(yn), yn.numel(), s1, L.ptr(im1),
                                                    _dtype_code(im1), B, H, W, L.ptr(g_w1),
                                                    L.ptr(g_nodes), L.ptr(g_im1), s),
                            "fi_dc_warp_backward")
                    if ctx.symmetric:
                        L.check(lib.fi_dc_warp_backward(L.ptr(nodes), L.ptr(xn), xn.numel(),
                                                        L.ptr(yn), yn.numel(), -0.5, L.ptr(im0),
                                                        _dtype_code(im0), B, H, W, L.ptr(g_w0),
                                                        L.ptr(g_nodes), None, s),
                                "fi_dc_warp_backward")
                    return g_nodes, None, g_im1, None, None, None, None

            cls._fn = _F
        return cls._fn

    @classmethod
    def apply(cls, nodes, im0, im1, xn, yn, temperature=0.1, symmetric=True):
        _check_nodes(nodes, xn, yn, im1)
        return cls.function().apply(nodes, im0, im1, xn, yn, temperature, symmetric)


def node_grid(height, width, spacing=WINDOW):
    """Node coordinates at the centres of the non-overlapping windows:
    ``spacing / 2 + spacing k``, as float32 numpy arrays (xn, yn)."""
    xn = (spacing / 2.0 + spacing * np.arange(width // spacing)).astype(np.float32)
    yn = (spacing / 2.0 + spacing * np.arange(height // spacing)).astype(np.float32)
    return xn, yn


def refine(nodes, im0, im1, xn, yn, steps=20, lr=0.05, temperature=0.1, history=False,
           symmetric=True):
    """Adam on the node field, minimising the mean squared soft-argmax residual of the
    windows; returns the refined nodes (and the loss per step when ``history``)."""
    import torch

    p = nodes.detach().clone().requires_grad_(True)
    opt = torch.optim.Adam([p], lr=lr)
    losses = []
    for _ in range(steps):
        opt.zero_grad(set_to_none=True)
        r = DeformCorrelate.apply(p, im0, im1, xn, yn, temperature, symmetric)
        loss = (r * r).sum(dim=-1).mean()
        loss.backward()
        opt.step()
        if history:
            losses.append(float(loss.detach()))
    out = p.detach()
    return (out, losses) if history else out
