"""Image deformation and the differentiable deform-and-correlate chain.

The reference measures each pass after the first with integer window shifts and
leaves the deformation of im1 as a to-do (works/piv/singlepass.py:736-738).  This
module provides, on device:

* ``warp(nodes, xn, yn, im1)``: im1 deformed by a displacement field given on nodes
  (bilinear in the field and in the image): ``im1w(x) = im1(x + d(x))``;
* ``DeformCorrelate``: a ``torch.autograd.Function`` mapping the node field to the
  residual displacement ``r`` of every non-overlapping 32 x 32 window, read out by a
  soft-argmax (temperature ``T``) from the normalised correlation plane of the
  window of im0 and the window of the deformed im1 (the plane of
  CorrelFFTNumpy.__call__, calcul/correl.py:671-685, over its norm).  Its backward
  pass is hand-written (``fi_dc_windows_backward``, ``fi_dc_warp_backward``): it
  recomputes the planes instead of storing them and returns the gradients with
  respect to the nodes and to the pixels of im1;
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


def warp(nodes, xn, yn, im1, stream=None):
    """im1 [batch, H, W] (uint8, uint16 as int16, float32) deformed by the node field:
    float32 [batch, H, W]."""
    import torch

    _check_nodes(nodes, xn, yn, im1)
    im1 = im1.contiguous()
    out = torch.empty(im1.shape, dtype=torch.float32, device=im1.device)
    B, H, W = im1.shape
    L.check(L.load().fi_dc_warp(L.ptr(nodes), L.ptr(xn), xn.numel(), L.ptr(yn), yn.numel(),
                                L.ptr(im1), _dtype_code(im1), B, H, W, L.ptr(out),
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
    """``apply(nodes, im0, im1, xn, yn, temperature) -> r`` (see the module doc);
    differentiable with respect to ``nodes`` and ``im1`` (float32)."""

    _fn = None

    @classmethod
    def function(cls):
        if cls._fn is None:
            import torch

            class _F(torch.autograd.Function):
                @staticmethod
                def forward(ctx, nodes, im0, im1, xn, yn, temperature):
                    im0 = im0.contiguous()
                    im1c = im1.contiguous()
                    im1w = warp(nodes, xn, yn, im1c)
                    r, _, _ = windows(im0, im1w, temperature)
                    ctx.save_for_backward(nodes, im0, im1c, xn, yn, im1w)
                    ctx.temperature = float(temperature)
                    return r

                @staticmethod
                def backward(ctx, grad_r):
                    nodes, im0, im1, xn, yn, im1w = ctx.saved_tensors
                    lib = L.load()
                    B, H, W = im0.shape
                    s = L.stream_handle()
                    grad_r = grad_r.contiguous().float()
                    g_w = torch.zeros_like(im1w)
                    L.check(lib.fi_dc_windows_backward(L.ptr(im0), L.ptr(im1w), B, H, W,
                                                       ctx.temperature, L.ptr(grad_r),
                                                       L.ptr(g_w), s),
                            "fi_dc_windows_backward")
                    g_nodes = torch.zeros_like(nodes)
                    want_im1 = ctx.needs_input_grad[2]
                    if want_im1 and im1.dtype != torch.float32:
                        raise TypeError("the gradient with respect to im1 needs a float32 im1")
                    g_im1 = torch.zeros_like(im1) if want_im1 else None
                    L.check(lib.fi_dc_warp_backward(L.ptr(nodes), L.ptr(xn), xn.numel(),
                                                    L.ptr(yn), yn.numel(), L.ptr(im1),
                                                    _dtype_code(im1), B, H, W, L.ptr(g_w),
                                                    L.ptr(g_nodes), L.ptr(g_im1), s),
                            "fi_dc_warp_backward")
                    return g_nodes, None, g_im1, None, None, None

            cls._fn = _F
        return cls._fn

    @classmethod
    def apply(cls, nodes, im0, im1, xn, yn, temperature=0.1):
        _check_nodes(nodes, xn, yn, im1)
        return cls.function().apply(nodes, im0, im1, xn, yn, temperature)


def node_grid(height, width, spacing=WINDOW):
    """Node coordinates at the centres of the non-overlapping windows:
    ``spacing / 2 + spacing k``, as float32 numpy arrays (xn, yn)."""
    xn = (spacing / 2.0 + spacing * np.arange(width // spacing)).astype(np.float32)
    yn = (spacing / 2.0 + spacing * np.arange(height // spacing)).astype(np.float32)
    return xn, yn


def refine(nodes, im0, im1, xn, yn, steps=20, lr=0.05, temperature=0.1, history=False):
    """Adam on the node field, minimising the mean squared soft-argmax residual of the
    windows; returns the refined nodes (and the loss per step when ``history``)."""
    import torch

    p = nodes.detach().clone().requires_grad_(True)
    opt = torch.optim.Adam([p], lr=lr)
    losses = []
    for _ in range(steps):
        opt.zero_grad(set_to_none=True)
        r = DeformCorrelate.apply(p, im0, im1, xn, yn, temperature)
        loss = (r * r).sum(dim=-1).mean()
        loss.backward()
        opt.step()
        if history:
            losses.append(float(loss.detach()))
    out = p.detach()
    return (out, losses) if history else out
