"""Pure-torch autograd restatement of the deform-and-correlate chain (float64):
the reference the hand-written adjoint of fluidimage_gb300.deform is checked
against, and the FP64 function differentiated by central finite differences."""

from __future__ import annotations

import torch

N = 32


def _cell(coords, v):
    n = coords.numel()
    j0 = (torch.searchsorted(coords, v, right=True) - 1).clamp(0, n - 2)
    t = ((v - coords[j0]) / (coords[j0 + 1] - coords[j0])).clamp(0.0, 1.0)
    return j0, t


def warp(nodes, xn, yn, im1, scale=1.0):
    """nodes [B, 2, ny, nx], im1 [B, H, W] -> im1 at (x + scale d) [B, H, W] (float64)."""
    B, H, W = im1.shape
    dev = im1.device
    xs = torch.arange(W, dtype=torch.float64, device=dev)
    ys = torch.arange(H, dtype=torch.float64, device=dev)
    j0, tx = _cell(xn.double(), xs)
    i0, ty = _cell(yn.double(), ys)
    comps = []
    for c in range(2):
        f = nodes[:, c]
        f00 = f[:, i0][:, :, j0]
        f01 = f[:, i0][:, :, j0 + 1]
        f10 = f[:, i0 + 1][:, :, j0]
        f11 = f[:, i0 + 1][:, :, j0 + 1]
        top = (1 - tx) * f00 + tx * f01
        bot = (1 - tx) * f10 + tx * f11
        comps.append((1 - ty)[:, None] * top + ty[:, None] * bot)
    px = (xs[None, None, :] + scale * comps[0]).clamp(-1e7, 1e7)
    py = (ys[None, :, None] + scale * comps[1]).clamp(-1e7, 1e7)
    x0 = torch.floor(px).detach()
    y0 = torch.floor(py).detach()
    fx, fy = px - x0, py - y0
    xa = x0.long().clamp(0, W - 1)
    xb = (x0.long() + 1).clamp(0, W - 1)
    ya = y0.long().clamp(0, H - 1)
    yb = (y0.long() + 1).clamp(0, H - 1)
    bi = torch.arange(B, device=dev)[:, None, None]
    top = (1 - fx) * im1[bi, ya, xa] + fx * im1[bi, ya, xb]
    bot = (1 - fx) * im1[bi, yb, xa] + fx * im1[bi, yb, xb]
    return (1 - fy) * top + fy * bot


def windows_r(im0, im1w, temperature):
    """Soft-argmax residual [B, H/32, W/32, 2] of the normalised correlation planes."""
    B, H, W = im0.shape
    nwy, nwx = H // N, W // N

    def tiles(a):
        a = a[:, :nwy * N, :nwx * N].reshape(B, nwy, N, nwx, N).permute(0, 1, 3, 2, 4)
        return a - a.mean(dim=(-1, -2), keepdim=True)

    w0, w1 = tiles(im0), tiles(im1w)
    n0 = torch.sqrt((w0 * w0).sum(dim=(-1, -2)))
    n1 = torch.sqrt((w1 * w1).sum(dim=(-1, -2)))
    u = torch.fft.ifft2(torch.conj(torch.fft.fft2(w0)) * torch.fft.fft2(w1)).real
    c = u / (n0 * n1)[..., None, None]
    m = torch.arange(N, device=im0.device)
    tau = torch.where(m < 16, m, m - 32).to(torch.float64)
    valid = m != 16
    mask = valid[:, None] & valid[None, :]
    cm = c.masked_fill(~mask, float("-inf"))
    p = torch.softmax(cm.flatten(-2) / temperature, dim=-1).view_as(c)
    rx = (p * tau[None, :]).sum(dim=(-1, -2))
    ry = (p * tau[:, None]).sum(dim=(-1, -2))
    return torch.stack([rx, ry], dim=-1)


def loss(nodes, im0, im1, xn, yn, temperature=0.1, symmetric=True):
    if symmetric:
        r = windows_r(warp(nodes, xn, yn, im0, -0.5), warp(nodes, xn, yn, im1, 0.5), temperature)
    else:
        r = windows_r(im0, warp(nodes, xn, yn, im1), temperature)
    return (r * r).sum(dim=-1).mean()
