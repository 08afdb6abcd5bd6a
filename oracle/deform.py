"""numpy restatement of the image deformation — TEST INFRASTRUCTURE ONLY.

The reference has no deformation (works/piv/singlepass.py:736-738 leaves it as a
to-do); this float64 restatement of the library's definition (bilinear field on
sorted node coordinates, constant beyond the outer nodes; bilinear sampling of im1
with replicated borders) checks the device warp and the deformation-mode passes.
"""

from __future__ import annotations

import numpy as np


def _cell(coords, v):
    coords = np.asarray(coords, np.float64)
    n = coords.size
    j0 = np.clip(np.searchsorted(coords, v, side="right") - 1, 0, n - 2)
    t = np.clip((v - coords[j0]) / (coords[j0 + 1] - coords[j0]), 0.0, 1.0)
    return j0, t


def field_at(nodes, xn, yn, H, W):
    """(u, v) [H, W] of a node field [2, ny, nx]."""
    j0, tx = _cell(xn, np.arange(W, dtype=np.float64))
    i0, ty = _cell(yn, np.arange(H, dtype=np.float64))
    out = []
    for f in np.asarray(nodes, np.float64):
        f00 = f[i0][:, j0]
        f01 = f[i0][:, j0 + 1]
        f10 = f[i0 + 1][:, j0]
        f11 = f[i0 + 1][:, j0 + 1]
        top = (1 - tx)[None] * f00 + tx[None] * f01
        bot = (1 - tx)[None] * f10 + tx[None] * f11
        out.append((1 - ty)[:, None] * top + ty[:, None] * bot)
    return out


def warp(nodes, xn, yn, im1, scale=1.0):
    """im1 [H, W] sampled bilinearly at (x + scale u, y + scale v), replicated borders
    (float64)."""
    im1 = np.asarray(im1, np.float64)
    H, W = im1.shape
    u, v = field_at(nodes, xn, yn, H, W)
    px = np.arange(W)[None, :] + scale * u
    py = np.arange(H)[:, None] + scale * v
    x0 = np.floor(px)
    y0 = np.floor(py)
    fx, fy = px - x0, py - y0
    xa = np.clip(x0.astype(np.int64), 0, W - 1)
    xb = np.clip(x0.astype(np.int64) + 1, 0, W - 1)
    ya = np.clip(y0.astype(np.int64), 0, H - 1)
    yb = np.clip(y0.astype(np.int64) + 1, 0, H - 1)
    top = (1 - fx) * im1[ya, xa] + fx * im1[ya, xb]
    bot = (1 - fx) * im1[yb, xa] + fx * im1[yb, xb]
    return (1 - fy) * top + fy * bot
