"""Seeded synthetic particle-image pairs for PIV tests and benchmarks.

Particle model (one image pair):

* particle centres uniform over the image extended by a margin of
  ``max|d| + 3 * diameter_max`` pixels, so that particles enter and leave the frame;
  the count is ``density * area_with_margin``;
* each particle is a Gaussian spot ``I0 * exp(-8 r^2 / d^2)`` (the ``e^-2`` level
  falls at ``r = d / 2``) with diameter ``d ~ U[d_min, d_max]`` and peak
  ``I0 ~ U[i_min, i_max]``;
* image 1 shows the same particles moved by the displacement field evaluated at the
  midpoint of the motion, ``x1 = x0 + d((x0 + x1) / 2)`` (three fixed-point
  iterations), which matches the convention that a PIV vector sits at the midpoint
  of its two windows;
* Gaussian noise of standard deviation ``noise`` counts is added, then the image is
  rounded and clipped to the range of the output dtype.

The pixel ``(iy, ix)`` is centred at ``(x, y) = (ix, iy)``.

This differs on purpose from the upstream helper
``fluidimage/synthetic.py:6-61`` (``exp(-r^2 / part_size^2)``, uniform shift only),
which cannot express the particle diameters, intensities and fields used here.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Callable, Optional, Tuple

import numpy as np

__all__ = [
    "ParticleModel",
    "uniform_shift",
    "oseen_vortex",
    "sinusoid",
    "make_pair",
]


@dataclass
class ParticleModel:
    density: float = 0.05
    diameter: Tuple[float, float] = (2.0, 3.0)
    intensity: Tuple[float, float] = (128.0, 255.0)
    noise: float = 2.0
    dtype: str = "uint8"
    max_value: Optional[float] = None  # clip level (default: dtype maximum)
    extra: dict = field(default_factory=dict)


def uniform_shift(dx: float, dy: float) -> Callable:
    def field_(x, y):
        return np.full_like(x, dx, dtype=np.float64), np.full_like(y, dy, dtype=np.float64)

    field_.max_displacement = float(np.hypot(dx, dy))
    return field_


def oseen_vortex(shape, d_max=8.0, rc=200.0, center=None) -> Callable:
    """Oseen vortex ``u_theta = G/(2 pi r) (1 - exp(-r^2/rc^2))`` scaled to max |d| = d_max."""
    ny, nx = shape
    if center is None:
        center = ((nx - 1) / 2.0, (ny - 1) / 2.0)
    xc, yc = center
    r = np.linspace(1e-6, 10 * rc, 200001)
    g = (1.0 - np.exp(-(r**2) / rc**2)) / r
    coef = d_max / g.max()

    def field_(x, y):
        x = np.asarray(x, dtype=np.float64) - xc
        y = np.asarray(y, dtype=np.float64) - yc
        r2 = x * x + y * y
        with np.errstate(invalid="ignore", divide="ignore"):
            u_over_r = np.where(r2 > 0, coef * (1.0 - np.exp(-r2 / rc**2)) / r2, coef / rc**2)
        return -u_over_r * y, u_over_r * x

    field_.max_displacement = float(d_max)
    return field_


def sinusoid(amplitude=5.0, wavelength=512.0) -> Callable:
    """``d = A (sin(2 pi y / L), cos(2 pi x / L))``."""

    def field_(x, y):
        x = np.asarray(x, dtype=np.float64)
        y = np.asarray(y, dtype=np.float64)
        k = 2 * np.pi / wavelength
        return amplitude * np.sin(k * y), amplitude * np.cos(k * x)

    field_.max_displacement = float(amplitude * np.sqrt(2.0))
    return field_


def _render(shape, xs, ys, diam, peak, chunk=65536):
    """Sum of Gaussian spots, as separable (rows x columns) patches per particle."""
    ny, nx = shape
    out = np.zeros(ny * nx, dtype=np.float64)
    radius = int(np.ceil(1.5 * diam.max())) + 1
    offs = np.arange(-radius, radius + 1)
    for c0 in range(0, xs.size, chunk):
        x = xs[c0:c0 + chunk]
        y = ys[c0:c0 + chunk]
        inv = -8.0 / (diam[c0:c0 + chunk] ** 2)
        ix = np.floor(x).astype(np.int64)[:, None] + offs[None, :]
        iy = np.floor(y).astype(np.int64)[:, None] + offs[None, :]
        gx = np.exp(inv[:, None] * (ix - x[:, None]) ** 2)
        gy = np.exp(inv[:, None] * (iy - y[:, None]) ** 2)
        gx[(ix < 0) | (ix >= nx)] = 0.0
        gy[(iy < 0) | (iy >= ny)] = 0.0
        vals = (peak[c0:c0 + chunk, None, None] * gy[:, :, None]) * gx[:, None, :]
        flat = np.clip(iy, 0, ny - 1)[:, :, None] * nx + np.clip(ix, 0, nx - 1)[:, None, :]
        out += np.bincount(flat.ravel(), weights=vals.ravel(), minlength=ny * nx)
    return out.reshape(shape)


def make_pair(
    shape,
    displacement: Callable,
    model: Optional[ParticleModel] = None,
    seed: int = 0,
    as_float32: bool = False,
):
    """Render one image pair; returns ``(im0, im1)``.

    ``as_float32`` converts the clipped integer images to float32 (the
    "float32 built from uint8" form).
    """
    if model is None:
        model = ParticleModel()
    rng = np.random.default_rng(seed)
    ny, nx = shape
    dmax = getattr(displacement, "max_displacement", 10.0)
    margin = dmax + 3.0 * model.diameter[1]
    area = (nx + 2 * margin) * (ny + 2 * margin)
    count = int(round(model.density * area))
    x0 = rng.uniform(-margin, nx - 1 + margin, count)
    y0 = rng.uniform(-margin, ny - 1 + margin, count)
    diam = rng.uniform(model.diameter[0], model.diameter[1], count)
    peak = rng.uniform(model.intensity[0], model.intensity[1], count)

    x1, y1 = x0.copy(), y0.copy()
    for _ in range(3):
        dx, dy = displacement(0.5 * (x0 + x1), 0.5 * (y0 + y1))
        x1 = x0 + dx
        y1 = y0 + dy

    info = np.iinfo(model.dtype)
    images = []
    for xs, ys in ((x0, y0), (x1, y1)):
        im = _render(shape, xs, ys, diam, peak)
        if model.noise > 0:
            im = im + rng.normal(0.0, model.noise, size=shape)
        top = info.max if model.max_value is None else model.max_value
        im = np.clip(np.rint(im), info.min, top).astype(model.dtype)
        if as_float32:
            im = im.astype(np.float32)
        images.append(im)
    return images[0], images[1]


def truth_at(displacement: Callable, xs, ys):
    """Ground-truth displacement at vector positions (midpoint convention)."""
    return displacement(np.asarray(xs, np.float64), np.asarray(ys, np.float64))
