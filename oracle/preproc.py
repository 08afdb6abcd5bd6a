"""scipy / numpy restatement of the upstream preprocessing tools — TEST INFRASTRUCTURE ONLY.

Restates works/preproc/_toolbox_py.py (fluidimage 0.5.3) for the tools the GPU
module provides, with upstream's stack handling (works/preproc/io.py:46-84): the
sliding tools, global_threshold and rescale_intensity_tanh run image by image into
a float64 stack; the temporal tools see the whole stack.  The arithmetic is
numpy's (NEP 50 scalar promotion), the filters scipy.ndimage's.
"""

from __future__ import annotations

import numpy as np
import scipy.ndimage as ndi


def _per_image(tool, img, **kw):
    """iterate_multiple_imgs (io.py:46-64)."""
    if img.ndim == 2:
        return tool(img, **kw)
    out = np.empty_like(img, dtype=np.float64)
    for i, im in enumerate(img):
        out[i] = tool(im, **kw)
    return out


def _clamped(img, filtered, weight):
    out = img - weight * filtered
    out[out < 0] = 0
    return out


def sliding_minima(img, weight=1.0, window_size=30, boundary_condition="reflect"):
    """_toolbox_py.py:129-155."""
    return _per_image(lambda im: _clamped(im, ndi.minimum_filter(
        im, size=window_size, mode=boundary_condition), weight), img)


def sliding_median(img, weight=1.0, window_size=30, boundary_condition="reflect"):
    """_toolbox_py.py:65-91."""
    return _per_image(lambda im: _clamped(im, ndi.median_filter(
        im, size=window_size, mode=boundary_condition), weight), img)


def sliding_percentile(img, percentile=10.0, weight=1.0, window_size=30,
                       boundary_condition="reflect"):
    """_toolbox_py.py:94-126."""
    return _per_image(lambda im: _clamped(im, ndi.percentile_filter(
        im, percentile, size=window_size, mode=boundary_condition), weight), img)


def _window(shape, window_shape):
    """_calcul_windowshape (_toolbox_py.py:163-185)."""
    if window_shape is None:
        return (shape[0], 1, 1)
    if isinstance(window_shape, int):
        return (window_shape, 1, 1)
    if len(window_shape) == 2:
        return (shape[0],) + tuple(window_shape)
    return tuple(window_shape)


def temporal_minima(img, weight=1.0, window_shape=None):
    """_toolbox_py.py:239-256."""
    return img - weight * ndi.minimum_filter(img, size=_window(img.shape, window_shape))


def temporal_median(img, weight=1.0, window_shape=None):
    """_toolbox_py.py:188-208."""
    return img - weight * ndi.median_filter(img, size=_window(img.shape, window_shape))


def temporal_percentile(img, percentile=10.0, weight=1.0, window_shape=None):
    """_toolbox_py.py:211-236."""
    return img - weight * ndi.percentile_filter(img, percentile,
                                                size=_window(img.shape, window_shape))


def global_threshold(img, minima=0, maxima=None):
    """_toolbox_py.py:264-289."""
    def one(im):
        out = im.copy()
        mx = maxima
        if mx is None:
            try:
                mx = np.iinfo(out.dtype).max
            except ValueError:
                mx = 65535
        out[out < minima] = minima
        out[out > mx] = mx
        return out
    return _per_image(one, img)


def rescale_intensity_tanh(img, threshold=None):
    """_toolbox_py.py:331-355."""
    def one(im):
        thr = threshold
        if thr is None:
            thr = 2 * np.sqrt(np.mean(im**2))
        if thr == 0:
            return im
        out = np.tanh(im / thr)
        return np.floor(np.max(im) / np.max(out) * out)
    return _per_image(one, img)


def sharpen(img, sigma1=3.0, sigma2=1.0, alpha=30.0):
    """_toolbox_py.py:472-490 (scipy.ndimage gaussian filters in the image dtype, numpy
    promotions in the combination)."""

    def one(im):
        blurred = ndi.gaussian_filter(im, sigma1)
        filter_blurred = ndi.gaussian_filter(blurred, sigma2)
        return blurred + alpha * (blurred - filter_blurred)

    return _per_image(one, img)
