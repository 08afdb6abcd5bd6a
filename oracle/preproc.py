"""scipy / numpy restatement of the upstream preprocessing tools — TEST INFRASTRUCTURE ONLY.

Restates works/preproc/_toolbox_py.py (fluidimage 0.5.3) for the tools the GPU
module provides, with upstream's stack handling (works/preproc/io.py:46-84): the
sliding tools, global_threshold and rescale_intensity_tanh run image by image into
a float64 stack; the temporal tools see the whole stack.  The arithmetic is
numpy's (NEP 50 scalar promotion), the filters scipy.ndimage's.

rescale_intensity, gamma_correction, adaptive_threshold and equalize_hist_global call
scikit-image (0.24.0 in the reference's lock file), which is not installed here: they
are restated from scikit-image's published definitions of ``exposure.equalize_hist``
(one histogram bin per integer value for integer images, numpy's uniform histogram
of nbins bins otherwise; np.interp of the cumulative distribution at the bin
centres), ``exposure.rescale_intensity``
(in_range='image', a numeric out_range; output float64 for integer images, the
float type otherwise), ``exposure.adjust_gamma`` (uint8 through a 256-entry table,
other dtypes scaled by the dtype's range, power law, cast back) and
``filters.threshold_local`` with method 'gaussian' (scipy's gaussian filter of the
float image, sigma = (block_size - 1) / 6, 'reflect', minus the offset).  Parity for
these four is unpinned: no scikit-image output exists here to record (the
gaussian filter itself is scipy's).
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


def rescale_intensity(img, minima=0.0, maxima=4096):
    """_toolbox_py.py:313-331 (skimage.exposure.rescale_intensity(img,
    out_range=(minima, maxima)))."""

    def one(im):
        out_dtype = np.float32 if im.dtype == np.float32 else np.float64
        imin, imax = float(im.min()), float(im.max())
        omin, omax = float(minima), float(maxima)
        im = np.clip(im, imin, imax)
        if imin != imax:
            im = (im - imin) / (imax - imin)
            return np.asarray(im * (omax - omin) + omin, dtype=out_dtype)
        return np.clip(im, omin, omax).astype(out_dtype)

    return _per_image(one, img)


def gamma_correction(img, gamma=1.0, gain=1.0, with_raw=False):
    """_toolbox_py.py:441-470 (skimage.exposure.adjust_gamma(img, gamma, gain)).
    ``with_raw``: also the float values before the cast to uint16 (for tests at
    truncation boundaries)."""
    if gamma < 0:
        raise ValueError("Gamma should be a non-negative real number.")
    raws = []

    def one(im):
        if im.dtype == np.uint8:
            lut = 255 * gain * (np.linspace(0, 1, 256) ** gamma)
            lut = np.minimum(np.rint(lut), 255).astype("uint8")
            return lut[im]
        if im.min() < 0:
            raise ValueError("Image Correction methods work correctly only on images with "
                             "non-negative values. Use skimage.exposure.rescale_intensity.")
        scale = 65535.0 if im.dtype == np.uint16 else 1.0
        raw = ((im / scale) ** gamma) * scale * gain
        raws.append(raw)
        return raw.astype(im.dtype)

    out = _per_image(one, img)
    return (out, raws) if with_raw else out


def adaptive_threshold(img, window_size=5, offset=0):
    """_toolbox_py.py:292-308 (skimage.filters.threshold_local(img, window_size,
    offset=offset), method 'gaussian')."""
    if int(window_size) % 2 == 0:
        raise ValueError("block_size must be odd")

    def one(im):
        ft = np.float32 if im.dtype == np.float32 else np.float64
        x = im.astype(ft, copy=False)
        out = np.zeros(x.shape, dtype=ft)
        ndi.gaussian_filter(x, (window_size - 1) / 6.0, output=out, mode="reflect", cval=0)
        return out - offset

    return _per_image(one, img)


def equalize_hist_global(img, nbins=256):
    """_toolbox_py.py:357-379 (skimage.exposure.equalize_hist(img, nbins=nbins))."""

    def one(im):
        if np.issubdtype(im.dtype, np.integer):
            lo, hi = int(im.min()), int(im.max())
            centers = np.arange(lo, hi + 1)
            hist = np.bincount((im.ravel().astype(np.int64) - lo), minlength=hi - lo + 1)
            cdf_dtype = np.float64
        else:
            hist, edges = np.histogram(im, bins=nbins)
            centers = (edges[:-1] + edges[1:]) / 2.0
            cdf_dtype = np.float32 if im.dtype == np.float32 else np.float64
        cdf = hist.cumsum()
        cdf = (cdf / float(cdf[-1])).astype(cdf_dtype, copy=False)
        out = np.interp(im.ravel(), centers, cdf).reshape(im.shape)
        return out.astype(np.float32 if im.dtype == np.float32 else np.float64, copy=False)

    return _per_image(one, img)
