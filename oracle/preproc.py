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


# ---------------------------------------------------------------- adaptive equalisation
#: grey levels of scikit-image's CLAHE (exposure/_adapthist.py: NR_OF_GRAY = 2**14)
NR_OF_GRAY = 2 ** 14


def _rescale_one(im, minima, maxima):
    return rescale_intensity(im, minima, maxima)


def clip_histogram(hist, clim):
    """Contrast limiting of one contextual-region histogram (Zuiderveld, "Contrast
    Limited Adaptive Histogram Equalization", Graphics Gems IV, 1994, in the
    variant of scikit-image 0.24's ``clip_histogram``): bins above the limit are
    cut and the excess is handed out again — first ``excess // nbins`` to every
    bin below ``clim - that``, bins between that and the limit filled to it, then
    one count at a time to bins below the limit, in strides of
    ``max(1, (bins below the limit) // excess)`` from every start bin in turn,
    until no excess is left or a full pass hands out nothing."""
    h = np.array(hist, dtype=np.int64)
    nb = h.size
    excess = int(np.maximum(h - clim, 0).sum())
    h = np.minimum(h, clim)
    incr = excess // nb
    upper = clim - incr
    for b in range(nb):
        if h[b] < upper:
            h[b] += incr
            excess -= incr
        if upper <= h[b] < clim:
            excess -= clim - h[b]
            h[b] = clim
    while excess > 0:
        before = excess
        for start in range(nb):
            under = h < clim
            stride = max(1, int(np.count_nonzero(under)) // excess)
            given = 0
            for p in range(start, nb, stride):
                if under[p]:
                    h[p] += 1
                    given += 1
            excess -= given
            if excess <= 0:
                break
        if before == excess:
            break
    return h


def _reflect(idx, size):
    """numpy's 'reflect' padding index (mirror without repeating the edge)."""
    if size == 1:
        return np.zeros_like(idx)
    period = 2 * (size - 1)
    m = np.mod(idx, period)
    return np.where(m >= size, period - m, m)


def clahe_levels(v, kernel_size, nbins, clip_limit=0.01):
    """scikit-image 0.24's ``_clahe`` restated (exposure/_adapthist.py) on a 2-D
    image ``v`` of grey levels in [0, NR_OF_GRAY): the image, extended at its end
    by reflection to whole regions of ``kernel_size``, is cut into contextual
    regions; each region's histogram of ``v // (1 + NR_OF_GRAY // nbins)`` is
    clipped at ``max(clip_limit * region size, 1)`` (truncated) and turned into the
    grey-level map ``min(cdf * ((NR_OF_GRAY - 1) / region size), NR_OF_GRAY - 1)``
    (float64, truncated); each pixel takes the bilinear blend of the maps of the
    four regions around it (coefficients ``r / k`` from the pixel's place in the
    block shifted by half a region, edge maps repeated), each term rounded to
    float32 and summed in float32 in the order (0, 0), (0, 1), (1, 0), (1, 1), the
    sum truncated to uint16."""
    s0, s1 = v.shape
    k0, k1 = (int(k) for k in kernel_size)
    m0, m1 = -(-s0 // k0), -(-s1 // k1)
    npix = k0 * k1
    clim = int(max(clip_limit * npix, 1)) if clip_limit > 0 else npix
    bins = v.astype(np.int64) // (1 + NR_OF_GRAY // nbins)
    ext = bins[np.ix_(_reflect(np.arange(m0 * k0), s0), _reflect(np.arange(m1 * k1), s1))]
    scale = np.float64(NR_OF_GRAY - 1) / np.float64(npix)
    maps = np.empty((m0, m1, nbins), np.int64)
    for i in range(m0):
        for j in range(m1):
            region = ext[i * k0:(i + 1) * k0, j * k1:(j + 1) * k1].ravel()
            h = clip_histogram(np.bincount(region, minlength=nbins), clim)
            cdf = np.cumsum(h).astype(np.float64)
            maps[i, j] = np.minimum(cdf * scale, NR_OF_GRAY - 1).astype(np.int64)
    yy, xx = np.meshgrid(np.arange(s0), np.arange(s1), indexing="ij")
    py, px = yy + k0 // 2, xx + k1 // 2
    bi, bj = py // k0, px // k1
    cy = (py - bi * k0) / np.float64(k0)
    cx = (px - bj * k1) / np.float64(k1)
    out = np.zeros((s0, s1), np.float32)
    for e0 in (0, 1):
        for e1 in (0, 1):
            ri = np.clip(bi + e0 - 1, 0, m0 - 1)
            rj = np.clip(bj + e1 - 1, 0, m1 - 1)
            mapped = maps[ri, rj, bins]
            w = (cx if e1 else 1.0 - cx) * (cy if e0 else 1.0 - cy)
            out += (mapped * w).astype(np.float32)
    return out.astype(np.uint16)


def equalize_hist_adapt(img, window_shape=(10, 10), nbins=256):
    """_toolbox_py.py:383-409: the image rescaled to [0, 1], scikit-image's
    ``exposure.equalize_adapthist`` (kernel_size=window_shape, clip_limit 0.01:
    rescaled to grey levels [0, NR_OF_GRAY - 1] and truncated, ``clahe_levels``,
    rescaled to [0, 1] in the float type), rescaled back to the image's [min, max].
    float32 images stay float32, others give float64."""

    def one(im):
        ft = np.float32 if im.dtype == np.float32 else np.float64
        if window_shape is None:  # scikit-image: 1/8 of each dimension
            kernel = tuple(max(s // 8, 1) for s in im.shape)
        elif np.isscalar(window_shape):
            kernel = (int(window_shape),) * 2
        else:
            kernel = tuple(int(k) for k in window_shape)
        lo, hi = im.min(), im.max()
        y = _rescale_one(_rescale_one(im, 0, 1), 0, NR_OF_GRAY - 1)
        levels = clahe_levels(y.astype(np.uint16), kernel, nbins)
        z = _rescale_one(levels.astype(ft), 0, 1)
        return _rescale_one(z, lo, hi)

    return _per_image(one, img)


def disk(radius):
    """scikit-image's ``morphology.disk(radius)``: x^2 + y^2 <= radius^2 on the
    (2 radius + 1)^2 grid."""
    r = np.arange(-radius, radius + 1)
    return ((r[:, None] ** 2 + r[None, :] ** 2) <= radius ** 2).astype(np.uint8)


def to_ubyte(y):
    """scikit-image's ``img_as_ubyte`` of a float image in [0, 1]: rint(y * 255)
    computed in the image's float type, clipped to [0, 255]."""
    prod = np.multiply(y, 255, dtype=y.dtype)
    return np.clip(np.rint(prod), 0, 255).astype(np.uint8)


def rank_equalize(u8, footprint):
    """scikit-image's ``filters.rank.equalize`` of a uint8 image: at each pixel, of
    the footprint's pixels inside the image (``pop``), the number ``n`` whose value
    is at most the centre's; the output is ``(256 - 1) * n / pop`` truncated to
    uint8."""
    s0, s1 = u8.shape
    fr = footprint.shape[0] // 2
    g = u8.astype(np.int64)
    n = np.zeros((s0, s1), np.int64)
    pop = np.zeros((s0, s1), np.int64)
    pad = np.full((s0 + 2 * fr, s1 + 2 * fr), -1, np.int64)
    pad[fr:fr + s0, fr:fr + s1] = g
    for dy, dx in zip(*np.nonzero(footprint)):
        win = pad[dy:dy + s0, dx:dx + s1]
        inside = win >= 0
        pop += inside
        n += inside & (win <= g)
    return ((255 * n) / pop.astype(np.float64)).astype(np.uint8)


def equalize_hist_local(img, radius=10):
    """_toolbox_py.py:412-438: the image rescaled to [0, 1], to uint8
    (``to_ubyte``), ``rank_equalize`` over ``disk(radius)``, rescaled to the image's
    [min, max] (float64)."""

    def one(im):
        lo, hi = im.min(), im.max()
        u8 = to_ubyte(_rescale_one(im, 0, 1))
        return _rescale_one(rank_equalize(u8, disk(radius)), lo, hi)

    return _per_image(one, img)
