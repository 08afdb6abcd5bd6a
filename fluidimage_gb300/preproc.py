"""Image preprocessing on the GPU, with the tools of fluidimage's toolbox.

Mirrors ``fluidimage.works.preproc`` (``WorkPreproc``, ``PreprocToolsPy``;
works/preproc/__init__.py:62-137, toolbox.py:24-120): the parameter tree
``params.tools`` (``available_tools``, ``sequence`` and one child per tool with its
arguments and ``enable``) and ``calcul({"arrays": ..., "names": ...})``.

The tools run in ``libfluidimage_gb300`` on device tensors (uint8, uint16 as int16
storage, float32, float64), with the arithmetic of the upstream functions in
works/preproc/_toolbox_py.py:

* ``sliding_minima / sliding_median / sliding_percentile`` (:66-155): a 2-D rank
  filter per image (scipy.ndimage window and boundary modes), then
  ``img - weight * filtered`` in numpy's result dtype, negatives set to 0;
* ``temporal_minima / temporal_median / temporal_percentile`` (:189-256): the rank
  filter over the stack with ``window_shape`` (nt, ny, nx), no clamping;
* ``global_threshold`` (:265-289) and ``rescale_intensity_tanh`` (:332-355);
* ``sharpen`` (:472-490): scipy.ndimage's gaussian filters (float64 line sums in
  scipy's order, each axis cast to the image dtype) and the final combination;
* ``rescale_intensity`` (:313-331), ``gamma_correction`` (:441-470),
  ``adaptive_threshold`` (:292-308) and ``equalize_hist_global`` (:357-379), which
  upstream takes from scikit-image 0.24 (``exposure.rescale_intensity`` with
  ``in_range='image'``, ``exposure.adjust_gamma``, ``filters.threshold_local`` with
  its gaussian method, ``exposure.equalize_hist``): their published definitions, in
  the dtypes scikit-image and numpy 2 use.

The adaptive equalisations, also built on scikit-image, are restated the same way:
``equalize_hist_adapt`` (:383-409, ``exposure.equalize_adapthist``: CLAHE on 2^14
grey levels, ``fi_clahe``) and ``equalize_hist_local`` (:412-438,
``filters.rank.equalize`` over ``morphology.disk``: ``fi_rank_equalize``).
"""

from __future__ import annotations

import math

import numpy as np

from . import _lib as L
from .params import ParamContainer

# Upstream tool signatures (works/preproc/_toolbox_py.py), without ``img``.
TOOL_DEFAULTS = {
    "sliding_median": dict(weight=1.0, window_size=30, boundary_condition="reflect"),
    "sliding_minima": dict(weight=1.0, window_size=30, boundary_condition="reflect"),
    "sliding_percentile": dict(percentile=10.0, weight=1.0, window_size=30,
                               boundary_condition="reflect"),
    "temporal_median": dict(weight=1.0, window_shape=None),
    "temporal_minima": dict(weight=1.0, window_shape=None),
    "temporal_percentile": dict(percentile=10.0, weight=1.0, window_shape=None),
    "global_threshold": dict(minima=0, maxima=None),
    "adaptive_threshold": dict(window_size=5, offset=0),
    "rescale_intensity": dict(minima=0.0, maxima=4096),
    "equalize_hist_global": dict(nbins=256),
    "equalize_hist_local": dict(radius=10),
    "equalize_hist_adapt": dict(window_shape=(10, 10), nbins=256),
    "gamma_correction": dict(gamma=1.0, gain=1.0),
    "sharpen": dict(sigma1=3.0, sigma2=1.0, alpha=30.0),
    "rescale_intensity_tanh": dict(threshold=None),
}
AVAILABLE_TOOLS = list(TOOL_DEFAULTS)

_DT = {np.dtype(np.uint8): L.PRE_U8, np.dtype(np.uint16): L.PRE_U16,
       np.dtype(np.float32): L.PRE_F32, np.dtype(np.float64): L.PRE_F64}


def _torch():
    import torch

    return torch


def _dtype_of(t):
    """numpy dtype of the image data of a device tensor (uint16 as int16 storage)."""
    torch = _torch()
    return {torch.uint8: np.dtype(np.uint8), torch.int16: np.dtype(np.uint16),
            torch.float32: np.dtype(np.float32), torch.float64: np.dtype(np.float64)}[t.dtype]


def _empty(shape, dtype, device):
    torch = _torch()
    td = {np.dtype(np.uint8): torch.uint8, np.dtype(np.uint16): torch.int16,
          np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}[np.dtype(dtype)]
    return torch.empty(shape, dtype=td, device=device)


def to_device(images, device=None):
    """Host image(s) -> device tensor (uint16 data kept bit for bit as int16)."""
    torch = _torch()
    if isinstance(images, torch.Tensor):
        return images.to(device or "cuda").contiguous()
    a = np.ascontiguousarray(images)
    if a.dtype == np.uint16:
        a = a.view(np.int16)
    elif a.dtype not in (np.uint8, np.float32, np.float64):
        raise TypeError(f"image dtype {a.dtype} not supported (uint8, uint16, float32, float64)")
    return torch.from_numpy(a).to(device or "cuda")


def to_host(t):
    """Device tensor -> numpy array (int16 storage of uint16 images viewed back)."""
    a = t.cpu().numpy()
    return a.view(np.uint16) if a.dtype == np.int16 else a


def _as_float64(t):
    """Values of a device image as float64 (uint16 data from its int16 storage)."""
    torch = _torch()
    if t.dtype == torch.int16:
        return (t.to(torch.int32) & 0xFFFF).to(torch.float64)
    return t.to(torch.float64)


def _per_image(tool):
    """Upstream's ``iterate_multiple_imgs`` (works/preproc/io.py:46-64): a 2-D image
    gives the tool's own dtype, a stack is filled image by image into float64."""

    def wrapper(img, *args, **kwargs):
        if img.dim() == 2:
            return tool(img, *args, **kwargs)
        return _as_float64(tool(img, *args, **kwargs))

    wrapper.__name__ = tool.__name__
    wrapper.__doc__ = tool.__doc__
    return wrapper


def _stack(img):
    """(nt, ny, nx) view of a 2-D image or a stack."""
    if img.dim() == 2:
        return img[None], True
    if img.dim() == 3:
        return img, False
    raise ValueError("images must be 2-D or a 3-D stack")


def _rank(size, rank_kind, percentile=None):
    """scipy.ndimage._rank_filter's rank for a box of ``size`` elements."""
    if rank_kind == "min":
        return 0
    if rank_kind == "median":
        return size // 2
    p = float(percentile)
    if p < 0.0:
        p += 100.0
    if p < 0 or p > 100:
        raise RuntimeError("invalid percentile")
    return size - 1 if p == 100.0 else int(float(size) * p / 100.0)


def rank_filter(img, window, rank_kind, percentile=None, mode="reflect", cval=0.0):
    """scipy.ndimage minimum_filter / median_filter / percentile_filter of a stack
    (nt, ny, nx) over the box ``window`` = (st, sy, sx); output in the input dtype."""
    torch = _torch()
    lib = L.load()
    x = img.contiguous()
    nt, ny, nx = x.shape
    st, sy, sx = (int(w) for w in window)
    r = _rank(st * sy * sx, rank_kind, percentile)
    if mode not in L.MODES:
        raise RuntimeError(f"boundary mode not supported: {mode}")
    dt = _DT[_dtype_of(x)]
    if dt in (L.PRE_F32, L.PRE_F64) and bool(torch.isnan(x).any()):
        raise ValueError("rank filters of images with NaN are not provided")
    out = torch.empty_like(x)
    scratch = None
    if r in (0, st * sy * sx - 1):
        scratch = torch.empty(2 * x.numel(), dtype=torch.int64, device=x.device)
    L.check(lib.fi_rank_filter(L.ptr(x), L.ptr(out), dt, nt, ny, nx, st, sy, sx, r,
                               L.MODES[mode], float(cval), L.ptr(scratch), L.stream_handle()),
            "fi_rank_filter")
    return out


def _result_dtype(dtype, weight):
    """numpy's dtype of ``img - weight * filtered`` (same dtype arrays)."""
    z = np.zeros(1, dtype=dtype)
    return (z - weight * z).dtype


def _subtract(img, filtered, weight, clamp):
    lib = L.load()
    dtype = _dtype_of(img)
    out_dt = _result_dtype(dtype, weight)
    if out_dt not in _DT:
        raise TypeError(f"result dtype {out_dt} not supported")
    out = _empty(tuple(img.shape), out_dt, img.device)
    L.check(lib.fi_subtract_weighted(L.ptr(img), L.ptr(filtered), _DT[dtype], img.numel(),
                                     float(weight), _DT[out_dt], int(clamp), L.ptr(out),
                                     L.stream_handle()), "fi_subtract_weighted")
    return out


def _window2d(window_size):
    if isinstance(window_size, (tuple, list)):
        sy, sx = (int(w) for w in window_size)
    else:
        sy = sx = int(window_size)
    return 1, sy, sx


def _sliding(img, weight, window_size, boundary_condition, kind, percentile=None):
    x, single = _stack(img)
    f = rank_filter(x, _window2d(window_size), kind, percentile, mode=boundary_condition)
    out = _subtract(x, f, weight, clamp=True)
    return out[0] if single else out


@_per_image
def sliding_minima(img, weight=1.0, window_size=30, boundary_condition="reflect"):
    """img - weight * minimum_filter(img), negatives -> 0 (_toolbox_py.py:129-155)."""
    return _sliding(img, weight, window_size, boundary_condition, "min")


@_per_image
def sliding_median(img, weight=1.0, window_size=30, boundary_condition="reflect"):
    """img - weight * median_filter(img), negatives -> 0 (_toolbox_py.py:65-91)."""
    return _sliding(img, weight, window_size, boundary_condition, "median")


@_per_image
def sliding_percentile(img, percentile=10.0, weight=1.0, window_size=30,
                       boundary_condition="reflect"):
    """img - weight * percentile_filter(img), negatives -> 0 (_toolbox_py.py:94-126)."""
    return _sliding(img, weight, window_size, boundary_condition, "percentile", percentile)


def _calcul_windowshape(arr_shape, window_shape):
    """_toolbox_py.py:163-185."""
    nb_imgs = arr_shape[0]
    if len(arr_shape) <= 2 or nb_imgs <= 1:
        raise ValueError(
            "Need more than one image to apply temporal filtering (use sliding filter?).")
    if window_shape is None:
        window_shape = (nb_imgs, 1, 1)
    elif isinstance(window_shape, int):
        window_shape = (window_shape, 1, 1)
    elif not isinstance(window_shape, (tuple, list)):
        raise ValueError("window_shape must be a tuple or a list.")
    elif len(window_shape) == 2:
        window_shape = (nb_imgs,) + tuple(window_shape)
    elif window_shape[0] <= 1:
        raise ValueError("Cannot perform temporal filtering, try spatial filtering.")
    return tuple(window_shape)


def _temporal(img, weight, window_shape, kind, percentile=None):
    window = _calcul_windowshape(tuple(img.shape), window_shape)
    f = rank_filter(img, window, kind, percentile)
    return _subtract(img, f, weight, clamp=False)


def temporal_minima(img, weight=1.0, window_shape=None):
    """img - weight * minimum_filter(img, window_shape) (_toolbox_py.py:239-256)."""
    return _temporal(img, weight, window_shape, "min")


def temporal_median(img, weight=1.0, window_shape=None):
    """img - weight * median_filter(img, window_shape) (_toolbox_py.py:188-208)."""
    return _temporal(img, weight, window_shape, "median")


def temporal_percentile(img, percentile=10.0, weight=1.0, window_shape=None):
    """img - weight * percentile_filter(img, window_shape) (_toolbox_py.py:211-236)."""
    return _temporal(img, weight, window_shape, "percentile", percentile)


@_per_image
def global_threshold(img, minima=0, maxima=None):
    """Clamp the intensities to [minima, maxima] (_toolbox_py.py:264-289)."""
    lib = L.load()
    dtype = _dtype_of(img)
    if maxima is None:
        maxima = np.iinfo(dtype).max if dtype.kind in "ui" else 65535
    out = _empty(tuple(img.shape), dtype, img.device)
    L.check(lib.fi_clamp(L.ptr(img.contiguous()), _DT[dtype], img.numel(), float(minima),
                         float(maxima), L.ptr(out), L.stream_handle()), "fi_clamp")
    return out


@_per_image
def rescale_intensity_tanh(img, threshold=None):
    """max(img) * tanh(img / threshold) / max(tanh(img / threshold)), floored
    (_toolbox_py.py:331-355); per image for a stack."""
    x, single = _stack(img)
    outs = [_tanh_one(x[i], threshold) for i in range(x.shape[0])]
    if single:
        return outs[0]
    return _torch().stack(outs)


def _tanh_one(img, threshold):
    torch = _torch()
    lib = L.load()
    dtype = _dtype_of(img)
    if dtype == np.float32:
        raise NotImplementedError("rescale_intensity_tanh of float32 images (upstream works "
                                  "in float32 there) is not provided")
    x = img.contiguous()
    nparts = 152
    part = torch.empty(2 * nparts, dtype=torch.float64, device=x.device)
    L.check(lib.fi_sq_sum_max(L.ptr(x), _DT[dtype], x.numel(), L.ptr(part),
                              L.ptr(part[nparts:]), nparts, L.stream_handle()), "fi_sq_sum_max")
    host = part.cpu().numpy()
    vmax = float(host[nparts:].max())
    if threshold is None:
        threshold = 2 * math.sqrt(float(host[:nparts].sum()) / x.numel())
    if threshold == 0:
        return img
    scale = vmax / math.tanh(vmax / threshold)
    out = torch.empty(tuple(x.shape), dtype=torch.float64, device=x.device)
    L.check(lib.fi_tanh_rescale(L.ptr(x), _DT[dtype], x.numel(), float(threshold), scale,
                                L.ptr(out), L.stream_handle()), "fi_tanh_rescale")
    return out


_NPARTS = 152


def _extremes(x):
    """Device partial (min, max) of ``x`` (fi_min_max), 2 x _NPARTS float64."""
    torch = _torch()
    part = torch.empty(2 * _NPARTS, dtype=torch.float64, device=x.device)
    L.check(L.load().fi_min_max(L.ptr(x), _DT[_dtype_of(x)], x.numel(), L.ptr(part), _NPARTS,
                                L.stream_handle()), "fi_min_max")
    return part


@_per_image
def rescale_intensity(img, minima=0.0, maxima=4096):
    """Intensities mapped linearly from [img.min(), img.max()] to [minima, maxima]
    (_toolbox_py.py:313-331); float32 for float32 images, float64 otherwise; per
    image for a stack."""
    x, single = _stack(img)
    outs = [_rescale_one(x[i], minima, maxima) for i in range(x.shape[0])]
    return outs[0] if single else _torch().stack(outs)


def _rescale_one(img, minima, maxima):
    torch = _torch()
    x = img.contiguous()
    dtype = _dtype_of(x)
    part = _extremes(x)
    out_dt = torch.float32 if dtype == np.float32 else torch.float64
    out = torch.empty(tuple(x.shape), dtype=out_dt, device=x.device)
    L.check(L.load().fi_rescale_intensity(L.ptr(x), _DT[dtype], x.numel(), L.ptr(part), _NPARTS,
                                          float(minima), float(maxima), L.ptr(out),
                                          L.stream_handle()), "fi_rescale_intensity")
    return out


def gamma_table(gamma, gain):
    """The 256-entry uint8 table of adjust_gamma for uint8 images, from the two
    parameters: rint(255 gain linspace(0, 1, 256) ** gamma), capped at 255."""
    lut = 255 * gain * (np.linspace(0, 1, 256) ** gamma)
    return np.minimum(np.rint(lut), 255).astype("uint8")


@_per_image
def gamma_correction(img, gamma=1.0, gain=1.0):
    """gain * img ** gamma on intensities scaled to [0, 1] by the dtype's range
    (_toolbox_py.py:441-470), in the image dtype."""
    torch = _torch()
    if gamma < 0:
        raise ValueError("Gamma should be a non-negative real number.")
    x = img.contiguous()
    dtype = _dtype_of(x)
    lut = None
    if dtype == np.uint8:
        lut = torch.as_tensor(gamma_table(gamma, gain), device=x.device)
    elif dtype.kind == "f":
        part = _extremes(x).cpu().numpy()
        if part[:_NPARTS].min() < 0:
            raise ValueError("Image Correction methods work correctly only on images with "
                             "non-negative values. Use skimage.exposure.rescale_intensity.")
    out = _empty(tuple(x.shape), dtype, x.device)
    L.check(L.load().fi_gamma(L.ptr(x), _DT[dtype], x.numel(), float(gamma), float(gain),
                              L.ptr(lut), L.ptr(out), L.stream_handle()), "fi_gamma")
    return out


def histogram_edges(vmin, vmax, nbins, dtype):
    """The outer edges, the bin edges and the range of numpy's uniform histogram
    (``np.histogram(a, bins=nbins)`` with the range taken from the data) of an
    array of float ``dtype`` with extremes vmin, vmax: computed on numpy scalars of
    that type, as numpy does."""
    dt = np.dtype(dtype).type
    first, last = dt(vmin), dt(vmax)
    if not (np.isfinite(first) and np.isfinite(last)):
        raise ValueError(f"autodetected range of [{first}, {last}] is not finite")
    if first == last:
        first = first - 0.5
        last = last + 0.5
    bin_type = np.result_type(first, last, np.dtype(dtype))
    edges = np.linspace(first, last, nbins + 1, endpoint=True, dtype=bin_type)
    denom = np.subtract(last, first, dtype=bin_type)
    return first, edges, denom


@_per_image
def equalize_hist_global(img, nbins=256):
    """Histogram equalisation (_toolbox_py.py:357-379; scikit-image's
    exposure.equalize_hist): the cumulative distribution of the image's histogram
    (one bin per integer value for integer images, ``nbins`` uniform bins for float
    images) interpolated at every pixel; float64 (float32 for float32 images); per
    image for a stack."""
    x, single = _stack(img)
    outs = [_equalize_one(x[i], nbins) for i in range(x.shape[0])]
    return outs[0] if single else _torch().stack(outs)


def _equalize_one(img, nbins):
    torch = _torch()
    lib = L.load()
    x = img.contiguous()
    dtype = _dtype_of(x)
    dev = x.device
    s = L.stream_handle()
    if dtype.kind in "ui":
        nb = 256 if dtype == np.uint8 else 65536
        hist = torch.empty(nb, dtype=torch.int32, device=dev)
        cdf = torch.empty(nb, dtype=torch.float64, device=dev)
        out = torch.empty(tuple(x.shape), dtype=torch.float64, device=dev)
        L.check(lib.fi_equalize_hist_int(L.ptr(x), _DT[dtype], x.numel(), L.ptr(hist), L.ptr(cdf),
                                         L.ptr(out), s), "fi_equalize_hist_int")
        return out
    part = _extremes(x).cpu().numpy()
    vmin, vmax = part[:_NPARTS].min(), part[_NPARTS:].max()
    if np.isnan(part).any():
        vmin = vmax = np.nan
    first, edges, denom = histogram_edges(vmin, vmax, int(nbins), dtype)
    centers = ((edges[:-1] + edges[1:]) / 2.0).astype(np.float64)
    d_edges = torch.as_tensor(edges, device=dev)
    d_centers = torch.as_tensor(centers, device=dev)
    hist = torch.empty(int(nbins), dtype=torch.int32, device=dev)
    cdf = torch.empty(int(nbins), dtype=torch.float64, device=dev)
    out = _empty(tuple(x.shape), dtype, dev)
    L.check(lib.fi_equalize_hist_float(L.ptr(x), _DT[dtype], x.numel(), L.ptr(d_edges), int(nbins),
                                       float(first), float(denom), L.ptr(d_centers), L.ptr(hist),
                                       L.ptr(cdf), L.ptr(out), s), "fi_equalize_hist_float")
    return out


def _gauss_weights(sigma, truncate=4.0):
    """scipy.ndimage's ``_gaussian_kernel1d`` (order 0, ndimage/_filters.py), reversed
    for the correlation as ``gaussian_filter1d`` does, and its radius."""
    radius = int(truncate * float(sigma) + 0.5)
    sigma2 = float(sigma) * float(sigma)
    x = np.arange(-radius, radius + 1)
    phi = np.exp(-0.5 / sigma2 * x ** 2)
    phi = phi / phi.sum()
    return np.ascontiguousarray(phi[::-1]), radius


def gaussian_filter(img, sigma):
    """scipy.ndimage.gaussian_filter(img, sigma) of each image of a stack (or of one
    image): axis y then x, 'reflect', truncate 4, the image dtype after each axis."""
    torch = _torch()
    x, single = _stack(img)
    x = x.contiguous()
    nt, ny, nx = x.shape
    w, radius = _gauss_weights(sigma)
    wd = torch.from_numpy(w).to(x.device)
    out = torch.empty_like(x)
    tmp = torch.empty_like(x)
    L.check(L.load().fi_gaussian_filter(L.ptr(x), L.ptr(out), L.ptr(tmp), _DT[_dtype_of(x)],
                                        nt, ny, nx, L.ptr(wd), radius, L.stream_handle()),
            "fi_gaussian_filter")
    return out[0] if single else out


def _as_float(x, ft):
    """A device image as float32 / float64 (uint16 travels as int16 storage)."""
    torch = _torch()
    if x.dtype == torch.int16:
        return (x.to(torch.int32) & 0xFFFF).to(ft)
    return x.to(ft)


@_per_image
def adaptive_threshold(img, window_size=5, offset=0):
    """The local threshold image of a gaussian-weighted neighbourhood
    (_toolbox_py.py:292-308; scikit-image's filters.threshold_local with method
    'gaussian'): the image as float64 (float32 images stay float32), scipy's
    gaussian filter with sigma = (window_size - 1) / 6 and 'reflect' borders,
    minus offset."""
    torch = _torch()
    if int(window_size) != window_size or int(window_size) % 2 == 0:
        raise ValueError(f"block_size must be odd! Given block_size {window_size} is even.")
    ft = torch.float32 if _dtype_of(img) == np.float32 else torch.float64
    x = _as_float(img.contiguous(), ft)
    sigma = (int(window_size) - 1) / 6.0
    out = gaussian_filter(x, sigma) if sigma > 1e-15 else x.clone()
    return out - offset


@_per_image
def sharpen(img, sigma1=3.0, sigma2=1.0, alpha=30.0):
    """_toolbox_py.py:472-490: two chained gaussian filters in the image dtype, then
    ``blurred + alpha * (blurred - filter_blurred)`` with numpy's promotions (integer
    images: the difference wraps in their type, the result is float64)."""
    blurred = gaussian_filter(img, sigma1)
    filtered = gaussian_filter(blurred, sigma2)
    dtype = _dtype_of(blurred)
    out_dt = np.dtype(np.float32) if dtype == np.float32 else np.dtype(np.float64)
    out = _empty(tuple(blurred.shape), out_dt, blurred.device)
    L.check(L.load().fi_sharpen_combine(L.ptr(blurred), L.ptr(filtered), _DT[dtype],
                                        blurred.numel(), float(alpha), L.ptr(out),
                                        L.stream_handle()), "fi_sharpen_combine")
    return out


#: grey levels of scikit-image's CLAHE (2^14)
NR_OF_GRAY = 2 ** 14


def _host_extremes(x):
    """(min, max) of a device image as Python floats (upstream's ``img.min()``,
    ``img.max()`` passed on as an output range)."""
    part = _extremes(x).cpu().numpy()
    return float(part[:_NPARTS].min()), float(part[_NPARTS:].max())


def _kernel_size(window_shape, shape):
    """``kernel_size`` as scikit-image's equalize_adapthist takes it: None gives
    1/8 of each dimension (at least 1), a number is used for both dimensions."""
    if window_shape is None:
        return tuple(max(s // 8, 1) for s in shape)
    if np.isscalar(window_shape):
        return (int(window_shape),) * 2
    if len(window_shape) != 2:
        raise ValueError(f"Incorrect value of `kernel_size`: {window_shape}")
    return tuple(int(k) for k in window_shape)


@_per_image
def equalize_hist_adapt(img, window_shape=(10, 10), nbins=256):
    """Contrast-limited adaptive histogram equalisation (_toolbox_py.py:383-409;
    scikit-image 0.24's exposure.equalize_adapthist with kernel_size=window_shape,
    clip_limit 0.01): the image rescaled to [0, 1], then to grey levels
    [0, 2^14 - 1] (truncated), ``fi_clahe``, rescaled to [0, 1] and back to the
    image's [min, max]; float32 for float32 images, float64 otherwise; per image
    for a stack."""
    x, single = _stack(img)
    outs = [_clahe_one(x[i], window_shape, nbins) for i in range(x.shape[0])]
    return outs[0] if single else _torch().stack(outs)


def _clahe_one(img, window_shape, nbins):
    torch = _torch()
    x = img.contiguous()
    ny, nx = x.shape
    k0, k1 = _kernel_size(window_shape, (ny, nx))
    if k0 < 1 or k1 < 1:
        raise ValueError(f"Incorrect value of `kernel_size`: {window_shape}")
    lo, hi = _host_extremes(x)
    levels = _rescale_one(_rescale_one(x, 0, 1), 0, NR_OF_GRAY - 1)
    m0, m1 = -(-ny // k0), -(-nx // k1)
    maps = torch.empty(m0 * m1 * int(nbins), dtype=torch.int16, device=x.device)
    eq = torch.empty_like(levels)
    L.check(L.load().fi_clahe(L.ptr(levels), _DT[_dtype_of(levels)], ny, nx, k0, k1, int(nbins),
                              0.01, L.ptr(maps), L.ptr(eq), L.stream_handle()), "fi_clahe")
    return _rescale_one(_rescale_one(eq, 0, 1), lo, hi)


@_per_image
def equalize_hist_local(img, radius=10):
    """Local histogram equalisation over a disk (_toolbox_py.py:412-438;
    scikit-image's filters.rank.equalize with morphology.disk(radius)): the image
    rescaled to [0, 1], to uint8 (img_as_ubyte), the rank equalisation
    (``fi_rank_equalize``), rescaled to the image's [min, max] (float64); per image
    for a stack."""
    x, single = _stack(img)
    outs = [_local_one(x[i], radius) for i in range(x.shape[0])]
    return outs[0] if single else _torch().stack(outs)


def _local_one(img, radius):
    torch = _torch()
    if int(radius) != radius or radius < 0:
        raise ValueError(f"radius must be a non-negative integer, not {radius!r}")
    x = img.contiguous()
    ny, nx = x.shape
    lo, hi = _host_extremes(x)
    unit = _rescale_one(x, 0, 1)
    lib, s = L.load(), L.stream_handle()
    u8 = torch.empty((ny, nx), dtype=torch.uint8, device=x.device)
    L.check(lib.fi_to_ubyte(L.ptr(unit), _DT[_dtype_of(unit)], unit.numel(), L.ptr(u8), s),
            "fi_to_ubyte")
    eq = torch.empty_like(u8)
    L.check(lib.fi_rank_equalize(L.ptr(u8), ny, nx, int(radius), L.ptr(eq), s),
            "fi_rank_equalize")
    return _rescale_one(eq, lo, hi)


TOOLS = {
    "sliding_median": sliding_median,
    "sliding_minima": sliding_minima,
    "sliding_percentile": sliding_percentile,
    "temporal_median": temporal_median,
    "temporal_minima": temporal_minima,
    "temporal_percentile": temporal_percentile,
    "global_threshold": global_threshold,
    "rescale_intensity_tanh": rescale_intensity_tanh,
    "rescale_intensity": rescale_intensity,
    "gamma_correction": gamma_correction,
    "adaptive_threshold": adaptive_threshold,
    "equalize_hist_global": equalize_hist_global,
    "equalize_hist_adapt": equalize_hist_adapt,
    "equalize_hist_local": equalize_hist_local,
    "sharpen": sharpen,
}
assert set(TOOLS) == set(AVAILABLE_TOOLS)


class PreprocToolsGB300:
    """``PreprocToolsPy`` on the GPU (works/preproc/toolbox.py:24-120)."""

    @classmethod
    def create_default_params(cls, params):
        tools = params._set_child("tools", {"available_tools": AVAILABLE_TOOLS,
                                            "sequence": None})
        for name in AVAILABLE_TOOLS:
            attribs = dict(TOOL_DEFAULTS[name])
            attribs["enable"] = False
            tools._set_child(name, attribs=attribs)
        return params

    def __init__(self, params):
        self.params = params.tools

    def apply(self, img):
        """Apply the enabled tools, in ``sequence`` order (or the tool list order)."""
        sequence = self.params.sequence
        if sequence is None:
            sequence = self.params.available_tools
        for name in sequence:
            p = getattr(self.params, name)
            if not p.enable:
                continue
            kwargs = {k: getattr(p, k) for k in TOOL_DEFAULTS[name]}
            img = TOOLS[name](img, **kwargs)
        return img


class PreprocResults:
    """Results of one series: ``data`` maps image names to arrays
    (data_objects/preproc.py)."""

    def __init__(self, params=None):
        self.params = params
        self.data = {}


class WorkPreproc:
    """``WorkPreproc`` on the GPU (works/preproc/__init__.py:62-137)."""

    @classmethod
    def create_default_params(cls, backend="gb300"):
        params = ParamContainer(tag="params")
        params._set_attrib("backend", backend)
        PreprocToolsGB300.create_default_params(params)
        return params

    def __init__(self, params=None, device=None):
        if params is None:
            params = type(self).create_default_params()
        self.params = params
        self.device = device
        self.tools = PreprocToolsGB300(params)

    def calcul_device(self, images):
        """Apply the tools to a device stack (nt, ny, nx) or image; returns a tensor."""
        return self.tools.apply(images)

    def calcul(self, serie):
        """``serie``: dict with ``arrays`` (a sequence of images) and ``names``."""
        arrays = serie["arrays"] if isinstance(serie, dict) else serie.get_arrays()
        names = serie["names"] if isinstance(serie, dict) else serie.names
        images = to_device(np.array(arrays), self.device)
        out = to_host(self.calcul_device(images))
        result = PreprocResults(self.params)
        result.data.update(dict(zip(names, out)))
        return result


Work = WorkPreproc
