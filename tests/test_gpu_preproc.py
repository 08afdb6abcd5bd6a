"""GPU preprocessing tools against the fixture recorded from the upstream tools.

Rank filters, the weighted subtraction, the clamp and sharpen's gaussian filters
are exact (integer keys and the same float arithmetic in the same order); rescale_intensity_tanh floors float64 values computed
with CUDA's tanh, which may differ from numpy's by one ulp, so at most 0.1 % of the
pixels may differ by one count.
"""

import json

import numpy as np
import pytest

import goldens

pytestmark = pytest.mark.gpu

Z = goldens.load("preproc")
CASES = sorted(k[len("args_"):] for k in Z.files if k.startswith("args_"))


@pytest.mark.parametrize("name", CASES)
def test_gpu_tool_matches_upstream(name):
    from fluidimage_gb300 import preproc as P

    a = json.loads(str(Z["args_" + name]))
    img = Z["img_" + a["image"]]
    got = P.to_host(getattr(P, a["function"])(P.to_device(img), **a["kwargs"]))
    want = Z["out_" + name]
    assert got.dtype == want.dtype, (got.dtype, want.dtype)
    if a["function"] == "rescale_intensity_tanh":
        diff = np.abs(got - want)
        assert diff.max() <= 1.0
        assert np.count_nonzero(diff) <= 1e-3 * diff.size
    else:
        np.testing.assert_array_equal(got, want)


def test_single_image_keeps_the_tool_dtype():
    """A 2-D image gives the tool's own dtype (upstream calls the tool directly)."""
    from fluidimage_gb300 import preproc as P
    from oracle import preproc as O

    img = Z["img_u8"][0]
    for fn, kw in (("sliding_minima", dict(window_size=5)),
                   ("global_threshold", dict(minima=20, maxima=180)),
                   ("sliding_median", dict(window_size=3, weight=1))):
        got = P.to_host(getattr(P, fn)(P.to_device(img), **kw))
        want = getattr(O, fn)(img.copy(), **kw)
        assert got.dtype == want.dtype
        np.testing.assert_array_equal(got, want)


def test_work_preproc_sequence():
    """WorkPreproc with two enabled tools in a given sequence, like upstream's
    PreprocToolsBase.apply (works/preproc/toolbox.py:90-115)."""
    from fluidimage_gb300.preproc import WorkPreproc
    from oracle import preproc as O

    params = WorkPreproc.create_default_params()
    params.tools.sequence = ["sliding_minima", "global_threshold"]
    params.tools.sliding_minima.enable = True
    params.tools.sliding_minima.window_size = 7
    params.tools.global_threshold.enable = True
    params.tools.global_threshold.minima = 5
    params.tools.global_threshold.maxima = 100
    imgs = Z["img_u16"]
    names = [f"im{i}" for i in range(len(imgs))]
    res = WorkPreproc(params).calcul({"arrays": list(imgs), "names": names})
    want = O.global_threshold(O.sliding_minima(imgs.copy(), window_size=7), minima=5,
                              maxima=100)
    got = np.array([res.data[n] for n in names])
    np.testing.assert_array_equal(got, want)


def _ulps(got, want):
    got, want = np.asarray(got), np.asarray(want)
    return np.abs(got - want) / np.spacing(np.maximum(np.abs(want), np.finfo(want.dtype).tiny))


@pytest.mark.parametrize("image", ["u8", "u16", "f32", "f64"])
@pytest.mark.parametrize("lo_hi", [(0.0, 4096.0), (-1.0, 1.0), (0.0, 65535.0)])
def test_rescale_intensity_matches_oracle(image, lo_hi):
    """rescale_intensity: the same IEEE operations in the same order as numpy, so the
    float64 and float32 results are equal to the oracle's."""
    from fluidimage_gb300 import preproc as P
    from oracle import preproc as O

    img = Z["img_f32"].astype(np.float64) * 1.37 if image == "f64" else Z["img_" + image]
    got = P.to_host(P.rescale_intensity(P.to_device(img), *lo_hi))
    want = O.rescale_intensity(img.copy(), *lo_hi)
    assert got.dtype == want.dtype
    np.testing.assert_array_equal(got, want)
    one = P.to_host(P.rescale_intensity(P.to_device(img[0]), *lo_hi))
    want1 = O.rescale_intensity(img[0].copy(), *lo_hi)
    assert one.dtype == want1.dtype
    np.testing.assert_array_equal(one, want1)


@pytest.mark.parametrize("image", ["u8", "u16", "f32", "f64"])
@pytest.mark.parametrize("gamma_gain", [(1.0, 1.0), (0.5, 1.0), (2.0, 0.8), (0.7, 1.0),
                                        (1.8, 1.3)])
def test_gamma_correction_matches_oracle(image, gamma_gain):
    """gamma_correction: uint8 exact (the same table); the exponents 0.5, 1 and 2 exact
    (numpy's sqrt, copy and product); other exponents through CUDA's pow, within
    2 ulps of the libm power for floats, and for uint16 equal except where the
    oracle's value before truncation lies within 1e-12 relative of an integer."""
    from fluidimage_gb300 import preproc as P
    from oracle import preproc as O

    gamma, gain = gamma_gain
    if image == "f64":
        img = np.abs(Z["img_f32"].astype(np.float64)) * 1.37
    elif image == "f32":
        img = np.abs(Z["img_f32"])
    else:
        img = Z["img_" + image]
    x = img[0]
    got = P.to_host(P.gamma_correction(P.to_device(x), gamma, gain))
    want, raws = O.gamma_correction(x.copy(), gamma, gain, with_raw=True)
    assert got.dtype == want.dtype
    exact = image == "u8" or gamma in (0.5, 1.0, 2.0)
    if exact:
        np.testing.assert_array_equal(got, want)
    elif image == "u16":
        raw = raws[0]
        near = np.abs(raw - np.rint(raw)) <= 1e-12 * np.maximum(np.abs(raw), 1.0)
        bad = (got != want) & ~near
        assert not bad.any(), int(bad.sum())
        assert np.abs(got.astype(np.int64) - want.astype(np.int64)).max() <= 1
    else:
        assert _ulps(got, want).max() <= 2.0
    stack = P.to_host(P.gamma_correction(P.to_device(img), gamma, gain))
    assert stack.dtype == np.float64
    np.testing.assert_array_equal(stack[0], got.astype(np.float64))


def test_gamma_correction_rejects_negative_float_images():
    from fluidimage_gb300 import preproc as P

    img = Z["img_f32"][0].copy()
    img[3, 4] = -1.0
    with pytest.raises(ValueError):
        P.gamma_correction(P.to_device(img), 0.7)


@pytest.mark.parametrize("image", ["u8", "u16", "f32"])
@pytest.mark.parametrize("window_offset", [(5, 0), (11, 3), (31, -2.5), (1, 1)])
def test_adaptive_threshold_matches_scipy(image, window_offset):
    """adaptive_threshold: scipy's gaussian filter of the float image (float64 line
    sums, the float type after each axis), so equal to the oracle bit for bit."""
    from fluidimage_gb300 import preproc as P
    from oracle import preproc as O

    ws, off = window_offset
    img = Z["img_" + image]
    got = P.to_host(P.adaptive_threshold(P.to_device(img[0]), ws, off))
    want = O.adaptive_threshold(img[0].copy(), ws, off)
    assert got.dtype == want.dtype
    np.testing.assert_array_equal(got, want)
    stack = P.to_host(P.adaptive_threshold(P.to_device(img), ws, off))
    np.testing.assert_array_equal(stack, O.adaptive_threshold(img.copy(), ws, off))


@pytest.mark.parametrize("image", ["u8", "u16", "f32", "f64"])
@pytest.mark.parametrize("nbins", [256, 100])
def test_equalize_hist_global_matches_oracle(image, nbins):
    """equalize_hist_global: integer images exactly (the cumulative fraction at the
    pixel's value); float images with the same bins as np.histogram and np.interp
    within 2 ulps (numpy's interpolation may contract the slope form into an FMA
    on some hosts)."""
    from fluidimage_gb300 import preproc as P
    from oracle import preproc as O

    img = Z["img_f32"].astype(np.float64) * 1.37 if image == "f64" else Z["img_" + image]
    x = img[0]
    got = P.to_host(P.equalize_hist_global(P.to_device(x), nbins))
    want = O.equalize_hist_global(x.copy(), nbins)
    assert got.dtype == want.dtype
    if image in ("u8", "u16"):
        np.testing.assert_array_equal(got, want)
    else:
        assert _ulps(got, want).max() <= 2.0
    stack = P.to_host(P.equalize_hist_global(P.to_device(img), nbins))
    assert stack.dtype == np.float64
    np.testing.assert_array_equal(stack[0], got.astype(np.float64))


def _adapt_image(image, shape=None):
    img = Z["img_f32"].astype(np.float64) * 1.37 if image == "f64" else Z["img_" + image]
    if shape is not None:
        rng = np.random.default_rng(11)
        hi = {"u8": 255, "u16": 4095}.get(image, 1)
        img = rng.integers(0, hi + 1, (2,) + shape).astype(img.dtype) if image in ("u8", "u16") \
            else (rng.random((2,) + shape) * 900.0).astype(img.dtype)
    return img


@pytest.mark.parametrize("image", ["u8", "u16", "f32", "f64"])
@pytest.mark.parametrize("window_nbins", [((10, 10), 256), ((7, 12), 100), ((16, 16), 256),
                                          (5, 64), (None, 256), ((64, 80), 256)])
def test_equalize_hist_adapt_matches_oracle(image, window_nbins):
    """equalize_hist_adapt (CLAHE): the same grey levels, clipped histograms, maps and
    float32 blend as the restatement of scikit-image's algorithm, so the result is
    equal to the oracle's (regions past the image's end reflected; a kernel as large
    as the image)."""
    from fluidimage_gb300 import preproc as P
    from oracle import preproc as O

    window, nbins = window_nbins
    img = _adapt_image(image)
    x = img[0]
    got = P.to_host(P.equalize_hist_adapt(P.to_device(x), window, nbins))
    want = O.equalize_hist_adapt(x.copy(), window, nbins)
    assert got.dtype == want.dtype
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("image", ["u8", "u16", "f32"])
@pytest.mark.parametrize("shape", [(97, 131), (33, 250), (9, 9)])
def test_equalize_hist_adapt_ragged_shapes(image, shape):
    """Images that are not multiples of the kernel, and smaller than it; a stack is
    equalised image by image (float64)."""
    from fluidimage_gb300 import preproc as P
    from oracle import preproc as O

    img = _adapt_image(image, shape)
    got = P.to_host(P.equalize_hist_adapt(P.to_device(img), (10, 10), 256))
    want = O.equalize_hist_adapt(img.copy(), (10, 10), 256)
    assert got.dtype == np.float64 and want.dtype == np.float64
    np.testing.assert_array_equal(got, want)


def test_equalize_hist_adapt_flat_image():
    from fluidimage_gb300 import preproc as P
    from oracle import preproc as O

    x = np.full((40, 50), 700, np.uint16)
    got = P.to_host(P.equalize_hist_adapt(P.to_device(x)))
    np.testing.assert_array_equal(got, O.equalize_hist_adapt(x.copy()))


@pytest.mark.parametrize("image", ["u8", "u16", "f32", "f64"])
@pytest.mark.parametrize("radius", [0, 1, 4, 10])
def test_equalize_hist_local_matches_oracle(image, radius):
    """equalize_hist_local: img_as_ubyte (rint in the image's float type), the rank
    equalisation over the disk with the pixels outside the image left out, and the
    rescaling, equal to the oracle's."""
    from fluidimage_gb300 import preproc as P
    from oracle import preproc as O

    img = _adapt_image(image)
    got = P.to_host(P.equalize_hist_local(P.to_device(img[:2]), radius))
    want = O.equalize_hist_local(img[:2].copy(), radius)
    assert got.dtype == want.dtype == np.float64
    np.testing.assert_array_equal(got, want)
    one = P.to_host(P.equalize_hist_local(P.to_device(img[0]), radius))
    np.testing.assert_array_equal(one, want[0])


def test_work_preproc_adaptive_equalisations():
    from fluidimage_gb300.preproc import WorkPreproc
    from oracle import preproc as O

    params = WorkPreproc.create_default_params()
    params.tools.sequence = ["equalize_hist_adapt", "equalize_hist_local"]
    params.tools.equalize_hist_adapt.enable = True
    params.tools.equalize_hist_local.enable = True
    params.tools.equalize_hist_local.radius = 3
    imgs = Z["img_u16"][:3]
    names = [f"im{i}" for i in range(len(imgs))]
    res = WorkPreproc(params).calcul({"arrays": list(imgs), "names": names})
    want = O.equalize_hist_local(O.equalize_hist_adapt(imgs.copy()), radius=3)
    got = np.array([res.data[n] for n in names])
    np.testing.assert_array_equal(got, want)
