"""The preprocessing oracle against the fixture recorded from the upstream tools
(bit for bit: same scipy.ndimage filters, same numpy arithmetic)."""

import json

import numpy as np
import pytest

import goldens
from oracle import preproc as O

Z = goldens.load("preproc")
CASES = sorted(k[len("args_"):] for k in Z.files if k.startswith("args_"))


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_upstream_tools(name):
    a = json.loads(str(Z["args_" + name]))
    img = Z["img_" + a["image"]]
    got = getattr(O, a["function"])(img.copy(), **a["kwargs"])
    want = Z["out_" + name]
    assert got.dtype == want.dtype
    np.testing.assert_array_equal(got, want)


def test_rescale_intensity_known_answers():
    """scikit-image's rescale_intensity(in_range='image', out_range=(lo, hi)) by its
    definition: the image's extremes go to lo and hi, linearly in between; float64
    for integer images, float32 for float32 images; a flat image is clipped."""
    a = np.array([[10, 20], [30, 50]], np.uint16)
    got = O.rescale_intensity(a, 0.0, 4.0)
    assert got.dtype == np.float64
    np.testing.assert_array_equal(got, [[0.0, 1.0], [2.0, 4.0]])
    f = np.array([[-1.0, 0.0, 3.0]], np.float32)
    got = O.rescale_intensity(f, 0.0, 8.0)
    assert got.dtype == np.float32
    np.testing.assert_array_equal(got, np.array([[0.0, 2.0, 8.0]], np.float32))
    flat = np.full((2, 3), 7, np.uint8)
    np.testing.assert_array_equal(O.rescale_intensity(flat, 0.0, 5.0), np.full((2, 3), 5.0))
    stack = np.stack([a, 2 * a])  # per image: both map to the same values
    got = O.rescale_intensity(stack, 0.0, 4.0)
    np.testing.assert_array_equal(got[0], got[1])


def test_gamma_correction_known_answers():
    """adjust_gamma by its definition: gain * (x / range) ** gamma * range, in the
    image dtype; uint8 through the rounded 256-entry table."""
    u8 = np.array([[0, 255, 128, 64]], np.uint8)
    got = O.gamma_correction(u8, 0.5, 1.0)
    want = np.minimum(np.rint(255 * np.sqrt(u8 / 255.0)), 255).astype(np.uint8)
    np.testing.assert_array_equal(got, want)
    assert got.dtype == np.uint8
    u16 = np.array([[0, 65535, 32768]], np.uint16)
    got = O.gamma_correction(u16, 2.0, 1.0)
    assert got.dtype == np.uint16
    assert got[0, 0] == 0 and got[0, 1] == 65535
    assert got[0, 2] == int(32768.0 ** 2 / 65535.0)
    f = np.array([[0.25, 1.0, 4.0]], np.float32)
    np.testing.assert_array_equal(O.gamma_correction(f, 2.0, 0.5),
                                  np.array([[0.03125, 0.5, 8.0]], np.float32))
    with pytest.raises(ValueError):
        O.gamma_correction(np.array([[-1.0]], np.float32))
    with pytest.raises(ValueError):
        O.gamma_correction(u8, -1.0)


def test_adaptive_threshold_definition():
    """threshold_local's gaussian method: a constant image is its own threshold (minus
    the offset); the weights sum to one; even windows are rejected."""
    flat = np.full((9, 11), 7, np.uint16)
    got = O.adaptive_threshold(flat, 5, 2)
    assert got.dtype == np.float64
    np.testing.assert_allclose(got, 5.0, rtol=0, atol=1e-12)
    f = np.full((9, 11), 3.0, np.float32)
    assert O.adaptive_threshold(f, 7, 0).dtype == np.float32
    with pytest.raises(ValueError):
        O.adaptive_threshold(flat, 4)


def test_equalize_hist_known_answers():
    """equalize_hist by its definition: integer images, one bin per value and the
    cumulative fraction of pixels at or below each pixel's value; float images, a
    uniform histogram over [min, max] interpolated at the bin centres."""
    a = np.array([[1, 2], [2, 5]], np.uint8)
    got = O.equalize_hist_global(a)
    assert got.dtype == np.float64
    np.testing.assert_array_equal(got, [[0.25, 0.75], [0.75, 1.0]])
    f = np.array([[0.0, 1.0], [1.0, 3.0]], np.float32)
    got = O.equalize_hist_global(f, nbins=3)
    assert got.dtype == np.float32
    np.testing.assert_array_equal(got, np.array([[0.25, 0.5], [0.5, 1.0]], np.float32))


def test_histogram_edges_follow_numpy():
    """The host computation of numpy's histogram edges (used by the device
    equalisation) equals np.histogram_bin_edges, flat images included."""
    from fluidimage_gb300.preproc import histogram_edges

    rng = np.random.default_rng(5)
    for dt in (np.float32, np.float64):
        for arr in (rng.random((7, 9)).astype(dt) * 3.7 - 1.1, np.full((3, 4), 2.5, dt)):
            for nb in (1, 7, 256):
                first, edges, denom = histogram_edges(arr.min(), arr.max(), nb, dt)
                want = np.histogram_bin_edges(arr, bins=nb)
                assert edges.dtype == want.dtype
                np.testing.assert_array_equal(edges, want)
                assert first == want[0]


def test_clip_histogram_known_answers():
    """Hand-traced cases of the contrast limiting: no increment (the remaining excess
    handed out in strides, overshooting by 2), a per-bin increment, and bins filled
    to the limit (the excess goes negative: no redistribution)."""
    from oracle import preproc as O

    np.testing.assert_array_equal(O.clip_histogram([5, 0, 0, 3, 0, 0, 0, 1], 2),
                                  [2, 1, 1, 2, 1, 1, 1, 2])
    np.testing.assert_array_equal(O.clip_histogram([10, 0, 0, 0], 4), [4, 2, 2, 2])
    np.testing.assert_array_equal(O.clip_histogram([20, 3, 2, 0, 0, 0, 0, 0], 4), [4] * 8)
    np.testing.assert_array_equal(O.clip_histogram([1, 2, 0], 5), [1, 2, 0])


def test_clahe_levels_flat_regions():
    """One grey level everywhere: each region's clipped histogram is [1, 1, 1, 1]
    (limit 1 for 2 x 2 regions), the map of bin 0 is floor(16383 / 4) and the blend
    weights sum to 1 exactly."""
    from oracle import preproc as O

    out = O.clahe_levels(np.zeros((4, 6), np.uint16), (2, 2), 4)
    np.testing.assert_array_equal(out, np.full((4, 6), 4095, np.uint16))


def test_rank_equalize_known_answer():
    from oracle import preproc as O

    u8 = np.array([[10, 20, 30], [40, 50, 60], [70, 80, 90]], np.uint8)
    out = O.rank_equalize(u8, O.disk(1))
    # (0, 0): 10, 20, 40 -> 1 of 3; (0, 1): 10, 20, 30, 50 -> 2 of 4; (1, 1): 5 of 5 -> 3
    assert out[0, 0] == 255 // 3 and out[0, 1] == 127 and out[1, 1] == 153
    assert out[2, 2] == 255
    np.testing.assert_array_equal(O.disk(1), [[0, 1, 0], [1, 1, 1], [0, 1, 0]])
    assert O.disk(10).sum() == 317


def test_to_ubyte_rounds_half_to_even():
    from oracle import preproc as O

    y = np.array([0.0, 1.0, 127.5 / 255, 0.5 / 255], np.float64)
    np.testing.assert_array_equal(O.to_ubyte(y), np.rint(y * 255).astype(np.uint8))
    assert O.to_ubyte(np.array([1.0], np.float32))[0] == 255
