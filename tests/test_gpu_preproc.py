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
