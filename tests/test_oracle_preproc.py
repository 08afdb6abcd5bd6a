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
