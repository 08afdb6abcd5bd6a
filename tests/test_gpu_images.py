"""Image decode into HBM (fi_image_unpack) against files of known content and the
CPU oracle."""

import numpy as np
import pytest

from imagefiles import cases, tiff_bytes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,data,expected", cases(), ids=[c[0] for c in cases()])
def test_imread_device_known_content(tmp_path, name, data, expected):
    import torch

    from fluidimage_gb300 import images

    path = tmp_path / f"{name}.{name.split('_')[0]}"
    path.write_bytes(data)
    got = images.imread_device(path, "cuda:0")
    assert got.device.type == "cuda" and got.shape == expected.shape
    want = torch.from_numpy(expected.astype(np.int32))
    assert torch.equal(got.cpu().to(torch.int32), want)


def test_imread_device_full_size_frame(tmp_path):
    """A 2048 x 2048 16-bit big-endian frame in 37-row strips, as a camera writes it."""
    import torch

    from fluidimage_gb300 import images
    from oracle import images as O

    rng = np.random.default_rng(12)
    img = rng.integers(0, 4096, (2048, 2048), dtype=np.uint16)
    path = tmp_path / "frame.tif"
    path.write_bytes(tiff_bytes(img, big_endian=True, rows_per_strip=37))
    assert np.array_equal(O.decode(path), img)
    got = images.imread_device(path, "cuda:0")
    assert torch.equal(got.cpu().to(torch.int32), torch.from_numpy(img.astype(np.int32)))
