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
    assert got.dtype == (torch.uint8 if expected.dtype == np.uint8 else torch.int16)
    assert np.array_equal(got.cpu().numpy().view(expected.dtype), expected)


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
    assert np.array_equal(got.cpu().numpy().view(np.uint16), img)


def test_decoded_frames_feed_the_pipeline(tmp_path):
    """imread_device output goes straight into WorkPIV.calcul_device: the same field
    as the host images through WorkPIV.calcul."""
    import torch

    from fluidimage_gb300 import WorkPIV, synthetic
    from fluidimage_gb300.images import imread_device

    model = synthetic.ParticleModel(density=0.05, noise=20.0, dtype="uint16")
    im0, im1 = synthetic.make_pair((256, 320), synthetic.uniform_shift(2.3, -1.4), model,
                                   seed=4)
    p0, p1 = tmp_path / "a.tif", tmp_path / "b.tif"
    p0.write_bytes(tiff_bytes(im0, rows_per_strip=16))
    p1.write_bytes(tiff_bytes(im1, big_endian=True))
    params = WorkPIV.create_default_params()
    params.piv0.shape_crop_im0 = 32
    params.multipass.number = 2
    work = WorkPIV(params, device="cuda:0")
    ref = work.calcul({"arrays": (im0, im1), "names": ("a", "b")})
    outs = work.calcul_device(imread_device(p0, "cuda:0"), imread_device(p1, "cuda:0"))
    torch.cuda.synchronize()
    got = work.results_to_host(outs, None)
    for k in range(2):
        np.testing.assert_array_equal(got.passes[k].deltaxs, ref.passes[k].deltaxs)
        np.testing.assert_array_equal(got.passes[k].deltays, ref.passes[k].deltays)
