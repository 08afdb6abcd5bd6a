"""Image decode: the oracle and the host reader against files of known content, the
reference's image samples (when present), and the error behaviour of upstream's
imread (util/util.py:46-59)."""

import os
from pathlib import Path

import numpy as np
import pytest

from fluidimage_gb300 import images
from oracle import images as O

from imagefiles import cases, png_bytes

SAMPLES = Path(os.environ.get("FLUIDIMAGE_SAMPLES", "/root/reference/image_samples"))
SAMPLE_FILES = [
    "Oseen/Images/Oseen_center_01.tif",  # 8-bit, one strip
    "4th_PIV-Challenge_Case_E/E_Particle_Images/Camera_01/im00001.tif",  # 16-bit, 64 strips
    "TomoPIV/particle/cam0.pre/im00001a.tif",
    "Karman/Images/Karman_01.bmp",  # 8-bit palette, bottom-up, 524-px rows
    "Jet/Images/c060a.png",  # 16-bit, Sub and Average rows
    "SurfTracking/Images/image1.png",  # 8-bit, Sub, Up and Paeth rows
]


@pytest.mark.parametrize("name,data,expected", cases(), ids=[c[0] for c in cases()])
def test_oracle_and_imread_known_content(tmp_path, name, data, expected):
    path = tmp_path / f"{name}.{name.split('_')[0]}"
    path.write_bytes(data)
    ref = O.decode(path)
    assert ref.dtype == expected.dtype and np.array_equal(ref, expected)
    got = images.imread(path)
    assert got.dtype == expected.dtype and np.array_equal(got, expected)


@pytest.mark.skipif(not SAMPLES.exists(), reason="upstream image_samples not present")
@pytest.mark.parametrize("rel", SAMPLE_FILES)
def test_imread_matches_oracle_on_samples(rel):
    path = SAMPLES / rel
    ref = O.decode(path)
    got = images.imread(path)
    p = images.read_payload(path)
    assert got.shape == ref.shape == (p.height, p.width)
    assert got.dtype == ref.dtype
    assert np.array_equal(got, ref)


def test_png_unfilter_every_filter_on_wide_pixels(tmp_path):
    rng = np.random.default_rng(3)
    img = rng.integers(0, 65536, (11, 7), dtype=np.uint16)
    for filt in range(5):
        path = tmp_path / f"f{filt}.png"
        path.write_bytes(png_bytes(img, filters=(filt,)))
        assert np.array_equal(images.imread(path), img)


def test_missing_file_raises_with_the_path():
    with pytest.raises(FileNotFoundError, match="__oups__.png"):
        images.imread("__oups__.png")


def test_unsupported_and_corrupt_files(tmp_path):
    img = np.zeros((4, 4), np.uint8)
    colour = tmp_path / "rgb.png"
    colour.write_bytes(png_bytes(img, color=2))
    with pytest.raises(NotImplementedError, match="colour type 2"):
        images.imread(colour)
    bad = bytearray(png_bytes(img))
    bad[40] ^= 0xFF  # inside the first IDAT chunk
    corrupt = tmp_path / "bad.png"
    corrupt.write_bytes(bytes(bad))
    with pytest.raises(ValueError, match="CRC"):
        images.imread(corrupt)
    unknown = tmp_path / "x.raw"
    unknown.write_bytes(b"\0" * 64)
    with pytest.raises(NotImplementedError, match="not supported"):
        images.imread(unknown)


def test_truncated_files_raise_value_error(tmp_path):
    from imagefiles import bmp_bytes, tiff_bytes

    img = np.arange(64, dtype=np.uint8).reshape(8, 8)
    for name, data in (("t.tif", tiff_bytes(img)[:40]), ("t.bmp", bmp_bytes(img)[:60]),
                       ("t.png", png_bytes(img)[:45])):
        path = tmp_path / name
        path.write_bytes(data)
        with pytest.raises(ValueError):
            images.imread(path)
