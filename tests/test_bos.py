"""WorkBOS (works/bos.py:19-91): PIV of each image against the reference image."""

import numpy as np
import pytest

from fluidimage_gb300 import WorkBOS, WorkPIV, workloads


def _images():
    (im0, im1), _ = workloads.config2_images(shape=(256, 256))
    return {"img_a.png": im0, "img_b.png": im1, "img_c.png": np.roll(im1, 3, axis=0)}


def test_params_and_reference():
    params = WorkBOS.create_default_params()
    assert params.reference == 0
    assert params.images.path == ""
    assert params.piv0.method_correl == "gb300"
    imgs = _images()
    work = WorkBOS(params, images=imgs)
    assert work.name_reference == "img_a.png"
    params.reference = "img_b.png"
    work = WorkBOS(params, images=imgs)
    assert work.name_reference == "img_b.png"
    assert work.image_reference is imgs["img_b.png"]
    params.reference = "missing.png"
    with pytest.raises(ValueError):
        WorkBOS(params, images=imgs)
    arr, name = WorkBOS(WorkBOS.create_default_params(), images=imgs).get_tuple_image_name(1)
    assert name == "img_b.png" and arr is imgs["img_b.png"]


@pytest.mark.gpu
def test_bos_matches_piv():
    imgs = _images()
    params = WorkBOS.create_default_params()
    params.piv0.shape_crop_im0 = 32
    params.multipass.number = 2
    params.multipass.use_tps = True
    params.multipass.smoothing_coef = 0.5
    work = WorkBOS(params, images=imgs)
    piv = WorkPIV(params)
    ref = imgs["img_a.png"]
    singles = {}
    for name in ("img_b.png", "img_c.png"):
        res = work.calcul((imgs[name], name))
        exp = piv.calcul({"arrays": (ref, imgs[name]), "names": ("img_a.png", name)})
        for pa, pb in zip(res.passes, exp.passes):
            np.testing.assert_array_equal(pa.deltaxs, pb.deltaxs)
            np.testing.assert_array_equal(pa.deltays, pb.deltays)
            assert pa.errors == pb.errors
        assert res.passes[-1].couple.name == name
        singles[name] = res
    series = list(work.calcul_series())
    assert len(series) == 3
    for res, name in zip(series[1:], ("img_b.png", "img_c.png")):
        np.testing.assert_array_equal(res.passes[-1].deltaxs_final,
                                      singles[name].passes[-1].deltaxs_final)
