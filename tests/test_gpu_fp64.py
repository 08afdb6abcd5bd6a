"""GPU results against the FP64 oracle (complex128 FFTs, float64 planes and fit).

The bar: displacements within 0.005 px of the FP64 oracle, outside near-ties and
windows cut at a different integer shift (both counted and printed); the final
interpolated field within 0.005 px; correlation planes within 2e-6 relative to
each plane's maximum (FP32 FFTs of mean-removed, power-of-two-scaled windows).
"""

import pytest

pytestmark = pytest.mark.gpu

TOL_PX = 5e-3
TOL_PLANE = 2e-6


def _run(work, im0, im1):
    import torch

    res = work.calcul({"arrays": (im0, im1), "names": ("im0", "im1")})
    torch.cuda.synchronize()
    return res


def test_config1_vs_fp64():
    from fluidimage_gb300 import WorkPIV, workloads
    from oracle import accuracy as A

    (im0, im1), _ = workloads.config1_images()
    params = workloads.config1_params(WorkPIV.create_default_params())
    res = _run(WorkPIV(params, keep_correls=True), im0, im1)
    ref = A.fp64_multipass(im0, im1, params, keep_planes=True)
    acc = A.summary(res.passes, ref)
    planes = A.plane_relative_error(res.passes[0].correls, ref[0].planes)
    print("config1 vs FP64:", acc, "planes:", planes)
    assert acc["compared"] > 900
    assert acc["max_px"] <= TOL_PX
    _check_final(acc)
    assert planes["max"] <= TOL_PLANE


def test_config2_vs_fp64():
    """The timed workload (2048^2, 3 passes, WorkFIX, TPS) against the FP64 oracle."""
    from fluidimage_gb300 import WorkPIV, workloads
    from oracle import accuracy as A

    (im0, im1), _ = workloads.config2_images(pair=0)
    params = workloads.config2_params(WorkPIV.create_default_params())
    res = _run(WorkPIV(params), im0, im1)
    ref = A.fp64_multipass(im0, im1, params)
    acc = A.summary(res.passes, ref)
    print("config2 vs FP64:", acc)
    assert acc["compared"] > 0.95 * res.passes[-1].deltaxs.size
    for p in acc["passes"]:
        assert p["max_px"] <= TOL_PX
    _check_final(acc)


def _check_final(acc):
    """The final field blends every kept vector of the last pass: exact to the bar
    when no vector was left out; otherwise a near-tie that took another peak moves
    the field near it, so the RMS is checked and the maximum printed."""
    excluded = sum(p["near_ties"] + p["other_shift"] for p in acc["passes"])
    if excluded == 0:
        assert acc["final_field_max_px"] <= TOL_PX
    else:
        assert acc["final_field_rms_px"] <= TOL_PX
